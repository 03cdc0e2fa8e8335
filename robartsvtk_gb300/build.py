"""Builds libhmf_gb300.so in-tree (robartsvtk_gb300/_build/) for sm_103a.

Eight translation units (the solver, its out-of-core driver, its FP64
evaluation, its adjoint and its schedules, the vote and energy, the
data-term producers, the C++ facade), compiled
in parallel with nvcc and linked into one shared library that exports the C
ABI of include/hmf.h and the C++ facade of csrc/hmf_segmentation.hpp.  The
kernel units are compiled with -fmad=false so the FP32 arithmetic follows the
reference kernels' operation order exactly.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(OUT_DIR, "libhmf_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fno-fast-math"]

UNITS = {
    "hmf_capi.o": ("hmf_capi.cu", ["-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false"]),
    "hmf_adjoint.o": ("hmf_adjoint.cu", ["-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false"]),
    "hmf_fp64.o": ("hmf_fp64.cu", ["-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false"]),
    "hmf_post.o": ("hmf_post.cu", ["-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false"]),
    "hmf_dataterm.o": ("hmf_dataterm.cu", ["-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
                                           "-Xcompiler", "-ffp-contract=off"]),
    "hmf_paged.o": ("hmf_paged.cu", []),
    "hmf_segmentation.o": ("hmf_segmentation.cpp", ["-x", "cu"]),
    "hmf_schedule.o": ("hmf_schedule.cpp", []),
}


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libhmf_gb300.so")
    return path


def _deps() -> list[str]:
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(INCLUDE, "hmf.h"))
    return [f for f in files if os.path.isfile(f)]


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd: list[str]) -> None:
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), p.stdout, p.stderr))


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    """Compile (if stale) and return the path of libhmf_gb300.so."""
    deps = _deps()
    if not force and not _stale(LIB_PATH, deps):
        return LIB_PATH
    os.makedirs(OUT_DIR, exist_ok=True)
    cc = nvcc()

    def compile_unit(item):
        obj, (src, extra) = item
        cmd = [cc, *NVCC_COMMON, *ARCH, *extra, "-c", os.path.join(CSRC, src),
               "-o", os.path.join(OUT_DIR, obj)]
        if verbose_ptxas and src.endswith(".cu"):
            cmd.insert(1, "-Xptxas=-v")
        _run(cmd)

    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        list(ex.map(compile_unit, UNITS.items()))
    tmp = LIB_PATH + ".tmp"
    _run([cc, "-shared", *ARCH, "-Xcompiler", "-fPIC", *[os.path.join(OUT_DIR, o) for o in UNITS],
          "-o", tmp])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force=True, verbose_ptxas=True))
