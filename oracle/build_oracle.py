"""Build recipe for the oracle (test infrastructure only).

Outputs (all git-ignored):
  oracle/_build/liboracle.so   -- the CPU restatements in hmf_oracle.cpp
                                  (REF_CUDA in FP32/FP64 and the REF_CPU port)
                                  and dag_oracle.cpp (the DAG solver).
  oracle/_ref/libhmf_ref_cpu.so -- only where the reference sources exist:
                                  the same REF_CPU driver linked against the
                                  reference's own, unmodified
                                  Common/vtkRobartsCommon/vtkMaxFlowSegmentationUtilities.cxx,
                                  compiled in place from the reference tree.
  oracle/_ref/hmf_ref_kernels.cubin -- only where the reference sources exist:
                                  the reference's own CUDA kernels
                                  (CUDA_hierarchicalmaxflow.cu + CUDA_commonKernels.cu)
                                  compiled for sm_103a, loaded by
                                  oracle/ref_kernels.py to produce golden vectors.

The reference needs VTK for its classes, which is absent; the two arithmetic
files above compile on their own given empty export-macro headers, which this
script writes into oracle/_ref/include/ (generated one-line stubs, not
reference sources).  Nothing here runs the reference's CMake build.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF_OUT = os.path.join(HERE, "_ref")
REFERENCE_ROOT = os.environ.get("HMF_REFERENCE_ROOT", "/root/reference")

CXXFLAGS = ["-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp",
            "-ffp-contract=off", "-fno-fast-math"]


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError("command failed: %s\n%s%s" % (" ".join(cmd), proc.stdout, proc.stderr))


def _newer(target: str, sources: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(s) <= t for s in sources if os.path.exists(s))


def build_port(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = [os.path.join(HERE, "hmf_oracle.cpp"), os.path.join(HERE, "dag_oracle.cpp")]
    out = os.path.join(BUILD, "liboracle.so")
    if force or not _newer(out, srcs):
        _run(["g++", *CXXFLAGS, *srcs, "-o", out + ".tmp"])
        os.replace(out + ".tmp", out)
    return out


def reference_available() -> bool:
    return os.path.isfile(os.path.join(
        REFERENCE_ROOT, "Common/vtkRobartsCommon/vtkMaxFlowSegmentationUtilities.cxx"))


def _write_stubs() -> str:
    inc = os.path.join(REF_OUT, "include")
    os.makedirs(inc, exist_ok=True)
    for name, macro in (("vtkRobartsCommonExport.h", "vtkRobartsCommonExport"),
                        ("vtkCudaCommonExport.h", "vtkCudaCommonExport"),
                        ("vtkCudaCommonStaticExport.h", "vtkCudaCommonStaticExport")):
        with open(os.path.join(inc, name), "w") as f:
            f.write("#pragma once\n#define %s\n" % macro)
    return inc


def build_reference_cpu(force: bool = False) -> str | None:
    if not reference_available():
        return None
    os.makedirs(REF_OUT, exist_ok=True)
    inc = _write_stubs()
    ref_dir = os.path.join(REFERENCE_ROOT, "Common/vtkRobartsCommon")
    ref_src = os.path.join(ref_dir, "vtkMaxFlowSegmentationUtilities.cxx")
    src = os.path.join(HERE, "hmf_oracle.cpp")
    out = os.path.join(REF_OUT, "libhmf_ref_cpu.so")
    if force or not _newer(out, [src, ref_src]):
        # The reference file is compiled single-threaded, as the reference runs it.
        _run(["g++", *CXXFLAGS, "-DHMF_ORACLE_WITH_REFERENCE", "-I", inc, "-I", ref_dir,
              src, ref_src, "-o", out + ".tmp"])
        os.replace(out + ".tmp", out)
    return out


def build_reference_cubin(force: bool = False) -> str | None:
    if not reference_available() or shutil.which("nvcc") is None:
        return None
    os.makedirs(REF_OUT, exist_ok=True)
    inc = _write_stubs()
    unit = os.path.join(HERE, "ref_kernels_unit.cu")
    d1 = os.path.join(REFERENCE_ROOT, "ImageProcessing/vtkCudaImageAnalytics")
    d2 = os.path.join(REFERENCE_ROOT, "Common/vtkCudaCommonStatic")
    d3 = os.path.join(REFERENCE_ROOT, "Common/vtkCudaCommon")
    out = os.path.join(REF_OUT, "hmf_ref_kernels.cubin")
    srcs = [unit, os.path.join(d1, "CUDA_hierarchicalmaxflow.cu"), os.path.join(d2, "CUDA_commonKernels.cu"),
            os.path.join(d1, "CUDA_hierarchicalmaxflowdecomp.cu"), os.path.join(d1, "CUDA_imagevote.cu")]
    if force or not _newer(out, srcs):
        # `saturate` was a legacy CUDA helper that CUDA 13 no longer ships.
        _run(["nvcc", "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3",
              "-Dsaturate=__saturatef", "-I", inc, "-I", d1, "-I", d2, "-I", d3,
              unit, "-o", out + ".tmp"])
        os.replace(out + ".tmp", out)
    return out


def build_all(force: bool = False) -> dict:
    with ThreadPoolExecutor(max_workers=3) as ex:
        f1 = ex.submit(build_port, force)
        f2 = ex.submit(build_reference_cpu, force)
        f3 = ex.submit(build_reference_cubin, force)
        return {"port": f1.result(), "reference_cpu": f2.result(), "reference_cubin": f3.result()}


if __name__ == "__main__":
    print(build_all(force="--force" in sys.argv))
