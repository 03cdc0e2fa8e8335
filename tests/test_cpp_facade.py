"""The C++ drop-in (robartsvtk_gb300/csrc/hmf_segmentation.hpp), compiled
into a caller program (tests/cpp/facade_main.cpp) and linked against
libhmf_gb300.so, as a VTK-free C++ application would use it.

CPU: the program compiles and links against the header and the library.
GPU: Update() on a seeded problem equals the oracle bit for bit, REF_CUDA
and REF_CPU semantics, in core and with SetMaxGPUUsage (out of core), and so
does Update() continued by ContinueUpdate(); a missing leaf input fails with
the reference's message and Update's -1.
"""
import os
import subprocess

import numpy as np
import pytest

from robartsvtk_gb300 import _capi, build
from robartsvtk_gb300.synthetic import random_tree_problem

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "cpp", "facade_main.cpp")


def _compile(out_dir) -> str:
    lib = build.build()
    exe = os.path.join(str(out_dir), "facade_main")
    cmd = ["g++", "-std=c++17", "-O1", "-I", build.CSRC, "-I", build.INCLUDE, SRC, "-o", exe,
           "-L", os.path.dirname(lib), "-l:" + os.path.basename(lib), "-Wl,-rpath," + os.path.dirname(lib)]
    p = subprocess.run(cmd, capture_output=True, text=True)
    assert p.returncode == 0, p.stderr
    return exe


def _write_spec(d, w, semantics, leaves_with_data=None, max_gpu_usage=None, continue_iterations=None):
    lines = ["%d %d %d" % w.dims, " ".join([str(len(w.parent))] + [str(p) for p in w.parent]),
             "%d %r %r %d" % (w.iterations, float(w.step), float(w.cc), semantics)]
    lines.append(" ".join([str(len(w.alpha))] + ["%d %r" % (v, float(a)) for v, a in w.alpha.items()]))
    data = [l for l in w.data if leaves_with_data is None or l in leaves_with_data]
    for l in data:
        w.data[l].astype(np.float32).tofile(os.path.join(d, "d%d.raw" % l))
    lines.append(" ".join([str(len(data))] + ["%d d%d.raw" % (l, l) for l in data]))
    for v, S in w.smooth.items():
        S.astype(np.float32).tofile(os.path.join(d, "s%d.raw" % v))
    lines.append(" ".join([str(len(w.smooth))] + ["%d s%d.raw" % (v, v) for v in w.smooth]))
    if max_gpu_usage is not None or continue_iterations is not None:
        line = "%r" % float(-1.0 if max_gpu_usage is None else max_gpu_usage)
        if continue_iterations is not None:
            line += " %d" % continue_iterations
        lines.append(line)
    with open(os.path.join(d, "spec.txt"), "w") as f:
        f.write("\n".join(lines) + "\n")


def test_facade_compiles_and_links(tmp_path):
    _compile(tmp_path)


@pytest.mark.gpu
@pytest.mark.parametrize("semantics,max_gpu_usage", [(0, None), (1, None), (0, 0.5), (1, 0.5)])
def test_facade_update_matches_the_oracle(tmp_path, semantics, max_gpu_usage):
    """Update() in core and, with SetMaxGPUUsage, out of core."""
    from oracle import oracle as O
    exe = _compile(tmp_path)
    w = random_tree_problem(61, (27, 14, 11), [-1, 0, 0, 1, 1, 2, 2], iterations=20, smooth_nodes=(1, 5))
    _write_spec(str(tmp_path), w, semantics, max_gpu_usage=max_gpu_usage)
    subprocess.run([exe, str(tmp_path)], check=True)
    status = open(os.path.join(tmp_path, "status.txt")).read().split("\n")
    assert status[0] == "1", status
    assert int(status[1]) == len(w.leaves)
    ref = O.solve(w.dims, w.parent, w.data, w.smooth, w.alpha, w.iterations, w.step, w.cc,
                  semantics=semantics)["u"]
    for leaf in w.leaves:
        got = np.fromfile(os.path.join(tmp_path, "out_%d.raw" % leaf), dtype=np.float32).reshape(w.dims[::-1])
        assert np.array_equal(got, ref[leaf].astype(np.float32)), leaf


@pytest.mark.gpu
@pytest.mark.parametrize("semantics,max_gpu_usage", [(0, None), (1, None), (0, 0.5)])
def test_facade_continue_update(tmp_path, semantics, max_gpu_usage):
    """Update() with 13 iterations, then ContinueUpdate() with 7: the
    oracle's 20-iteration solve, bit for bit."""
    from oracle import oracle as O
    exe = _compile(tmp_path)
    w = random_tree_problem(63, (27, 14, 11), [-1, 0, 0, 1, 1, 2, 2], iterations=13, smooth_nodes=(1, 5))
    _write_spec(str(tmp_path), w, semantics, max_gpu_usage=max_gpu_usage, continue_iterations=7)
    subprocess.run([exe, str(tmp_path)], check=True)
    status = open(os.path.join(tmp_path, "status.txt")).read().split("\n")
    assert status[0] == "1", status
    ref = O.solve(w.dims, w.parent, w.data, w.smooth, w.alpha, 20, w.step, w.cc, semantics=semantics)["u"]
    for leaf in w.leaves:
        got = np.fromfile(os.path.join(tmp_path, "out_%d.raw" % leaf), dtype=np.float32).reshape(w.dims[::-1])
        assert np.array_equal(got, ref[leaf].astype(np.float32)), leaf


@pytest.mark.gpu
def test_facade_missing_input_fails_like_the_reference(tmp_path):
    exe = _compile(tmp_path)
    w = random_tree_problem(62, (8, 7, 6), [-1, 0, 0, 0], iterations=3)
    _write_spec(str(tmp_path), w, 0, leaves_with_data={1, 2})
    subprocess.run([exe, str(tmp_path)], check=True)
    status = open(os.path.join(tmp_path, "status.txt")).read().split("\n")
    assert status[0] == "-1"
    assert "Missing data prior for leaf node." in status[2]
    _capi.load()
