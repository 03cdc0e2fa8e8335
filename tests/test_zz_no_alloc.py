"""hmf_solve_noalloc: the allocation-free solve for callers that must not
allocate device memory while they run (for example a plugin in a streaming
image-guidance application that reserves all GPU memory at start-up, where a
cudaMalloc or cudaFree could synchronise the device and stall the
application's other streams).  The entry point keeps its state in a static
64 MiB device array of the library; these tests call it through the C ABI and
check it against the allocating entry points (hmf_create / hmf_solve /
hmf_get_labels), which the other tests pin to the oracle.  The file is named
so that pytest collects it last."""
import ctypes

import numpy as np
import pytest

from robartsvtk_gb300 import HMFSolver, _capi
from robartsvtk_gb300.synthetic import random_tree_problem

pytestmark = pytest.mark.gpu


def _context_labels(w, semantics=0):
    with HMFSolver(w.dims, w.parent, semantics) as s:
        for leaf, d in w.data.items():
            s.set_data(leaf, d)
        for v, S in w.smooth.items():
            s.set_smoothness(v, S)
        for v, a in w.alpha.items():
            s.set_smoothness_scalar(v, a)
        s.set_params(w.iterations, w.step, w.cc)
        s.solve()
        return {v: s.labels(v) for v in range(len(w.parent)) if w.parent[v] >= 0}


def _noalloc_labels(w, semantics=0, stream=None, capture=False):
    """Labels of a hmf_solve_noalloc call; with `capture`, the return code of
    the call made inside a CUDA graph capture of `stream` instead."""
    import torch
    lib = _capi.load()
    n = len(w.parent)
    keep = []
    data = (ctypes.c_void_p * n)()
    smooth = (ctypes.c_void_p * n)()
    for v, d in w.data.items():
        t = torch.from_numpy(d).cuda()
        keep.append(t)
        data[v] = t.data_ptr()
    for v, S in w.smooth.items():
        t = torch.from_numpy(S).cuda()
        keep.append(t)
        smooth[v] = t.data_ptr()
    alpha = (ctypes.c_double * n)(*[w.alpha.get(v, 1.0) for v in range(n)])
    outs = {v: torch.full(w.dims[::-1], -7.0, device="cuda") for v in range(n) if w.parent[v] >= 0}
    labels = (ctypes.c_void_p * n)()
    for v, t in outs.items():
        labels[v] = t.data_ptr()
    par = (ctypes.c_int * n)(*w.parent)
    torch.cuda.synchronize()
    handle = stream.cuda_stream if stream is not None else None
    if capture:
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=stream):
            rc = lib.hmf_solve_noalloc(*w.dims, par, n, semantics, data, smooth, alpha, w.iterations, w.step,
                                       w.cc, labels, handle)
        return rc
    rc = lib.hmf_solve_noalloc(*w.dims, par, n, semantics, data, smooth, alpha, w.iterations, w.step, w.cc,
                               labels, handle)
    assert rc == 0, lib.hmf_last_error(None)
    return {v: t.cpu().numpy() for v, t in outs.items()}


def test_noalloc_matches_the_allocating_path_on_two_calls_in_a_row():
    a = random_tree_problem(41, (37, 19, 23), [-1, 0, 0, 1, 1, 2, 2], iterations=30, smooth_nodes=(1, 4, 6))
    b = random_tree_problem(42, (64, 24, 16), [-1, 0, 0, 0], iterations=45)
    for w in (a, b):
        ref = _context_labels(w)
        got = _noalloc_labels(w)
        for v in ref:
            # the same kernels run on the same inputs: results are bit-identical
            assert np.array_equal(got[v], ref[v]), v


def test_noalloc_rejects_a_problem_beyond_its_scratch():
    import torch
    lib = _capi.load()
    dims = (256, 256, 256)  # 4 leaves would need ~2.6 GB of state
    par = (ctypes.c_int * 5)(-1, 0, 0, 0, 0)
    t = torch.zeros(1, device="cuda")
    data = (ctypes.c_void_p * 5)(*([None] + [t.data_ptr()] * 4))
    rc = lib.hmf_solve_noalloc(*dims, par, 5, 0, data, None, None, 10, 0.1, 0.25, None, None)
    assert rc == -1
    assert b"64 MiB" in lib.hmf_last_error(None)


def test_noalloc_ref_cpu_semantics_and_a_caller_stream():
    """REF_CPU semantics (the per-voxel leaf iteration of the reference's CPU
    class) on a caller's non-default stream, twice in a row, against the
    allocating path."""
    import torch
    w = random_tree_problem(43, (29, 17, 13), [-1, 0, 0, 1, 1, 1], iterations=25, smooth_nodes=(1,))
    ref = _context_labels(w, semantics=1)
    stream = torch.cuda.Stream()
    for _ in range(2):
        got = _noalloc_labels(w, semantics=1, stream=stream)
        for v in ref:
            assert np.array_equal(got[v], ref[v]), v


def test_noalloc_reports_negative_input():
    """A negative data term is reported after the solve (the reference
    rejects such inputs), and the next call with valid input succeeds."""
    import torch
    lib = _capi.load()
    w = random_tree_problem(44, (12, 9, 7), [-1, 0, 0], iterations=4)
    bad = {k: v.copy() for k, v in w.data.items()}
    bad[1][3, 4, 5] = -1.0
    w_bad = random_tree_problem(44, (12, 9, 7), [-1, 0, 0], iterations=4)
    w_bad.data = bad
    with pytest.raises(AssertionError):
        _noalloc_labels(w_bad)
    assert b"non-negative" in lib.hmf_last_error(None)
    ref = _context_labels(w)
    got = _noalloc_labels(w)
    for v in ref:
        assert np.array_equal(got[v], ref[v]), v


def test_noalloc_refuses_a_stream_capture():
    """Inside a CUDA graph capture the call returns HMF_ERR_INVALID_ARGUMENT
    before queuing anything (it stages its tables from its own stack frame and
    waits for its stream), and the next call outside the capture succeeds."""
    import torch
    lib = _capi.load()
    w = random_tree_problem(45, (12, 9, 7), [-1, 0, 0], iterations=3)
    rc = _noalloc_labels(w, stream=torch.cuda.Stream(), capture=True)
    assert rc == -1
    assert b"capture" in lib.hmf_last_error(None)
    ref = _context_labels(w)
    got = _noalloc_labels(w)
    for v in ref:
        assert np.array_equal(got[v], ref[v]), v
