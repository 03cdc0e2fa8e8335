"""Parity of the CUDA path (through the C ABI) with the oracle.  GPU only.

Bar: REF_CUDA labels and sinks bit-identical to the FP32 restatement of the
reference kernels (the kernels use the same operation order, no FMA
contraction, IEEE sqrt/division); REF_CPU bit-identical to the reference's
compiled CPU code.  End-to-end workloads additionally state max |u - u_fp64|.
"""
import os

import numpy as np
import pytest

from oracle import oracle as O
from robartsvtk_gb300 import REF_CPU, REF_CUDA, HierarchicalMaxFlowSegmentation, HMFError, HMFSolver
from robartsvtk_gb300.synthetic import boxes_flat3, ellipsoids_tree4, random_tree_problem
from tests.golden.cases import CASES, problem

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
LABEL_TOL = 1e-4  # per-voxel max |u_gpu - u_oracle| accepted for end-to-end workloads


def run_gpu(w, semantics=REF_CUDA, device_inputs=False, iterations=None, window=0, zchunk=0, pipeline=False,
            units=0):
    import torch
    with HMFSolver(w.dims, w.parent, semantics) as s:
        if window:
            s.set_flow_window(window)
        if units:
            s.set_flow_units(units)
        if zchunk:
            s.set_zchunk(zchunk)
        if pipeline:
            s.set_pipeline(True)
        keep = []
        for leaf, d in w.data.items():
            if device_inputs:
                t = torch.from_numpy(d).cuda()
                keep.append(t)
                s.set_data(leaf, t)
            else:
                s.set_data(leaf, d)
        for v, S in w.smooth.items():
            if device_inputs:
                t = torch.from_numpy(S).cuda()
                keep.append(t)
                s.set_smoothness(v, t)
            else:
                s.set_smoothness(v, S)
        for v, a in w.alpha.items():
            s.set_smoothness_scalar(v, a)
        s.set_params(w.iterations if iterations is None else iterations, w.step, w.cc)
        s.solve()
        n = len(w.parent)
        u = np.zeros((n,) + w.dims[::-1], np.float32)
        sink = np.zeros_like(u)
        for v in range(n):
            sink[v] = s.sink(v)
            if w.parent[v] >= 0:
                u[v] = s.labels(v)
        return {"u": u, "sink": sink, "stats": s.stats()}


def oracle(w, iterations=None, **kw):
    it = w.iterations if iterations is None else iterations
    return O.solve(w.dims, w.parent, w.data, w.smooth, w.alpha, it, w.step, w.cc, want_sink=True, **kw)


def assert_same(gpu, ref, what=""):
    for k in ("u", "sink"):
        a, b = gpu[k], ref[k].astype(np.float32)
        diff = np.abs(a.astype(np.float64) - b.astype(np.float64))
        assert np.array_equal(a, b), "%s %s: max |diff| %.3g at %s" % (
            what, k, diff.max(), np.unravel_index(diff.argmax(), diff.shape))


@pytest.mark.parametrize("name", sorted(CASES))
def test_ref_cuda_bitexact_golden_cases(name):
    w = problem(name)
    assert_same(run_gpu(w), oracle(w), name)


@pytest.mark.parametrize("dims,parent,smooth_nodes,iters", [
    ((5, 4, 3), [-1, 0, 0, 0], (), 7),
    ((1, 1, 9), [-1, 0, 0], (), 12),            # single column
    ((40, 1, 1), [-1, 0, 0], (1,), 12),         # single row
    ((31, 17, 1), [-1, 0, 0, 0], (2,), 15),     # single plane
    ((64, 16, 40), [-1, 0, 0, 1, 1, 2, 2], (1, 2, 3, 4, 5, 6), 9),  # z split into chunks
    ((70, 19, 23), [-1, 0, 1, 2, 2, 1, 0], (3, 4), 11),            # partial tiles, deep tree
    ((33, 65, 12), [-1, 0, 0, 0, 0, 0, 0, 0, 0], (), 6),           # wide root
])
def test_ref_cuda_bitexact_shapes(dims, parent, smooth_nodes, iters):
    w = random_tree_problem(21, dims, parent, iterations=iters, smooth_nodes=smooth_nodes)
    assert_same(run_gpu(w), oracle(w), str(dims))


@pytest.mark.parametrize("dims,parent,smooth_nodes,iters,zchunk", [
    ((5, 4, 3), [-1, 0, 0, 0], (), 7, 0),
    ((31, 17, 1), [-1, 0, 0, 0], (2,), 9, 0),
    ((70, 130, 23), [-1, 0, 1, 2, 2, 1, 0], (3, 4), 6, 0),     # interior 64-row windows and partial ones
    ((40, 64, 40), [-1, 0, 0, 1, 1, 2, 2], (1, 2, 3), 5, 7),  # exactly one window row, short z chunks
    ((33, 61, 12), [-1, 0, 0, 0, 0], (), 6, 0),                # 61 rows: two windows of 59 + 2
])
def test_ref_cuda_bitexact_64_row_windows(dims, parent, smooth_nodes, iters, zchunk):
    w = random_tree_problem(26, dims, parent, iterations=iters, smooth_nodes=smooth_nodes)
    assert_same(run_gpu(w, window=64, zchunk=zchunk), oracle(w), "64 rows " + str(dims))


@pytest.mark.parametrize("dims,parent,smooth_nodes,iters,zchunk,window", [
    ((40, 30, 50), [-1, 0, 0, 1, 1, 2, 2], (1, 2), 19, 7, 0),    # 8 slabs, 19 iterations: 8 + 8 + 2 + 1
    ((33, 61, 23), [-1, 0, 0, 0], (), 10, 5, 64),                # 5 slabs of 5 planes, the last of 3
    ((64, 16, 40), [-1, 0, 0, 1, 1, 2, 2], (1, 3, 5), 9, 0, 0),   # the default plan's chunks
    ((20, 12, 6), [-1, 0, 0], (), 4, 0, 0),                      # a single slab
    ((27, 14, 11), [-1, 0, 0, 1, 1, 2, 2], (1, 5), 20, 3, 0),    # slabs of 3 planes, the last of 2
    ((27, 14, 11), [-1, 0, 0, 1, 1, 2, 2], (1, 5), 20, 2, 0),    # 2-plane chunks: the pipeline stays off
])
def test_ref_cuda_bitexact_slab_pipeline(dims, parent, smooth_nodes, iters, zchunk, window):
    w = random_tree_problem(28, dims, parent, iterations=iters, smooth_nodes=smooth_nodes)
    assert_same(run_gpu(w, window=window, zchunk=zchunk, pipeline=True), oracle(w), "pipelined " + str(dims))


@pytest.mark.parametrize("dims,parent,smooth_nodes,iters,zchunk,window,pipeline,units", [
    ((40, 30, 50), [-1, 0, 0, 1, 1, 2, 2], (1, 2), 9, 7, 0, True, 2),     # pipelined slabs, 2 marches per CTA
    ((64, 16, 40), [-1, 0, 0, 1, 1, 2, 2], (1, 3, 5), 7, 0, 0, False, 3),  # 3 marches: CTAs span windows
    ((33, 61, 12), [-1, 0, 0, 0, 0], (), 6, 0, 64, False, 4),             # 64-row windows
    ((70, 19, 23), [-1, 0, 1, 2, 2, 1, 0], (3, 4), 8, 4, 0, True, 64),    # one CTA per slab launch or fewer
])
def test_ref_cuda_bitexact_units_per_cta(dims, parent, smooth_nodes, iters, zchunk, window, pipeline, units):
    """Several (window, vertex) marches per flow-kernel CTA, one after another."""
    w = random_tree_problem(31, dims, parent, iterations=iters, smooth_nodes=smooth_nodes)
    assert_same(run_gpu(w, window=window, zchunk=zchunk, pipeline=pipeline, units=units), oracle(w),
                "units %d %s" % (units, dims))


def test_slab_pipeline_with_device_inputs_that_move():
    """The per-slab tables follow inputs that move between solves."""
    import torch
    w = random_tree_problem(29, (36, 20, 30), [-1, 0, 0, 1, 1], iterations=9, smooth_nodes=(1,))
    ref = oracle(w)
    with HMFSolver(w.dims, w.parent) as s:
        s.set_zchunk(6)
        s.set_pipeline(True)
        for v, a in w.alpha.items():
            s.set_smoothness_scalar(v, a)
        s.set_params(w.iterations, w.step, w.cc)
        for attempt in range(2):
            keep = [torch.from_numpy(d).cuda() for d in w.data.values()]  # new device buffers each time
            for leaf, t in zip(w.data, keep):
                s.set_data(leaf, t)
            for v, S in w.smooth.items():
                s.set_smoothness(v, S)
            s.solve()
            assert s.pipeline
            for v in range(len(w.parent)):
                if w.parent[v] >= 0:
                    assert np.array_equal(s.labels(v), ref["u"][v].astype(np.float32)), (attempt, v)


def test_autotuned_plan_is_bitexact():
    w = random_tree_problem(27, (90, 75, 33), [-1, 0, 0, 1, 1], iterations=8, smooth_nodes=(1,))
    ref = oracle(w)
    with HMFSolver(w.dims, w.parent) as s:
        for leaf, d in w.data.items():
            s.set_data(leaf, d)
        for v, S in w.smooth.items():
            s.set_smoothness(v, S)
        for v, a in w.alpha.items():
            s.set_smoothness_scalar(v, a)
        s.set_params(w.iterations, w.step, w.cc)
        s.autotune()
        assert s.flow_window in (32, 64) and s.zchunk() >= 1
        s.solve()
        for v in range(len(w.parent)):
            if w.parent[v] >= 0:
                assert np.array_equal(s.labels(v), ref["u"][v].astype(np.float32)), v


def test_ref_cuda_shared_smoothness_image():
    w = random_tree_problem(22, (20, 12, 10), [-1, 0, 0, 1, 1], iterations=10)
    S = np.random.default_rng(1).uniform(0, 1, size=(10, 12, 20)).astype(np.float32)
    w.smooth = {v: S for v in (1, 2, 3, 4)}
    assert_same(run_gpu(w), oracle(w))


def test_ref_cuda_zero_iterations_is_the_initialisation():
    w = random_tree_problem(23, (9, 8, 7), [-1, 0, 0, 1, 1], iterations=0)
    w.data[2][0, 0, 0] = w.data[3][0, 0, 0] = w.data[4][0, 0, 0] = 0.5  # a three-way tie
    assert_same(run_gpu(w), oracle(w))


def test_device_inputs_equal_host_inputs():
    w = random_tree_problem(24, (36, 10, 9), [-1, 0, 0, 1, 1], iterations=8, smooth_nodes=(1, 3))
    a, b = run_gpu(w), run_gpu(w, device_inputs=True)
    assert np.array_equal(a["u"], b["u"]) and np.array_equal(a["sink"], b["sink"])
    w2 = random_tree_problem(24, (35, 10, 9), [-1, 0, 0, 1, 1], iterations=8, smooth_nodes=(1, 3))
    assert_same(run_gpu(w2, device_inputs=True), oracle(w2), "pitched device inputs")


def test_ref_cpu_mode_matches_reference_cpu_golden():
    g = np.load(os.path.join(GOLDEN, "ref_cpu_golden.npz"))
    for name in sorted(CASES):
        w = problem(name)
        r = run_gpu(w, semantics=REF_CPU)
        assert np.array_equal(r["u"], g[name + "/u"]), name
        assert np.array_equal(r["sink"], g[name + "/sink"]), name


def test_ref_cpu_mode_matches_port_odd_shape():
    w = random_tree_problem(25, (37, 11, 6), [-1, 0, 0, 1, 1, 1], iterations=40, smooth_nodes=(1,))
    r = run_gpu(w, semantics=REF_CPU)
    o = oracle(w, semantics=O.REF_CPU)
    assert np.array_equal(r["u"], o["u"].astype(np.float32))


def test_boxes64_flat3_end_to_end():
    """64^3, 3 boxes, flat 3 leaves, alpha 0.1, 200 iterations."""
    w = boxes_flat3(seed=0)
    g = run_gpu(w)
    o32 = oracle(w)
    o64 = oracle(w, precision=64)
    leaves = w.leaves
    err = np.abs(g["u"][leaves] - o32["u"][leaves]).max()
    err64 = np.abs(g["u"][leaves].astype(np.float64) - o64["u"][leaves]).max()
    agree = (np.argmax(g["u"][leaves], 0) == np.argmax(o32["u"][leaves], 0)).mean()
    print("boxes64: max|u-u32| %.3g  max|u-u64| %.3g  argmax agreement %.6f" % (err, err64, agree))
    assert err <= LABEL_TOL and agree >= 0.999
    assert err64 < 1e-3


def test_ellipsoids256_tree4_full_size_first_iterations_bitexact():
    """The 256^3 two-level workload at full size: 3 iterations against the oracle."""
    w = ellipsoids_tree4(seed=0)
    assert_same(run_gpu(w, iterations=3), oracle(w, iterations=3), "256^3")


def test_ellipsoids256_tree4_full_solve_properties():
    w = ellipsoids_tree4(seed=0)
    a = run_gpu(w)
    u = a["u"][w.leaves]
    assert np.isfinite(u).all() and u.min() >= 0 and u.max() <= 1
    assert (np.argmax(u, 0) == w.truth).mean() > 0.95
    b = run_gpu(w)
    assert np.array_equal(a["u"], b["u"])  # deterministic


def test_missing_leaf_data_is_an_error():
    with HMFSolver((4, 4, 4), [-1, 0, 0]) as s:
        s.set_data(1, np.ones((4, 4, 4), np.float32))
        with pytest.raises(HMFError, match="Missing data"):
            s.solve()


def test_negative_data_is_reported():
    with HMFSolver((4, 4, 4), [-1, 0, 0]) as s:
        d = np.ones((4, 4, 4), np.float32)
        d[1, 2, 3] = -1
        s.set_data(1, d)
        s.set_data(2, np.ones((4, 4, 4), np.float32))
        s.solve()
        with pytest.raises(HMFError, match="non-negative"):
            s.labels(1)


def test_host_memory_labelled_as_device_memory_is_refused():
    """A host buffer passed as HMF_DEVICE is refused by the calls that take
    it (none of these calls launches a kernel); device tensors still pass."""
    import torch

    from robartsvtk_gb300._capi import HMF_DEVICE
    host = np.ones((4, 4, 4), np.float32)
    with HMFSolver((4, 4, 4), [-1, 0, 0]) as s:
        with pytest.raises(HMFError, match="host memory passed as device memory"):
            s.set_data_pointer(1, host.ctypes.data, HMF_DEVICE)
        rc = s._lib.hmf_set_smoothness(s._ctx, 1, host.ctypes.data, HMF_DEVICE)
        assert rc != 0 and b"device memory" in s._lib.hmf_last_error(s._ctx)
        dev = torch.ones((4, 4, 4), dtype=torch.float32, device="cuda")
        s.set_data(1, dev)
        s.set_data(2, dev)
        s.set_smoothness(1, dev)
        s.solve()
        out = np.empty((4, 4, 4), np.float32)
        rc = s._lib.hmf_get_labels(s._ctx, 1, out.ctypes.data, HMF_DEVICE, None)
        assert rc != 0 and b"device memory" in s._lib.hmf_last_error(s._ctx)
        assert np.all(np.isfinite(s.labels(1)))


def test_filter_api_end_to_end():
    w = random_tree_problem(26, (12, 10, 8), [-1, 0, 0, 1, 1], iterations=20, smooth_nodes=(2,))
    f = HierarchicalMaxFlowSegmentation()
    f.SetHierarchy(w.parent)
    for leaf, d in w.data.items():
        f.SetDataInputDataObject(leaf, d)
    for v, S in w.smooth.items():
        f.SetSmoothnessInputDataObject(v, S)
    for v, a in w.alpha.items():
        f.AddSmoothnessScalar(v, a)
    f.SetNumberOfIterations(w.iterations)
    assert f.Update() == 1, f.GetLastError()
    o = oracle(w)
    assert f.GetNumberOfOutputPorts() == len(w.leaves)
    for leaf in w.leaves:
        assert np.array_equal(f.GetOutputDataObject(leaf), o["u"][leaf].astype(np.float32))
    assert f.GetOutputDataObject(1) is None  # branch: no output port


def test_launch_count_per_iteration():
    w = random_tree_problem(27, (16, 16, 16), [-1, 0, 0, 0], iterations=10)
    r = run_gpu(w)
    assert r["stats"]["launches"] == 1 + 2 * 10  # init + (flow, tree) per iteration


@pytest.mark.skipif(not os.path.exists(os.path.join(GOLDEN, "ref_cuda_golden.npz")),
                    reason="REF_CUDA golden vectors not generated yet")
@pytest.mark.parametrize("name", sorted(CASES))
def test_against_reference_cuda_kernels_golden(name):
    """Golden vectors produced by the reference's own CUDA kernels (compiled
    from CUDA_hierarchicalmaxflow.cu with nvcc's default FMA contraction)."""
    g = np.load(os.path.join(GOLDEN, "ref_cuda_golden.npz"))
    w = problem(name)
    r = run_gpu(w)
    assert np.abs(r["u"] - g[name + "/u"]).max() <= LABEL_TOL


@pytest.mark.parametrize("flow,tree", [("tma", "bulk"), ("ring", "bulk"), ("tma", "quad"), ("ring", "scalar")])
def test_kernel_variants_are_bitexact(flow, tree, monkeypatch):
    """Every flow / tree kernel variant gives the oracle's results."""
    monkeypatch.setenv("HMF_FLOW_KERNEL", flow)
    monkeypatch.setenv("HMF_TREE_KERNEL", tree)
    for dims, parent in (((45, 30, 21), [-1, 0, 0, 1, 1, 2, 2]), ((29, 58, 9), [-1, 0, 0, 0])):
        w = random_tree_problem(31, dims, parent, iterations=12, smooth_nodes=(1, 2))
        assert_same(run_gpu(w), oracle(w), "%s/%s %s" % (flow, tree, dims))


def test_large_tree_uses_small_chunks():
    """A 20-vertex tree: the tree kernel's chunk shrinks to fit shared memory."""
    parent = [-1] + [0] * 4 + [1, 1, 2, 2, 3, 3, 4, 4] + [5, 5, 6, 6, 7, 7, 8]
    w = random_tree_problem(32, (40, 21, 13), parent, iterations=6, smooth_nodes=(3, 9))
    assert_same(run_gpu(w), oracle(w), "20-vertex tree")


@pytest.mark.parametrize("z", [1, 2, 3, 5, 16, 0])
def test_z_chunk_lengths_are_bitexact(z):
    """The flow kernel's work plan does not change results: chunks of a few
    planes (halo planes of both neighbours recomputed), the default plan and
    the 15-vertex tree of the large workload."""
    for dims, parent in (((45, 30, 23), [-1, 0, 0, 1, 1, 2, 2]),
                         ((33, 29, 19), [-1, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6])):
        w = random_tree_problem(41, dims, parent, iterations=7, smooth_nodes=(1, 4))
        with HMFSolver(w.dims, w.parent) as s:
            for leaf, d in w.data.items():
                s.set_data(leaf, d)
            for v, S in w.smooth.items():
                s.set_smoothness(v, S)
            for v, a in w.alpha.items():
                s.set_smoothness_scalar(v, a)
            s.set_params(w.iterations, w.step, w.cc)
            s.set_zchunk(z)
            assert s.zchunk() == (z if z else s.zchunk()) and 1 <= s.zchunk() <= dims[2]
            s.solve()
            ref = oracle(w)
            for v in range(len(parent)):
                assert np.array_equal(s.sink(v), ref["sink"][v].astype(np.float32)), (z, dims, v)
                if parent[v] >= 0:
                    assert np.array_equal(s.labels(v), ref["u"][v].astype(np.float32)), (z, dims, v)
