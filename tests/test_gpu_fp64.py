"""FP64 evaluation of the REF_CUDA iteration on the GPU (hmf_solve_fp64), the
measurements taken against it, and the full-length parity of the 256^3
two-level workload.  GPU only.

Bars: the FP64 GPU solve equals the oracle's FP64 restatement bit for bit
(same operations in the same order, in double); the FP32 GPU solve of the
256^3 tree4 workload over all 500 iterations is within LABEL_TOL of the FP32
oracle per voxel with >= 99.9 % argmax agreement, and its distance from the
FP64 solve is stated.
"""
import numpy as np
import pytest

from oracle import oracle as O
from robartsvtk_gb300 import REF_CPU, HMFBatchSolver, HMFError, HMFSolver
from robartsvtk_gb300._capi import HMF_FP64_PROBE_ALPHA, HMF_FP64_PROBE_DATA, check
from robartsvtk_gb300.synthetic import ellipsoids_tree4, ellipsoids_tree8, random_tree_problem
from tests.golden.cases import CASES, problem

pytestmark = pytest.mark.gpu
LABEL_TOL = 1e-4  # per-voxel max |u_gpu - u_oracle| accepted for end-to-end workloads


def _configure(s, w, iterations=None):
    for leaf, d in w.data.items():
        s.set_data(leaf, d)
    for v, S in w.smooth.items():
        s.set_smoothness(v, S)
    for v, a in w.alpha.items():
        s.set_smoothness_scalar(v, a)
    s.set_params(w.iterations if iterations is None else iterations, w.step, w.cc)


def fp64_gpu(w, probes=()):
    with HMFSolver(w.dims, w.parent) as s:
        _configure(s, w)
        for p in probes:
            s.set_fp64_probe(*p)
        s.solve_fp64()
        return {v: s.labels_fp64(v) for v in range(len(w.parent)) if w.parent[v] >= 0}


def fp64_oracle(w, data=None, alpha=None):
    return O.solve(w.dims, w.parent, data if data is not None else w.data, w.smooth,
                   alpha if alpha is not None else w.alpha, w.iterations, w.step, w.cc, precision=64)["u"]


def assert_fp64_same(got, ref, what=""):
    for v, u in got.items():
        diff = np.abs(u - ref[v])
        assert np.array_equal(u, ref[v]), "%s vertex %d: max |diff| %.3g" % (what, v, diff.max())


@pytest.mark.parametrize("name", sorted(CASES))
def test_fp64_bitexact_golden_cases(name):
    w = problem(name)
    assert_fp64_same(fp64_gpu(w), fp64_oracle(w), name)


@pytest.mark.parametrize("dims,parent,smooth_nodes,iters", [
    ((5, 4, 3), [-1, 0, 0, 0], (), 7),
    ((1, 1, 9), [-1, 0, 0], (), 12),
    ((40, 1, 1), [-1, 0, 0], (1,), 12),
    ((31, 17, 1), [-1, 0, 0, 0], (2,), 15),
    ((70, 19, 23), [-1, 0, 1, 2, 2, 1, 0], (3, 4), 11),
    ((33, 65, 12), [-1, 0, 0, 0, 0, 0, 0, 0, 0], (), 6),
])
def test_fp64_bitexact_shapes(dims, parent, smooth_nodes, iters):
    w = random_tree_problem(31, dims, parent, iterations=iters, smooth_nodes=smooth_nodes)
    assert_fp64_same(fp64_gpu(w), fp64_oracle(w), str(dims))


def test_fp64_zero_iterations_tie():
    w = random_tree_problem(32, (9, 8, 7), [-1, 0, 0, 1, 1], iterations=0)
    w.data[2][0, 0, 0] = w.data[3][0, 0, 0] = w.data[4][0, 0, 0] = 0.5
    assert_fp64_same(fp64_gpu(w), fp64_oracle(w))


def test_fp64_data_probe_equals_modified_input():
    w = random_tree_problem(33, (12, 10, 9), [-1, 0, 0, 1, 1], iterations=20, smooth_nodes=(1,))
    leaf, (z, y, x) = 3, (4, 5, 6)
    vox = (z * w.dims[1] + y) * w.dims[0] + x
    # the unchanged value is a no-op
    same = fp64_gpu(w, [(HMF_FP64_PROBE_DATA, leaf, vox, float(w.data[leaf][z, y, x]))])
    assert_fp64_same(same, fp64_oracle(w), "probe = D")
    # a float-representable new value equals the oracle on the modified float input
    val = np.float32(w.data[leaf][z, y, x] * 0.5 + 0.125)
    data = {k: v.copy() for k, v in w.data.items()}
    data[leaf][z, y, x] = val
    got = fp64_gpu(w, [(HMF_FP64_PROBE_DATA, leaf, vox, float(val))])
    assert_fp64_same(got, fp64_oracle(w, data=data), "probe data")


def test_fp64_alpha_probe_equals_modified_alpha():
    w = random_tree_problem(34, (11, 9, 8), [-1, 0, 0, 0], iterations=15)
    new = float(np.float32(0.37))
    alpha = dict(w.alpha)
    alpha[2] = new
    got = fp64_gpu(w, [(HMF_FP64_PROBE_ALPHA, 2, 0, new)])
    assert_fp64_same(got, fp64_oracle(w, alpha=alpha), "probe alpha")


def test_fp64_error_and_loss_match_host_computation():
    w = random_tree_problem(35, (20, 14, 11), [-1, 0, 0, 1, 1, 2, 2], iterations=30, smooth_nodes=(1, 5))
    truth = np.random.default_rng(5).integers(0, len(w.leaves), size=w.dims[::-1]).astype(np.int32)
    with HMFSolver(w.dims, w.parent) as s:
        _configure(s, w)
        s.solve()
        s.solve_fp64()
        err = s.fp64_error()
        u32 = np.stack([s.labels(l).astype(np.float64) for l in w.leaves])
        u64 = np.stack([s.labels_fp64(l) for l in w.leaves])
        loss = s.fp64_loss(truth, eps=1e-6)
    assert err["max_abs_err"] == np.abs(u32 - u64).max()
    assert err["argmax_agreement"] == (np.argmax(u32, 0) == np.argmax(u64, 0)).mean()
    picked = np.take_along_axis(u64, truth[None], 0)[0]
    ref = -np.sum(np.log(np.maximum(picked, 1e-6))) / truth.size
    assert loss == pytest.approx(ref, rel=1e-12)


def test_fp64_refuses_what_it_does_not_evaluate():
    w = random_tree_problem(36, (6, 5, 4), [-1, 0, 0], iterations=3)
    with HMFSolver(w.dims, w.parent, REF_CPU) as s:
        _configure(s, w)
        with pytest.raises(HMFError, match="REF_CUDA"):
            s.solve_fp64()
    with HMFSolver(w.dims, w.parent) as s:
        _configure(s, w)
        with pytest.raises(HMFError, match="has not run"):
            s.labels_fp64(1)
        with pytest.raises(HMFError, match="leaf"):
            s.set_fp64_probe(HMF_FP64_PROBE_DATA, 0, 0, 1.0)
        with pytest.raises(HMFError, match="out of range"):
            s.set_fp64_probe(HMF_FP64_PROBE_DATA, 1, 6 * 5 * 4, 1.0)
    with HMFBatchSolver([(6, 5, 4), (4, 4, 4)], [-1, 0, 0]) as b:
        with pytest.raises(HMFError, match="single-volume"):
            check(b._lib.hmf_solve_fp64(b._ctx, None), b._ctx)


def test_ellipsoids256_tree4_full_length_parity():
    """The 256^3 two-level workload over all 500 iterations: the GPU's FP32
    labels against the FP32 oracle (host cores), and against the FP64 GPU
    solve, whose distance is stated."""
    w = ellipsoids_tree4(seed=0)
    with HMFSolver(w.dims, w.parent) as s:
        _configure(s, w)
        s.solve()
        u32 = np.stack([s.labels(l) for l in w.leaves])
        s.solve_fp64()
        e64 = s.fp64_error()
    ref = O.solve(w.dims, w.parent, w.data, w.smooth, w.alpha, w.iterations, w.step, w.cc)["u"][w.leaves]
    err = float(np.abs(u32.astype(np.float64) - ref).max())
    agree = float((np.argmax(u32, 0) == np.argmax(ref, 0)).mean())
    identical = bool(np.array_equal(u32, ref.astype(np.float32)))
    print("ellipsoids256_tree4 500 it: max|u_gpu - u_oracle32| %.3g (bit-identical: %s), argmax agreement %.6f; "
          "max|u_gpu - u_fp64| %.3g, argmax agreement with FP64 %.6f"
          % (err, identical, agree, e64["max_abs_err"], e64["argmax_agreement"]))
    assert err <= LABEL_TOL and agree >= 0.999
    assert e64["argmax_agreement"] >= 0.999


def test_ellipsoids_tree8_three_level_tree_parity():
    """The three-level tree of the 512x512x384 workload (root -> 2 -> 4 -> 8,
    14 flows, 15-entry sweep) on a 256x256x192 crop of its phantom
    generator, 40 iterations: the GPU's FP32 labels bit-identical to the
    FP32 oracle, and the FP64 GPU solve's distance stated."""
    w = ellipsoids_tree8(seed=5, dims=(256, 256, 192), iterations=40)
    with HMFSolver(w.dims, w.parent) as s:
        _configure(s, w)
        s.solve()
        u32 = np.stack([s.labels(l) for l in w.leaves])
        s.solve_fp64()
        e64 = s.fp64_error()
    ref = O.solve(w.dims, w.parent, w.data, w.smooth, w.alpha, w.iterations, w.step, w.cc)["u"][w.leaves]
    identical = bool(np.array_equal(u32, ref.astype(np.float32)))
    print("ellipsoids256x256x192_tree8 40 it: bit-identical to the oracle: %s; max|u_gpu - u_fp64| %.3g, argmax "
          "agreement with FP64 %.6f" % (identical, e64["max_abs_err"], e64["argmax_agreement"]))
    assert identical
    assert e64["argmax_agreement"] >= 0.999

