"""The bounded copy waits' failure path, made to run on healthy hardware.
GPU only.

hmf_inject_wait_stall makes one CTA of the next launch of a kernel wait on an
mbarrier that no copy completes; its bounded wait runs out, the kernel stops
issuing copies, drains the copies in flight into its shared memory and
leaves, and the call reports HMF_ERR_CUDA.  Nothing faults or hangs: the
context stays usable and the next solve is bit-identical to the oracle.
"""
import numpy as np
import pytest

from oracle import oracle as O
from robartsvtk_gb300 import DAGSolver, HMFError, HMFSolver
from robartsvtk_gb300._capi import (HMF_STALL_FLOW, HMF_STALL_REVERSE_FLOW, HMF_STALL_REVERSE_SWEEP,
                                    HMF_STALL_SWEEP)
from robartsvtk_gb300.synthetic import random_tree_problem

pytestmark = pytest.mark.gpu


def _configure(s, w):
    for leaf, d in w.data.items():
        s.set_data(leaf, d)
    for v, S in w.smooth.items():
        s.set_smoothness(v, S)
    for v, a in w.alpha.items():
        s.set_smoothness_scalar(v, a)
    s.set_params(w.iterations, w.step, w.cc)


def _labels(s, w):
    return {v: s.labels(v) for v in range(len(w.parent)) if w.parent[v] >= 0}


def _problem():
    # several windows and z chunks per vertex, so the stalled CTA is one of many
    return random_tree_problem(41, (70, 40, 30), [-1, 0, 0, 1, 1, 2, 2], iterations=6, smooth_nodes=(1, 4))


@pytest.mark.parametrize("kernel", [HMF_STALL_FLOW, HMF_STALL_SWEEP])
def test_stalled_wait_is_reported_and_the_context_recovers(kernel):
    w = _problem()
    ref = O.solve(w.dims, w.parent, w.data, w.smooth, w.alpha, w.iterations, w.step, w.cc)["u"]
    with HMFSolver(w.dims, w.parent) as s:
        _configure(s, w)
        s.solve()  # captures the iteration graphs
        s.set_wait_limit(2_000_000)  # 2 ms
        s.inject_wait_stall(kernel)
        s.solve()
        with pytest.raises(HMFError, match="timed out"):
            s.labels(w.leaves[0])
        s.set_wait_limit(0)
        s.solve()
        for v, u in _labels(s, w).items():
            assert np.array_equal(u, ref[v].astype(np.float32)), v


def test_stalled_dag_sweep_is_reported_and_the_context_recovers():
    dims, n = (40, 30, 20), 5
    edges = [(0, 1), (0, 2), (1, 3), (1, 4), (2, 4)]
    rng = np.random.default_rng(3)
    data = {v: rng.uniform(0, 2, size=dims[::-1]).astype(np.float32) for v in (3, 4)}
    with DAGSolver(dims, n, edges) as s:
        for v, d in data.items():
            s.set_data(v, d)
        for v in range(1, n):
            s.set_smoothness_scalar(v, 0.3)
        s.set_params(5, 0.1, 0.25)
        s.solve()
        good = {v: s.labels(v) for v in (1, 2, 3, 4)}
        s.inject_wait_stall(HMF_STALL_SWEEP)
        s.solve()
        with pytest.raises(HMFError, match="timed out"):
            s.labels(3)
        s.solve()
        for v, u in good.items():
            assert np.array_equal(s.labels(v), u), v


@pytest.mark.parametrize("kernel", [HMF_STALL_REVERSE_FLOW, HMF_STALL_REVERSE_SWEEP])
def test_stalled_adjoint_wait_is_reported_and_the_context_recovers(kernel):
    w = random_tree_problem(42, (60, 40, 24), [-1, 0, 0, 0], iterations=5)
    truth = np.random.default_rng(4).integers(0, 3, size=w.dims[::-1]).astype(np.int32)
    with HMFSolver(w.dims, w.parent) as s:
        _configure(s, w)
        loss = s.solve_adjoint(truth, checkpoint_every=5)
        grad = s.data_gradient(w.leaves[0])
        s.set_wait_limit(2_000_000)
        s.inject_wait_stall(kernel)
        with pytest.raises(HMFError, match="timed out"):
            s.solve_adjoint(truth, checkpoint_every=5)
        s.set_wait_limit(0)
        assert s.solve_adjoint(truth, checkpoint_every=5) == pytest.approx(loss, rel=1e-12)
        assert np.array_equal(s.data_gradient(w.leaves[0]), grad)


def test_wait_controls_validate_their_arguments():
    w = random_tree_problem(43, (6, 5, 4), [-1, 0, 0], iterations=2)
    with HMFSolver(w.dims, w.parent) as s:
        with pytest.raises(HMFError):
            s.set_wait_limit(-1)
        with pytest.raises(HMFError):
            s.inject_wait_stall(7)
        s.inject_wait_stall(HMF_STALL_FLOW)
        s.inject_wait_stall(-1)  # cancelled: the solve runs normally
        _configure(s, w)
        s.solve()
        s.labels(1)
