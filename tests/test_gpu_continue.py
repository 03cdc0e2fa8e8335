"""Continued solves (hmf_solve_continue): k2 more iterations from the state a
solve of k1 ended in must equal, bit for bit, one solve of k1 + k2 -- and the
oracle's.  Covers odd k1 (flows left in the second set), the slab pipeline,
the launch-by-launch path, batches, REF_CPU, out-of-core contexts, the
convergence log per call and the refusals.  GPU only."""
import numpy as np
import pytest

from oracle import oracle as O
from robartsvtk_gb300 import REF_CPU, REF_CUDA, HierarchicalMaxFlowSegmentation, HMFBatchSolver, HMFError, HMFSolver
from robartsvtk_gb300.segmentation import DAGSolver, DirectedAcyclicGraphMaxFlowSegmentation
from robartsvtk_gb300.synthetic import random_tree_problem

pytestmark = pytest.mark.gpu

HMF_ERR_INVALID_ARGUMENT = -1
HMF_ERR_STATE = -6


def _configure(s, w, iterations):
    for leaf, d in w.data.items():
        s.set_data(leaf, d)
    for v, S in w.smooth.items():
        s.set_smoothness(v, S)
    for v, a in w.alpha.items():
        s.set_smoothness_scalar(v, a)
    s.set_params(iterations, w.step, w.cc)


def _state(s, w):
    n = len(w.parent)
    u = np.zeros((n,) + w.dims[::-1], np.float32)
    sink = np.zeros_like(u)
    for v in range(n):
        sink[v] = s.sink(v)
        if w.parent[v] >= 0:
            u[v] = s.labels(v)
    return {"u": u, "sink": sink}


def _same(a, b, what):
    for k in ("u", "sink"):
        assert np.array_equal(a[k], b[k].astype(np.float32)), "%s %s max |diff| %.3g" % (
            what, k, np.abs(a[k] - b[k]).max())


def _oracle(w, iterations, semantics=O.REF_CUDA):
    return O.solve(w.dims, w.parent, w.data, w.smooth, w.alpha, iterations, w.step, w.cc, want_sink=True,
                   semantics=semantics)


def _in_rounds(w, rounds, semantics=REF_CUDA, pipeline=False, zchunk=0, timing=False):
    """The state after solve(rounds[0]), solve_continue(rounds[1]), ..."""
    with HMFSolver(w.dims, w.parent, semantics) as s:
        _configure(s, w, rounds[0])
        s.set_pipeline(pipeline)
        if zchunk:
            s.set_zchunk(zchunk)
        s.set_timing(timing)
        s.solve()
        for k in rounds[1:]:
            s.set_params(k, w.step, w.cc)
            s.solve_continue()
        if pipeline:
            assert s.pipeline
        return _state(s, w)


@pytest.mark.parametrize("dims,parent,smooth_nodes,rounds", [
    ((37, 19, 11), [-1, 0, 0, 1, 1, 2, 2], (1, 5), (7, 5)),     # odd first round: flows moved to set 0
    ((37, 19, 11), [-1, 0, 0, 1, 1, 2, 2], (1, 5), (6, 6)),
    ((24, 16, 9), [-1, 0, 0, 0], (), (1, 1, 3, 0, 4)),           # several rounds, one of none
    ((23, 9, 8), [-1] + [0] * 17 + [1, 1], (3,), (5, 4)),       # 20 vertices: the table-driven sweep
])
def test_continue_equals_one_longer_solve(dims, parent, smooth_nodes, rounds):
    w = random_tree_problem(61, dims, parent, iterations=sum(rounds), smooth_nodes=smooth_nodes)
    ref = _oracle(w, sum(rounds))
    _same(_in_rounds(w, rounds), ref, "graphs %s" % (rounds,))
    _same(_in_rounds(w, rounds, timing=True), ref, "launch by launch %s" % (rounds,))


@pytest.mark.parametrize("rounds", [(9, 10), (8, 3)])
def test_continue_through_the_slab_pipeline(rounds):
    # 50 planes in chunks of 7: 8 slabs, replayed in graphs of several iterations
    w = random_tree_problem(62, (40, 30, 50), [-1, 0, 0, 1, 1, 2, 2], iterations=sum(rounds), smooth_nodes=(1, 2))
    _same(_in_rounds(w, rounds, pipeline=True, zchunk=7), _oracle(w, sum(rounds)), "pipelined %s" % (rounds,))


def test_continue_ref_cpu():
    w = random_tree_problem(63, (29, 13, 7), [-1, 0, 0, 1, 1], iterations=11, smooth_nodes=(1,))
    _same(_in_rounds(w, (4, 7), semantics=REF_CPU), _oracle(w, 11, semantics=O.REF_CPU), "REF_CPU")


def test_continue_a_batch():
    dims = [(21, 13, 9), (8, 30, 5)]
    parent = [-1, 0, 0, 1, 1]
    ws = [random_tree_problem(64 + i, d, parent, iterations=12, smooth_nodes=(1, 3)) for i, d in enumerate(dims)]
    for w in ws[1:]:
        w.alpha = dict(ws[0].alpha)
    with HMFBatchSolver(dims, parent) as b:
        for i, w in enumerate(ws):
            for leaf, d in w.data.items():
                b.set_data(i, leaf, d)
            for v, S in w.smooth.items():
                b.set_smoothness(i, v, S)
        for v, a in ws[0].alpha.items():
            b.set_smoothness_scalar(v, a)
        b.set_params(5, ws[0].step, ws[0].cc)
        b.solve()
        b.set_params(7, ws[0].step, ws[0].cc)
        b.solve_continue()
        for i, w in enumerate(ws):
            ref = _oracle(w, 12)
            n = len(parent)
            got = {"u": np.zeros((n,) + w.dims[::-1], np.float32), "sink": np.zeros((n,) + w.dims[::-1], np.float32)}
            for v in range(n):
                got["sink"][v] = b.sink(i, v)
                if parent[v] >= 0:
                    got["u"][v] = b.labels(i, v)
            _same(got, ref, "batch volume %d" % i)


def test_convergence_log_per_round_is_the_long_solves_log():
    w = random_tree_problem(65, (36, 20, 17), [-1, 0, 0, 1, 1, 2, 2], iterations=13, smooth_nodes=(1, 5))
    with HMFSolver(w.dims, w.parent) as s:
        _configure(s, w, 13)
        s.set_convergence_log(True)
        s.solve()
        whole = s.convergence()["max"]
        # rounds of 5, 5, 3 with an early-stopping style loop
        s.set_params(5, w.step, w.cc)
        s.solve()
        parts = [s.convergence()["max"]]
        s.solve_continue()
        parts.append(s.convergence()["max"])
        s.set_params(3, w.step, w.cc)
        s.solve_continue()
        parts.append(s.convergence()["max"])
        state = _state(s, w)
    assert [len(p) for p in parts] == [5, 5, 3]
    assert np.array_equal(np.concatenate(parts), whole)
    _same(state, _oracle(w, 13), "three rounds with the log")


def test_refusals():
    w = random_tree_problem(66, (12, 10, 6), [-1, 0, 0], iterations=3)
    with HMFSolver(w.dims, w.parent) as s:
        _configure(s, w, 3)
        with pytest.raises(HMFError) as e:
            s.solve_continue()
        assert e.value.code == HMF_ERR_STATE
        s.solve()
        s.solve_continue()
    with DAGSolver((12, 10, 6), 4, [(0, 1), (0, 2), (1, 3), (2, 3)]) as d:
        with pytest.raises(HMFError) as e:
            d.solve_continue()
        assert e.value.code == HMF_ERR_INVALID_ARGUMENT
    with HMFSolver(w.dims, w.parent, max_gpu_usage=0.5) as p:
        _configure(p, w, 3)
        with pytest.raises(HMFError) as e:
            p.solve_continue()
        assert e.value.code == HMF_ERR_STATE


@pytest.mark.parametrize("semantics,dims,plans,rounds", [
    (REF_CUDA, (37, 19, 45), ((20, 2), (20, 2)), (5, 6)),        # 4 blocks; odd rounds: flows of set 1 stored
    (REF_CUDA, (37, 19, 45), ((20, 2), (28, 3)), (4, 7)),        # another layout for the continuation
    (REF_CUDA, (32, 16, 20), ((64, 0), (64, 0), (64, 0)), (3, 1, 4)),  # one block: single rounds
    (REF_CUDA, (37, 19, 45), ((20, 2), (20, 2)), (6, 0)),        # a continuation of no iterations
    (REF_CPU, (29, 13, 17), ((0, 0), (0, 0)), (4, 7)),
])
def test_continue_out_of_core(semantics, dims, plans, rounds):
    """Out-of-core contexts continue from the host copy their last solve
    ended in: equal to one in-core solve of all the rounds' iterations."""
    w = random_tree_problem(67, dims, [-1, 0, 0, 1, 1, 2, 2], iterations=sum(rounds), smooth_nodes=(1, 4))
    ref = _in_rounds(w, (sum(rounds),), semantics=semantics)
    with HMFSolver(w.dims, w.parent, semantics, max_gpu_usage=0.75) as p:
        _configure(p, w, rounds[0])
        p.set_paged_plan(*plans[0])
        p.solve()
        for plan, k in zip(plans[1:], rounds[1:]):
            p.set_paged_plan(*plan)
            p.set_params(k, w.step, w.cc)
            p.solve_continue()
        got = _state(p, w)
    _same(got, ref, "out of core %s %s" % (plans, rounds))


def test_filter_continue_update():
    """The filter facade: Update() with 8 iterations, ContinueUpdate() with 5
    equals the oracle's 13; changing the extent in between is refused, and so
    is ContinueUpdate on the graph filter."""
    w = random_tree_problem(68, (21, 17, 9), [-1, 0, 0, 1, 1], iterations=13, smooth_nodes=(2,))
    f = HierarchicalMaxFlowSegmentation()
    f.SetHierarchy(w.parent)
    for leaf, d in w.data.items():
        f.SetDataInputDataObject(leaf, d)
    for v, S in w.smooth.items():
        f.SetSmoothnessInputDataObject(v, S)
    for v, a in w.alpha.items():
        f.AddSmoothnessScalar(v, a)
    f.SetNumberOfIterations(8)
    assert f.Update() == 1, f.GetLastError()
    f.SetNumberOfIterations(5)
    assert f.ContinueUpdate() == 1, f.GetLastError()
    ref = _oracle(w, 13)
    for leaf in w.leaves:
        assert np.array_equal(f.GetOutputDataObject(leaf), ref["u"][leaf].astype(np.float32)), leaf
    small = random_tree_problem(69, (7, 6, 5), [-1, 0, 0, 1, 1], iterations=2)
    for leaf, d in small.data.items():
        f.SetDataInputDataObject(leaf, d)
    f.SetSmoothnessInputDataObject(2, None)
    assert f.ContinueUpdate() == -1
    assert "ContinueUpdate follows an Update" in f.GetLastError()
    g = DirectedAcyclicGraphMaxFlowSegmentation()
    assert g.ContinueUpdate() == -1
