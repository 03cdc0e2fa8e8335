"""hmf_create_dag (the directed-acyclic-graph solver of
vtkCudaDirectedAcyclicGraphMaxFlowSegmentation) against the oracle
(oracle/dag_oracle.cpp) and, through it, the reference's own kernels
(tests/golden/ref_dag_golden.npz).  The kernels evaluate the oracle's FP32
operations in the same order: labels and sinks must be bit-identical.
GPU only."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from robartsvtk_gb300 import REF_CPU, DAGSolver, DirectedAcyclicGraphMaxFlowSegmentation, HMFError, vote
from tests.golden.cases import DAG_CASES, DagProblem, dag_problem

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ref_dag_golden.npz")


def gpu_solve(w, timing=False, device_inputs=False):
    s = DAGSolver(w.dims, w.n, w.edges, w.weights)
    keep = []
    for leaf, d in w.data.items():
        if device_inputs:
            import torch

            d = torch.from_numpy(d).cuda()
            keep.append(d)
        s.set_data(leaf, d)
    for v, S in w.smooth.items():
        s.set_smoothness(v, S)
    for v, a in w.alpha.items():
        s.set_smoothness_scalar(v, a)
    s.set_params(w.iterations, w.step, w.cc)
    if timing:
        s.set_timing(True)
    s.solve()
    root = O.dag_forward(w.n, w.edges, w.weights)[0]
    out = {"u": {v: s.labels(v) for v in range(w.n) if v != root}, "sink": {v: s.sink(v) for v in range(w.n)},
           "leaves": s.leaves, "root": root}
    s.close()
    return out


def oracle_solve(w, precision=32):
    return O.dag_solve(w.dims, w.n, w.edges, w.data, w.weights, w.smooth, w.alpha, w.iterations, w.step, w.cc,
                       precision=precision)


def assert_exact(g, o, what):
    for v, u in g["u"].items():
        assert np.array_equal(u, o["u"][v].astype(np.float32)), "%s label %d: max |diff| %.3g" % (
            what, v, np.abs(u - o["u"][v]).max())
    for v, s in g["sink"].items():
        assert np.array_equal(s, o["sink"][v].astype(np.float32)), "%s sink %d: max |diff| %.3g" % (
            what, v, np.abs(s - o["sink"][v]).max())


@pytest.fixture(params=["default", "generic", "simple"])
def dag_kernel(request, monkeypatch):
    """The default graph sweep (graph in kernel parameters for up to 8
    nodes), the table-driven bulk-staged one and the direct one."""
    if request.param == "default":
        monkeypatch.delenv("HMF_DAG_KERNEL", raising=False)
    else:
        monkeypatch.setenv("HMF_DAG_KERNEL", request.param)
    return request.param


@pytest.mark.parametrize("name", sorted(DAG_CASES))
def test_dag_matches_oracle_and_reference_kernels(name, dag_kernel):
    w = dag_problem(name)
    g = gpu_solve(w)
    assert_exact(g, oracle_solve(w), name)
    gold = np.load(GOLDEN)
    for v, u in g["u"].items():
        assert np.abs(u - gold[name + "/u"][v]).max() <= 2e-6
    assert g["leaves"] == [v for v in O.dag_forward(w.n, w.edges, w.weights) if v in w.data]


def random_dag(seed, dims, n, edges, weights=None, iterations=30, smooth_nodes=()):
    rng = np.random.default_rng(seed)
    shape = dims[::-1]
    kids = {p for p, _ in edges}
    data = {v: rng.uniform(0, 3.0, size=shape).astype(np.float32) for v in range(n) if v not in kids}
    smooth = {v: rng.uniform(0, 1, size=shape).astype(np.float32) for v in smooth_nodes}
    alpha = {v: float(rng.uniform(0.05, 1.0)) for v in range(1, n)}
    return DagProblem(dims, n, edges, weights, data, smooth, alpha, iterations)


DIAMOND = [(0, 1), (0, 2), (1, 3), (2, 3), (1, 4), (2, 5)]


@pytest.mark.parametrize("dims", [(37, 29, 21), (61, 45, 37), (1, 7, 11), (55, 1, 9), (28, 27, 1), (5, 4, 3)])
def test_dag_shapes(dims, dag_kernel):
    w = random_dag(3, dims, 6, DIAMOND, iterations=17, smooth_nodes=(2, 3))
    assert_exact(gpu_solve(w), oracle_solve(w), str(dims))


def test_dag_many_iterations_deep_graph_and_weights(dag_kernel):
    # three levels, a skip edge from the root, a leaf with three parents
    edges = [(0, 1), (0, 2), (1, 3), (2, 3), (1, 4), (3, 5), (3, 6), (4, 6), (2, 6), (0, 7), (4, 8)]
    weights = [1.0, 0.5, 0.7, 1.3, 1.0, 0.9, 0.4, 0.8, 1.1, 2.0, 0.6]
    w = random_dag(5, (33, 20, 17), 9, edges, weights, iterations=120, smooth_nodes=(1, 5))
    g = gpu_solve(w)
    assert_exact(g, oracle_solve(w), "deep")
    # FP64 error of the FP32 solve, stated
    o64 = oracle_solve(w, precision=64)
    err = max(np.abs(g["u"][v] - o64["u"][v]).max() for v in g["u"])
    print("DAG FP32 vs FP64 label error after 120 iterations: %.3g" % err)
    assert err <= 1e-4


def test_dag_timing_path_and_device_inputs_agree():
    w = random_dag(7, (24, 18, 12), 6, DIAMOND, iterations=9)
    a = gpu_solve(w)
    b = gpu_solve(w, timing=True, device_inputs=True)
    for v in a["u"]:
        assert np.array_equal(a["u"][v], b["u"][v])


@pytest.mark.parametrize("iterations", [0, 1, 2])
def test_dag_few_iterations(iterations, dag_kernel):
    w = random_dag(9, (13, 11, 7), 6, DIAMOND, iterations=iterations, smooth_nodes=(4,))
    assert_exact(gpu_solve(w), oracle_solve(w), "T=%d" % iterations)


def test_dag_vote_and_facade():
    w = dag_problem("dag_weighted_11x6x7")
    f = DirectedAcyclicGraphMaxFlowSegmentation()
    f.SetStructure(w.n, w.edges, w.weights)
    for v, a in w.alpha.items():
        f.AddSmoothnessScalar(v, a)
    for v, d in w.data.items():
        f.SetDataInputDataObject(v, d)
    for v, S in w.smooth.items():
        f.SetSmoothnessInputDataObject(v, S)
    f.SetNumberOfIterations(w.iterations)
    assert f.Update() == 1
    o = oracle_solve(w)
    for leaf in w.data:
        assert np.array_equal(f.GetOutputDataObject(leaf), o["u"][leaf].astype(np.float32))
    leaves = f._solver.leaves
    got = f._solver.vote()
    want = O.vote([o["u"][l].astype(np.float32) for l in leaves], leaves)
    assert np.array_equal(got, want)
    assert np.array_equal(vote([f.GetOutputDataObject(l) for l in leaves], leaves), want)


def test_dag_errors():
    w = dag_problem("dag_diamond_9x7x5")
    with pytest.raises(HMFError, match="cycle"):
        DAGSolver(w.dims, 4, [(0, 1), (1, 2), (2, 3), (3, 1)])
    with pytest.raises(HMFError, match="more than one root"):
        DAGSolver(w.dims, 3, [(0, 1), (2, 1)])
    with pytest.raises(HMFError, match="positive"):
        DAGSolver(w.dims, 3, [(0, 1), (0, 2)], [1.0, -1.0])
    import ctypes

    from robartsvtk_gb300 import _capi

    lib = _capi.load()
    ctx = ctypes.c_void_p()
    ep = (ctypes.c_int * 2)(0, 0)
    ec = (ctypes.c_int * 2)(1, 2)
    assert lib.hmf_create_dag(ctypes.byref(ctx), 4, 4, 4, 3, 2, ep, ec, None, REF_CPU, 0) < 0
    assert b"REF_CPU" in lib.hmf_last_error(None)
    s = DAGSolver(w.dims, w.n, w.edges)
    for leaf, d in w.data.items():
        s.set_data(leaf, d)
    s.set_params(3, 0.1, 0.25)
    s.solve()
    with pytest.raises(HMFError, match="trees"):
        s.energy()
    truth = np.zeros(w.dims[::-1], np.int32)
    with pytest.raises(HMFError, match="trees"):
        s.solve_adjoint(truth)
    s.close()
