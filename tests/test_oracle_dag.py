"""The DAG solver oracle (oracle/dag_oracle.cpp) against the reference's own
kernels run in the same task order (tests/golden/ref_dag_golden.npz, made by
tests/golden/make_golden.py --ref-dag from CUDA_hierarchicalmaxflow.cu and
CUDA_commonKernels.cu compiled unmodified), and its graph handling.  The
reference kernels are compiled with fused multiply-adds, the oracle without:
labels agree to 2e-6, sinks and source buffers to 2e-6 relative.  CPU only."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from tests.golden.cases import DAG_CASES, dag_problem

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ref_dag_golden.npz")


def run(w, **kw):
    return O.dag_solve(w.dims, w.n, w.edges, w.data, w.weights, w.smooth, w.alpha, w.iterations, w.step, w.cc, **kw)


@pytest.mark.parametrize("name", sorted(DAG_CASES))
def test_oracle_matches_reference_kernels(name):
    g = np.load(GOLDEN)
    w = dag_problem(name)
    r = run(w)
    root = O.dag_forward(w.n, w.edges, w.weights)[0]
    nr = [v for v in range(w.n) if v != root]
    scale = np.abs(g[name + "/sink"]).max()
    assert np.abs(r["u"][nr] - g[name + "/u"][nr]).max() <= 2e-6
    assert np.abs(r["sink"] - g[name + "/sink"]).max() <= 2e-6 * scale
    assert np.abs(r["inc"][nr] - g[name + "/inc"][nr]).max() <= 2e-6 * scale
    # the FP64 oracle is as close: the difference is rounding, not order
    r64 = run(w, precision=64)
    assert np.abs(r64["u"][nr] - g[name + "/u"][nr]).max() <= 2e-6


def test_forward_order_is_level_by_level():
    # 4 is a child of the root and of 2; its level is 3 (the longest path)
    edges = [(0, 1), (1, 2), (2, 3), (2, 4), (0, 4), (1, 5)]
    assert O.dag_forward(6, edges) == [0, 1, 2, 5, 3, 4]


def test_zero_iterations_is_the_initial_labelling():
    w = dag_problem("dag_diamond_9x7x5")
    w.iterations = 0
    r = run(w)
    leaves = [3, 4, 5]
    m = np.minimum.reduce([w.data[l] for l in leaves])
    ind = np.stack([(w.data[l] == m).astype(np.float64) for l in leaves])
    np.testing.assert_array_equal(r["u"][leaves], (ind / ind.sum(0)).astype(np.float32))
    # branches: sum of w * child label, w = 1 / #parents of the child
    np.testing.assert_allclose(r["u"][1], r["u"][3] * 0.5 + r["u"][4], rtol=1e-6)
    for v in range(1, 6):
        np.testing.assert_array_equal(r["sink"][v], m)


@pytest.mark.parametrize("edges,weights,msg", [
    ([(0, 1), (1, 2), (2, 1)], None, "cycle"),
    ([(0, 1), (2, 1)], None, "more than one root"),
    ([(0, 1), (1, 2), (2, 3), (3, 1)], None, "cycle"),
    ([(0, 1), (0, 5)], None, "out of range"),
    ([(0, 1), (0, 2)], [1.0, 0.0], "positive"),
])
def test_graph_errors(edges, weights, msg):
    n = 1 + max(max(p, c) for p, c in edges if c < 5)
    with pytest.raises(RuntimeError, match=msg):
        O.dag_forward(n, edges, weights)
