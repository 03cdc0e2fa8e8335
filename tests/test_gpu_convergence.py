"""Per-iteration convergence log (hmf_set_convergence_log): max and mean of
|u_new - u_old| over non-root vertices and voxels, reduced inside the label
sweep.  GPU only.

Bar: the per-iteration maximum equals the one computed on the host from the
FP32 oracle's state after each iteration (the labels are bit-identical, the
differences are formed in float), the mean agrees to 1e-6 relative (its sum
runs in another order).
"""
import numpy as np
import pytest

from oracle import oracle as O
from robartsvtk_gb300 import HMFBatchSolver, HMFError, HMFSolver
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


def oracle_changes(w):
    """max and mean |du| per iteration from the oracle's FP32 state."""
    n = len(w.parent)
    nonroot = [v for v in range(n) if w.parent[v] >= 0]
    st = O.new_state(w.dims, n)
    O.iterate(w.dims, w.parent, w.data, st, w.smooth or None, w.alpha, iterations=0, step=w.step, cc=w.cc,
              init=True)
    mx, mean = [], []
    for _ in range(w.iterations):
        before = st["u"][nonroot].copy()
        O.iterate(w.dims, w.parent, w.data, st, w.smooth or None, w.alpha, iterations=1, step=w.step, cc=w.cc)
        d = np.abs(st["u"][nonroot] - before)  # float32, as the kernel forms it
        mx.append(float(d.max()))
        mean.append(float(d.astype(np.float64).sum()) / d.size)
    return np.array(mx), np.array(mean)


@pytest.mark.parametrize("dims,parent,smooth_nodes", [
    ((36, 20, 17), [-1, 0, 0, 1, 1, 2, 2], (1, 5)),   # VX a multiple of 4
    ((37, 19, 11), [-1, 0, 0, 0], ()),                # padded rows
    ((23, 9, 8), [-1] + [0] * 17 + [1, 1], (3,)),     # 20 vertices: the table-driven sweep
])
def test_convergence_log_matches_the_oracle(dims, parent, smooth_nodes):
    w = random_tree_problem(51, dims, parent, iterations=12, smooth_nodes=smooth_nodes)
    mx, mean = oracle_changes(w)
    with HMFSolver(w.dims, w.parent) as s:
        _configure(s, w)
        s.set_convergence_log(True)
        s.solve()
        got = s.convergence()
        # a second solve logs afresh (graph replay, same numbers)
        s.solve()
        again = s.convergence()
    assert len(got["max"]) == w.iterations
    assert np.array_equal(got["max"], mx)
    np.testing.assert_allclose(got["mean"], mean, rtol=1e-6)
    assert np.array_equal(again["max"], got["max"])


def test_convergence_log_off_and_timed_path():
    w = random_tree_problem(52, (20, 12, 9), [-1, 0, 0, 1, 1], iterations=7)
    with HMFSolver(w.dims, w.parent) as s:
        _configure(s, w)
        s.solve()
        assert len(s.convergence()["max"]) == 0
        s.set_convergence_log(True)
        s.set_timing(True)  # launches one by one: the same log
        s.solve()
        timed = s.convergence()
        s.set_timing(False)
        s.solve()
        graphed = s.convergence()
        assert np.array_equal(timed["max"], graphed["max"])
        s.set_convergence_log(False)
        s.solve()
        assert len(s.convergence()["max"]) == 0


def test_convergence_log_of_a_batch_pools_its_volumes():
    ws = [random_tree_problem(53 + k, d, [-1, 0, 0, 0], iterations=6) for k, d in
          enumerate([(16, 10, 9), (24, 7, 12)])]
    ws[1].alpha = dict(ws[0].alpha)  # a batch shares one set of smoothness weights
    with HMFBatchSolver([w.dims for w in ws], ws[0].parent) as b:
        for k, w in enumerate(ws):
            for leaf, d in w.data.items():
                b.set_data(k, leaf, d)
        for v, a in ws[0].alpha.items():
            b.set_smoothness_scalar(v, a)
        b.set_params(6, ws[0].step, ws[0].cc)
        b.set_convergence_log(True)
        b.solve()
        got = b.convergence()
    per = [oracle_changes(w) for w in ws]
    assert np.array_equal(got["max"], np.maximum(per[0][0], per[1][0]))
    sizes = [w.nvox * (len(w.parent) - 1) for w in ws]
    pooled = (per[0][1] * sizes[0] + per[1][1] * sizes[1]) / sum(sizes)
    np.testing.assert_allclose(got["mean"], pooled, rtol=1e-6)


def test_convergence_log_refusals():
    with HMFBatchSolver([(15, 8, 8), (16, 8, 8)], [-1, 0, 0]) as b:
        with pytest.raises(HMFError, match="multiple of 4"):
            b.set_convergence_log(True)
    from robartsvtk_gb300 import REF_CPU
    with HMFSolver((8, 8, 8), [-1, 0, 0], REF_CPU) as s:
        with pytest.raises(HMFError, match="REF_CUDA"):
            s.set_convergence_log(True)
