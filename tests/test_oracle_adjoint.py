"""The oracle's reverse-mode adjoint (oracle.adjoint, FP64) against central
finite differences of its own forward loss.  CPU only.

The inputs are float32 (as the solver takes them), so each difference
quotient divides by the perturbation that float32 actually represents."""
import numpy as np
import pytest

from oracle import oracle as O
from robartsvtk_gb300.synthetic import random_tree_problem

PARENT = [-1, 0, 0, 1, 1]


def _problem(seed=3, dims=(9, 8, 7), iterations=30):
    w = random_tree_problem(seed, dims, PARENT, iterations=iterations, smooth_nodes=(1, 3), data_hi=2.0)
    rng = np.random.default_rng(seed)
    truth = rng.integers(0, len(w.leaves), size=w.dims[::-1]).astype(np.int32)
    return w, truth


def _loss(w, truth, data=None, alpha=None):
    return O.adjoint(w.dims, w.parent, data or w.data, truth, w.smooth, alpha or w.alpha, w.iterations, w.step,
                     w.cc)["loss"]


def test_adjoint_data_gradient_matches_central_differences():
    w, truth = _problem()
    base = O.adjoint(w.dims, w.parent, w.data, truth, w.smooth, w.alpha, w.iterations, w.step, w.cc)
    rng = np.random.default_rng(11)
    h = 3e-5  # small enough that a step rarely crosses a kink of the iteration
    good, tried = 0, 0
    for _ in range(24):
        leaf = w.leaves[rng.integers(len(w.leaves))]
        idx = tuple(int(rng.integers(0, s)) for s in truth.shape)
        x = float(w.data[leaf][idx])
        xp, xm = np.float32(x + h), np.float32(x - h)
        if xm < 0:
            continue
        dp = {k: v.copy() for k, v in w.data.items()}
        dm = {k: v.copy() for k, v in w.data.items()}
        dp[leaf][idx] = xp
        dm[leaf][idx] = xm
        fd = (_loss(w, truth, data=dp) - _loss(w, truth, data=dm)) / (float(xp) - float(xm))
        ad = base["dD"][leaf][idx]
        tried += 1
        good += abs(fd - ad) <= 1e-4 * max(abs(fd), abs(ad)) + 1e-9
    # a probe whose +-h step crosses a kink of the iteration (a clamp or a
    # saturation switching) legitimately disagrees; nearly all must agree
    assert tried >= 20 and good >= tried - 2, (good, tried)


def test_adjoint_alpha_gradient_matches_central_differences():
    w, truth = _problem()
    base = O.adjoint(w.dims, w.parent, w.data, truth, w.smooth, w.alpha, w.iterations, w.step, w.cc)
    h = 3e-5
    for v in range(1, len(PARENT)):
        a = float(w.alpha[v])
        ap, am = float(np.float32(a + h)), float(np.float32(a - h))  # the solver stores alpha as float
        fd = (_loss(w, truth, alpha={**w.alpha, v: ap}) - _loss(w, truth, alpha={**w.alpha, v: am})) / (ap - am)
        ad = base["dalpha"][v]
        assert abs(fd - ad) <= 1e-4 * max(abs(fd), abs(ad)) + 1e-9, (v, fd, ad)
    assert base["dalpha"][0] == 0.0


def test_adjoint_fp32_close_to_fp64():
    w, truth = _problem(seed=5, dims=(11, 7, 6), iterations=20)
    a64 = O.adjoint(w.dims, w.parent, w.data, truth, w.smooth, w.alpha, w.iterations, w.step, w.cc, precision=64)
    a32 = O.adjoint(w.dims, w.parent, w.data, truth, w.smooth, w.alpha, w.iterations, w.step, w.cc, precision=32)
    assert abs(a32["loss"] - a64["loss"]) <= 1e-5 * abs(a64["loss"])
    scale = np.abs(a64["dD"]).max()
    assert np.abs(a32["dD"] - a64["dD"]).max() <= 1e-3 * scale
    np.testing.assert_allclose(a32["dalpha"], a64["dalpha"], rtol=1e-2, atol=1e-6 * np.abs(a64["dalpha"]).max())


def test_adjoint_zero_iterations_and_bad_truth():
    w, truth = _problem(iterations=0)
    r = O.adjoint(w.dims, w.parent, w.data, truth, w.smooth, w.alpha, 0, w.step, w.cc)
    assert np.all(r["dD"] == 0.0) and np.all(r["dalpha"] == 0.0)
    bad = truth.copy()
    bad[0, 0, 0] = len(w.leaves)
    with pytest.raises(RuntimeError, match="truth class"):
        O.adjoint(w.dims, w.parent, w.data, bad, w.smooth, w.alpha, 3, w.step, w.cc)
