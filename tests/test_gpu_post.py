"""Vote and energy decomposition (hmf_vote, hmf_get_vote,
hmf_decomposition_energy, hmf_get_energy) against the oracle's restatement
and the reference kernels' golden vectors.  Votes are integer work: exact.
Energies are FP64 sums of FP32 per-voxel terms formed in the reference's
order, summed in another order than the oracle: relative tolerance 1e-11.
GPU only."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from robartsvtk_gb300 import REF_CPU, REF_CUDA, HMFBatchSolver, HMFError, HMFSolver, decomposition_energy, vote
from robartsvtk_gb300.synthetic import random_tree_problem

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ref_post_golden.npz")
PARENT = [-1, 0, 0, 1, 1, 2, 2]


def tie_images(seed, shape, n):
    rng = np.random.default_rng(seed)
    return [(rng.integers(0, 3, size=shape) / 3.0).astype(np.float32) for _ in range(n)]


@pytest.mark.parametrize("semantics", [REF_CUDA, REF_CPU])
def test_vote_host_and_device(semantics):
    torch = pytest.importorskip("torch")
    ins = tie_images(1, (11, 9, 7), 5)
    vals = [4, 9, 2, 7, 0]
    want = O.vote(ins, vals, semantics=semantics)
    assert np.array_equal(vote(ins, vals, semantics=semantics), want)
    dev = [torch.from_numpy(a).cuda() for a in ins]
    got = vote(dev, vals, semantics=semantics)
    assert got.is_cuda and np.array_equal(got.cpu().numpy(), want)


def test_vote_matches_reference_kernel_golden():
    g = np.load(GOLDEN)
    names = sorted({k.split("/")[0] for k in g.files})
    for name in names:
        ins = list(g[name + "/vote_inputs"])
        vals = g[name + "/vote_values"]
        assert np.array_equal(vote(ins, vals, semantics=REF_CUDA), g[name + "/vote"]), name


def test_energy_matches_reference_kernel_golden():
    g = np.load(GOLDEN)
    names = sorted({k.split("/")[0] for k in g.files})
    for name in names:
        lab = g[name + "/label"]
        sm = g[name + "/smooth"]
        dims = lab.shape[::-1]
        zero = np.zeros_like(lab)
        # root -> {1: leaf with the labelling, 2: leaf at zero}: f[1] = sum of the gradient terms
        _, f = decomposition_energy(dims, [-1, 0, 0], {1: zero, 2: zero}, {1: lab, 2: zero})
        want = g[name + "/grad"].astype(np.float64).sum()
        assert abs(f[1] - want) <= 1e-11 * abs(want), name
        _, f = decomposition_energy(dims, [-1, 0, 0], {1: zero, 2: zero}, {1: lab, 2: zero}, smooth={1: sm})
        want = g[name + "/grad_smooth"].astype(np.float64).sum()
        assert abs(f[1] - want) <= 1e-11 * abs(want), name


def solved(w, semantics=REF_CUDA):
    s = HMFSolver(w.dims, w.parent, semantics)
    for leaf, d in w.data.items():
        s.set_data(leaf, d)
    for v, S in w.smooth.items():
        s.set_smoothness(v, S)
    for v, a in w.alpha.items():
        s.set_smoothness_scalar(v, a)
    s.set_params(w.iterations, w.step, w.cc)
    s.solve()
    return s


@pytest.mark.parametrize("semantics", [REF_CUDA, REF_CPU])
def test_context_vote_matches_oracle(semantics):
    w = random_tree_problem(5, (29, 17, 13), PARENT, iterations=20, smooth_nodes=(1, 4))
    o = O.solve(w.dims, w.parent, w.data, w.smooth, w.alpha, w.iterations, w.step, w.cc, semantics=semantics)
    with solved(w, semantics) as s:
        got = s.vote()
        leaves = s.leaves
    want = O.vote([o["u"][l].astype(np.float32) for l in leaves], leaves, semantics=semantics)
    assert np.array_equal(got, want)


def test_energy_standalone_matches_oracle():
    rng = np.random.default_rng(7)
    dims = (23, 19, 11)
    shape = dims[::-1]
    leaves = [3, 4, 5, 6]
    lab = {l: rng.random(shape).astype(np.float32) for l in leaves}
    dat = {l: rng.random(shape).astype(np.float32) for l in leaves}
    sm = {1: rng.random(shape).astype(np.float32), 4: rng.random(shape).astype(np.float32)}
    o = O.energy(dims, PARENT, dat, lab, sm)
    f0, f = decomposition_energy(dims, PARENT, dat, lab, sm)
    assert abs(f0 - o["f0"]) <= 1e-11 * abs(o["f0"])
    np.testing.assert_allclose(f, o["f"], rtol=1e-11, atol=0)
    torch = pytest.importorskip("torch")
    cuda = lambda d: {k: torch.from_numpy(v).cuda() for k, v in d.items()}  # noqa: E731
    f0d, fd = decomposition_energy(dims, PARENT, cuda(dat), cuda(lab), cuda(sm))
    assert abs(f0d - o["f0"]) <= 1e-11 * abs(o["f0"])
    np.testing.assert_allclose(fd, o["f"], rtol=1e-11, atol=0)


@pytest.mark.parametrize("dims", [(1, 1, 1), (1, 7, 5), (33, 9, 3), (64, 17, 70), (5, 40, 1), (40, 1, 33),
                                  (97, 23, 41)])
def test_energy_march_shapes(dims):
    """The z-marching kernel's tiles (32 x 8 columns) and z chunks on ragged
    and degenerate volumes: partial tiles, one-voxel axes, chunk borders."""
    rng = np.random.default_rng(sum(dims))
    shape = dims[::-1]
    leaves = [3, 4, 5, 6]
    lab = {l: rng.random(shape).astype(np.float32) for l in leaves}
    dat = {l: rng.random(shape).astype(np.float32) for l in leaves}
    sm = {2: rng.random(shape).astype(np.float32), 5: rng.random(shape).astype(np.float32)}
    o = O.energy(dims, PARENT, dat, lab, sm)
    f0, f = decomposition_energy(dims, PARENT, dat, lab, sm)
    assert abs(f0 - o["f0"]) <= 1e-11 * abs(o["f0"])
    np.testing.assert_allclose(f, o["f"], rtol=1e-11, atol=1e-30)


def test_energy_large_tree_and_dense_quads():
    """Eleven non-root vertices (past the register-resident kernels' eight) and
    rows a multiple of four wide (the four-voxel vote)."""
    rng = np.random.default_rng(17)
    parent = [-1, 0, 0, 1, 1, 1, 2, 2, 3, 3, 6, 6]
    dims = (16, 9, 7)
    shape = dims[::-1]
    leaves = [v for v in range(1, len(parent)) if v not in parent]
    lab = {l: rng.random(shape).astype(np.float32) for l in leaves}
    dat = {l: rng.random(shape).astype(np.float32) for l in leaves}
    sm = {4: rng.random(shape).astype(np.float32), 6: rng.random(shape).astype(np.float32)}
    o = O.energy(dims, parent, dat, lab, sm)
    f0, f = decomposition_energy(dims, parent, dat, lab, sm)
    assert abs(f0 - o["f0"]) <= 1e-11 * abs(o["f0"])
    np.testing.assert_allclose(f, o["f"], rtol=1e-11, atol=0)
    ins = tie_images(3, shape, 6)
    vals = [11, 3, 8, 1, 5, 2]
    for semantics in (REF_CUDA, REF_CPU):
        assert np.array_equal(vote(ins, vals, semantics=semantics), O.vote(ins, vals, semantics=semantics))


def test_context_energy_matches_oracle():
    w = random_tree_problem(9, (31, 22, 15), PARENT, iterations=15, smooth_nodes=(1, 4, 5))
    o = O.solve(w.dims, w.parent, w.data, w.smooth, w.alpha, w.iterations, w.step, w.cc)
    with solved(w) as s:
        f0, f = s.energy()
        leaves = s.leaves
    want = O.energy(w.dims, w.parent, w.data, {l: o["u"][l].astype(np.float32) for l in leaves}, w.smooth)
    assert abs(f0 - want["f0"]) <= 1e-11 * abs(want["f0"])
    np.testing.assert_allclose(f, want["f"], rtol=1e-11, atol=0)


def test_batch_vote_and_energy_per_volume():
    ws = [random_tree_problem(30 + i, d, [-1, 0, 0, 0], iterations=10, smooth_nodes=(2,))
          for i, d in enumerate([(17, 9, 8), (8, 21, 5), (12, 12, 12)])]
    for w in ws[1:]:
        w.alpha = dict(ws[0].alpha)
    with HMFBatchSolver([w.dims for w in ws], ws[0].parent) as b:
        for i, w in enumerate(ws):
            for leaf, d in w.data.items():
                b.set_data(i, leaf, d)
            for v, S in w.smooth.items():
                b.set_smoothness(i, v, S)
        for v, a in ws[0].alpha.items():
            b.set_smoothness_scalar(v, a)
        b.set_params(ws[0].iterations, ws[0].step, ws[0].cc)
        b.solve()
        for i, w in enumerate(ws):
            o = O.solve(w.dims, w.parent, w.data, w.smooth, w.alpha, w.iterations, w.step, w.cc)
            leaves = b.leaves
            labs = {l: o["u"][l].astype(np.float32) for l in leaves}
            assert np.array_equal(b.vote(i), O.vote([labs[l] for l in leaves], leaves))
            f0, f = b.energy(i)
            want = O.energy(w.dims, w.parent, w.data, labs, w.smooth)
            assert abs(f0 - want["f0"]) <= 1e-11 * abs(want["f0"])
            np.testing.assert_allclose(f, want["f"], rtol=1e-11, atol=0)


def test_post_errors():
    with pytest.raises(HMFError):
        vote([], [])
    with HMFSolver((4, 4, 4), [-1, 0, 0]) as s:
        with pytest.raises(HMFError, match="has not run"):
            s.vote()
        with pytest.raises(HMFError, match="has not run"):
            s.energy()
    with pytest.raises(HMFError, match="root"):
        decomposition_energy((3, 3, 3), [-1, -1], {}, {})
