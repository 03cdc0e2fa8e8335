"""hmf_solve_adjoint (CUDA) against the oracle's adjoint restatement.

The forward states come from the solver's own kernels (bit-identical to the
FP32 oracle) and the backward kernels evaluate the oracle's FP32 operations
in the same order, so the per-voxel data gradients must agree exactly.  The
alpha gradients are sums over voxels reduced in a different order (double
precision): relative tolerance 1e-9.  GPU only."""
import numpy as np
import pytest

from oracle import oracle as O
from robartsvtk_gb300 import REF_CPU, HMFBatchSolver, HMFError, HMFSolver, adjoint_schedule
from robartsvtk_gb300.synthetic import random_tree_problem

pytestmark = pytest.mark.gpu

PARENT = [-1, 0, 0, 1, 1]


def problem(seed, dims, parent=PARENT, iterations=12, smooth_nodes=(1, 3)):
    w = random_tree_problem(seed, dims, parent, iterations=iterations, smooth_nodes=smooth_nodes, data_hi=2.0)
    rng = np.random.default_rng(seed + 1000)
    truth = rng.integers(0, len(w.leaves), size=w.dims[::-1]).astype(np.int32)
    return w, truth


def solver_for(w):
    s = HMFSolver(w.dims, w.parent)
    for leaf, d in w.data.items():
        s.set_data(leaf, d)
    for v, S in w.smooth.items():
        s.set_smoothness(v, S)
    for v, a in w.alpha.items():
        s.set_smoothness_scalar(v, a)
    s.set_params(w.iterations, w.step, w.cc)
    return s


def run_gpu(w, truth, checkpoint_every=0, max_slots=0):
    with solver_for(w) as s:
        if max_slots:
            s.set_adjoint_memory(max_state_slots=max_slots)
        loss = s.solve_adjoint(truth, checkpoint_every=checkpoint_every)
        dD = {l: s.data_gradient(l) for l in s.leaves}
        da = s.alpha_gradient()
        u = {v: s.labels(v) for v in range(len(w.parent)) if w.parent[v] >= 0}
        plan = s.adjoint_plan()
    return {"loss": loss, "dD": dD, "dalpha": da, "u": u, "plan": plan}


def run_oracle(w, truth):
    return O.adjoint(w.dims, w.parent, w.data, truth, w.smooth, w.alpha, w.iterations, w.step, w.cc, precision=32)


def assert_matches(g, o, w, what=""):
    assert abs(g["loss"] - o["loss"]) <= 1e-12 * abs(o["loss"]), (what, g["loss"], o["loss"])
    for l in w.leaves:
        diff = np.abs(g["dD"][l] - o["dD"][l]).max()
        assert np.array_equal(g["dD"][l], o["dD"][l]), "%s leaf %d: max |diff| %.3g (max |grad| %.3g)" % (
            what, l, diff, np.abs(o["dD"][l]).max())
    np.testing.assert_allclose(g["dalpha"], o["dalpha"], rtol=1e-9, atol=1e-15 * max(1.0, np.abs(o["dalpha"]).max()))


@pytest.fixture(params=["fused", "chain"])
def reverse_kernel(request, monkeypatch):
    """The fused reverse flow kernel (default) and the unfused per-vertex chain."""
    if request.param == "chain":
        monkeypatch.setenv("HMF_ADJOINT_KERNEL", "chain")
    else:
        monkeypatch.delenv("HMF_ADJOINT_KERNEL", raising=False)
    return request.param


@pytest.mark.parametrize("dims", [(9, 8, 7), (37, 29, 21), (61, 45, 37), (28, 27, 1), (1, 7, 11), (55, 1, 9),
                                  (5, 4, 3), (64, 50, 40)])
def test_adjoint_matches_oracle(dims, reverse_kernel):
    w, truth = problem(7, dims)
    g = run_gpu(w, truth)
    o = run_oracle(w, truth)
    assert_matches(g, o, w, "%s %s" % (dims, reverse_kernel))
    assert g["plan"]["recomputed_segments"] == 0  # everything fits: no recomputation


@pytest.mark.parametrize("k", [1, 3, 5])
def test_adjoint_checkpointing_recomputes_exactly(k, reverse_kernel):
    w, truth = problem(11, (33, 20, 17), iterations=13)
    o = run_oracle(w, truth)
    g = run_gpu(w, truth, checkpoint_every=k)
    n_ckpt = (13 + k - 1) // k
    assert g["plan"]["checkpoint_every"] == k and g["plan"]["recomputed_segments"] == n_ckpt - 1
    assert g["plan"]["state_slots"] == n_ckpt + k
    assert g["plan"]["forward_iterations"] == 13 + (n_ckpt - 1) * (k - 1)
    assert g["plan"]["backward_steps"] == 13
    assert_matches(g, o, w, "k=%d" % k)
    # the labels read after the adjoint are the forward solve's
    f = O.solve(w.dims, w.parent, w.data, w.smooth, w.alpha, w.iterations, w.step, w.cc)
    for v, u in g["u"].items():
        assert np.array_equal(u, f["u"][v].astype(np.float32)), v


@pytest.mark.parametrize("slots", [3, 4, 6])
def test_adjoint_fewest_forward_schedule_recomputes_exactly(slots, reverse_kernel):
    """Too few state slots for every state: the revolve-style schedule keeps
    and recomputes states recursively; the gradients do not change."""
    w, truth = problem(13, (33, 20, 17), iterations=13)
    g = run_gpu(w, truth, max_slots=slots)
    sched = adjoint_schedule(13, slots)
    assert g["plan"]["checkpoint_every"] == 0 and g["plan"]["state_slots"] == slots
    assert g["plan"]["forward_iterations"] == sum(1 for a in sched if a[0] == 0) > 13
    assert_matches(g, run_oracle(w, truth), w, "slots=%d" % slots)


def test_adjoint_config5_tree_with_few_slots():
    """The 15-vertex tree of the large workload (root -> 2 -> 4 -> 8), whose
    sweep reverse takes the table-driven kernel, under a 5-slot schedule."""
    parent = [-1, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6]
    w, truth = problem(17, (26, 21, 15), parent=parent, iterations=11, smooth_nodes=(1, 4, 9))
    g = run_gpu(w, truth, max_slots=5)
    assert g["plan"]["state_slots"] == 5
    assert_matches(g, run_oracle(w, truth), w, "tree8, 5 slots")


def test_adjoint_twenty_vertex_tree(reverse_kernel):
    """Twenty vertices (the staged sweep reverse for 9..32 vertices, leaves
    at several depths, ids not in pre-order) and the unfused chain."""
    parent = [-1, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 6, 6, 7, 8, 9, 9, 9]
    w, truth = problem(23, (27, 19, 14), parent=parent, iterations=8, smooth_nodes=(2, 7, 13))
    assert_matches(run_gpu(w, truth), run_oracle(w, truth), w, "tree20")


def test_adjoint_flat_tree_without_smoothness_images(reverse_kernel):
    w, truth = problem(21, (40, 24, 18), parent=[-1, 0, 0, 0, 0], iterations=10, smooth_nodes=())
    assert_matches(run_gpu(w, truth), run_oracle(w, truth), w, "flat4")


def test_adjoint_two_level_tree_in_preorder(reverse_kernel):
    """Vertex ids in pre-order (the sweep reverse's compile-time order)."""
    w, truth = problem(71, (45, 31, 26), parent=[-1, 0, 1, 1, 0, 4, 4], iterations=9, smooth_nodes=(1, 2, 5))
    assert_matches(run_gpu(w, truth), run_oracle(w, truth), w, "tree4")


def test_adjoint_deep_tree(reverse_kernel):
    parent = [-1, 0, 0, 1, 1, 2, 2, 3, 3]
    w, truth = problem(31, (23, 19, 13), parent=parent, iterations=9, smooth_nodes=(1, 4, 6))
    assert_matches(run_gpu(w, truth), run_oracle(w, truth), w, "deep")


def test_adjoint_zero_iterations():
    w, truth = problem(41, (12, 10, 8), iterations=0)
    g = run_gpu(w, truth)
    o = run_oracle(w, truth)
    assert abs(g["loss"] - o["loss"]) <= 1e-12 * abs(o["loss"])
    for l in w.leaves:
        assert np.all(g["dD"][l] == 0.0)


def test_adjoint_device_truth_and_torch_autograd():
    torch = pytest.importorskip("torch")
    from robartsvtk_gb300.autograd import hmf_loss

    w, truth = problem(51, (30, 22, 14), iterations=8)
    o = run_oracle(w, truth)
    with solver_for(w) as s:
        data = torch.stack([torch.from_numpy(w.data[l]) for l in s.leaves]).cuda().requires_grad_(True)
        alpha = torch.tensor([w.alpha.get(v, 1.0) for v in range(len(w.parent))], dtype=torch.float64,
                             requires_grad=True)
        loss = hmf_loss(s, data, alpha, torch.from_numpy(truth).cuda())
        (2.0 * loss).backward()
    assert abs(loss.item() - o["loss"]) <= 1e-12 * abs(o["loss"])
    for j, l in enumerate(w.leaves):
        np.testing.assert_array_equal(data.grad[j].cpu().numpy(), (2.0 * o["dD"][l]).astype(np.float32))
    np.testing.assert_allclose(alpha.grad.numpy(), 2.0 * o["dalpha"], rtol=1e-9, atol=1e-15)


def test_adjoint_errors():
    w, truth = problem(61, (10, 9, 8), iterations=3)
    with solver_for(w) as s:
        with pytest.raises(HMFError, match="has not run"):
            s.data_gradient(w.leaves[0])
        bad = truth.copy()
        bad[0, 0, 0] = len(w.leaves)
        with pytest.raises(HMFError, match="class index"):
            s.solve_adjoint(bad)
        s.solve_adjoint(truth)
        with pytest.raises(HMFError, match="leaves only"):
            s.data_gradient(1)
        with pytest.raises(HMFError, match="eps"):
            s.solve_adjoint(truth, eps=0.0)
        s.set_adjoint_memory(max_state_slots=2)  # x_0 and one more: no schedule for 3 iterations
        with pytest.raises(HMFError, match="state slots"):
            s.solve_adjoint(truth)
        with pytest.raises(HMFError, match="more than the 2 allowed"):
            s.solve_adjoint(truth, checkpoint_every=1)
        with pytest.raises(HMFError, match=">= 0"):
            s.set_adjoint_memory(max_bytes=-1)
    with HMFSolver(w.dims, w.parent, semantics=REF_CPU) as s:
        with pytest.raises(HMFError, match="REF_CUDA"):
            s.solve_adjoint(truth)
    with HMFBatchSolver([(4, 4, 4), (3, 3, 3)], [-1, 0, 0]) as b:
        lib = b._lib
        import ctypes
        t = np.zeros(64, np.int32)
        rc = lib.hmf_solve_adjoint(b._ctx, t.ctypes.data, 0, 0, 1e-6, ctypes.byref(ctypes.c_double()), None)
        assert rc == -1 and b"single-volume" in lib.hmf_last_error(b._ctx)
