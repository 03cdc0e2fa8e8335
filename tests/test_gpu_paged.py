"""Out-of-core solves (hmf_create_paged) on the GPU against the in-core solve.

The state lives in pinned host memory and blocks of z-planes are iterated on
the device in rounds; the blocks run the in-core kernels, so labels and sinks
must equal hmf_create + hmf_solve's bit for bit (which the parity tests pin
to the oracle).  Covers plans of several blocks with short last rounds, one
block, a plan derived from a MaxGPUUsage budget, device inputs with a
shared smoothness image, REF_CPU semantics, repeated solves on one context,
the negative-input report, refused in-core-only calls and the filter
facade."""

import numpy as np
import pytest

from robartsvtk_gb300 import REF_CPU, REF_CUDA, HierarchicalMaxFlowSegmentation, HMFError, HMFSolver
from robartsvtk_gb300.synthetic import random_tree_problem

pytestmark = pytest.mark.gpu

PARENT = [-1, 0, 0, 1, 1, 2, 2]


def _fill(s, w, device_inputs=False, shared_smooth=False):
    import torch
    keep = []
    for leaf, d in w.data.items():
        if device_inputs:
            t = torch.from_numpy(d).cuda()
            keep.append(t)
            s.set_data(leaf, t)
        else:
            s.set_data(leaf, d)
    smooth = dict(w.smooth)
    if shared_smooth and smooth:
        first = next(iter(smooth.values()))
        smooth = {v: first for v in range(1, len(w.parent))}
    tensors = {}
    for v, S in smooth.items():
        if device_inputs:
            if id(S) not in tensors:
                tensors[id(S)] = torch.from_numpy(S).cuda()
            s.set_smoothness(v, tensors[id(S)])
        else:
            s.set_smoothness(v, S)
    keep.extend(tensors.values())
    for v, a in w.alpha.items():
        s.set_smoothness_scalar(v, a)
    s.set_params(w.iterations, w.step, w.cc)
    return keep


def _outputs(s, w):
    n = len(w.parent)
    u = {v: s.labels(v) for v in range(n) if w.parent[v] >= 0}
    sink = {v: s.sink(v) for v in range(n)}
    return u, sink


def _in_core(w, semantics=REF_CUDA, **kw):
    with HMFSolver(w.dims, w.parent, semantics) as s:
        keep = _fill(s, w, **kw)
        s.solve()
        out = _outputs(s, w)
        del keep
        return out


def _paged(w, semantics=REF_CUDA, plan=(0, 0), usage=0.75, inputs="auto", **kw):
    with HMFSolver(w.dims, w.parent, semantics, max_gpu_usage=usage) as s:
        s.set_paged_plan(*plan, inputs=inputs)
        keep = _fill(s, w, **kw)
        s.solve()
        out = _outputs(s, w)
        info = s.paged_plan()
        del keep
        return out, info


def _assert_same(a, b):
    for part in (0, 1):
        for v in a[part]:
            assert np.array_equal(a[part][v], b[part][v]), (part, v)


@pytest.mark.parametrize("inputs", ["host", "device"])
@pytest.mark.parametrize("dims,plan,iterations,blocks", [
    ((37, 19, 45), (20, 2), 13, 4),   # rounds 2,2,2,2,2,2,1
    ((37, 19, 50), (20, 2), 13, 4),   # every block owns planes exactly 2k+1 from its top face
    ((40, 24, 61), (28, 3), 10, 4),   # rounds 3,3,3,1
    ((33, 17, 29), (12, 1), 4, 4),    # the thinnest blocks for one iteration per round
    ((44, 20, 96), (20, 2), 9, 9),    # nine blocks: each block context takes three
    ((32, 16, 20), (64, 0), 12, 1),   # one block covers the volume: one round
    ((37, 19, 45), (64, 3), 13, 1),   # one block, rounds of 3: the state crosses the host link
])
def test_paged_plans_equal_the_in_core_solve(dims, plan, iterations, blocks, inputs):
    w = random_tree_problem(21, dims, PARENT, iterations=iterations, smooth_nodes=(1, 4))
    ref = _in_core(w)
    got, info = _paged(w, plan=plan, inputs=inputs)
    assert info["blocks"] == blocks
    _assert_same(got, ref)
    assert info["link_bytes"] > 0


def test_paged_device_inputs_and_shared_smoothness():
    w = random_tree_problem(22, (48, 20, 52), [-1, 0, 0, 0, 0], iterations=11, smooth_nodes=(1, 2, 3, 4))
    ref = _in_core(w, device_inputs=True, shared_smooth=True)
    got, info = _paged(w, plan=(20, 2), device_inputs=True, shared_smooth=True)
    assert info["blocks"] == 5 and info["rounds"] == 6
    _assert_same(got, ref)


def test_paged_pinned_host_inputs_read_over_the_link():
    """Inputs in pinned host memory (torch pin_memory) are read in place by
    every block of every round."""
    import torch
    w = random_tree_problem(30, (36, 20, 48), PARENT, iterations=7, smooth_nodes=(2,))
    ref = _in_core(w)
    pinned = {k: torch.from_numpy(v).pin_memory() for k, v in w.data.items()}
    spinned = {k: torch.from_numpy(v).pin_memory() for k, v in w.smooth.items()}
    with HMFSolver(w.dims, w.parent, REF_CUDA, max_gpu_usage=0.75) as s:
        s.set_paged_plan(20, 2, inputs="host")
        for leaf, t in pinned.items():
            s.set_data(leaf, t)
        for v, t in spinned.items():
            s.set_smoothness(v, t)
        for v, a in w.alpha.items():
            s.set_smoothness_scalar(v, a)
        s.set_params(w.iterations, w.step, w.cc)
        s.solve()
        got = _outputs(s, w)
    _assert_same(got, ref)


def test_paged_plan_from_a_memory_budget():
    """A MaxGPUUsage budget that holds three blocks of ~20 planes and the
    inputs: the plan comes from the budget, and the device memory stays
    within it."""
    import torch
    w = random_tree_problem(23, (64, 48, 80), [-1, 0, 0, 1, 1, 2, 2], iterations=9, smooth_nodes=(1,))
    total = torch.cuda.get_device_properties(0).total_memory
    pitch = 64
    per_plane = (9 * 6 + 1 + 4 + 1) * pitch * 48 * 4
    inputs = 5 * 64 * 48 * 80 * 4
    budget = 3 * (16 << 20) + inputs + 3 * 20 * per_plane
    usage = budget / total
    ref = _in_core(w)
    with HMFSolver(w.dims, w.parent, REF_CUDA, max_gpu_usage=usage) as s:
        keep = _fill(s, w)
        s.solve()
        got = _outputs(s, w)
        info = s.paged_plan()
        assert s.device_bytes() <= budget
        del keep
    assert info["blocks"] > 1 and 16 <= info["block_planes"] <= 20
    _assert_same(got, ref)


def test_paged_ref_cpu_semantics():
    w = random_tree_problem(24, (29, 17, 40), PARENT, iterations=15, smooth_nodes=(1,))
    ref = _in_core(w, semantics=REF_CPU)
    got, info = _paged(w, semantics=REF_CPU, plan=(12, 0))
    assert info["blocks"] == 4 and info["rounds"] == 1
    _assert_same(got, ref)


def test_paged_context_solves_twice():
    w = random_tree_problem(25, (35, 21, 44), PARENT, iterations=7, smooth_nodes=(2,))
    w2 = random_tree_problem(26, (35, 21, 44), PARENT, iterations=12, smooth_nodes=(1, 5))
    with HMFSolver(w.dims, w.parent, REF_CUDA, max_gpu_usage=0.75) as s:
        s.set_paged_plan(20, 2)
        keep = _fill(s, w)
        s.solve()
        first = _outputs(s, w)
        keep2 = _fill(s, w2)
        s.set_smoothness(2, None)
        s.solve()
        second = _outputs(s, w2)
        del keep, keep2
    _assert_same(first, _in_core(w))
    _assert_same(second, _in_core(w2))


def test_paged_reports_negative_input_and_refuses_in_core_calls():
    w = random_tree_problem(27, (20, 12, 30), [-1, 0, 0], iterations=4)
    w.data[1][5, 3, 2] = -0.5
    with HMFSolver(w.dims, w.parent, REF_CUDA, max_gpu_usage=0.75) as s:
        s.set_paged_plan(12, 1)
        keep = _fill(s, w)
        s.solve()
        with pytest.raises(HMFError, match="non-negative"):
            s.labels(1)
        with pytest.raises(HMFError, match="out-of-core"):
            s.autotune()
        with pytest.raises(HMFError, match="out-of-core"):
            s.solve_fp64()
        del keep


def test_paged_layout_too_thin_is_an_error():
    w = random_tree_problem(28, (20, 12, 40), [-1, 0, 0], iterations=4)
    with HMFSolver(w.dims, w.parent, REF_CUDA, max_gpu_usage=0.75) as s:
        s.set_paged_plan(16, 2)  # needs at least 20 planes for 2 iterations per round
        keep = _fill(s, w)
        with pytest.raises(HMFError, match="four times the halo"):
            s.solve()
        del keep


def test_filter_facade_with_max_gpu_usage():
    w = random_tree_problem(29, (30, 18, 36), PARENT, iterations=6, smooth_nodes=(1,))
    outs = []
    for usage in (None, 0.75):
        f = HierarchicalMaxFlowSegmentation()
        f.SetStructure(w.parent)
        f.SetMaxGPUUsage(usage)
        for leaf, d in w.data.items():
            f.SetDataInputDataObject(leaf, d)
        for v, S in w.smooth.items():
            f.SetSmoothnessInputDataObject(v, S)
        for v, a in w.alpha.items():
            f.AddSmoothnessScalar(v, a)
        f.SetNumberOfIterations(w.iterations)
        assert f.Update() == 1
        outs.append({leaf: f.GetOutputDataObject(leaf).copy() for leaf in w.leaves})
    for leaf in w.leaves:
        assert np.array_equal(outs[0][leaf], outs[1][leaf])


def test_paged_zero_iterations_and_a_budget_too_small():
    """Zero iterations: every block initialises only, equal to the in-core
    initialisation.  A budget below three blocks of planes is refused before
    any device work."""
    w = random_tree_problem(32, (30, 16, 40), PARENT, iterations=0, smooth_nodes=(1,))
    ref = _in_core(w)
    got, info = _paged(w, plan=(12, 0))
    assert info["rounds"] == 1 and info["round_iterations"] == 0
    _assert_same(got, ref)
    with HMFSolver(w.dims, w.parent, REF_CUDA, max_gpu_usage=1e-9) as s:
        keep = _fill(s, w)
        with pytest.raises(HMFError, match="MaxGPUUsage"):
            s.solve()
        del keep

