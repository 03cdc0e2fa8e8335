"""Batched solves (hmf_create_batch): volumes of different sizes sharing one
tree, solved in the same launches.  Every volume must equal the oracle's solve
of that volume alone.  GPU only."""
import numpy as np
import pytest

from oracle import oracle as O
from robartsvtk_gb300 import REF_CPU, REF_CUDA, HMFBatchSolver, HMFError, HMFSolver
from robartsvtk_gb300.synthetic import random_tree_problem

pytestmark = pytest.mark.gpu

PARENT = [-1, 0, 0, 1, 1]


def make_batch(seed, dims_list, parent=PARENT, iterations=15, smooth_nodes=(1, 3)):
    ws = [random_tree_problem(seed + i, d, parent, iterations=iterations, smooth_nodes=smooth_nodes)
          for i, d in enumerate(dims_list)]
    for w in ws[1:]:  # one tree, one set of weights for the whole batch
        w.alpha = dict(ws[0].alpha)
    return ws


def solve_batch(ws, semantics=REF_CUDA, autotune=False, device_inputs=False, pipeline=True, units=0):
    import torch
    keep = []
    with HMFBatchSolver([w.dims for w in ws], ws[0].parent, semantics) as b:
        b.set_pipeline(pipeline)
        if units:
            b.set_flow_units(units)
        for i, w in enumerate(ws):
            for leaf, d in w.data.items():
                if device_inputs:
                    t = torch.from_numpy(d).cuda()
                    keep.append(t)
                    b.set_data(i, leaf, t)
                else:
                    b.set_data(i, leaf, d)
            for v, S in w.smooth.items():
                b.set_smoothness(i, v, S)
        for v, a in ws[0].alpha.items():
            b.set_smoothness_scalar(v, a)
        b.set_params(ws[0].iterations, ws[0].step, ws[0].cc)
        if autotune:
            b.autotune()
        b.solve()
        out = []
        for i, w in enumerate(ws):
            n = len(w.parent)
            u = np.zeros((n,) + w.dims[::-1], np.float32)
            s = np.zeros_like(u)
            for v in range(n):
                s[v] = b.sink(i, v)
                if w.parent[v] >= 0:
                    u[v] = b.labels(i, v)
            out.append({"u": u, "sink": s})
        return out, b.stats()


def oracle(w, semantics=O.REF_CUDA):
    return O.solve(w.dims, w.parent, w.data, w.smooth, w.alpha, w.iterations, w.step, w.cc, want_sink=True,
                   semantics=semantics)


def same(a, b, what):
    for k in ("u", "sink"):
        assert np.array_equal(a[k], b[k].astype(np.float32)), "%s %s max |diff| %.3g" % (
            what, k, np.abs(a[k] - b[k]).max())


def test_batch_of_uneven_volumes_matches_oracle_per_volume():
    dims = [(37, 19, 23), (48, 48, 48), (5, 4, 3), (61, 30, 9), (1, 7, 11), (33, 65, 12)]
    ws = make_batch(100, dims)
    refs = [oracle(w) for w in ws]
    # the whole batch in 2 launches per iteration, or (slab pipeline, the
    # default) 2 per group of consecutive volumes, the groups as independent
    # graph chains
    for pipeline, per_iter in ((False, 2), (True, 2 * min(6, len(dims)))):
        res, stats = solve_batch(ws, pipeline=pipeline)
        for i, w in enumerate(ws):
            same(res[i], refs[i], "volume %d %s pipeline %s" % (i, w.dims, pipeline))
        assert stats["launches"] == 1 + per_iter * ws[0].iterations


@pytest.mark.parametrize("units", [2, 5])
def test_batch_with_several_marches_per_cta(units):
    """Flow CTAs that march several (window, vertex) units, crossing from one
    volume's units to the next, with and without the volume-group pipeline."""
    dims = [(37, 19, 23), (5, 4, 3), (61, 30, 9), (33, 65, 12)]
    ws = make_batch(150, dims)
    refs = [oracle(w) for w in ws]
    for pipeline in (False, True):
        res, _ = solve_batch(ws, pipeline=pipeline, units=units)
        for i, w in enumerate(ws):
            same(res[i], refs[i], "volume %d units %d pipeline %s" % (i, units, pipeline))


def test_batch_with_device_inputs_and_autotune():
    dims = [(70, 50, 40), (36, 36, 80), (100, 21, 17)]
    ws = make_batch(200, dims, parent=[-1, 0, 0, 0], smooth_nodes=(2,))
    res, _ = solve_batch(ws, autotune=True, device_inputs=True)
    for i, w in enumerate(ws):
        same(res[i], oracle(w), "volume %d" % i)


def test_batch_ref_cpu():
    ws = make_batch(300, [(9, 8, 7), (13, 4, 6)], iterations=20)
    res, _ = solve_batch(ws, semantics=REF_CPU)
    for i, w in enumerate(ws):
        same(res[i], oracle(w, semantics=O.REF_CPU), "volume %d" % i)


def test_batch_volume_without_smoothness_on_a_vertex():
    ws = make_batch(400, [(20, 18, 9), (17, 22, 10)], smooth_nodes=(1, 3))
    del ws[1].smooth[3]  # vertex 3 has an image in volume 0 only
    res, _ = solve_batch(ws)
    for i, w in enumerate(ws):
        same(res[i], oracle(w), "volume %d" % i)


def test_batch_equals_single_volume_solves():
    ws = make_batch(500, [(40, 30, 20), (25, 44, 16)])
    res, _ = solve_batch(ws)
    for i, w in enumerate(ws):
        with HMFSolver(w.dims, w.parent) as s:
            for leaf, d in w.data.items():
                s.set_data(leaf, d)
            for v, S in w.smooth.items():
                s.set_smoothness(v, S)
            for v, a in w.alpha.items():
                s.set_smoothness_scalar(v, a)
            s.set_params(w.iterations, w.step, w.cc)
            s.solve()
            for v in range(1, len(w.parent)):
                assert np.array_equal(res[i]["u"][v], s.labels(v))


def test_batch_errors():
    with pytest.raises(HMFError):
        HMFBatchSolver([(4, 4, 4), (0, 3, 3)], [-1, 0, 0])
    with HMFBatchSolver([(4, 4, 4), (3, 3, 3)], [-1, 0, 0]) as b:
        b.set_data(0, 1, np.ones((4, 4, 4), np.float32))
        b.set_data(0, 2, np.ones((4, 4, 4), np.float32))
        b.set_data(1, 1, np.ones((3, 3, 3), np.float32))
        with pytest.raises(HMFError, match="Missing data"):
            b.solve()
        with pytest.raises(ValueError):
            b.set_data(1, 2, np.ones((4, 4, 4), np.float32))
