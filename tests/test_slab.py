"""The z-slab decomposition of one solve (robartsvtk_gb300/replicas.py:
slab_bounds, exchange_halos) on CPU: gloo ranks each iterate their slab plus
halo planes with the oracle as the solver and trade halos after every
iteration; the assembled state must equal the monolithic solve's bit for bit
(flows, divergence, labels and sinks of every vertex)."""
import os
import socket

import numpy as np
import pytest

from robartsvtk_gb300 import replicas
from robartsvtk_gb300.synthetic import random_tree_problem

PARENT = [-1, 0, 0, 1, 1, 2, 2]
KEYS = ("fx", "fy", "fz", "div", "u", "sink")


def problem():
    return random_tree_problem(5, (13, 11, 17), PARENT, iterations=9, smooth_nodes=(1, 4))


def test_slab_bounds():
    for vz, world in ((17, 1), (17, 2), (17, 3), (64, 8), (9, 4)):
        spans = [replicas.slab_bounds(vz, world, r) for r in range(world)]
        assert spans[0][0] == 0 and spans[-1][1] == vz
        for (a0, a1, alo, ahi), (b0, b1, blo, bhi) in zip(spans, spans[1:]):
            assert a1 == b0 and ahi == blo == replicas.HALO_PLANES
        sizes = [z1 - z0 for z0, z1, _, _ in spans]
        assert max(sizes) - min(sizes) <= 1
        assert spans[0][2] == 0 and spans[-1][3] == 0
    with pytest.raises(ValueError):
        replicas.slab_bounds(5, 3, 0)  # slabs thinner than the halo


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import torch
    import torch.distributed as dist

    from oracle import oracle as O

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w = problem()
        vx, vy, vz = w.dims
        z0, z1, lo, hi = b = replicas.slab_bounds(vz, world, rank)
        sl = slice(z0 - lo, z1 + hi)
        dims = (vx, vy, z1 + hi - (z0 - lo))
        data = {v: np.ascontiguousarray(d[sl]) for v, d in w.data.items()}
        smooth = {v: np.ascontiguousarray(S[sl]) for v, S in w.smooth.items()}
        st = O.new_state(dims, len(PARENT))
        O.iterate(dims, PARENT, data, st, smooth, w.alpha, iterations=0, step=w.step, cc=w.cc, init=True,
                  threads=1)
        views = [torch.from_numpy(st[k]) for k in KEYS]
        for _ in range(w.iterations):
            O.iterate(dims, PARENT, data, st, smooth, w.alpha, iterations=1, step=w.step, cc=w.cc, threads=1)
            replicas.exchange_halos(views, b, rank, world)
        q.put((rank, z0, z1, {k: st[k][:, lo:lo + (z1 - z0)].copy() for k in KEYS}))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_slabs_with_halo_exchange_equal_the_monolithic_solve(world):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    from oracle import oracle as O

    if not torch.distributed.is_available():
        pytest.skip("torch.distributed is not available")
    w = problem()
    mono = O.new_state(w.dims, len(PARENT))
    O.iterate(w.dims, PARENT, w.data, mono, w.smooth, w.alpha, iterations=w.iterations, step=w.step, cc=w.cc,
              init=True)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    parts = [q.get(timeout=300) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    covered = np.zeros(w.dims[2], bool)
    for rank, z0, z1, st in parts:
        covered[z0:z1] = True
        for k in KEYS:
            rows = [v for v in range(len(PARENT)) if k == "sink" or PARENT[v] >= 0]
            for v in rows:
                assert np.array_equal(st[k][v], mono[k][v, z0:z1]), (world, rank, k, v)
    assert covered.all()
