"""Multi-rank host logic of the replica runs (robartsvtk_gb300/replicas.py),
on CPU: two gloo ranks agree on the volume sharding, the slowest rank's time
and the whole-job throughput, as bench.py computes them under torchrun."""
import os
import socket

import pytest

from robartsvtk_gb300 import replicas


def test_shard_volumes_covers_every_volume_once_and_balances():
    sizes = [48 * 48 * 48, 192 * 100 * 77, 64 ** 3, 150 ** 3, 90 * 60 * 120, 1, 120 ** 3, 77 * 77 * 77, 5000]
    for world in (1, 2, 3, 4, 8, 12):
        shards = replicas.shard_volumes(sizes, world)
        assert len(shards) == world
        flat = sorted(i for s in shards for i in s)
        assert flat == list(range(len(sizes)))
        loads = [sum(sizes[i] for i in s) for s in shards]
        # greedy largest-first: the heaviest rank exceeds the mean by at most one volume
        assert max(loads) <= sum(sizes) / world + max(sizes)
    assert replicas.shard_volumes([], 2) == [[], []]
    with pytest.raises(ValueError):
        replicas.shard_volumes(sizes, 0)


def test_single_process_without_a_process_group():
    assert replicas.max_over_ranks(3.5) == 3.5
    assert replicas.sum_over_ranks(2.0) == 2.0
    assert replicas.job_throughput(1000.0, 500.0) == 2000.0
    replicas.barrier()  # no-op


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, sizes, q):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, local = replicas.rank_env()
        shards = replicas.shard_volumes(sizes, w)
        mine = shards[r]
        gathered = [None] * w
        dist.all_gather_object(gathered, mine)
        replicas.barrier()
        ms = 100.0 + 50.0 * r  # rank 1 is the slowest
        units = float(sum(sizes[i] for i in mine))
        out = {"rank": r, "local": local, "gathered": gathered,
               "max_ms": replicas.max_over_ranks(ms), "total": replicas.sum_over_ranks(units),
               "value": replicas.job_throughput(units, ms)}
        replicas.barrier()
        q.put(out)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    if not torch.distributed.is_available():
        pytest.skip("torch.distributed is not available")
    sizes = [48 ** 3, 192 ** 3, 64 ** 3, 150 ** 3, 90 ** 3]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, sizes, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort(key=lambda d: d["rank"])
    shards = replicas.shard_volumes(sizes, 2)
    for d in res:
        assert d["gathered"] == shards  # every rank computed the same sharding
        assert d["local"] == d["rank"]
        assert d["max_ms"] == 150.0
        assert d["total"] == float(sum(sizes))
        assert d["value"] == pytest.approx(sum(sizes) / 0.150)
