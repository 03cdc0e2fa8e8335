"""Multi-GPU runs of this path: one process per GPU, no data-path collective.

A solve shards only by whole volumes (independent objects): each rank solves
its own volumes on its own GPU, and the ranks meet only to time the job (a
barrier on both sides of the timed region, the slowest rank's time).  A
spatial slab decomposition of one volume would need a per-iteration halo
exchange of the flows, sinks and labels; it is not built (every run of this
project has one GPU).

Works with any torch.distributed backend: NCCL on GPUs, gloo on the host
(the tests run two gloo ranks on CPU).
"""
from __future__ import annotations

import os


def rank_env():
    """(rank, world size, local rank) from the torchrun environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def shard_volumes(voxels, world):
    """Assign volumes (their voxel counts) to `world` ranks: largest first,
    each to the least loaded rank (ties: lowest rank), so that the slowest
    rank's share is within one volume of the mean.  Deterministic: every rank
    computes the same assignment.  Returns a list of index lists, one per
    rank, each in increasing index order."""
    if world < 1:
        raise ValueError("world size must be >= 1")
    load = [0] * world
    out = [[] for _ in range(world)]
    for i in sorted(range(len(voxels)), key=lambda k: (-int(voxels[k]), k)):
        r = min(range(world), key=lambda q: (load[q], q))
        out[r].append(i)
        load[r] += int(voxels[i])
    return [sorted(s) for s in out]


def barrier():
    import torch.distributed as dist

    if dist.is_available() and dist.is_initialized():
        dist.barrier()


def max_over_ranks(value, device=None):
    """The largest `value` over the ranks (the job's time is its slowest
    rank's); the value itself without an initialised process group."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value, device=None):
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def job_throughput(units, ms, device=None):
    """Whole-job throughput: the units every rank processed over the slowest
    rank's time (units per second)."""
    total = sum_over_ranks(units, device)
    slowest = max_over_ranks(ms, device)
    return total / (slowest / 1000.0)
