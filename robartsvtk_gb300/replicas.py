"""Multi-GPU runs of this path: one process per GPU, no data-path collective.

A solve shards by whole volumes (independent objects): each rank solves its
own volumes on its own GPU, and the ranks meet only to time the job (a
barrier on both sides of the timed region, the slowest rank's time).

One volume shards by z-slab with a halo exchange after every iteration:
one iteration's new state at plane z reads the old state at planes z-2 ..
z+2 (gradient step g -> descent p' -> projection multiplier m -> projected
flows P -> divergence), so a rank that holds its slab plus two halo planes on
each side computes its slab exactly, and then trades its two outermost slab
planes with each neighbour.  slab_bounds and exchange_halos are that
protocol; the GPU solver itself runs whole volumes (every run of this project
has one GPU), and tests/test_slab.py checks the protocol bit for bit with the
oracle as each rank's solver.

Works with any torch.distributed backend: NCCL on GPUs, gloo on the host
(the tests run gloo ranks on CPU).
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


HALO_PLANES = 2  # old-state planes one iteration reads on each side of a plane


def slab_bounds(vz, world, rank, halo=HALO_PLANES):
    """The balanced z-slab of `rank` among `world` ranks: (z0, z1, lo, hi) --
    its planes [z0, z1) and the halo planes held below (lo) and above (hi),
    clipped at the volume's faces.  Every slab must have at least `halo`
    planes (the halo comes from the direct neighbours only)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank / world size")
    base, extra = divmod(int(vz), world)
    if base < halo and world > 1:
        raise ValueError("%d planes cannot give %d slabs of at least %d planes" % (vz, world, halo))
    z0 = rank * base + min(rank, extra)
    z1 = z0 + base + (1 if rank < extra else 0)
    return z0, z1, min(halo, z0), min(halo, int(vz) - z1)


def exchange_halos(arrays, bounds, rank, world, axis=1):
    """Refresh the halo planes of `arrays` (tensors holding planes
    [z0 - lo, z1 + hi) along `axis`, bounds = slab_bounds(...)) from the
    neighbours' slabs: the first hi_lower slab planes go to rank - 1 (its
    upper halo), the last lo_upper to rank + 1 (its lower halo).  All arrays
    travel in one message per direction (non-blocking sends and receives, so
    the order between ranks cannot deadlock)."""
    import torch
    import torch.distributed as dist

    z0, z1, lo, hi = bounds
    nz = z1 - z0
    if world == 1:
        return
    reqs, recvs = [], []
    if rank > 0:  # planes z0 .. z0 + lo - 1 to the lower neighbour (its hi == our lo)
        down = torch.cat([a.narrow(axis, lo, lo).contiguous().reshape(-1) for a in arrays])
        reqs.append(dist.isend(down, rank - 1))
        buf = torch.empty_like(down)
        reqs.append(dist.irecv(buf, rank - 1))
        recvs.append((buf, 0, lo))
    if rank < world - 1:  # planes z1 - hi .. z1 - 1 to the upper neighbour (its lo == our hi)
        up = torch.cat([a.narrow(axis, lo + nz - hi, hi).contiguous().reshape(-1) for a in arrays])
        reqs.append(dist.isend(up, rank + 1))
        buf = torch.empty_like(up)
        reqs.append(dist.irecv(buf, rank + 1))
        recvs.append((buf, lo + nz, hi))
    for r in reqs:
        r.wait()
    for buf, start, count in recvs:
        off = 0
        for a in arrays:
            dst = a.narrow(axis, start, count)
            k = dst.numel()
            dst.copy_(buf[off:off + k].reshape(dst.shape))
            off += k
