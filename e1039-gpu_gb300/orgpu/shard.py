"""Event sharding across processes (one process per GPU).

Events are independent in every stage of the path (one reference block per
event, online_reconstruction.cu:776-894), so a batch splits into contiguous
event ranges with no exchange during the work: replicas only.  The only
collective is on the host side after the work: the max of the per-rank times
(the job takes as long as its slowest rank) and, where a caller wants them in
one place, the per-rank outputs.

Works with any torch.distributed backend (gloo on CPU in the tests, NCCL on
GPUs); with no process group every function degrades to the single-rank
answer.
"""
import numpy as np


def world_rank():
    """(world size, rank) of the default process group, (1, 0) without one."""
    try:
        import torch.distributed as dist
        if dist.is_available() and dist.is_initialized():
            return dist.get_world_size(), dist.get_rank()
    except ImportError:
        pass
    return 1, 0


def shard_range(n_events, world, rank):
    """Contiguous [start, stop) of `rank` among `world` ranks; the first
    n_events % world ranks take one event more."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} outside a world of {world}")
    q, r = divmod(int(n_events), world)
    start = rank * q + min(rank, r)
    return start, start + q + (1 if rank < r else 0)


def shard_records(records, offsets, world, rank):
    """This rank's part of a record batch: (records, offsets rebased to 0,
    first event index)."""
    n = len(offsets) - 1
    a, b = shard_range(n, world, rank)
    lo, hi = int(offsets[a]), int(offsets[b])
    return records[lo:hi], (offsets[a:b + 1] - offsets[a]).astype(offsets.dtype), a


def rank_seed(seed, rank):
    """Seed of rank's own synthetic events when every rank generates a full
    batch (weak scaling)."""
    return int(seed) + 1000 * int(rank)


def max_over_ranks(x, device=None):
    """Max of a float over all ranks (the job time of a timed region)."""
    world, _ = world_rank()
    if world == 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x, device=None):
    world, _ = world_rank()
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return type(x)(t.item())


def gather_to_rank0(arr):
    """Concatenate a 1-D numpy array of every rank, in rank order, on rank 0
    (None elsewhere).  Host-side, after the work."""
    world, rank = world_rank()
    if world == 1:
        return np.asarray(arr)
    import torch.distributed as dist
    out = [None] * world if rank == 0 else None
    dist.gather_object(np.asarray(arr), out, dst=0)
    return np.concatenate(out) if rank == 0 else None
