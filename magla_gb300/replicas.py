"""Independent replicas on several GPUs (one process per GPU).

The numeric phase does not exchange data between GPUs: a batch of
independent systems is split by system, one contiguous share per rank, and
each rank factorises and solves its share alone.  The only cross-rank
operations are the timing reduction (the slowest rank defines the step
time) and optional checks; both go through ``torch.distributed`` (NCCL on
GPUs, gloo on CPUs).
"""
from __future__ import annotations


def shard(count: int, rank: int, world: int) -> range:
    """Contiguous, balanced share of ``count`` items for ``rank`` of ``world``
    (the first ``count % world`` ranks take one item more)."""
    if world < 1 or not 0 <= rank < world or count < 0:
        raise ValueError("invalid shard request")
    base, extra = divmod(count, world)
    lo = rank * base + min(rank, extra)
    return range(lo, lo + base + (1 if rank < extra else 0))


def max_over_ranks(value: float) -> float:
    """The maximum of ``value`` over all ranks (``value`` itself without a process group)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float) -> float:
    """The sum of ``value`` over all ranks (``value`` itself without a process group)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())
