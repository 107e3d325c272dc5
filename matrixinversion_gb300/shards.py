"""Batch shards across ranks (one process per GPU).

Matrices are independent, so N GPUs run N shards of the batch with no
collective on the data path; only timings are reduced (maximum over ranks,
as the benchmark contract wants).  Works with any torch.distributed backend
(NCCL on GPUs, gloo on the host).
"""
from __future__ import annotations


def shard_range(total: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous [lo, hi) of `total` matrices for `rank` (strong scaling):
    shards differ in size by at most one matrix and cover the batch."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank must be in [0, world)")
    base, extra = divmod(int(total), int(world))
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def shard_seed(seed: int, rank: int) -> int:
    """Seed of a rank's own batch (weak scaling: every rank inverts a full
    batch of different matrices)."""
    return int(seed) + 7919 * int(rank)


def max_over_ranks(value: float, device=None) -> float:
    """Maximum of `value` over all ranks (the value itself without a process
    group)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(units_per_rank: int, seconds_max: float, world: int) -> float:
    """Whole-job throughput: the units all ranks processed over the slowest
    rank's time."""
    return float(world) * float(units_per_rank) / float(seconds_max)
