"""Replica sharding of independent images across ranks (one process per GPU).

The FFT / phaseCorrelate path has no exchange step: every image (or request)
is an independent unit, so N GPUs run N replicas over disjoint unit sets.
The only collectives are the timing barrier and the max-over-ranks reduction
of the step time; no collective ever touches image data.
"""
from __future__ import annotations


def shard(n_units: int, rank: int, world: int) -> range:
    """Contiguous, balanced block of unit indices for `rank` (strong scaling:
    the total is fixed).  Blocks are disjoint and cover range(n_units)."""
    if world < 1 or not 0 <= rank < world or n_units < 0:
        raise ValueError("bad shard arguments")
    q, r = divmod(n_units, world)
    start = rank * q + min(rank, r)
    return range(start, start + q + (1 if rank < r else 0))


def seeds_for(rank: int, per_rank: int, base: int = 1000) -> list[int]:
    """Input seeds of a rank's own batch (weak scaling: each rank gets
    `per_rank` fresh images; no two ranks share a seed)."""
    if rank < 0 or per_rank < 0:
        raise ValueError("bad seed arguments")
    return [base + rank * per_rank + i for i in range(per_rank)]


def max_over_ranks(value: float, dist=None, device=None) -> float:
    """The slowest rank's value (step time): all_reduce MAX on one float64."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_rate(units_per_rank: float, world: int, max_seconds: float) -> float:
    """Whole-job throughput: the units all ranks processed over the slowest
    rank's time."""
    if max_seconds <= 0:
        raise ValueError("time must be positive")
    return units_per_rank * world / max_seconds
