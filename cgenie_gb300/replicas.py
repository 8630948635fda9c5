"""Ranks of a multi-GPU run: members are independent, so every rank advances its own
ensemble (weak scaling) and the only collective is the timing reduction.

- `rank_seed` gives each rank a distinct, reproducible member set;
- `job_time` is the whole job's time: the slowest rank;
- `job_units` is the work of all ranks (tracer cell-updates).
"""
from __future__ import annotations


def rank_seed(seed: int, rank: int) -> int:
    return int(seed) + 7919 * int(rank)


def job_time(seconds: float, dist=None, device=None) -> float:
    """Max over ranks of the local time (the local time without a process group)."""
    if dist is None or not dist.is_initialized():
        return float(seconds)
    import torch
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_units(units: int, dist=None, device=None) -> int:
    """Sum over ranks of the local work."""
    if dist is None or not dist.is_initialized():
        return int(units)
    import torch
    t = torch.tensor([int(units)], dtype=torch.int64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return int(t.item())
