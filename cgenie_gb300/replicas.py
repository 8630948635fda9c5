"""Ranks of a multi-GPU run.  Members are independent, so one ensemble is partitioned
across ranks (rank r advances members r, r + N, r + 2N, ... of the ensemble, on its own GPU,
with no collective on the data path), the results are gathered on one rank, and the timing is
reduced over ranks.

- `partition` gives the members of a rank;
- `gather` brings the per-member results of every rank to one rank, in member order;
- `job_time` is the whole job's time: the slowest rank;
- `job_units` is the work of all ranks (tracer cell-updates).
"""
from __future__ import annotations


def partition(n: int, rank: int, world: int) -> list:
    """Indices of the members of an `n`-member ensemble that rank `rank` of `world` advances."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} of {world}")
    return list(range(int(rank), int(n), int(world)))


def gather(local: dict, n: int, dist=None, dst: int = 0):
    """Per-member results of all ranks on rank `dst`, as a list in member order (None on the
    other ranks).  `local` maps a member index to this rank's result for it; every index
    0..n-1 must come from exactly one rank.  Without a process group: the local results."""
    if dist is None or not dist.is_initialized():
        parts = [local]
        rank = dst
    else:
        rank = dist.get_rank()
        parts = [None] * dist.get_world_size() if rank == dst else None
        dist.gather_object(local, parts, dst=dst)
    if rank != dst:
        return None
    out = [None] * n
    seen = set()
    for part in parts:
        for i, v in part.items():
            if i in seen or not 0 <= i < n:
                raise ValueError(f"member {i} gathered twice or out of range")
            seen.add(i)
            out[i] = v
    if len(seen) != n:
        raise ValueError(f"{n - len(seen)} members missing from the gather")
    return out


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
