"""Replicas across ranks: one process per GPU, no collective on the data path.

Flood scenarios share nothing, so a job of N scenarios is split across the
ranks of a torch.distributed group, each rank advances its share on its own
GPU, and the ranks communicate only to report: the units they processed
(summed) and the seconds they took (the maximum, since the job ends with
its slowest rank).  A single domain is not split across GPUs.

    units = replicas.shard(len(scenarios), rank, world)     # this rank's indices
    value = replicas.job_throughput(local_units, local_seconds)
"""
from __future__ import annotations

from typing import Optional


def shard(n: int, rank: int, world: int) -> range:
    """Contiguous block of the n items for `rank` of `world`; the blocks of
    all ranks cover 0..n-1 once, and their sizes differ by at most one."""
    if world < 1 or not 0 <= rank < world or n < 0:
        raise ValueError(f"bad shard request n={n} rank={rank} world={world}")
    return range(n * rank // world, n * (rank + 1) // world)


def rank_seed(seed: int, rank: int) -> int:
    """Seed of the synthetic inputs of one rank's replica."""
    return seed + rank


def job_totals(local_units: float, local_seconds: float, group=None, device=None):
    """(units summed over ranks, seconds maximised over ranks).  Without an
    initialised process group this is the local pair."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(local_units), float(local_seconds)
    u = torch.tensor([float(local_units)], dtype=torch.float64, device=device)
    s = torch.tensor([float(local_seconds)], dtype=torch.float64, device=device)
    dist.all_reduce(u, op=dist.ReduceOp.SUM, group=group)
    dist.all_reduce(s, op=dist.ReduceOp.MAX, group=group)
    return float(u.item()), float(s.item())


def job_throughput(local_units: float, local_seconds: float, group=None, device=None) -> Optional[float]:
    """Whole-job rate: units of all ranks / seconds of the slowest rank."""
    u, s = job_totals(local_units, local_seconds, group, device)
    return u / s if s > 0 else None
