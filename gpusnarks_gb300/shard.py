"""Sharding of independent transforms across ranks (one GPU per rank).

The NTT path has no exchange step between independent transforms, so a
multi-GPU run partitions the jobs and each rank runs its own batch with no
data-path collective.  Jobs are assigned greedily by work (largest first to
the least-loaded rank), with work = (n/2) log2 n butterflies.
"""
from __future__ import annotations


def job_work(log_n: int) -> float:
    return float((1 << max(log_n - 1, 0)) * max(log_n, 1))


def shard_jobs(sizes: list[int], world: int) -> list[list[int]]:
    """Indices of `sizes` for each rank, balanced by work (deterministic)."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(sizes)), key=lambda i: (-sizes[i], i))
    load = [0.0] * world
    parts: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        parts[r].append(i)
        load[r] += job_work(sizes[i])
    for p in parts:
        p.sort()
    return parts


def rank_jobs(sizes: list[int], rank: int, world: int) -> list[int]:
    return shard_jobs(sizes, world)[rank]
