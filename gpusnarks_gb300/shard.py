"""Sharding of independent transforms across ranks (one GPU per rank).

The NTT path has no exchange step between independent transforms, so a
multi-GPU run partitions the jobs and each rank runs its own batch with no
data-path collective.  Jobs are assigned greedily by work (largest first to
the least-loaded rank), with work = (n/2) log2 n butterflies, each one
Montgomery product of 2 s^2 + s word multiply-adds for an s-limb field, so a
list that mixes fields (the serving mix of BLS12-381 and MNT4-753) balances by
the integer-pipe time its jobs take rather than by element count.
"""
from __future__ import annotations


def job_work(log_n: int, limbs: int = 1) -> float:
    """Word multiply-adds of one transform: (n/2) log2 n butterflies x (2 s^2 + s)."""
    return float((1 << max(log_n - 1, 0)) * max(log_n, 1)) * (2 * limbs * limbs + limbs)


def shard_jobs(sizes: list[int], world: int, limbs: list[int] | None = None) -> list[list[int]]:
    """Indices of `sizes` for each rank, balanced by work (deterministic).  `limbs` gives each job's limb
    count when the list mixes fields (default: all jobs in one field)."""
    if world < 1:
        raise ValueError("world must be >= 1")
    if limbs is not None and len(limbs) != len(sizes):
        raise ValueError("limbs must give one limb count per job")
    work = [job_work(k, 1 if limbs is None else limbs[i]) for i, k in enumerate(sizes)]
    order = sorted(range(len(sizes)), key=lambda i: (-work[i], i))
    load = [0.0] * world
    parts: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        parts[r].append(i)
        load[r] += work[i]
    for p in parts:
        p.sort()
    return parts


def rank_jobs(sizes: list[int], rank: int, world: int, limbs: list[int] | None = None) -> list[int]:
    return shard_jobs(sizes, world, limbs)[rank]
