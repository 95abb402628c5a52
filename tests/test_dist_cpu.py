"""Multi-rank host logic on CPU with gloo, world_size 2.

Each rank takes its shard of a batch of independent transforms (no data-path
collective) and the max-over-ranks timing reduction bench.py uses; the shards
are disjoint, cover every job and are balanced by work.
"""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, sizes, q):
    import torch
    import torch.distributed as dist

    import bench
    from gpusnarks_gb300.shard import job_work, rank_jobs
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = rank_jobs(sizes, rank, world)
    gathered = [None] * world
    dist.all_gather_object(gathered, mine)
    t = bench.max_over_ranks(float(rank + 1), world)
    bench.barrier(world)
    work = sum(job_work(sizes[i]) for i in mine)
    w = torch.tensor([work], dtype=torch.float64)
    dist.all_reduce(w, op=dist.ReduceOp.MAX)
    if rank == 0:
        q.put((gathered, t, float(w.item())))
    dist.destroy_process_group()


def test_two_rank_sharding_gloo():
    import multiprocessing as mp
    import numpy as np

    from gpusnarks_gb300.shard import job_work
    rng = np.random.default_rng(4)
    sizes = [int(k) for k in rng.integers(10, 21, size=512)]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, sizes, q)) for r in range(2)]
    for p in procs:
        p.start()
    gathered, tmax, wmax = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    a, b = gathered
    assert not set(a) & set(b)
    assert sorted(a + b) == list(range(len(sizes)))
    assert tmax == 2.0
    total = sum(job_work(k) for k in sizes)
    assert wmax <= 0.5 * total * 1.02  # balanced within 2%


def test_shard_single_rank_is_identity():
    from gpusnarks_gb300.shard import shard_jobs
    assert shard_jobs([3, 1, 2], 1) == [[0, 1, 2]]
    with pytest.raises(ValueError):
        shard_jobs([1], 0)


def test_mixed_field_sharding_balances_integer_work():
    """A BLS12-381 / MNT4-753 mix balances by multiply-adds: an MNT4 transform of the same size costs
    (2*24^2+24)/(2*8^2+8) = 8.6x a BLS one, so balancing by element count would leave one rank ~2x loaded."""
    import numpy as np

    from gpusnarks_gb300.shard import job_work, shard_jobs
    rng = np.random.default_rng(5)
    sizes = [int(k) for k in rng.integers(12, 23, size=400)]
    limbs = [int(s) for s in rng.choice([8, 24], size=400)]
    parts = shard_jobs(sizes, 2, limbs)
    assert sorted(parts[0] + parts[1]) == list(range(400))
    loads = [sum(job_work(sizes[i], limbs[i]) for i in p) for p in parts]
    assert max(loads) <= 0.5 * sum(loads) * 1.02
    with pytest.raises(ValueError):
        shard_jobs([10, 11], 2, [8])
