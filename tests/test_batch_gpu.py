"""Batched persistent launch: bit-exact against the plain per-call path and
the oracle, with and without CUDA-graph capture."""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def _make_jobs(g, torch, f, sizes, dirs, seed):
    from gpusnarks_gb300.batch import fill_random
    total = sum(1 << k for k in sizes)
    pool = torch.empty(total * f.limbs, dtype=torch.int32, device="cuda")
    fill_random(f, pool, seed)
    views, jobs, off = [], [], 0
    for k, d in zip(sizes, dirs):
        v = pool[off * f.limbs:(off + (1 << k)) * f.limbs]
        views.append(v)
        jobs.append((v.data_ptr(), k, d, None, None))
        off += 1 << k
    return pool, views, jobs


@pytest.mark.parametrize("fname,lo,hi,count", [("bls12_381_fr", 2, 14, 48), ("mnt4753_fr", 1, 11, 24),
                                               ("p32", 3, 16, 40)])
@pytest.mark.parametrize("graph", [True, False])
def test_batch_matches_per_call(gsn, cuda_device, fname, lo, hi, count, graph):
    import torch
    from gpusnarks_gb300.batch import Batch
    f = gsn.FIELDS[fname]
    rng = np.random.default_rng(count + lo)
    sizes = [int(k) for k in rng.integers(lo, hi + 1, size=count)]
    dirs = [int(d) for d in rng.choice([0, 1, 2, 3], size=count)]
    pool, views, jobs = _make_jobs(gsn, torch, f, sizes, dirs, 0x5EED0400 + count)
    ref = [v.clone() for v in views]
    for r, k, d in zip(ref, sizes, dirs):
        gsn.ntt(f, r, direction=d)
    b = Batch(f, jobs, graph=graph)
    b.launch()
    torch.cuda.synchronize()
    b.status()
    for v, r, k in zip(views, ref, sizes):
        assert torch.equal(v, r), k
    # a second launch (graph replay) applies the transforms again
    again = [v.clone() for v in views]
    for r, d in zip(again, dirs):
        gsn.ntt(f, r, direction=d)
    b.launch()
    torch.cuda.synchronize()
    b.status()
    for v, r in zip(views, again):
        assert torch.equal(v, r)
    info = b.info()
    assert info["jobs"] == count and info["elements"] == sum(1 << k for k in sizes)
    b.close()


def test_batch_matches_oracle(gsn, cuda_device):
    import torch
    from gpusnarks_gb300.batch import Batch
    f = gsn.BLS12_381
    sizes = [9, 3, 12, 0, 1, 10]
    pool, views, jobs = _make_jobs(gsn, torch, f, sizes, [0] * len(sizes), 0x5EED0444)
    host = [gsn.to_host(v).reshape(-1, f.limbs).copy() for v in views]
    b = Batch(f, jobs)
    b.launch()
    torch.cuda.synchronize()
    for v, x in zip(views, host):
        assert np.array_equal(gsn.to_host(v).reshape(x.shape), O.ntt(1, x).reshape(x.shape))
    b.close()


def test_device_random_matches_host_replica(gsn, cuda_device):
    import torch
    from gpusnarks_gb300.batch import fill_random
    for f in (gsn.P32, gsn.BLS12_381, gsn.MNT4_753):
        d = torch.empty(1000 * f.limbs, dtype=torch.int32, device="cuda")
        fill_random(f, d, 1234)
        assert np.array_equal(gsn.to_host(d).reshape(f.shape(1000)), f.device_random(1000, 1234))


@pytest.mark.parametrize("fid", [0, 1, 2])
def test_bounded_wait_expires_without_fault(gsn, cuda_device, fid):
    """Failure detection on the GPU without a fault: a batch whose first pass
    is missing from the queue can never satisfy its dependency; every wait
    runs out after ~1 ms, the kernel records GSN_ERR_TIMEOUT and ends, and the
    context stays usable (the control run right after succeeds)."""
    import ctypes
    lib = gsn.load()
    st = ctypes.c_uint32(123)
    assert lib.gsn_batch_selftest_wait(fid, 1, ctypes.byref(st)) == 0, lib.gsn_last_error()
    assert st.value == 8  # GSN_ERR_TIMEOUT
    assert lib.gsn_batch_selftest_wait(fid, 0, ctypes.byref(st)) == 0, lib.gsn_last_error()
    assert st.value == 0


def test_batch_rejects_bad_jobs(gsn, cuda_device):
    import torch
    from gpusnarks_gb300.batch import Batch
    f = gsn.BLS12_381
    d = torch.empty(64 * f.limbs, dtype=torch.int32, device="cuda")
    with pytest.raises(gsn.GsnError, match="ARG"):
        Batch(f, [(d.data_ptr() + 4, 4, 0, None, None)])
    with pytest.raises(gsn.GsnError, match="SIZE"):
        Batch(f, [(d.data_ptr(), 40, 0, None, None)])
    with pytest.raises(gsn.GsnError, match="OMEGA"):
        Batch(f, [(d.data_ptr(), 4, 0, 2, None)])


def test_batch_rejects_empty_job_list(gsn, cuda_device):
    from gpusnarks_gb300.batch import Batch
    with pytest.raises(gsn.GsnError, match="ARG"):
        Batch(gsn.BLS12_381, [])


def test_one_shot_ntt_batch(gsn, cuda_device):
    """gsn_ntt_batch equals a kept Batch's launch and returns with the work done."""
    import torch
    from gpusnarks_gb300.batch import Batch, ntt_batch
    f = gsn.MNT4_753
    sizes = [9, 3, 12, 0, 1, 10, 6]
    dirs = [0, 1, 2, 0, 1, 2, 0]
    xs = [f.random_array(1 << k, seed=7300 + i) for i, k in enumerate(sizes)]
    a = [gsn.to_device(x) for x in xs]
    b = [gsn.to_device(x) for x in xs]
    ntt_batch(f, [(t.data_ptr(), k, d, None, None) for t, k, d in zip(a, sizes, dirs)])
    kept = Batch(f, [(t.data_ptr(), k, d, None, None) for t, k, d in zip(b, sizes, dirs)], graph=False)
    try:
        kept.launch()
        torch.cuda.synchronize()
        kept.status()
    finally:
        kept.close()
    for ta, tb in zip(a, b):
        assert torch.equal(ta, tb)
    for x, t, k, d in zip(xs, a, sizes, dirs):
        if d == 0:
            assert np.array_equal(gsn.to_host(t).reshape(x.shape), O.ntt(f.fid, x).reshape(x.shape))
    with pytest.raises(gsn.GsnError, match="ARG"):
        ntt_batch(f, [])


def test_batch_at_configured_sizes(gsn, cuda_device):
    """The batched workload at its configured sizes: 64 BLS12-381 forward jobs with log n drawn from
    10..20 (every size present), one graph-captured persistent launch with the batched tuning table.
    Every job equals the per-call path bit for bit; the jobs up to 2^14 also equal the oracle."""
    import torch
    from gpusnarks_gb300.batch import Batch, job_sizes
    f = gsn.BLS12_381
    sizes = list(range(10, 21)) + job_sizes(64 - 11, 10, 20, 0x5EED0404)
    pool, views, jobs = _make_jobs(gsn, torch, f, sizes, [0] * len(sizes), 0x5EED0405)
    small = {i: gsn.to_host(v).reshape(-1, f.limbs).copy() for i, (v, k) in enumerate(zip(views, sizes)) if k <= 14}
    ref = [v.clone() for v in views]
    for r in ref:
        gsn.ntt(f, r)
    b = Batch(f, jobs, graph=True)
    try:
        b.launch()
        torch.cuda.synchronize()
        b.status()
    finally:
        b.close()
    for i, (v, r, k) in enumerate(zip(views, ref, sizes)):
        assert torch.equal(v, r), (i, k)
    for i, x in small.items():
        assert np.array_equal(gsn.to_host(views[i]).reshape(x.shape), O.ntt(1, x).reshape(x.shape)), i


def test_batch_mixed_directions_at_large_sizes_mnt4(gsn, cuda_device):
    """MNT4-753 jobs up to 2^18 in every direction through one persistent launch, against the per-call
    path (the batched kernel's multi-pass plans with pre/post scaling at sizes above one tile)."""
    import torch
    from gpusnarks_gb300.batch import Batch
    f = gsn.MNT4_753
    sizes = [18, 16, 14, 12, 17, 15, 13, 11]
    dirs = [0, 1, 2, 3, 3, 2, 1, 0]
    pool, views, jobs = _make_jobs(gsn, torch, f, sizes, dirs, 0x5EED0406)
    ref = [v.clone() for v in views]
    for r, d in zip(ref, dirs):
        gsn.ntt(f, r, direction=d)
    b = Batch(f, jobs, graph=False)
    try:
        b.launch()
        torch.cuda.synchronize()
        b.status()
    finally:
        b.close()
    for v, r, k in zip(views, ref, sizes):
        assert torch.equal(v, r), k
