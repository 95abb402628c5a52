"""Serving: every result equals the plain path, alone and in a mix, under an
HBM budget that forces requests to wait for memory."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _plain(g, f, x, d):
    t = g.to_device(x)
    g.ntt(f, t, direction=d)
    return g.to_host(t).reshape(x.shape)


def _requests(g, count, seed, lo=5, hi=12):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        f = (g.BLS12_381, g.MNT4_753)[int(rng.integers(0, 2))]
        k = int(rng.integers(lo, hi + 1))
        d = int(rng.integers(0, 3))
        x = f.random_array(1 << k, seed=seed * 1000 + i)
        out.append((f, k, d, x))
    return out


def test_results_match_plain_path_alone_and_in_mix(gsn, cuda_device):
    from gpusnarks_gb300.serve import Server
    reqs = _requests(gsn, 40, 7)
    want = [_plain(gsn, f, x, d) for f, k, d, x in reqs]
    srv = Server(1 << 30, max_inflight=3)
    try:
        # alone: one request at a time
        alone = []
        for f, k, d, x in reqs[:6]:
            out = np.empty_like(x)
            rid = srv.submit(f, x, d, host_out=out)
            srv.wait(rid)
            srv.release(rid)
            alone.append(out)
        # in the mix: everything at once
        outs = [np.empty_like(x) for _, _, _, x in reqs]
        ids = [srv.submit(f, x, d, host_out=o) for (f, k, d, x), o in zip(reqs, outs)]
        for rid in ids:
            srv.wait(rid)
            srv.release(rid)
        for o, w in zip(outs, want):
            assert np.array_equal(o, w)
        for a, o in zip(alone, outs[:6]):
            assert np.array_equal(a, o)
        st = srv.stats()
        assert st["completed"] == 46 and st["failed"] == 0
    finally:
        srv.close()


def test_requests_over_the_work_cap_run_per_pass(gsn, cuda_device):
    """With max_launch_work = 1 every request exceeds the cap and runs alone through the per-pass kernels
    (forward, inverse and coset forward, both fields, resident and copied-out results); mixed with a
    second server's packed launches, results equal the plain path."""
    from gpusnarks_gb300.serve import Server
    reqs = _requests(gsn, 24, 11, lo=8, hi=16)
    want = [_plain(gsn, f, x, d) for f, k, d, x in reqs]
    lone = Server(1 << 31, max_inflight=2, max_launch_work=1)
    packed = Server(1 << 31, max_inflight=2)
    try:
        outs = [np.empty_like(x) for _, _, _, x in reqs]
        ids = []
        for i, ((f, k, d, x), o) in enumerate(zip(reqs, outs)):
            srv = lone if i % 3 else packed
            ids.append((srv, srv.submit(f, x, d, host_out=None if i % 4 == 0 else o)))
        for i, (srv, rid) in enumerate(ids):
            srv.wait(rid)
            if i % 4 == 0:
                srv.fetch(rid, outs[i])
            srv.release(rid)
        for o, w in zip(outs, want):
            assert np.array_equal(o, w)
        st = lone.stats()
        assert st["failed"] == 0 and st["launches"] == st["completed"]  # one launch per request
    finally:
        lone.close()
        packed.close()


def test_budget_admission_and_resident_results(gsn, cuda_device):
    from gpusnarks_gb300.serve import Server
    f = gsn.MNT4_753
    xs = [f.random_array(1 << 12, seed=300 + i) for i in range(12)]
    want = [_plain(gsn, f, x, 0) for x in xs]
    per = (1 << 12) * 96 * 2
    srv = Server(3 * per + 4096, max_inflight=2)  # about three requests fit at once
    try:
        ids = [srv.submit(f, x, 0) for x in xs]  # results stay resident
        for rid, w, x in zip(ids, want, xs):
            srv.wait(rid)
            out = np.empty_like(x)
            srv.fetch(rid, out)
            srv.release(rid)
            assert np.array_equal(out, w)
        assert srv.stats()["device_bytes_peak"] <= 3 * per + 4096
        with pytest.raises(gsn.GsnError, match="NOMEM"):
            srv.submit(f, f.random_array(1 << 14, seed=1), 0)
    finally:
        srv.close()


def test_run_trace_small(gsn, cuda_device):
    from gpusnarks_gb300.serve import Request, Server, TraceEntry, poisson_trace
    trace = poisson_trace(30, 2000.0, 5, lo=6, hi=11)
    ins, outs, entries, want = [], [], [], []
    for i, (t, fid, k, d) in enumerate(trace):
        f = gsn.BY_ID[fid]
        x = f.random_array(1 << k, seed=900 + i)
        o = np.empty_like(x)
        ins.append(x)
        outs.append(o)
        want.append(_plain(gsn, f, x, d))
        entries.append(TraceEntry(t, Request(fid, k, d, None, x.ctypes.data, o.ctypes.data)))
    srv = Server(1 << 30, max_inflight=4)
    try:
        srv.warmup(1, 6, 11)
        srv.warmup(2, 6, 11)
        lat, makespan, ph = srv.run_trace(entries, phases=True)
    finally:
        srv.close()
    assert (lat > 0).all() and makespan > 0
    for o, w in zip(outs, want):
        assert np.array_equal(o, w)
    # phase times: each non-negative, and together the request's latency (clock reads differ by ~us)
    assert ph.shape == (len(entries), 5)
    assert (ph[:, 1:] >= 0).all() and (ph[:, 0] > -1e-3).all()
    assert np.allclose(ph.sum(axis=1), lat, atol=1e-4)


def test_run_trace_empty(gsn, cuda_device):
    from gpusnarks_gb300.serve import Server
    srv = Server(1 << 24, max_inflight=2)
    try:
        lat, makespan = srv.run_trace([])
        lat2, makespan2, ph = srv.run_trace([], phases=True)
    finally:
        srv.close()
    assert lat.shape == (0,) and lat2.shape == (0,) and ph.shape == (0, 5)
    assert makespan == 0.0 and makespan2 == 0.0


def test_least_work_first_policy_results_and_order(gsn, cuda_device):
    """GSN_SERVE_LEAST_WORK_FIRST: every result equals the plain path, and under a backlog
    the small requests finish before the large ones that arrived first."""
    from gpusnarks_gb300.serve import LEAST_WORK_FIRST, Request, Server, TraceEntry
    f = gsn.MNT4_753
    sizes = [16, 16, 16, 16, 8, 8, 8, 8]  # large ones arrive first, all at once
    ins = [f.random_array(1 << k, seed=4400 + i) for i, k in enumerate(sizes)]
    outs = [np.empty_like(x) for x in ins]
    want = [_plain(gsn, f, x, 0) for x in ins]
    entries = [TraceEntry(0.0, Request(f.fid, k, 0, None, x.ctypes.data, o.ctypes.data))
               for k, x, o in zip(sizes, ins, outs)]
    srv = Server(1 << 30, max_inflight=1, max_launch_work=1, policy=LEAST_WORK_FIRST)
    try:
        srv.warmup(f.fid, 8, 16)
        lat, _ = srv.run_trace(entries)
    finally:
        srv.close()
    for o, w in zip(outs, want):
        assert np.array_equal(o, w)
    assert lat[4:].max() < lat[:4].max()


def test_request_lifecycle_errors(gsn, cuda_device):
    """Every misuse of a request id comes back as its own error, and the server stays usable."""
    import ctypes

    from gpusnarks_gb300.serve import Request, Server
    f = gsn.BLS12_381
    x = f.random_array(1 << 10, seed=4500)
    want = _plain(gsn, f, x, 0)
    srv = Server(1 << 28, max_inflight=2)
    try:
        with pytest.raises(gsn.GsnError, match="ARG"):
            srv.wait(987654321)
        with pytest.raises(gsn.GsnError, match="ARG"):
            srv.release(987654321)
        with pytest.raises(gsn.GsnError, match="ARG"):
            srv.submit(f, x, 7)  # no such direction
        rid_c = ctypes.c_uint64()
        too_big = Request(f.fid, 40, 0, None, x.ctypes.data, None)
        assert srv.lib.gsn_server_submit(srv.h, ctypes.byref(too_big), ctypes.byref(rid_c)) == 3  # SIZE
        assert srv.lib.gsn_server_submit(srv.h, None, ctypes.byref(rid_c)) == 1  # ARG
        out = np.empty_like(x)
        rid = srv.submit(f, x, 0, host_out=out)  # result copied out: nothing stays resident
        srv.wait(rid)
        with pytest.raises(gsn.GsnError, match="STATE"):
            srv.fetch(rid, np.empty_like(x))
        srv.release(rid)
        with pytest.raises(gsn.GsnError, match="ARG"):
            srv.release(rid)  # already released
        assert np.array_equal(out, want)
        rid = srv.submit(f, x, 0)  # resident result
        srv.wait(rid)
        got = srv.fetch(rid, np.empty_like(x))
        srv.release(rid)
        assert np.array_equal(got, want)
    finally:
        srv.close()


def test_serving_mix_at_configured_sizes(gsn, cuda_device):
    """Requests at the serving workload's sizes: both fields, 2^12..2^22 (the largest of each field
    included), forward, inverse, coset forward and coset inverse, submitted at once under a budget that
    makes the large ones wait for memory; every result equals the plain path bit for bit."""
    from gpusnarks_gb300.serve import Server
    rng = np.random.default_rng(0x5EED0505)
    reqs = []
    for f in (gsn.BLS12_381, gsn.MNT4_753):
        for i, k in enumerate([22, 21, 20, 18, 16, 14, 12] + [int(v) for v in rng.integers(12, 23, size=5)]):
            d = (i + f.fid) % 4
            x = f.device_random(1 << k, 0x5EED0500 + 100 * f.fid + i)
            reqs.append((f, k, d, x))
    want = [_plain(gsn, f, x, d) for f, k, d, x in reqs]
    srv = Server(3 << 30, max_inflight=4)  # 3 GiB: an MNT4 2^22 request holds 0.8 GiB
    try:
        outs = [np.empty_like(x) for _, _, _, x in reqs]
        ids = [srv.submit(f, x, d, host_out=o) for (f, k, d, x), o in zip(reqs, outs)]
        for rid in ids:
            srv.wait(rid, timeout_s=120.0)
            srv.release(rid)
        st = srv.stats()
    finally:
        srv.close()
    for (f, k, d, _), o, w in zip(reqs, outs, want):
        assert np.array_equal(o, w), (f.name, k, d)
    assert st["failed"] == 0 and st["device_bytes_peak"] <= 3 << 30
