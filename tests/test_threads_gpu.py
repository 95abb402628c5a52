"""The C ABI is thread-safe per stream: host threads issuing transforms on their own streams at the same
time (ctypes releases the GIL for every call) all get the oracle's results, and concurrent gsn_ntt_host
calls serialise correctly."""
import threading

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

SEED = 0x5EED7000


def test_concurrent_streams(gsn, cuda_device):
    import torch
    cases = [(gsn.P32, 18), (gsn.BLS12_381, 12), (gsn.MNT4_753, 10), (gsn.P32, 14),
             (gsn.BLS12_381, 16), (gsn.MNT4_753, 8), (gsn.P32, 22), (gsn.BLS12_381, 9)]
    inputs = [f.random_array(1 << k, seed=SEED + i) for i, (f, k) in enumerate(cases)]
    want = [O.ntt(f.fid, x).reshape(x.shape) for (f, _), x in zip(cases, inputs)]
    got = [None] * len(cases)
    errors = []

    def worker(t):
        try:
            s = torch.cuda.Stream()
            for i in range(t, len(cases), 4):
                f, _ = cases[i]
                d = gsn.to_device(inputs[i])
                torch.cuda.current_stream().synchronize()
                for _ in range(3):  # forward, inverse, forward: all on this thread's stream
                    gsn.ntt(f, d, stream=s)
                    gsn.ntt(f, d, direction=gsn.INVERSE, stream=s)
                gsn.ntt(f, d, stream=s)
                s.synchronize()
                got[i] = gsn.to_host(d).reshape(inputs[i].shape)
        except Exception as exc:  # reported below
            errors.append(exc)

    threads = [threading.Thread(target=worker, args=(t,)) for t in range(4)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    assert not errors, errors
    for g_, w in zip(got, want):
        assert np.array_equal(g_, w)


def test_concurrent_host_calls(gsn, cuda_device):
    cases = [(gsn.P32, 15), (gsn.BLS12_381, 11), (gsn.MNT4_753, 9), (gsn.BLS12_381, 13)]
    arrays = [f.random_array(1 << k, seed=SEED + 50 + i) for i, (f, k) in enumerate(cases)]
    want = [O.ntt(f.fid, x).reshape(x.shape) for (f, _), x in zip(cases, arrays)]
    work = [a.copy() for a in arrays]
    errors = []

    def worker(i):
        try:
            f, k = cases[i]
            gsn.best_fft(work[i], None, field=f)
        except Exception as exc:
            errors.append(exc)

    threads = [threading.Thread(target=worker, args=(i,)) for i in range(len(cases))]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    assert not errors, errors
    for a, w in zip(work, want):
        assert np.array_equal(a, w)


def test_server_clients_on_several_threads(gsn, cuda_device):
    """Four client threads submit to one server and wait on their own requests at the same time."""
    from gpusnarks_gb300.serve import Server
    rng = np.random.default_rng(SEED + 77)
    reqs = []
    for i in range(32):
        f = (gsn.BLS12_381, gsn.MNT4_753)[int(rng.integers(0, 2))]
        k = int(rng.integers(6, 13))
        d = int(rng.integers(0, 3))
        reqs.append((f, k, d, f.random_array(1 << k, seed=SEED + 500 + i)))
    want = []
    for f, k, d, x in reqs:
        t = gsn.to_device(x)
        gsn.ntt(f, t, direction=d)
        want.append(gsn.to_host(t).reshape(x.shape))
    got = [None] * len(reqs)
    errors = []
    srv = Server(1 << 30, max_inflight=3)

    def client(t):
        try:
            for i in range(t, len(reqs), 4):
                f, k, d, x = reqs[i]
                out = np.empty_like(x)
                rid = srv.submit(f, x, d, host_out=out)
                srv.wait(rid)
                srv.release(rid)
                got[i] = out
        except Exception as exc:  # reported below
            errors.append(exc)

    try:
        threads = [threading.Thread(target=client, args=(t,)) for t in range(4)]
        for th in threads:
            th.start()
        for th in threads:
            th.join(120)
    finally:
        srv.close()
    assert not errors, errors
    for g_, w in zip(got, want):
        assert np.array_equal(g_, w)


def test_one_shot_batches_on_several_threads(gsn, cuda_device):
    """gsn_ntt_batch from four threads, each on its own stream, at the same time."""
    import torch
    from gpusnarks_gb300.batch import ntt_batch
    f = gsn.BLS12_381
    sizes = [[10, 4, 8], [12, 6], [9, 9, 9, 3], [11, 0, 7]]
    xs = [[f.random_array(1 << k, seed=SEED + 900 + 10 * t + j) for j, k in enumerate(ks)]
          for t, ks in enumerate(sizes)]
    want = [[O.ntt(f.fid, x).reshape(x.shape) for x in row] for row in xs]
    got = [None] * len(sizes)
    errors = []

    def worker(t):
        try:
            s = torch.cuda.Stream()
            ds = [gsn.to_device(x) for x in xs[t]]
            torch.cuda.current_stream().synchronize()
            ntt_batch(f, [(d.data_ptr(), k, 0, None, None) for d, k in zip(ds, sizes[t])], stream=s)
            got[t] = [gsn.to_host(d).reshape(x.shape) for d, x in zip(ds, xs[t])]
        except Exception as exc:  # reported below
            errors.append(exc)

    threads = [threading.Thread(target=worker, args=(t,)) for t in range(4)]
    for th in threads:
        th.start()
    for th in threads:
        th.join(120)
    assert not errors, errors
    for grow, wrow in zip(got, want):
        for g_, w in zip(grow, wrow):
            assert np.array_equal(g_, w)
