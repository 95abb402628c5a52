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
