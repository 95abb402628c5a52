"""GPU parity: the CUDA NTT through the C ABI against the oracle.

Integer work, so every comparison is bit-exact.  Sizes where the oracle
finishes in seconds are compared element by element; the largest sizes are
checked through size-independent properties (inverse round trip, X[0] = sum,
direct evaluation of sampled outputs, linearity).
"""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

SEED = 0x5EED0000


def _dev(g, x):
    return g.to_device(x)


def _run(g, f, x, **kw):
    d = g.to_device(x)
    g.ntt(f, d, **kw)
    return g.to_host(d).reshape(x.shape)


@pytest.mark.parametrize("fname,log_n", [
    ("p32", 0), ("p32", 1), ("p32", 2), ("p32", 5), ("p32", 8), ("p32", 11), ("p32", 12), ("p32", 13),
    ("p32", 17), ("p32", 20), ("p32", 22), ("p32", 23),
    ("bls12_381_fr", 0), ("bls12_381_fr", 1), ("bls12_381_fr", 3), ("bls12_381_fr", 9),
    ("bls12_381_fr", 10), ("bls12_381_fr", 14), ("bls12_381_fr", 17), ("bls12_381_fr", 19),
    ("mnt4753_fr", 0), ("mnt4753_fr", 1), ("mnt4753_fr", 4), ("mnt4753_fr", 8), ("mnt4753_fr", 9),
    ("mnt4753_fr", 12), ("mnt4753_fr", 16), ("mnt4753_fr", 17),
])
def test_forward_matches_oracle(gsn, cuda_device, fname, log_n):
    f = gsn.FIELDS[fname]
    x = f.random_array(1 << log_n, seed=SEED + 17 * log_n + f.fid)
    got = _run(gsn, f, x)
    want = O.ntt(f.fid, x).reshape(x.shape)
    assert np.array_equal(got, want)


@pytest.mark.parametrize("fname,max_log", [("p32", 22), ("bls12_381_fr", 20), ("mnt4753_fr", 19)])
def test_every_size_matches_oracle(gsn, cuda_device, fname, max_log):
    """Every size from 2^0 up, so every plan of the tuned table in that range runs: forward against the
    oracle, then the inverse back to the input."""
    f = gsn.FIELDS[fname]
    for log_n in range(max_log + 1):
        x = f.random_array(1 << log_n, seed=SEED + 1000 + 31 * log_n + f.fid)
        d = gsn.to_device(x)
        gsn.ntt(f, d)
        got = gsn.to_host(d).reshape(x.shape)
        assert np.array_equal(got, O.ntt(f.fid, x).reshape(x.shape)), log_n
        gsn.ntt(f, d, direction=gsn.INVERSE)
        assert np.array_equal(gsn.to_host(d).reshape(x.shape), x), log_n


def test_config1_p32_n65536(gsn, cuda_device):
    """p = 3*2^30+1, n = 2^16, seeded uniform inputs, omega = 5^((p-1)/n)."""
    f = gsn.P32
    x = f.random_array(1 << 16, seed=SEED + 0)
    w = pow(5, (f.p - 1) >> 16, f.p)
    assert gsn.root_of_unity(f, 16) == w
    got = _run(gsn, f, x, omega=w)
    assert np.array_equal(got, O.fft(0, x, w, log_cpus=3))


def test_config2_mnt4_n262144(gsn, cuda_device):
    """MNT4-753 r, n = 2^18: bit-exact against the oracle and INTT round trip."""
    f = gsn.MNT4_753
    x = f.random_array(1 << 18, seed=SEED + 1)
    d = gsn.to_device(x)
    gsn.ntt(f, d)
    got = gsn.to_host(d).reshape(x.shape)
    want = O.ntt(2, x).reshape(x.shape)
    assert np.array_equal(got, want)
    gsn.ntt(f, d, direction=gsn.INVERSE)
    assert np.array_equal(gsn.to_host(d).reshape(x.shape), x)


@pytest.mark.parametrize("fname,log_n", [("p32", 10), ("p32", 16), ("bls12_381_fr", 9), ("bls12_381_fr", 12),
                                         ("mnt4753_fr", 7), ("mnt4753_fr", 10)])
def test_inverse_and_coset_match_oracle(gsn, cuda_device, fname, log_n):
    f = gsn.FIELDS[fname]
    x = f.random_array(1 << log_n, seed=SEED + 99 + log_n)
    inv = _run(gsn, f, x, direction=gsn.INVERSE)
    assert np.array_equal(inv, O.intt(f.fid, x).reshape(x.shape))
    cos = _run(gsn, f, x, direction=gsn.COSET_FORWARD)
    assert np.array_equal(cos, O.coset_ntt(f.fid, x, f.generator).reshape(x.shape))
    # coset inverse undoes coset forward, with an explicit shift too
    s = 3
    y = _run(gsn, f, x, direction=gsn.COSET_FORWARD, shift=s)
    assert np.array_equal(y, O.coset_ntt(f.fid, x, s).reshape(x.shape))
    back = _run(gsn, f, y, direction=gsn.COSET_INVERSE, shift=s)
    assert np.array_equal(back, x)


@pytest.mark.parametrize("fname,log_n", [("p32", 9), ("bls12_381_fr", 8), ("mnt4753_fr", 6)])
def test_custom_omega(gsn, cuda_device, fname, log_n):
    """A root other than the default (omega^3 is also primitive) is honoured."""
    f = gsn.FIELDS[fname]
    x = f.random_array(1 << log_n, seed=SEED + 5)
    w = pow(gsn.root_of_unity(f, log_n), 3, f.p)
    got = _run(gsn, f, x, omega=w)
    assert np.array_equal(got, O.fft(f.fid, x, w, log_cpus=2).reshape(x.shape))


def test_extreme_values(gsn, cuda_device):
    for f in (gsn.P32, gsn.BLS12_381, gsn.MNT4_753):
        n = 1 << 9
        vals = [0, 1, f.p - 1, f.p - 2, (f.p - 1) // 2] * (n // 5) + [f.p - 1] * (n % 5)
        x = f.ints_to_array(vals)
        assert np.array_equal(_run(gsn, f, x), O.ntt(f.fid, x).reshape(x.shape))


def test_errors(gsn, cuda_device):
    import torch
    f = gsn.P32
    x = gsn.to_device(f.random_array(16, seed=1))
    with pytest.raises(gsn.GsnError, match="OMEGA"):
        gsn.ntt(f, x, omega=2)  # not a root of unity
    with pytest.raises(gsn.GsnError, match="OMEGA"):
        gsn.ntt(f, x, omega=pow(gsn.root_of_unity(f, 4), 2, f.p))  # order 8, not 16
    with pytest.raises(gsn.GsnError, match="OMEGA"):
        gsn.ntt(f, x, omega=f.p + 1)  # not reduced
    lib = gsn.load()
    assert lib.gsn_ntt(7, x.data_ptr(), 4, None, 0, None, None) == 2
    assert lib.gsn_ntt(0, x.data_ptr(), 31, None, 0, None, None) == 3
    assert lib.gsn_ntt(0, x.data_ptr(), 4, None, 9, None, None) == 1
    b = gsn.to_device(gsn.BLS12_381.random_array(16, seed=2))
    assert lib.gsn_ntt(1, b.data_ptr() + 4, 2, None, 0, None, None) == 1  # misaligned
    assert lib.gsn_ntt(0, None, 4, None, 0, None, None) == 1
    torch.cuda.synchronize()


def test_host_path_best_fft(gsn, cuda_device):
    """gsn_ntt_host: the best_fft drop-in on a host array, in place."""
    for f, log_n in ((gsn.P32, 14), (gsn.BLS12_381, 11), (gsn.MNT4_753, 9)):
        x = f.random_array(1 << log_n, seed=SEED + 3)
        a = x.copy()
        out = gsn.best_fft(a, gsn.root_of_unity(f, log_n))
        assert out is a
        assert np.array_equal(a, O.ntt(f.fid, x).reshape(x.shape))
        gsn.best_fft(a, None, direction=gsn.INVERSE)
        assert np.array_equal(a, x)


def test_host_path_pinned(gsn, cuda_device):
    """gsn_ntt_host on page-locked host memory (the buffer bench.py's e2e uses): forward, inverse and
    coset forward match the oracle."""
    import ctypes
    cases = ((gsn.P32, 16), (gsn.BLS12_381, 8), (gsn.BLS12_381, 13), (gsn.MNT4_753, 4),
             (gsn.MNT4_753, 12), (gsn.MNT4_753, 15))
    for f, log_n in cases:
        n = 1 << log_n
        x = f.random_array(n, seed=SEED + 5 * log_n + f.fid)
        buf = gsn.host_buffer(x.nbytes)
        try:
            arr = np.ctypeslib.as_array(ctypes.cast(buf, ctypes.POINTER(ctypes.c_uint32)),
                                        shape=(x.size,)).reshape(x.shape)
            arr[...] = x
            gsn._lib.check(gsn.load().gsn_ntt_host(f.fid, buf.value, log_n, None, gsn.FORWARD, None))
            assert np.array_equal(arr, O.ntt(f.fid, x).reshape(x.shape)), (f.name, log_n)
            gsn._lib.check(gsn.load().gsn_ntt_host(f.fid, buf.value, log_n, None, gsn.INVERSE, None))
            assert np.array_equal(arr, x), (f.name, log_n)
            s = np.ascontiguousarray(f.to_limbs(f.generator), dtype=np.uint32)
            gsn._lib.check(gsn.load().gsn_ntt_host(f.fid, buf.value, log_n, None, gsn.COSET_FORWARD,
                                                   gsn._lib.u32p(s)))
            assert np.array_equal(arr, O.coset_ntt(f.fid, x, f.generator).reshape(x.shape)), (f.name, log_n)
        finally:
            gsn.free_host_buffer(buf)


@pytest.mark.parametrize("fname,log_n,count", [("mnt4753_fr", 12, 7), ("bls12_381_fr", 14, 5),
                                               ("p32", 18, 4), ("mnt4753_fr", 15, 2)])
def test_host_batch_pipelined(gsn, cuda_device, fname, log_n, count):
    """gsn_ntt_host_batch: several host arrays through the copy/compute pipeline, each equal to its own
    oracle transform; pageable numpy arrays and page-locked buffers; forward, then inverse back."""
    import ctypes
    f = gsn.FIELDS[fname]
    xs = [f.random_array(1 << log_n, seed=SEED + 400 + 13 * i + log_n) for i in range(count)]
    work = [x.copy() for x in xs]
    gsn.best_fft_many(work, field=f)
    for w, x in zip(work, xs):
        assert np.array_equal(w, O.ntt(f.fid, x).reshape(x.shape))
    gsn.best_fft_many(work, field=f, direction=gsn.INVERSE)
    for w, x in zip(work, xs):
        assert np.array_equal(w, x)
    bufs = [gsn.host_buffer(x.nbytes) for x in xs]
    try:
        views = []
        for b, x in zip(bufs, xs):
            v = np.ctypeslib.as_array(ctypes.cast(b, ctypes.POINTER(ctypes.c_uint32)), shape=(x.size,))
            v[:] = x.reshape(-1)
            views.append(v)
        gsn.best_fft_many([(b.value, log_n) for b in bufs], field=f, direction=gsn.COSET_FORWARD)
        for v, x in zip(views, xs):
            assert np.array_equal(v.reshape(x.shape), O.coset_ntt(f.fid, x, f.generator).reshape(x.shape))
    finally:
        for b in bufs:
            gsn.free_host_buffer(b)


def test_release_caches_then_reuse(gsn, cuda_device):
    """gsn_release_caches frees tables, scratch and the host-path buffers; every path rebuilds what it needs
    on the next call and still matches the oracle."""
    f = gsn.MNT4_753
    x = f.random_array(1 << 11, seed=SEED + 77)
    a = x.copy()
    gsn.best_fft(a, None)
    gsn.best_fft_many([a.copy(), a.copy()], field=f)
    gsn._lib.check(gsn.load().gsn_release_caches())
    b, c = x.copy(), x.copy()
    gsn.best_fft(b, None)
    gsn.best_fft_many([c], field=f)
    d = gsn.to_device(x)
    gsn.ntt(f, d)
    want = O.ntt(f.fid, x).reshape(x.shape)
    for got in (b, c, gsn.to_host(d).reshape(x.shape)):
        assert np.array_equal(got, want)


def test_host_batch_errors(gsn, cuda_device):
    import ctypes
    lib = gsn.load()
    assert lib.gsn_ntt_host_batch(1, None, 0, 4, None, 0, None) == 0
    assert lib.gsn_ntt_host_batch(1, None, 2, 4, None, 0, None) == 1
    arr = (ctypes.c_void_p * 2)(None, None)
    assert lib.gsn_ntt_host_batch(1, arr, 2, 4, None, 0, None) == 1
    x = gsn.BLS12_381.random_array(16, seed=3)
    arr = (ctypes.c_void_p * 1)(x.ctypes.data)
    assert lib.gsn_ntt_host_batch(1, arr, 1, 40, None, 0, None) == 3
    assert lib.gsn_ntt_host_batch(9, arr, 1, 4, None, 0, None) == 2


@pytest.mark.parametrize("log_n", [12, 18, 22])
def test_p32_four_byte_aligned_arrays(gsn, cuda_device, log_n):
    """p32 data and scratch only 4-byte aligned (offset by one element) take the generic pass instead of
    the 16-byte-vector kernel, and still match the oracle."""
    import torch
    f = gsn.P32
    n = 1 << log_n
    x = f.random_array(n, seed=SEED + log_n)
    big = torch.zeros(n + 4, dtype=torch.int32, device="cuda")
    d = big[1:n + 1]
    d.copy_(torch.from_numpy(x.view(np.int32)))
    scr = torch.zeros(n + 4, dtype=torch.int32, device="cuda")[1:n + 1]
    assert d.data_ptr() % 16 == 4 and scr.data_ptr() % 16 == 4
    gsn.ntt(f, d)
    assert np.array_equal(gsn.to_host(d), O.ntt(0, x))
    gsn.ntt(f, d, direction=gsn.INVERSE, scratch=scr)
    assert np.array_equal(gsn.to_host(d), x)


def test_deterministic_rerun(gsn, cuda_device):
    f = gsn.BLS12_381
    x = f.random_array(1 << 15, seed=SEED + 8)
    assert np.array_equal(_run(gsn, f, x), _run(gsn, f, x))


def test_pointwise_mul(gsn, cuda_device):
    for f in (gsn.P32, gsn.BLS12_381, gsn.MNT4_753):
        a = f.random_array(257, seed=11)
        b = f.random_array(257, seed=12)
        da, db = gsn.to_device(a), gsn.to_device(b)
        gsn.pointwise_mul(f, da, db)
        got = f.array_to_ints(gsn.to_host(da))
        want = [(x * y) % f.p for x, y in zip(f.array_to_ints(a), f.array_to_ints(b))]
        assert got == want
