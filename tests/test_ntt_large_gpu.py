"""GPU checks at the largest sizes (32-bit sweep up to 2^28) and the
polynomial-product companion run.

Where the oracle would take minutes, size-independent properties are used:
inverse round trip, X[0] = sum x, direct evaluation X[k] = sum_j x_j w^(jk)
at sampled k (numpy uint64, exact because p < 2^32), and linearity.
"""
import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

P = 3 * 2**30 + 1


def _eval_at(x: np.ndarray, w: int, k: int) -> int:
    """sum_j x_j * w^(j*k) mod p, chunked numpy with exact uint64 products."""
    n = x.size
    step = pow(w, k, P)
    total = 0
    chunk = 1 << 22
    start_pow = 1
    for s in range(0, n, chunk):
        m = min(chunk, n - s)
        # powers step^(s..s+m-1): by doubling within the chunk
        pw = np.empty(m, dtype=np.uint64)
        pw[0] = start_pow
        filled = 1
        mult = step
        while filled < m:
            c = min(filled, m - filled)
            pw[filled:filled + c] = (pw[:c] * np.uint64(mult)) % np.uint64(P)
            filled += c
            mult = (mult * mult) % P
        total = (total + int(np.sum((x[s:s + m].astype(np.uint64) * pw) % np.uint64(P), dtype=np.uint64) % P)) % P
        start_pow = (start_pow * pow(step, m, P)) % P
    return total % P


def test_p32_2_24_matches_oracle(gsn, cuda_device):
    f = gsn.P32
    x = f.random_array(1 << 24, seed=0x5EED0003)
    d = gsn.to_device(x)
    gsn.ntt(f, d)
    assert np.array_equal(gsn.to_host(d), O.ntt(0, x))


@pytest.mark.parametrize("log_n", [20, 22, 24, 26, 28])
def test_p32_sweep_properties(gsn, cuda_device, log_n):
    import torch
    f = gsn.P32
    n = 1 << log_n
    x = f.random_array(n, seed=0x5EED0003 + log_n)
    d = gsn.to_device(x)
    gsn.ntt(f, d)
    X = gsn.to_host(d)
    w = gsn.root_of_unity(f, log_n)
    assert int(X[0]) == int(np.sum(x.astype(np.uint64)) % P)
    rng = np.random.default_rng(log_n)
    for k in [1, n - 1] + [int(v) for v in rng.integers(2, n - 1, size=2)]:
        assert int(X[k]) == _eval_at(x, w, k), k
    # linearity on the device: NTT(x + y) = NTT(x) + NTT(y)
    y = f.random_array(n, seed=0x5EEDBEEF + log_n)
    s = ((x.astype(np.uint64) + y.astype(np.uint64)) % P).astype(np.uint32)
    ds, dy = gsn.to_device(s), gsn.to_device(y)
    gsn.ntt(f, ds)
    gsn.ntt(f, dy)
    lhs = ds.view(torch.int32).to(torch.int64) & 0xFFFFFFFF
    rhs = ((d.to(torch.int64) & 0xFFFFFFFF) + (dy.to(torch.int64) & 0xFFFFFFFF)) % P
    assert torch.equal(lhs, rhs)
    # inverse round trip
    gsn.ntt(f, d, direction=gsn.INVERSE)
    assert np.array_equal(gsn.to_host(d), x)


def test_p32_poly_product_2_21(gsn, cuda_device):
    """Two seeded polynomials with 2^20 coefficients (degree < 2^20) multiplied
    by forward NTTs of size 2^21, a pointwise product and an inverse NTT; the
    product is checked against the oracle's NTT product and at sampled
    coefficients by direct convolution sums."""
    import torch
    f = gsn.P32
    m = 1 << 20
    a = f.random_array(m, seed=0x5EED0013)
    b = f.random_array(m, seed=0x5EED0023)
    A = np.zeros(2 * m, dtype=np.uint32)
    B = np.zeros(2 * m, dtype=np.uint32)
    A[:m], B[:m] = a, b
    dA, dB = gsn.to_device(A), gsn.to_device(B)
    gsn.ntt(f, dA)
    gsn.ntt(f, dB)
    gsn.pointwise_mul(f, dA, dB)
    gsn.ntt(f, dA, direction=gsn.INVERSE)
    c = gsn.to_host(dA)
    # oracle product (the restated host FFT, fixed butterfly)
    Ao, Bo = O.ntt(0, A), O.ntt(0, B)
    prod = ((Ao.astype(np.uint64) * Bo.astype(np.uint64)) % P).astype(np.uint32)
    assert np.array_equal(c, _oracle_intt_p32(prod))
    assert int(c[-1]) == 0
    a64, b64 = a.astype(np.uint64), b.astype(np.uint64)
    for k in (0, 1, 7, m - 1, m, 2 * m - 2):
        lo, hi = max(0, k - (m - 1)), min(k, m - 1)
        idx = np.arange(lo, hi + 1)
        want = int(np.sum((a64[idx] * b64[k - idx]) % np.uint64(P), dtype=np.uint64) % np.uint64(P)) \
            if idx.size < (1 << 20) else _chunked_conv(a64, b64, k, lo, hi)
        assert int(c[k]) == want % P, k
    torch.cuda.synchronize()


def _chunked_conv(a64, b64, k, lo, hi):
    total = 0
    for s in range(lo, hi + 1, 1 << 18):
        e = min(hi + 1, s + (1 << 18))
        idx = np.arange(s, e)
        total += int(np.sum((a64[idx] * b64[k - idx]) % np.uint64(P), dtype=np.uint64))
    return total % P


def _oracle_intt_p32(X: np.ndarray) -> np.ndarray:
    """Inverse NTT with the oracle: forward with w^-1, then n^-1 (numpy exact)."""
    n = X.size
    log_n = n.bit_length() - 1
    w = O.root(0, log_n)
    y = O.fft(0, X, pow(w, P - 2, P), log_cpus=3)
    ninv = pow(n, P - 2, P)
    return ((y.astype(np.uint64) * np.uint64(ninv)) % np.uint64(P)).astype(np.uint32)


def _limb_sum(arr: np.ndarray, sign: np.ndarray | None = None) -> int:
    """sum_j s_j x_j as an integer, x given as (n, L) little-endian uint32 limbs, s_j in {+1, -1}: column
    sums in uint64 (each < 2^32 * n <= 2^58), combined as a big integer."""
    a = arr.astype(np.uint64)
    if sign is None:
        cols = a.sum(axis=0, dtype=np.uint64)
        return sum(int(c) << (32 * i) for i, c in enumerate(cols))
    pos = a[sign > 0].sum(axis=0, dtype=np.uint64)
    neg = a[sign < 0].sum(axis=0, dtype=np.uint64)
    return sum((int(c) - int(d)) << (32 * i) for i, (c, d) in enumerate(zip(pos, neg)))


@pytest.mark.parametrize("fname,log_n", [("bls12_381_fr", 26), ("mnt4753_fr", 24), ("bls12_381_fr", 23)])
def test_big_field_max_size_properties(gsn, cuda_device, fname, log_n):
    """The largest transforms of the multi-limb fields (2^26 x 32 B = 2 GiB, 2^24 x 96 B = 1.5 GiB):
    X[0] = sum x and X[n/2] = sum (-1)^j x_j (w^(n/2) = -1), both from exact limb-column sums, and the
    inverse round trip, bit for bit on the device."""
    import torch
    from gpusnarks_gb300.batch import fill_random
    f = gsn.FIELDS[fname]
    n = 1 << log_n
    d = torch.empty(n * f.limbs, dtype=torch.int32, device="cuda")
    fill_random(f, d, 0x5EED0000 + log_n)
    x0 = d.clone()
    x = gsn.to_host(d).reshape(n, f.limbs)
    gsn.ntt(f, d)
    X = gsn.to_host(d).reshape(n, f.limbs)
    assert f.from_limbs(X[0]) == _limb_sum(x) % f.p
    sign = np.where(np.arange(n) % 2 == 0, 1, -1)
    assert f.from_limbs(X[n // 2]) == _limb_sum(x, sign) % f.p
    gsn.ntt(f, d, direction=gsn.INVERSE)
    assert torch.equal(d, x0)
