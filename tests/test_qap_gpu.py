"""GPU parity of the QAP H computation (gsn_coset_quotient, gsn_qap_h) against the oracle.

Integer work: bit-exact.  Small sizes element by element against oracle.qap_h;
a larger satisfied system through size-independent properties (top coefficient
zero, H(r) Z(r) = A(r) B(r) - C(r) at a random point).
"""
import random

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

SEED = 0x5EED0000


def _rand(f, n, seed):
    return f.random_array(n, seed=seed)


@pytest.mark.parametrize("fname,log_n", [("p32", 6), ("p32", 12), ("bls12_381_fr", 5), ("bls12_381_fr", 10),
                                         ("mnt4753_fr", 4), ("mnt4753_fr", 8)])
def test_coset_quotient_matches_oracle(gsn, cuda_device, fname, log_n):
    f = gsn.FIELDS[fname]
    n = 1 << log_n
    a, b, c = (_rand(f, n, SEED + 100 * k + log_n) for k in range(3))
    for shift in (None, 3):
        da, db, dc = gsn.to_device(a), gsn.to_device(b), gsn.to_device(c)
        gsn.coset_quotient(f, da, db, dc, shift=shift)
        s = f.generator if shift is None else shift
        zinv = pow((pow(s, n, f.p) - 1) % f.p, f.p - 2, f.p)
        want = [((x * y - z) * zinv) % f.p for x, y, z in zip(f.array_to_ints(a), f.array_to_ints(b),
                                                               f.array_to_ints(c))]
        assert f.array_to_ints(gsn.to_host(da)) == want


@pytest.mark.parametrize("fname,log_n", [("p32", 10), ("p32", 14), ("bls12_381_fr", 9), ("bls12_381_fr", 12),
                                         ("mnt4753_fr", 7), ("mnt4753_fr", 10)])
def test_qap_h_matches_oracle(gsn, cuda_device, fname, log_n):
    f = gsn.FIELDS[fname]
    n = 1 << log_n
    a, b, c = (_rand(f, n, SEED + 7 * k + 3 * log_n) for k in range(3))
    da, db, dc = gsn.to_device(a), gsn.to_device(b), gsn.to_device(c)
    gsn.qap_h(f, da, db, dc)
    want = O.qap_h(f.fid, a, b, c)
    assert np.array_equal(gsn.to_host(da).reshape(a.shape), want.reshape(a.shape))


def _eval_from_domain(p, vals, n, w, r):
    """A(r) for the interpolant of vals on <w>: (r^n - 1)/n * sum v_i w^i / (r - w^i)."""
    pts, x = [], 1
    for _ in range(n):
        pts.append(x)
        x = x * w % p
    dens = [(r - t) % p for t in pts]
    pref = [1] * (n + 1)
    for i, d in enumerate(dens):
        pref[i + 1] = pref[i] * d % p
    inv_all = pow(pref[n], p - 2, p)
    acc = 0
    for i in range(n - 1, -1, -1):  # batch inversion
        inv_i = inv_all * pref[i] % p
        inv_all = inv_all * dens[i] % p
        acc = (acc + vals[i] * pts[i] % p * inv_i) % p
    return (pow(r, n, p) - 1) * pow(n, p - 2, p) % p * acc % p


@pytest.mark.parametrize("fname,log_n", [("bls12_381_fr", 16), ("mnt4753_fr", 14)])
def test_qap_h_satisfied_system(gsn, cuda_device, fname, log_n):
    """c = a*b on the domain (computed on the GPU): H is the exact quotient."""
    f = gsn.FIELDS[fname]
    n = 1 << log_n
    a, b = _rand(f, n, SEED + 1), _rand(f, n, SEED + 2)
    da, db = gsn.to_device(a), gsn.to_device(b)
    dc = gsn.to_device(a)
    gsn.pointwise_mul(f, dc, db)
    c = gsn.to_host(dc).reshape(a.shape)
    gsn.qap_h(f, da, db, dc)
    H = f.array_to_ints(gsn.to_host(da))
    assert H[n - 1] == 0
    p, w = f.p, gsn.root_of_unity(f, log_n)
    r = random.Random(log_n).randrange(2, p)
    hr = 0
    for coef in reversed(H):
        hr = (hr * r + coef) % p
    A, B, C = (_eval_from_domain(p, f.array_to_ints(v), n, w, r) for v in (a, b, c))
    assert hr * (pow(r, n, p) - 1) % p == (A * B - C) % p


def test_qap_errors(gsn, cuda_device):
    import ctypes
    f = gsn.BLS12_381
    n = 16
    da, db, dc = (gsn.to_device(_rand(f, n, k)) for k in range(3))
    lib = gsn.load()
    one = gsn._lib.u32p(f.to_limbs(1))
    zero = gsn._lib.u32p(f.to_limbs(0))
    assert lib.gsn_coset_quotient(f.fid, da.data_ptr(), db.data_ptr(), dc.data_ptr(), 4, one, None) == 1
    assert lib.gsn_coset_quotient(f.fid, da.data_ptr(), db.data_ptr(), dc.data_ptr(), 4, zero, None) == 1
    assert lib.gsn_qap_h(f.fid, da.data_ptr(), da.data_ptr(), dc.data_ptr(), 4, None, None) == 1
    assert lib.gsn_coset_quotient(9, da.data_ptr(), db.data_ptr(), dc.data_ptr(), 4, None, None) == 2
    del ctypes
