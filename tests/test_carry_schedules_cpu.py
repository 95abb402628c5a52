"""CPU emulation of the two carry schedules the device arithmetic relies on, word by word with an explicit
carry flag, checked against Python integers on random and carry-heavy operands (limbs of 0xFFFFFFFF):

* the even/odd Montgomery product with the pending merge carry (arith.cuh fe_mul_eo): every pair chain's
  final carry fits its top word, the reduction row zeroes word 0, and the result is a*b*R^-1 mod p;
* the register-pair-aligned plain product of the multi-exponentiation (multiexp.cuh mul_acc): no carry is
  lost into a word that already holds one, and A + 2^32 B = a*b.

These are the bounds arguments of the two kernels' comments, run on the CPU for BLS12-381 r and
MNT4-753 r."""
import random

import pytest

import oracle as O

M = 0xFFFFFFFF


def _pair_chain(acc, x, off, y, n):
    c = 0
    for k in range(n // 2):
        prod = x[2 * k + off] * y
        s = acc[2 * k] + (prod & M) + c
        acc[2 * k], c = s & M, s >> 32
        s = acc[2 * k + 1] + (prod >> 32) + c
        acc[2 * k + 1], c = s & M, s >> 32
    s = acc[n] + c
    assert s >> 32 == 0, "pair chain overflowed its top word"
    acc[n] = s


def mont_eo_pending(a, b, p, pinv, n):
    E, Od, q = [0] * (n + 1), [0] * (n + 1), 0
    for i in range(n):
        _pair_chain(E, a, 0, b[i], n)
        _pair_chain(Od, a, 1, b[i], n)
        m = (E[0] * pinv) & M
        _pair_chain(E, p, 0, m, n)
        _pair_chain(Od, p, 1, m, n)
        assert E[0] == 0
        onew = E[2:n + 1] + [0, 0]
        s = Od[0] + E[1]
        e0, c = s & M, s >> 32
        s = Od[1] + q + c
        e1, q = s & M, s >> 32
        E, Od = [e0, e1] + Od[2:n + 1], onew
    t = sum(v << (32 * k) for k, v in enumerate(E)) + (sum(v << (32 * k) for k, v in enumerate(Od)) << 32) + (q << 64)
    pp = sum(v << (32 * k) for k, v in enumerate(p))
    assert t < 2 * pp
    return t - pp if t >= pp else t


def plain_pairs(a, b, n):
    A, B = [0] * (2 * n + 1), [0] * (2 * n - 1)
    for i in range(n):
        for into_a, acc, off in ((True, A, 0), (False, B, 1)):
            j0 = (i & 1) if into_a else ((i + 1) & 1)
            jlast = ((n - 1 - j0) // 2) * 2 + j0
            c = 0
            for j in range(j0, jlast + 1, 2):
                prod = a[j] * b[i]
                s = acc[i + j - off] + (prod & M) + c
                acc[i + j - off], c = s & M, s >> 32
                s = acc[i + j + 1 - off] + (prod >> 32) + c
                acc[i + j + 1 - off], c = s & M, s >> 32
            s = acc[i + jlast + 2 - off] + c
            assert s <= M, "carry lost"
            acc[i + jlast + 2 - off] = s
    return sum(v << (32 * k) for k, v in enumerate(A)) + (sum(v << (32 * k) for k, v in enumerate(B)) << 32)


def _operands(fid, count, seed):
    p = O.MODULI[fid]
    n = O.LIMBS[fid]
    rnd = random.Random(seed)
    vals = [0, 1, p - 1, p - 2, p >> 1] + [rnd.randrange(p) for _ in range(count)]
    vals += [sum((M if rnd.random() < 0.85 else 0) << (32 * k) for k in range(n)) % p for _ in range(count)]
    return vals


@pytest.mark.parametrize("fid", [1, 2])
def test_montgomery_pending_merge_emulation(fid):
    n, p = O.LIMBS[fid], O.MODULI[fid]
    pl = [(p >> (32 * k)) & M for k in range(n)]
    pinv = (-pow(p, -1, 1 << 32)) & M
    rinv = pow(1 << (32 * n), -1, p)
    vals = _operands(fid, 60, 11 + fid)
    for x in vals:
        for y in vals[:25]:
            a = [(x >> (32 * k)) & M for k in range(n)]
            b = [(y >> (32 * k)) & M for k in range(n)]
            assert mont_eo_pending(a, b, pl, pinv, n) == x * y * rinv % p


@pytest.mark.parametrize("fid", [1, 2])
def test_pair_aligned_plain_product_emulation(fid):
    n = O.LIMBS[fid]
    vals = _operands(fid, 60, 21 + fid) + [(1 << (32 * n)) - 1]
    for x in vals:
        for y in vals[:25]:
            a = [(x >> (32 * k)) & M for k in range(n)]
            b = [(y >> (32 * k)) & M for k in range(n)]
            assert plain_pairs(a, b, n) == x * y
