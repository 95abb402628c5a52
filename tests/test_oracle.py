"""The oracle checked against definitions, KATs and the reference's own output.

CPU only.  Three independent anchors:
  1. pure-Python big-integer math (naive DFT, modular arithmetic, schoolbook);
  2. golden fixtures produced by the reference's headers compiled unmodified
     (tests/golden/make_golden.py);
  3. when the reference checkout is present, the compiled reference itself.
"""
import hashlib
import pathlib
import random

import numpy as np
import pytest

import oracle as O

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden"
REF_Q = O.to_limbs(3, O.MODULI[3])


@pytest.mark.parametrize("fid", [0, 1, 2, 3])
def test_arith_matches_bigint(fid):
    rnd = random.Random(fid)
    p = O.MODULI[fid]
    for _ in range(50):
        a, b = rnd.randrange(p), rnd.randrange(p)
        assert O.arith(fid, "mul", a, b) == a * b % p
        assert O.arith(fid, "add", a, b) == (a + b) % p
        assert O.arith(fid, "sub", a, b) == (a - b) % p
        e = rnd.randrange(1 << 48)
        assert O.arith(fid, "pow", a, 0, e) == pow(a, e, p)


@pytest.mark.parametrize("fid", [0, 1, 2, 3])
def test_field_kats(fid):
    """Known answers of cuda/device_field_operator_test.cpp:222-298, on correct fields.

    The 2^35 case is checked as the integer 2^35; the reference spells it with
    a big-endian limb pattern (tmp[SIZE-2] = 8, :295-297) that does not match
    its own little-endian layout.
    """
    assert O.arith(fid, "add", 1234, 1234) == 2468
    assert O.arith(fid, "sub", 1234, 1234) == 0
    assert O.arith(fid, "sub", 1235, 1234) == 1
    assert O.arith(fid, "mul", 1234, 1234) == 1522756
    assert O.arith(fid, "mul", 1522756, 1234) == 1879080904
    assert O.arith(fid, "pow", 2, 0, 0) == 1
    assert O.arith(fid, "pow", 2, 0, 2) == 4
    assert O.arith(fid, "pow", 4, 0, 10) == 1048576
    assert O.arith(fid, "pow", 2, 0, 20) == 1048576
    assert O.arith(fid, "pow", 2, 0, 35) == (1 << 35) % O.MODULI[fid]


def test_field_constants():
    """Generators are quadratic non-residues; 2-adicity as documented."""
    for fid, s in ((0, 30), (1, 32), (2, 30), (3, 15)):
        p = O.MODULI[fid]
        assert (p - 1) % (1 << s) == 0 and ((p - 1) >> s) % 2 == 1
        assert pow(O.GENERATORS[fid], (p - 1) // 2, p) == p - 1
    assert O.MODULI[3] == O.from_limbs(REF_Q)
    assert O.MODULI[0] == 3 * 2**30 + 1


@pytest.mark.parametrize("fid", [0, 1, 2])
@pytest.mark.parametrize("log_n", [0, 1, 2, 4, 7])
def test_fixed_fft_is_dft(fid, log_n):
    rnd = random.Random(100 + fid * 10 + log_n)
    p = O.MODULI[fid]
    n = 1 << log_n
    xs = [rnd.randrange(p) for _ in range(n)]
    w = O.root(fid, log_n)
    want = O.naive_dft(fid, xs, w)
    for serial in (True, False):
        for lc in (0, 1, 3):
            got = O.ints(fid, O.fft(fid, O.array(fid, xs), w, log_cpus=lc, serial=serial))
            assert got == want


@pytest.mark.parametrize("fid", [0, 1, 2])
def test_intt_roundtrip_and_coset(fid):
    rnd = random.Random(7 + fid)
    p = O.MODULI[fid]
    log_n = 6
    xs = [rnd.randrange(p) for _ in range(1 << log_n)]
    x = O.array(fid, xs)
    assert O.ints(fid, O.intt(fid, O.ntt(fid, x))) == xs
    g = O.GENERATORS[fid]
    want = O.naive_dft(fid, [(v * pow(g, i, p)) % p for i, v in enumerate(xs)], O.root(fid, log_n))
    assert O.ints(fid, O.coset_ntt(fid, x, g)) == want


@pytest.mark.parametrize("fid", [0, 1, 2])
def test_qap_h_is_exact_quotient(fid):
    """For a satisfied system (c_i = a_i b_i on the domain) the oracle's H is the exact polynomial
    quotient (A B - C) / (x^n - 1), checked with schoolbook products; its top coefficient is zero.
    Also the coset inverse undoes the coset transform."""
    rnd = random.Random(31 + fid)
    p = O.MODULI[fid]
    n = 32
    a = [rnd.randrange(p) for _ in range(n)]
    b = [rnd.randrange(p) for _ in range(n)]
    c = [(x * y) % p for x, y in zip(a, b)]
    H = O.ints(fid, O.qap_h(fid, O.array(fid, a), O.array(fid, b), O.array(fid, c)))
    assert H[n - 1] == 0
    A, B, C = (O.ints(fid, O.intt(fid, O.array(fid, v))) for v in (a, b, c))
    lhs = O.schoolbook(fid, A, B)
    for i, v in enumerate(C):
        lhs[i] = (lhs[i] - v) % p
    z = [p - 1] + [0] * (n - 1) + [1]  # x^n - 1
    rhs = O.schoolbook(fid, H[: n - 1], z)
    assert lhs[: len(rhs)] == rhs and all(v == 0 for v in lhs[len(rhs):])
    x = O.array(fid, a)
    s = rnd.randrange(2, p)
    assert O.ints(fid, O.coset_intt(fid, O.coset_ntt(fid, x, s), s)) == a


@pytest.mark.parametrize("fid", [0, 1])
def test_ntt_polynomial_product(fid):
    rnd = random.Random(11 + fid)
    p = O.MODULI[fid]
    deg = 37
    a = [rnd.randrange(p) for _ in range(deg + 1)]
    b = [rnd.randrange(p) for _ in range(deg + 1)]
    n = 128
    A = O.ntt(fid, O.array(fid, a + [0] * (n - len(a))))
    B = O.ntt(fid, O.array(fid, b + [0] * (n - len(b))))
    prod = [(x * y) % p for x, y in zip(O.ints(fid, A), O.ints(fid, B))]
    c = O.ints(fid, O.intt(fid, O.array(fid, prod)))
    assert c[: 2 * deg + 1] == O.schoolbook(fid, a, b)
    assert all(v == 0 for v in c[2 * deg + 1:])


def test_refscalar_arith_golden():
    g = np.load(GOLDEN / "refscalar_arith.npz")
    for i in range(len(g["a"])):
        a, b = g["a"][i], g["b"][i]
        assert (O.refscalar_arith("mul", a, b) == g["mul"][i]).all()
        assert (O.refscalar_arith("add", a, b) == g["add"][i]).all()
        assert (O.refscalar_arith("sub", a, b) == g["sub"][i]).all()
        assert (O.refscalar_arith("pow", a, None, int(g["e"][i])) == g["pow"][i]).all()


def test_refscalar_mul_is_not_modular():
    """The reference product is not a*b*R^-1 mod q (m_inv and normalisation quirks)."""
    q = O.MODULI[3]
    a = np.zeros(24, dtype=np.uint32)
    b = np.zeros(24, dtype=np.uint32)
    a[0], b[0] = 1234, 5678
    got = O.from_limbs(O.refscalar_arith("mul", a, b))
    assert got != (1234 * 5678 * pow(1 << 768, -1, q)) % q


def test_refscalar_fft_golden_n4096():
    g = np.load(GOLDEN / "refscalar_fft_n4096.npz")
    data = np.zeros((4096, 24), dtype=np.uint32)
    data[:, 0] = 1234
    out = O.refscalar_fft(data, REF_Q, log_cpus=10)
    assert (out == g["out"]).all()
    assert hashlib.sha256(out.tobytes()).hexdigest() == str(g["sha256"])


@pytest.mark.slow
def test_refscalar_fft_golden_shipped_config():
    """test/main.cpp:45-71 at n = 2^16 (about a minute on 8 cores)."""
    g = np.load(GOLDEN / "refscalar_fft_n65536.npz")
    data = np.zeros((65536, 24), dtype=np.uint32)
    data[:, 0] = 1234
    out = O.refscalar_fft(data, REF_Q, log_cpus=10)
    assert (out[:32] == g["head"]).all()
    assert hashlib.sha256(out.tobytes()).hexdigest() == str(g["sha256"])


@pytest.mark.parametrize("name,fid", [("p32", 0), ("bls12_381_fr", 1), ("mnt4753_fr", 2)])
def test_ref_butterfly_golden(name, fid):
    """The restatement with the reference butterfly equals fft_host.h as shipped."""
    g = np.load(GOLDEN / f"ref_butterfly_{name}.npz")
    w = O.from_limbs(g["omega"])
    lc = int(g["log_cpus"])
    assert (O.fft(fid, g["x"], w, serial=True, ref_butterfly=True) == g["serial"]).all()
    assert (O.fft(fid, g["x"], w, log_cpus=lc, ref_butterfly=True) == g["parallel"]).all()


def test_against_compiled_reference_when_present():
    ref = O.ref()
    if ref is None:
        pytest.skip("reference checkout absent; golden fixtures cover this")
    rnd = random.Random(5)
    for fid, log_n in ((0, 9), (1, 6), (2, 5)):
        p = O.MODULI[fid]
        x = O.array(fid, [rnd.randrange(p) for _ in range(1 << log_n)])
        w = O.root(fid, log_n)
        wl = O.to_limbs(fid, w)
        y = x.copy()
        ref.ref_fft_oracle_field(fid, O._ptr(y), log_n, O._ptr(wl), 3, 0, 0)
        assert (O.fft(fid, x, w, log_cpus=3, ref_butterfly=True) == y).all()


@pytest.mark.parametrize("fid,name", [(0, "p32"), (1, "bls12_381_fr"), (2, "mnt4753_fr")])
def test_multiexp_oracle_against_reference_fixtures(fid, name):
    """The restated multi_exp (test/multiexp.h:3-13) equals the compiled reference's own multi_exp over
    the same field type (golden fixtures) and the definition sum a_i b_i (Python integers)."""
    g = np.load(pathlib.Path(__file__).parent / "golden" / f"ref_multiexp_{name}.npz")
    for n in g["lengths"]:
        a, b = g[f"a_{n}"], g[f"b_{n}"]
        for mode in (0, 1):
            got = O.multiexp(fid, a, b, mode)
            assert np.array_equal(got, g[f"out_{n}_mode{mode}"]), (n, mode)
            if n <= 257:
                assert O.from_limbs(got) == O.multiexp_definition(fid, a, b, mode), (n, mode)


def test_multiexp_oracle_against_compiled_reference_when_present():
    ref = O.ref()
    if ref is None:
        pytest.skip("reference checkout not present")
    import random
    for fid in (0, 1, 2):
        rnd = random.Random(77 + fid)
        p = O.MODULI[fid]
        n = 333
        a = O.array(fid, [rnd.randrange(p) for _ in range(n)])
        b = O.array(fid, [rnd.randrange(p) for _ in range(n)])
        for mode in (0, 1):
            out = np.zeros(O.LIMBS[fid], dtype=np.uint32)
            assert ref.ref_multi_exp_oracle_field(fid, O._ptr(a), O._ptr(b), n, mode, O._ptr(out)) == 0
            assert np.array_equal(O.multiexp(fid, a, b, mode), out)
