"""ORACLE — test infrastructure only.

The CPU checker for the NTT path.  Only tests/, ``__graft_entry__.smoke()`` and
bench.py's CPU-baseline / reference legs may import this package, and only to
check or to time the CPU restatement; the product (gpusnarks_gb300) never
imports it.

Contents:

* ctypes bindings to oracle/_build/liboracle.so (oracle.cpp): the restated
  reference host FFT (test/fft_host.h:18-118) over correct fields, with the
  fixed or the reference butterfly, and the restated reference ``Scalar``
  arithmetic (cuda/device_field_operators.h:92-258);
* ctypes bindings to oracle/_ref/libref.so (ref_driver.cpp), the reference's
  own headers compiled unmodified, when it was built;
* pure-Python big-integer definitions: naive DFT, inverse, coset DFT and
  schoolbook polynomial product for small sizes.  These are the mathematical
  definitions and pin the restatement.

The moduli below are written out independently of gpusnarks_gb300/fields.py
(from the task configuration and cuda/device_field.h:443-446) so that a wrong
product constant cannot hide behind a shared definition.
"""
from __future__ import annotations

import ctypes
import pathlib

import numpy as np

from . import build as _build

MODULI = {
    0: 3221225473,
    1: 0x73EDA753299D7D483339D80809A1D80553BDA402FFFE5BFEFFFFFFFF00000001,
    2: int("41898490967918953402344214791240637128170709919953949071783502921025352812571106773058"
           "893763790338921418070971888458477323173057491593855069696241854796396165721416325350"
           "064441470418137846398469611935719059908164220784476160001"),
    3: int("41898490967918953402344214791240637128170709919953949071783502921025352812571106773058"
           "893763790338921418070971888253786114353726529584385201591605722013126468931404347949"
           "840543007986327743462853720628051692141265303114721689601"),
}
LIMBS = {0: 1, 1: 8, 2: 24, 3: 24}
GENERATORS = {0: 5, 1: 7, 2: 11, 3: 13}

_lib = None
_ref = None
_u32p = ctypes.POINTER(ctypes.c_uint32)


def lib():
    global _lib
    if _lib is None:
        so = _build.build_oracle()
        _lib = ctypes.CDLL(str(so))
        _lib.oracle_fft.argtypes = [ctypes.c_int, _u32p, ctypes.c_int, _u32p, ctypes.c_int,
                                    ctypes.c_int, ctypes.c_int, ctypes.c_int]
        _lib.oracle_arith.argtypes = [ctypes.c_int, ctypes.c_int, _u32p, _u32p, ctypes.c_uint64, _u32p]
        _lib.oracle_refscalar_arith.argtypes = [ctypes.c_int, _u32p, _u32p, ctypes.c_uint64, _u32p]
        _lib.oracle_refscalar_fft.argtypes = [_u32p, ctypes.c_int, _u32p, ctypes.c_int, ctypes.c_int]
        _lib.oracle_multiexp.argtypes = [ctypes.c_int, _u32p, _u32p, ctypes.c_uint64, ctypes.c_int, _u32p]
    return _lib


def ref():
    """The reference's own headers compiled unmodified, or None when absent."""
    global _ref
    if _ref is None:
        so = _build.build_ref()
        if so is None or not so.exists():
            return None
        _ref = ctypes.CDLL(str(so))
        _ref.ref_scalar_arith.argtypes = [ctypes.c_int, _u32p, _u32p, ctypes.c_uint32, _u32p]
        _ref.ref_scalar_fft.argtypes = [_u32p, ctypes.c_int, _u32p, ctypes.c_int, ctypes.c_int]
        _ref.ref_fft_oracle_field.argtypes = [ctypes.c_int, _u32p, ctypes.c_int, _u32p, ctypes.c_int,
                                              ctypes.c_int, ctypes.c_int]
        _ref.ref_multi_exp_oracle_field.argtypes = [ctypes.c_int, _u32p, _u32p, ctypes.c_uint64, ctypes.c_int,
                                                    _u32p]
    return _ref


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(_u32p)


def to_limbs(fid: int, x: int) -> np.ndarray:
    return np.array([(x >> (32 * i)) & 0xFFFFFFFF for i in range(LIMBS[fid])], dtype=np.uint32)


def from_limbs(limbs) -> int:
    return sum(int(v) << (32 * i) for i, v in enumerate(np.asarray(limbs).reshape(-1)))


def root(fid: int, log_n: int) -> int:
    p = MODULI[fid]
    return pow(GENERATORS[fid], (p - 1) >> log_n, p)


# --- C restatement ------------------------------------------------------------

def fft(fid: int, data: np.ndarray, omega: int, *, log_cpus: int = 0, nthreads: int = 0,
        ref_butterfly: bool = False, serial: bool = False) -> np.ndarray:
    """Restated fft_host.h over field ``fid``; returns a new array (same shape)."""
    a = np.ascontiguousarray(data, dtype=np.uint32).copy()
    n = a.size // LIMBS[fid]
    log_n = n.bit_length() - 1
    assert 1 << log_n == n
    w = to_limbs(fid, omega)
    rc = lib().oracle_fft(fid, _ptr(a), log_n, _ptr(w), log_cpus, nthreads, int(ref_butterfly), int(serial))
    if rc != 0:
        raise RuntimeError(f"oracle_fft failed rc={rc}")
    return a


def ntt(fid: int, data: np.ndarray, omega: int | None = None, *, nthreads: int = 0, log_cpus: int | None = None):
    """Forward NTT with the fixed butterfly (natural order in and out)."""
    n = np.asarray(data).size // LIMBS[fid]
    log_n = n.bit_length() - 1
    if omega is None:
        omega = root(fid, log_n)
    if log_cpus is None:
        log_cpus = min(3, log_n)
    return fft(fid, data, omega, log_cpus=log_cpus, nthreads=nthreads)


def intt(fid: int, data: np.ndarray, omega: int | None = None, *, nthreads: int = 0):
    """Inverse NTT: forward with omega^-1, then scale by n^-1."""
    p = MODULI[fid]
    n = np.asarray(data).size // LIMBS[fid]
    log_n = n.bit_length() - 1
    if omega is None:
        omega = root(fid, log_n)
    out = ntt(fid, data, pow(omega, p - 2, p), nthreads=nthreads)
    return scale(fid, out, pow(n, p - 2, p))


def scale(fid: int, data: np.ndarray, c: int) -> np.ndarray:
    """Multiply every element by the constant c (Python ints; small/medium n)."""
    p = MODULI[fid]
    xs = ints(fid, data)
    return array(fid, [(x * c) % p for x in xs], like=data)


def coset_ntt(fid: int, data: np.ndarray, shift: int, omega: int | None = None, *, nthreads: int = 0):
    """NTT of x_i * shift^i."""
    p = MODULI[fid]
    xs = ints(fid, data)
    pre, s = [], 1
    for x in xs:
        pre.append((x * s) % p)
        s = (s * shift) % p
    return ntt(fid, array(fid, pre, like=data), omega, nthreads=nthreads)


def coset_intt(fid: int, data: np.ndarray, shift: int, omega: int | None = None, *, nthreads: int = 0):
    """Inverse of coset_ntt: inverse NTT, then x_i * shift^-i."""
    p = MODULI[fid]
    xs = ints(fid, intt(fid, data, omega, nthreads=nthreads))
    sinv, s, out = pow(shift, p - 2, p), 1, []
    for x in xs:
        out.append((x * s) % p)
        s = (s * sinv) % p
    return array(fid, out, like=data)


def qap_h(fid: int, a: np.ndarray, b: np.ndarray, c: np.ndarray, shift: int | None = None) -> np.ndarray:
    """H = (A B - C) / (x^n - 1) of the QAP witness map, from the evaluations of A, B, C on the size-n
    domain (the published algorithm of libsnark's r1cs_to_qap_witness_map, a third-party prover
    that the reference's MNT4-753 types serve, cuda/device_field.h:443-447): interpolate A, B, C
    (inverse NTT), evaluate them on the coset shift*<w> (coset NTT), divide A*B - C pointwise by
    Z(shift w^i) = shift^n - 1, interpolate on the coset (coset inverse NTT)."""
    p = MODULI[fid]
    if shift is None:
        shift = GENERATORS[fid]
    n = np.asarray(a).size // LIMBS[fid]
    ev = [ints(fid, coset_ntt(fid, intt(fid, x), shift)) for x in (a, b, c)]
    zinv = pow((pow(shift, n, p) - 1) % p, p - 2, p)
    h = [((x * y - z) * zinv) % p for x, y, z in zip(*ev)]
    return coset_intt(fid, array(fid, h, like=a), shift)


def arith(fid: int, op: str, a: int, b: int = 0, e: int = 0) -> int:
    code = {"mul": 0, "add": 1, "sub": 2, "pow": 3}[op]
    out = np.zeros(LIMBS[fid], dtype=np.uint32)
    la, lb = to_limbs(fid, a), to_limbs(fid, b)
    lib().oracle_arith(fid, code, _ptr(la), _ptr(lb), e, _ptr(out))
    return from_limbs(out)


def refscalar_arith(op: str, a: np.ndarray, b: np.ndarray | None = None, e: int = 0) -> np.ndarray:
    code = {"mul": 0, "add": 1, "sub": 2, "pow": 3}[op]
    a = np.ascontiguousarray(a, dtype=np.uint32)
    b = np.zeros(24, dtype=np.uint32) if b is None else np.ascontiguousarray(b, dtype=np.uint32)
    out = np.zeros(24, dtype=np.uint32)
    lib().oracle_refscalar_arith(code, _ptr(a), _ptr(b), e, _ptr(out))
    return out


def refscalar_fft(data: np.ndarray, omega_limbs: np.ndarray, log_cpus: int, nthreads: int = 0) -> np.ndarray:
    a = np.ascontiguousarray(data, dtype=np.uint32).copy()
    n = a.size // 24
    w = np.ascontiguousarray(omega_limbs, dtype=np.uint32)
    lib().oracle_refscalar_fft(_ptr(a), n.bit_length() - 1, _ptr(w), log_cpus, nthreads)
    return a


MULTIEXP_CANONICAL, MULTIEXP_MONTGOMERY = 0, 1


def multiexp(fid: int, a: np.ndarray, b: np.ndarray, mode: int = MULTIEXP_CANONICAL) -> np.ndarray:
    """sum_i a[i] * b[i], the restated multi_exp of test/multiexp.h:3-13 (serial, index order).  mode 0:
    canonical integers in and out; mode 1: the words are Montgomery forms (each term is the Montgomery
    product of the stored words, as the reference's Scalar::operator* is)."""
    a = np.ascontiguousarray(a, dtype=np.uint32)
    b = np.ascontiguousarray(b, dtype=np.uint32)
    n = a.size // LIMBS[fid]
    assert b.size == a.size
    out = np.zeros(LIMBS[fid], dtype=np.uint32)
    rc = lib().oracle_multiexp(fid, _ptr(a), _ptr(b), n, mode, _ptr(out))
    if rc != 0:
        raise RuntimeError(f"oracle_multiexp failed rc={rc}")
    return out


def multiexp_definition(fid: int, a, b, mode: int = MULTIEXP_CANONICAL) -> int:
    """The mathematical definition with Python integers: sum a_i b_i mod p (canonical), or
    sum a_i b_i R^-1 mod p (Montgomery forms, R = 2^(32 limbs))."""
    p = MODULI[fid]
    s = sum(x * y for x, y in zip(ints(fid, a), ints(fid, b))) % p
    if mode == MULTIEXP_MONTGOMERY:
        s = s * pow(1 << (32 * LIMBS[fid]), p - 2, p) % p
    return s


def max_threads() -> int:
    return lib().oracle_max_threads()


# --- pure-Python definitions --------------------------------------------------

def ints(fid: int, arr) -> list[int]:
    a = np.ascontiguousarray(arr, dtype=np.uint32).reshape(-1, LIMBS[fid])
    return [from_limbs(row) for row in a]


def array(fid: int, xs, like=None) -> np.ndarray:
    L = LIMBS[fid]
    out = np.zeros((len(xs), L), dtype=np.uint32)
    for i, x in enumerate(xs):
        for j in range(L):
            out[i, j] = (x >> (32 * j)) & 0xFFFFFFFF
    if like is not None:
        return out.reshape(np.asarray(like).shape)
    return out if L > 1 else out.reshape(-1)


def naive_dft(fid: int, xs: list[int], omega: int) -> list[int]:
    """X[k] = sum_j x[j] omega^(jk) mod p, O(n^2)."""
    p = MODULI[fid]
    n = len(xs)
    pw = [pow(omega, e, p) for e in range(n)]
    return [sum(x * pw[(j * k) % n] for j, x in enumerate(xs)) % p for k in range(n)]


def schoolbook(fid: int, a: list[int], b: list[int]) -> list[int]:
    p = MODULI[fid]
    out = [0] * (len(a) + len(b) - 1)
    for i, x in enumerate(a):
        if x:
            for j, y in enumerate(b):
                out[i + j] += x * y
    return [v % p for v in out]
