"""Generate the golden fixtures in tests/golden/ from the reference itself.

Requires the reference checkout (default /root/reference, or
GSN_REFERENCE_ROOT): oracle/build.py compiles its own headers, unmodified,
into oracle/_ref/libref.so, and every output below comes from that library —
not from the oracle restatement.  The tests then check the oracle against
these files, so the oracle stays pinned on machines without the checkout.

Fixtures (all numpy .npz, little-endian uint32 limbs):

* ``refscalar_arith.npz``  the reference ``fields::Scalar`` operators
  (cuda/device_field.h:115-158) on seeded 24-limb operands.
* ``refscalar_fft_n4096.npz``  the reference host FFT over the reference
  Scalar at its shipped call (test/main.cpp:45-71: every input Scalar(1234),
  omega = Scalar(_mod), one = Scalar::one(), log_cpus = 10), at n = 2^12.
* ``refscalar_fft_n65536.npz``  the same at the shipped n = 2^16: a SHA-256 of
  the full output and its first 32 elements (the full output is 6 MiB).
* ``ref_butterfly_<field>.npz``  the reference host FFT (test/fft_host.h, its
  own butterfly) over the oracle's correct field type, on seeded inputs, both
  the serial loop and the num_cpus decomposition with log_cpus = 2.
* ``ref_multiexp_<field>.npz``  the reference's CPU multi-exponentiation
  multi_exp (test/multiexp.h:3-13) over the oracle's correct field type on
  seeded vectors of several lengths (0, 1, 257, 1024), canonical integers and
  stored Montgomery forms.  ``--only multiexp`` writes just these.

Run: ``python tests/golden/make_golden.py`` (about a minute, mostly the
2^16 reference run).
"""
from __future__ import annotations

import hashlib
import pathlib
import random
import sys

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

import oracle  # noqa: E402

FIELD_NAMES = {0: "p32", 1: "bls12_381_fr", 2: "mnt4753_fr"}
REF_Q_LIMBS = np.array([610172929, 1586521054, 752685471, 3818738770, 2596546032, 1669861489,
                        1987204260, 1750781161, 3411246648, 3087994277, 4061660573, 2971133814,
                        2707093405, 2580620505, 3902860685, 134068517, 1821890675, 1589111033,
                        1536143341, 3086587728, 4007841197, 270700578, 764593169, 115910],
                       dtype=np.uint32)


def _seeded_elements(fid: int, n: int, seed: int) -> np.ndarray:
    rnd = random.Random(seed)
    p = oracle.MODULI[fid]
    return oracle.array(fid, [rnd.randrange(p) for _ in range(n)])


MULTIEXP_LENGTHS = (0, 1, 257, 1024)


def write_multiexp(ref) -> None:
    p_ = oracle._ptr
    for fid in (0, 1, 2):
        L = oracle.LIMBS[fid]
        kw = {}
        for n in MULTIEXP_LENGTHS:
            a = _seeded_elements(fid, n, 0x5EED0300 + 16 * fid + n % 16).reshape(n, L) if n else \
                np.zeros((0, L), dtype=np.uint32)
            b = _seeded_elements(fid, n, 0x5EED0380 + 16 * fid + n % 16).reshape(n, L) if n else \
                np.zeros((0, L), dtype=np.uint32)
            a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
            kw[f"a_{n}"], kw[f"b_{n}"] = a, b
            for mode in (0, 1):
                out = np.zeros(L, dtype=np.uint32)
                rc = ref.ref_multi_exp_oracle_field(fid, p_(a), p_(b), n, mode, p_(out))
                assert rc == 0
                kw[f"out_{n}_mode{mode}"] = out
        np.savez_compressed(HERE / f"ref_multiexp_{FIELD_NAMES[fid]}.npz", lengths=np.array(MULTIEXP_LENGTHS), **kw)


def main() -> None:
    ref = oracle.ref()
    if ref is None:
        raise SystemExit("reference checkout not found; cannot generate golden fixtures")
    if "--only" in sys.argv and sys.argv[sys.argv.index("--only") + 1] == "multiexp":
        write_multiexp(ref)
        print("multiexp fixtures written to", HERE)
        return
    p_ = oracle._ptr

    # 1. Scalar operator KATs
    rnd = random.Random(0x5EED0100)
    A, B, MUL, ADD, SUB, POW, E = [], [], [], [], [], [], []
    for k in range(32):
        a = np.array([rnd.getrandbits(32) for _ in range(24)], dtype=np.uint32)
        b = np.array([rnd.getrandbits(32) for _ in range(24)], dtype=np.uint32)
        # keep operands below 2^753 like reduced field elements; a few small ones
        a[23] &= 0x1FFFF
        b[23] &= 0x1FFFF
        if k < 4:
            a[:] = 0
            b[:] = 0
            a[0], b[0] = 1234 + k, 5678 + k
        e = rnd.randrange(0, 200)
        outs = []
        for code, bb, ee in ((0, b, 0), (1, b, 0), (2, b, 0), (3, a, e)):
            o = np.zeros(24, dtype=np.uint32)
            ref.ref_scalar_arith(code, p_(a), p_(bb), ee, p_(o))
            outs.append(o)
        A.append(a); B.append(b); E.append(e)
        MUL.append(outs[0]); ADD.append(outs[1]); SUB.append(outs[2]); POW.append(outs[3])
    np.savez_compressed(HERE / "refscalar_arith.npz", a=np.array(A), b=np.array(B), e=np.array(E, dtype=np.uint32),
                        mul=np.array(MUL), add=np.array(ADD), sub=np.array(SUB), pow=np.array(POW))

    # 2/3. the shipped FFT call
    for log_n, full in ((12, True), (16, False)):
        n = 1 << log_n
        data = np.zeros((n, 24), dtype=np.uint32)
        data[:, 0] = 1234
        ref.ref_scalar_fft(p_(data), log_n, p_(REF_Q_LIMBS), 10, 0)
        digest = hashlib.sha256(data.tobytes()).hexdigest()
        kw = {"log_n": log_n, "log_cpus": 10, "input_value": 1234, "sha256": digest}
        if full:
            kw["out"] = data
        else:
            kw["head"] = data[:32].copy()
        np.savez_compressed(HERE / f"refscalar_fft_n{n}.npz", **kw)
        print(f"refscalar fft n=2^{log_n}: {digest}")

    # 4. reference butterfly over correct fields
    for fid, log_n in ((0, 10), (1, 8), (2, 7)):
        x = _seeded_elements(fid, 1 << log_n, 0x5EED0200 + fid)
        w = oracle.root(fid, log_n)
        wl = oracle.to_limbs(fid, w)
        outs = {}
        for serial in (1, 0):
            y = x.copy()
            rc = ref.ref_fft_oracle_field(fid, p_(y), log_n, p_(wl), 2, 0, serial)
            assert rc == 0
            outs["serial" if serial else "parallel"] = y
        np.savez_compressed(HERE / f"ref_butterfly_{FIELD_NAMES[fid]}.npz", x=x, omega=wl, log_cpus=2,
                            **outs)
    # 5. multi-exponentiation
    write_multiexp(ref)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
