"""Field definitions for the NTT path (product side).

Every field element is stored the way the reference stores ``fields::Scalar``
(cuda/device_field.h:75): an array of little-endian 32-bit limbs
``uint32_t im_rep[LIMBS]``.  Here that is a numpy ``uint32`` array of shape
``(n, LIMBS)`` (``(n,)`` for the one-limb field).

Fields:

* ``P32``        p = 3*2^30 + 1, one limb, generator 5 (2-adicity 30).
* ``BLS12_381``  BLS12-381 scalar field r, 8 limbs, generator 7 (2-adicity 32).
* ``MNT4_753``   MNT4-753 scalar field r, 24 limbs, generator 11 (2-adicity 30).
                 The decimal value is the second modulus listed in
                 cuda/device_field.h:445-446.
* ``MNT4_753_Q`` MNT4-753 base field q, the modulus the reference actually
                 compiles in (cuda/device_field.h:62-65); 2-adicity 15.  It is
                 carried for the reference-arithmetic comparison only.

The generator of each NTT field is a quadratic non-residue, so
``g^((p-1)/2^k)`` has exact order ``2^k`` for every ``k`` up to the 2-adicity.
The reference ships no generator and ignores the ``omg`` argument of
``best_fft`` (cuda/fft_kernel.cu:117-147; the kernel uses the raw modulus limbs, :65-68); these are this library's choices.
"""
from __future__ import annotations

from dataclasses import dataclass, field as dc_field

import numpy as np

# Limbs of the reference modulus, as written in cuda/device_field.h:62-65.
_REF_Q_LIMBS = (
    610172929, 1586521054, 752685471, 3818738770, 2596546032, 1669861489,
    1987204260, 1750781161, 3411246648, 3087994277, 4061660573, 2971133814,
    2707093405, 2580620505, 3902860685, 134068517, 1821890675, 1589111033,
    1536143341, 3086587728, 4007841197, 270700578, 764593169, 115910)

_MNT4_R = int(
    "41898490967918953402344214791240637128170709919953949071783502921025352812"
    "57110677305889376379033892141807097188845847732317305749159385506969624185"
    "4796396165721416325350064441470418137846398469611935719059908164220784476160001")


def _limbs_to_int(limbs) -> int:
    return sum(int(v) << (32 * i) for i, v in enumerate(limbs))


@dataclass(frozen=True)
class Field:
    name: str
    fid: int                 # id used by the C ABI (gsn_field)
    limbs: int
    p: int
    generator: int | None
    two_adicity: int = dc_field(init=False)

    def __post_init__(self):
        s, t = 0, self.p - 1
        while t % 2 == 0:
            t //= 2
            s += 1
        object.__setattr__(self, "two_adicity", s)

    # --- integer helpers -------------------------------------------------
    @property
    def R(self) -> int:
        return 1 << (32 * self.limbs)

    @property
    def pinv(self) -> int:
        """-p^-1 mod 2^32 (the CIOS constant)."""
        return (-pow(self.p, -1, 1 << 32)) % (1 << 32)

    def root(self, log_n: int) -> int:
        """Primitive 2^log_n-th root of unity g^((p-1)/2^log_n)."""
        if log_n > self.two_adicity:
            raise ValueError(f"{self.name}: 2^{log_n} exceeds 2-adicity {self.two_adicity}")
        return pow(self.generator, (self.p - 1) >> log_n, self.p)

    def to_limbs(self, x: int) -> np.ndarray:
        return np.array([(x >> (32 * i)) & 0xFFFFFFFF for i in range(self.limbs)], dtype=np.uint32)

    def from_limbs(self, arr) -> int:
        return _limbs_to_int(np.asarray(arr, dtype=np.uint32).reshape(-1)[: self.limbs])

    def to_mont(self, x: int) -> int:
        return (x * self.R) % self.p

    def from_mont(self, x: int) -> int:
        return (x * pow(self.R, -1, self.p)) % self.p

    # --- arrays ------------------------------------------------------------
    def shape(self, n: int):
        return (n,) if self.limbs == 1 else (n, self.limbs)

    def ints_to_array(self, xs) -> np.ndarray:
        xs = list(xs)
        out = np.zeros((len(xs), self.limbs), dtype=np.uint32)
        for i, x in enumerate(xs):
            for j in range(self.limbs):
                out[i, j] = (x >> (32 * j)) & 0xFFFFFFFF
        return out.reshape(self.shape(len(xs)))

    def array_to_ints(self, arr) -> list[int]:
        a = np.ascontiguousarray(arr, dtype=np.uint32).reshape(-1, self.limbs).astype(object)
        shifts = [1 << (32 * j) for j in range(self.limbs)]
        return [sum(int(row[j]) * shifts[j] for j in range(self.limbs)) for row in a]

    def random_array(self, n: int, seed: int) -> np.ndarray:
        """Uniform elements of [0, p) by rejection sampling on limb-wise bits.

        splitmix64 seeded with ``seed`` fills the limbs, the top limb is masked
        to ``bitlen(p)`` and values >= p are redrawn.  Vectorised in numpy so a
        2^22 x 24-limb input takes well under a second.
        """
        nbits = self.p.bit_length()
        top_bits = nbits - 32 * (self.limbs - 1)
        top_mask = np.uint32((1 << top_bits) - 1)
        p_limbs = self.to_limbs(self.p)
        out = np.empty((n, self.limbs), dtype=np.uint32)
        need = np.arange(n)
        state = np.uint64(seed)
        while need.size:
            words, state = _splitmix_words(state, need.size * self.limbs)
            cand = words.reshape(need.size, self.limbs)
            cand[:, -1] &= top_mask
            ok = _lt_limbs(cand, p_limbs)
            out[need[ok]] = cand[ok]
            need = need[~ok]
        return out.reshape(self.shape(n))


    def device_random(self, n: int, seed: int, start: int = 0) -> np.ndarray:
        """Host replica of gsn_fill_random: elements [start, start+n) of the stream.

        Limb j of attempt a of element i is the low word of splitmix64's
        finaliser of seed + (i*64*N + a*N + j + 1) * 0x9E3779B97F4A7C15; the
        top limb is masked to bitlen(p) and the first attempt below p wins.
        """
        N = self.limbs
        top_bits = self.p.bit_length() - 32 * (N - 1)
        top_mask = np.uint64((1 << top_bits) - 1) if top_bits < 32 else np.uint64(0xFFFFFFFF)
        p_limbs = self.to_limbs(self.p)
        idx = np.arange(start, start + n, dtype=np.uint64)
        out = np.zeros((n, N), dtype=np.uint32)
        done = np.zeros(n, dtype=bool)
        golden = np.uint64(0x9E3779B97F4A7C15)
        with np.errstate(over="ignore"):
            for a in range(64):
                if done.all():
                    break
                cand = np.empty((n, N), dtype=np.uint32)
                for j in range(N):
                    ctr = idx * np.uint64(64 * N) + np.uint64(a * N + j + 1)
                    z = np.uint64(seed) + ctr * golden
                    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
                    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
                    z = z ^ (z >> np.uint64(31))
                    w = z & np.uint64(0xFFFFFFFF)
                    if j == N - 1:
                        w &= top_mask
                    cand[:, j] = w.astype(np.uint32)
                ok = _lt_limbs(cand, p_limbs) & ~done
                out[ok] = cand[ok]
                done |= ok
        return out.reshape(self.shape(n))


def _splitmix_words(state: np.uint64, count: int):
    """``count`` 32-bit words from a splitmix64 stream (two per output)."""
    m = (count + 1) // 2
    with np.errstate(over="ignore"):
        idx = np.arange(1, m + 1, dtype=np.uint64)
        z = state + idx * np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
        new_state = state + np.uint64(m) * np.uint64(0x9E3779B97F4A7C15)
    w = np.empty(2 * m, dtype=np.uint32)
    w[0::2] = (z & np.uint64(0xFFFFFFFF)).astype(np.uint32)
    w[1::2] = (z >> np.uint64(32)).astype(np.uint32)
    return w[:count], new_state


def _lt_limbs(cand: np.ndarray, p_limbs: np.ndarray) -> np.ndarray:
    """Row-wise cand < p for little-endian limb rows."""
    lt = np.zeros(cand.shape[0], dtype=bool)
    eq = np.ones(cand.shape[0], dtype=bool)
    for j in range(cand.shape[1] - 1, -1, -1):
        c = cand[:, j]
        lt |= eq & (c < p_limbs[j])
        eq &= c == p_limbs[j]
    return lt


P32 = Field("p32", 0, 1, 3 * 2**30 + 1, 5)
BLS12_381 = Field("bls12_381_fr", 1, 8,
                  0x73EDA753299D7D483339D80809A1D80553BDA402FFFE5BFEFFFFFFFF00000001, 7)
MNT4_753 = Field("mnt4753_fr", 2, 24, _MNT4_R, 11)
MNT4_753_Q = Field("mnt4753_fq", 3, 24, _limbs_to_int(_REF_Q_LIMBS), 13)

FIELDS = {f.name: f for f in (P32, BLS12_381, MNT4_753, MNT4_753_Q)}
BY_ID = {f.fid: f for f in FIELDS.values()}
