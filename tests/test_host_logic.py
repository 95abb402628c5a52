"""Host-side generators and helpers (no GPU): the seeded inputs every benchmark and test uses."""
import numpy as np

import gpusnarks_gb300.fields as F
from gpusnarks_gb300.batch import job_sizes
from gpusnarks_gb300.serve import poisson_trace

GOLDEN = 0x9E3779B97F4A7C15
MASK64 = (1 << 64) - 1


def _splitmix(z):
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9 & MASK64
    z = (z ^ (z >> 27)) * 0x94D049BB133111EB & MASK64
    return z ^ (z >> 31)


def _device_random_scalar(f, i, seed):
    """The documented stream of gsn_fill_random for element i, in plain Python integers."""
    n_limbs = f.limbs
    top_bits = f.p.bit_length() - 32 * (n_limbs - 1)
    for a in range(64):
        limbs = []
        for j in range(n_limbs):
            ctr = i * 64 * n_limbs + a * n_limbs + j + 1
            w = _splitmix((seed + ctr * GOLDEN) & MASK64) & 0xFFFFFFFF
            if j == n_limbs - 1 and top_bits < 32:
                w &= (1 << top_bits) - 1
            limbs.append(w)
        v = sum(w << (32 * j) for j, w in enumerate(limbs))
        if v < f.p:
            return v
    return 0


def test_device_random_follows_its_documented_stream():
    for f in (F.P32, F.BLS12_381, F.MNT4_753):
        seed = 0x5EED0000 + f.fid
        got = f.device_random(40, seed, start=1000)
        for i in range(40):
            assert f.from_limbs(got.reshape(40, -1)[i]) == _device_random_scalar(f, 1000 + i, seed)


def test_device_random_is_canonical_and_chunkable():
    for f in (F.P32, F.BLS12_381, F.MNT4_753):
        a = f.device_random(300, 7)
        b = np.concatenate([f.device_random(100, 7, start=s).reshape(100, -1) for s in (0, 100, 200)])
        assert np.array_equal(a.reshape(300, -1), b)
        assert all(v < f.p for v in f.array_to_ints(a))


def test_poisson_trace_is_seeded_and_shaped():
    t1 = poisson_trace(2000, 2000.0, 5)
    t2 = poisson_trace(2000, 2000.0, 5)
    assert t1 == t2 and t1 != poisson_trace(2000, 2000.0, 6)
    arrivals = np.array([e[0] for e in t1])
    assert arrivals[0] == 0.0 and np.all(np.diff(arrivals) >= 0)
    assert abs(arrivals[-1] - 1.0) < 0.15  # 2000 arrivals at 2000/s
    assert {e[1] for e in t1} == {1, 2} and {e[3] for e in t1} == {0, 1, 2}
    ks = np.array([e[2] for e in t1])
    assert ks.min() == 12 and ks.max() == 22


def test_job_sizes_are_seeded_and_in_range():
    a = job_sizes(4096, 10, 20, 0x5EED0004)
    assert a == job_sizes(4096, 10, 20, 0x5EED0004)
    assert min(a) == 10 and max(a) == 20 and len(set(a)) == 11
