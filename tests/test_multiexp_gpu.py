"""Multi-exponentiation over field elements on the GPU (gsn_multiexp / gsn_multiexp_host, the reference's
multiexp of cuda/multi_exp.cu:104-137 for field elements) against the oracle's restatement of
test/multiexp.h:3-13 and the compiled reference's own outputs (golden fixtures).  Integer results: every
comparison is exact.

At sizes where the serial oracle would take too long, size-independent properties are checked:
with b constant c, the result is c * sum(a) (sum from exact limb-column sums), and the sum over the whole
array equals the sum of the sums over two parts.
"""
import pathlib

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu
GOLDEN = pathlib.Path(__file__).parent / "golden"


def _dev(g, x):
    return g.to_device(np.ascontiguousarray(x))


@pytest.mark.parametrize("fid,name", [(0, "p32"), (1, "bls12_381_fr"), (2, "mnt4753_fr")])
def test_multiexp_matches_reference_fixtures(gsn, cuda_device, fid, name):
    fx = np.load(GOLDEN / f"ref_multiexp_{name}.npz")
    f = gsn.BY_ID[fid]
    for n in fx["lengths"]:
        a, b = fx[f"a_{n}"], fx[f"b_{n}"]
        for mode in (0, 1):
            if n == 0:
                import torch
                da = torch.empty(f.limbs, dtype=torch.int32, device="cuda")
                out = gsn.multiexp(f, da[:0], da[:0], mode=mode)
            else:
                out = gsn.multiexp(f, _dev(gsn, a), _dev(gsn, b), mode=mode)
            got = gsn.to_host(out)
            assert np.array_equal(got, fx[f"out_{n}_mode{mode}"]), (n, mode)
            host = gsn.multiexp_host(a.reshape(-1, f.limbs) if f.limbs > 1 else a.reshape(-1),
                                     b.reshape(-1, f.limbs) if f.limbs > 1 else b.reshape(-1), field=f, mode=mode)
            assert np.array_equal(host, got), (n, mode)


@pytest.mark.parametrize("fid", [0, 1, 2])
@pytest.mark.parametrize("n", [2, 3, 31, 255, 256, 4097, 65541])
def test_multiexp_matches_oracle(gsn, cuda_device, fid, n):
    """Ragged lengths (tails of the 4-element loads of p32, partially filled blocks and warps)."""
    f = gsn.BY_ID[fid]
    if fid == 2 and n > 4097:
        n = 16411
    a = f.random_array(n, seed=0x5EED0C00 + 7 * fid + n)
    b = f.random_array(n, seed=0x5EED0D00 + 7 * fid + n)
    for mode in (0, 1):
        got = gsn.to_host(gsn.multiexp(f, _dev(gsn, a), _dev(gsn, b), mode=mode))
        assert np.array_equal(got, O.multiexp(fid, a, b, mode)), mode


def test_multiexp_extreme_values(gsn, cuda_device):
    """All elements p-1: every product and every partial sum takes its largest value."""
    for f in (gsn.P32, gsn.BLS12_381, gsn.MNT4_753):
        n = 3001
        pm1 = f.to_limbs(f.p - 1)
        a = np.tile(pm1, (n, 1)) if f.limbs > 1 else np.full(n, pm1[0], dtype=np.uint32)
        for mode in (0, 1):
            got = gsn.to_host(gsn.multiexp(f, _dev(gsn, a), _dev(gsn, a), mode=mode))
            assert np.array_equal(got, O.multiexp(f.fid, a, a, mode)), (f.name, mode)


def test_p32_unaligned_arrays(gsn, cuda_device):
    """p32 arrays only need 4-byte alignment: offset views take the scalar loads."""
    import torch
    f = gsn.P32
    n = 10001
    a = f.random_array(n + 1, seed=0x5EED0E01)
    b = f.random_array(n + 1, seed=0x5EED0E02)
    da, db = _dev(gsn, a), _dev(gsn, b)
    out = torch.empty(1, dtype=torch.int32, device="cuda")
    gsn.multiexp(f, da[1:], db[1:], out)
    assert np.array_equal(gsn.to_host(out), O.multiexp(0, a[1:], b[1:]))


def _limb_sum(arr: np.ndarray) -> int:
    cols = arr.astype(np.uint64).sum(axis=0, dtype=np.uint64)
    return sum(int(c) << (32 * i) for i, c in enumerate(cols))


@pytest.mark.parametrize("fid,log_n", [(0, 26), (1, 24), (2, 21)])
def test_multiexp_large_properties(gsn, cuda_device, fid, log_n):
    """Large arrays: with b = c everywhere the result is c * sum(a) mod p, and splitting the array in
    two uneven parts gives two results that add up to the whole."""
    import torch
    from gpusnarks_gb300.batch import fill_random
    f = gsn.BY_ID[fid]
    n = 1 << log_n
    a = torch.empty(n * f.limbs, dtype=torch.int32, device="cuda")
    b = torch.empty(n * f.limbs, dtype=torch.int32, device="cuda")
    fill_random(f, a, 0x5EED0F00 + fid)
    fill_random(f, b, 0x5EED0F80 + fid)
    whole = f.from_limbs(gsn.to_host(gsn.multiexp(f, a, b)))
    k = (n // 3) & ~3
    part1 = f.from_limbs(gsn.to_host(gsn.multiexp(f, a[:k * f.limbs], b[:k * f.limbs])))
    part2 = f.from_limbs(gsn.to_host(gsn.multiexp(f, a[k * f.limbs:], b[k * f.limbs:])))
    assert whole == (part1 + part2) % f.p
    c = f.random_array(1, seed=0x5EED0FFF + fid).reshape(-1)[:f.limbs]
    cc = torch.from_numpy(np.tile(c, n).view(np.int32)).to("cuda")
    got = f.from_limbs(gsn.to_host(gsn.multiexp(f, a, cc)))
    sa = _limb_sum(gsn.to_host(a).reshape(n, f.limbs))
    assert got == (f.from_limbs(c) * sa) % f.p
