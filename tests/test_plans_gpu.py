"""Every kernel variant through forced plans: a tuning table naming the plans is loaded, transforms are
checked bit for bit against the oracle (small sizes) and against the committed plans' output (large
sizes), forward and inverse, and the committed table is restored afterwards.

The register-blocked multi-limb pass (kernel 2) runs here for one to three passes, 4- and 8-row
sub-steps, 1, 2 and 4 columns per tile, radices that are and are not multiples of the sub-step."""
import json

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def rb_plan(log_n, radix, lj, e_log):
    """The plan make_rb_plan builds (runtime.cu): tile widths of make_split_plan, threads per pass."""
    npass = len(radix)
    log_j, block = [], []
    for i, r in enumerate(radix):
        last = i == npass - 1
        inner = sum(radix[i + 1:])
        j = (0 if npass == 1 else min(lj, radix[0])) if last else min(lj, inner)
        log_j.append(j)
        block.append(max(32, min(256, (1 << (r + j)) >> min(e_log, r))))
    pad = lambda v: v + [0] * (4 - len(v))
    return {"field": 1, "mode": 0, "log_n": log_n, "kernel": 2, "e_log": e_log, "npass": npass,
            "radix_log": pad(list(radix)), "log_j": pad(log_j), "block": pad(block), "ms": 1.0}


def _use(gsn, tmp_path, plans):
    path = tmp_path / "plans.json"
    path.write_text(json.dumps({"device": "test", "plans": plans}))
    gsn.clear_tuning()
    gsn.load_tuning(path)


def _restore(gsn):
    from gpusnarks_gb300._lib import TUNING_FILE
    gsn.clear_tuning()
    if TUNING_FILE.exists():
        gsn.load_tuning(TUNING_FILE)


SMALL = [(1, [1]), (3, [3]), (5, [5]), (8, [8]), (10, [10]), (6, [3, 3]), (9, [4, 5]), (12, [5, 7]),
         (14, [7, 7]), (13, [3, 4, 6])]


@pytest.mark.parametrize("e_log", [2, 3])
@pytest.mark.parametrize("lj", [0, 1, 2])
def test_rb_plans_match_oracle(gsn, cuda_device, tmp_path, e_log, lj):
    f = gsn.BLS12_381
    try:
        _use(gsn, tmp_path, [rb_plan(k, radix, lj, e_log) for k, radix in SMALL])
        for k, radix in SMALL:
            assert gsn.plan(f, k)["kernel"] == 2
            x = f.random_array(1 << k, seed=0x5EED1000 + 32 * k + 4 * lj + e_log)
            d = gsn.to_device(x)
            gsn.ntt(f, d)
            assert np.array_equal(gsn.to_host(d).reshape(x.shape), O.ntt(1, x).reshape(x.shape)), (k, radix)
            for direction in (gsn.INVERSE, gsn.COSET_FORWARD, gsn.COSET_INVERSE):
                y = gsn.to_device(x)
                gsn.ntt(f, y, direction=direction)
                want = {gsn.INVERSE: lambda: O.intt(1, x),
                        gsn.COSET_FORWARD: lambda: O.coset_ntt(1, x, O.GENERATORS[1]),
                        gsn.COSET_INVERSE: lambda: O.coset_intt(1, x, O.GENERATORS[1])}[direction]()
                assert np.array_equal(gsn.to_host(y).reshape(x.shape), want.reshape(x.shape)), (k, radix, direction)
    finally:
        _restore(gsn)


LARGE = [(16, [8, 8]), (18, [9, 9]), (20, [10, 10]), (20, [6, 7, 7]), (22, [7, 7, 8]), (24, [8, 8, 8])]


@pytest.mark.parametrize("k,radix", LARGE)
def test_rb_plans_match_committed_plans(gsn, cuda_device, tmp_path, k, radix):
    import torch
    from gpusnarks_gb300.batch import fill_random
    f = gsn.BLS12_381
    n = 1 << k
    x = torch.empty(n * f.limbs, dtype=torch.int32, device="cuda")
    fill_random(f, x, 0x5EED1100 + k)
    want = {}
    _restore(gsn)
    for direction in (gsn.FORWARD, gsn.INVERSE, gsn.COSET_FORWARD):
        y = x.clone()
        gsn.ntt(f, y, direction=direction)
        want[direction] = y
    try:
        _use(gsn, tmp_path, [rb_plan(k, radix, lj, e) for lj in (2,) for e in (3,)])
        for direction, w in want.items():
            y = x.clone()
            gsn.ntt(f, y, direction=direction)
            assert torch.equal(y, w), direction
        _use(gsn, tmp_path, [rb_plan(k, radix, 1, 2)])
        y = x.clone()
        gsn.ntt(f, y)
        assert torch.equal(y, want[gsn.FORWARD])
    finally:
        _restore(gsn)


def generic_plan(fid, log_n, radix, lj, block):
    """A plan for the generic tile (kernel 0) with the tile widths make_split_plan gives (runtime.cu)."""
    npass = len(radix)
    log_j = []
    for i, r in enumerate(radix):
        last = i == npass - 1
        inner = sum(radix[i + 1:])
        log_j.append((0 if npass == 1 else min(lj, radix[0])) if last else min(lj, inner))
    pad = lambda v: v + [0] * (4 - len(v))
    return {"field": fid, "mode": 0, "log_n": log_n, "kernel": 0, "e_log": 4, "npass": npass,
            "radix_log": pad(list(radix)), "log_j": pad(log_j), "block": pad([block] * npass), "ms": 1.0}


# Passes of radix 2^1 (the fused last stage is the tile's only stage), 2^2 (the smallest tile whose stage 0
# reads global memory) and larger, in every position of the pass sequence.
GENERIC_SMALL = [(2, [1, 1]), (3, [1, 2]), (3, [2, 1]), (4, [2, 2]), (5, [2, 3]), (5, [1, 1, 3]), (6, [1, 2, 3]),
                 (7, [3, 4]), (9, [3, 3, 3]), (9, [2, 5, 2])]


@pytest.mark.parametrize("fname", ["p32", "bls12_381_fr", "mnt4753_fr"])
@pytest.mark.parametrize("lj,block", [(0, 32), (1, 64), (2, 32)])
def test_generic_small_radix_plans_match_oracle(gsn, cuda_device, tmp_path, fname, lj, block):
    f = gsn.FIELDS[fname]
    try:
        for k, radix in GENERIC_SMALL:  # one plan per size in a table, so one table per case
            _use(gsn, tmp_path, [generic_plan(f.fid, k, radix, lj, block)])
            p = gsn.plan(f, k)
            assert p["kernel"] == 0 and p["radix_log"][:len(radix)] == radix, (k, radix, p)
            x = f.random_array(1 << k, seed=0x5EED1200 + 16 * k + 4 * lj + f.fid)
            for direction in (gsn.FORWARD, gsn.INVERSE, gsn.COSET_FORWARD, gsn.COSET_INVERSE):
                y = gsn.to_device(x)
                gsn.ntt(f, y, direction=direction)
                want = {gsn.FORWARD: lambda: O.ntt(f.fid, x),
                        gsn.INVERSE: lambda: O.intt(f.fid, x),
                        gsn.COSET_FORWARD: lambda: O.coset_ntt(f.fid, x, O.GENERATORS[f.fid]),
                        gsn.COSET_INVERSE: lambda: O.coset_intt(f.fid, x, O.GENERATORS[f.fid])}[direction]()
                assert np.array_equal(gsn.to_host(y).reshape(x.shape), want.reshape(x.shape)), (k, radix, direction)
    finally:
        _restore(gsn)
