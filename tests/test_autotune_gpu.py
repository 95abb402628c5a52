"""The autotuner itself on the GPU: a short tune over a small range for single transforms and for the
batched kernel, every chosen plan valid, and transforms with the freshly tuned table equal to the oracle.
The committed tuning table is restored afterwards so later tests run the committed plans."""
import json

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def _restore(gsn):
    from gpusnarks_gb300._lib import TUNING_FILE
    gsn.clear_tuning()
    if TUNING_FILE.exists():
        gsn.load_tuning(TUNING_FILE)


def test_autotune_small_range_then_parity(gsn, cuda_device, tmp_path):
    import torch
    from gpusnarks_gb300.batch import Batch
    try:
        gsn.clear_tuning()
        gsn.autotune(gsn.BLS12_381, 8, 12, reps=2)
        gsn.autotune(gsn.P32, 10, 13, reps=2)
        gsn.autotune(gsn.MNT4_753, 6, 9, reps=2)
        gsn.autotune(gsn.BLS12_381, 8, 10, reps=2, batched=True)
        path = tmp_path / "tuned.json"
        gsn.save_tuning(path)
        saved = json.loads(path.read_text())["plans"]
        keys = {(p["field"], p["log_n"], p.get("mode", 0)) for p in saved}
        assert {(1, k, 0) for k in range(8, 13)} <= keys
        assert {(0, k, 0) for k in range(10, 14)} <= keys
        assert {(2, k, 0) for k in range(6, 10)} <= keys
        assert {(1, k, 1) for k in range(8, 11)} <= keys
        for p in saved:
            assert p["ms"] > 0 and sum(p["radix_log"][:p["npass"]]) == p["log_n"]
        for f, lo, hi in ((gsn.BLS12_381, 8, 12), (gsn.P32, 10, 13), (gsn.MNT4_753, 6, 9)):
            for k in range(lo, hi + 1):
                plan = gsn.plan(f, k)
                assert plan["log_n"] == k
                x = f.random_array(1 << k, seed=0x5EED0A00 + 16 * f.fid + k)
                d = gsn.to_device(x)
                gsn.ntt(f, d)
                assert np.array_equal(gsn.to_host(d).reshape(x.shape), O.ntt(f.fid, x).reshape(x.shape)), (f.name, k)
                gsn.ntt(f, d, direction=gsn.INVERSE)
                assert np.array_equal(gsn.to_host(d).reshape(x.shape), x), (f.name, k)
        # the batched plans: one persistent launch over jobs of the tuned sizes
        f = gsn.BLS12_381
        xs = [f.random_array(1 << k, seed=0x5EED0B00 + k) for k in (8, 9, 10, 10, 9)]
        ds = [gsn.to_device(x) for x in xs]
        b = Batch(f, [(d.data_ptr(), x.shape[0].bit_length() - 1, 0, None, None) for d, x in zip(ds, xs)])
        try:
            b.launch()
            torch.cuda.synchronize()
            b.status()
        finally:
            b.close()
        for d, x in zip(ds, xs):
            assert np.array_equal(gsn.to_host(d).reshape(x.shape), O.ntt(1, x).reshape(x.shape))
        # a saved table loads back to the same plans
        gsn.clear_tuning()
        gsn.load_tuning(path)
        path2 = tmp_path / "again.json"
        gsn.save_tuning(path2)
        assert json.loads(path2.read_text())["plans"] == saved
    finally:
        _restore(gsn)
