"""GPU parity of the reference-compatible transform (gsn_fft_ref_compat).

It must equal, bit for bit, the reference's own host FFT over its own Scalar
arithmetic: the golden fixtures made from the compiled reference at the
shipped call (test/main.cpp:45-71: inputs Scalar(1234), omega = Scalar(_mod),
log_cpus = 10) at n = 2^12 (full) and 2^16 (SHA-256), and the oracle's
restatement (oracle.refscalar_fft) on seeded inputs for other sizes and
log_cpus values, including the serial branch (log_n < log_cpus).
"""
import hashlib
import pathlib

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

GOLDEN = pathlib.Path(__file__).resolve().parent / "golden"
REF_Q = O.to_limbs(3, O.MODULI[3])


def _run(gsn, data, omega, log_cpus):
    d = gsn.to_device(data)
    gsn.fft_ref_compat(d, omega, log_cpus)
    return gsn.to_host(d).reshape(data.shape)


@pytest.mark.parametrize("n,key", [(4096, "out"), (65536, "head")])
def test_shipped_call_golden(gsn, cuda_device, n, key):
    g = np.load(GOLDEN / f"refscalar_fft_n{n}.npz")
    data = np.zeros((n, 24), dtype=np.uint32)
    data[:, 0] = int(g["input_value"])
    out = _run(gsn, data, REF_Q, int(g["log_cpus"]))
    assert (out[: len(g[key])] == g[key]).all()
    assert hashlib.sha256(out.tobytes()).hexdigest() == str(g["sha256"])


@pytest.mark.parametrize("log_n,log_cpus", [(4, 6), (6, 2), (8, 3), (10, 5), (10, 10), (11, 4)])
def test_matches_restatement(gsn, cuda_device, log_n, log_cpus):
    rng = np.random.default_rng(1000 + 17 * log_n + log_cpus)
    data = rng.integers(0, 2 ** 32, size=(1 << log_n, 24), dtype=np.uint64).astype(np.uint32)
    data[:, 23] &= 0x1FFFF  # below 2^753, like the reference's inputs
    omega = rng.integers(0, 2 ** 32, size=24, dtype=np.uint64).astype(np.uint32)
    omega[23] &= 0x1FFFF
    want = O.refscalar_fft(data, omega, log_cpus)
    got = _run(gsn, data, omega, log_cpus)
    assert np.array_equal(got, want.reshape(data.shape))


def test_ref_compat_errors(gsn, cuda_device):
    import torch
    lib = gsn.load()
    d = torch.zeros(64 * 24, dtype=torch.int32, device="cuda")
    w = gsn._lib.u32p(REF_Q)
    assert lib.gsn_fft_ref_compat(None, 6, w, 2, None) == 1
    assert lib.gsn_fft_ref_compat(d.data_ptr() + 4, 6, w, 2, None) == 1
    assert lib.gsn_fft_ref_compat(d.data_ptr(), 25, w, 2, None) == 3
    assert lib.gsn_fft_ref_compat(d.data_ptr(), 6, w, 17, None) == 1
    torch.cuda.synchronize()
