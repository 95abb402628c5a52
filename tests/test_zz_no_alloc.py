"""gsn_ntt_noalloc: the transform for callers that cannot allocate device
memory at call time (loops that must not take an allocation's implicit
device synchronisation, or memory owned by another allocator).  It uses a fixed
scratch array compiled into the library instead of the per-stream scratch
gsn_ntt grows with cudaMalloc.

Called through the C ABI and compared with gsn_ntt on the same inputs, on two
calls in a row (the shared scratch keeps the previous call's contents, so the
second call checks that nothing depends on it).  Integer results: the
comparison is exact.  This file is collected last on purpose.
"""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("fname,log_n", [("p32", 20), ("p32", 24), ("bls12_381_fr", 16), ("mnt4753_fr", 14)])
def test_noalloc_matches_gsn_ntt_twice(gsn, cuda_device, fname, log_n):
    import torch
    from gpusnarks_gb300.batch import fill_random
    f = gsn.FIELDS[fname]
    lib = gsn.load()
    gsn.prepare(f, log_n)  # builds the twiddle table (this allocates; set-up time)
    stream = torch.cuda.current_stream().cuda_stream
    for call in range(2):
        for direction in (gsn.FORWARD, gsn.INVERSE):
            x = torch.empty((1 << log_n) * f.limbs, dtype=torch.int32, device="cuda")
            fill_random(f, x, 0x5EED0900 + 10 * call + direction)
            want = x.clone()
            gsn.ntt(f, want, direction=direction)
            rc = lib.gsn_ntt_noalloc(f.fid, x.data_ptr(), log_n, direction, stream)
            assert rc == 0, lib.gsn_last_error()
            torch.cuda.synchronize()
            assert torch.equal(x, want), (call, direction)


def test_noalloc_allocates_nothing_and_rejects_oversize(gsn, cuda_device):
    import torch
    f = gsn.BLS12_381
    lib = gsn.load()
    gsn.prepare(f, 18)
    x = torch.zeros((1 << 18) * f.limbs, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    assert lib.gsn_ntt_noalloc(f.fid, x.data_ptr(), 18, 0, stream) == 0  # first call: address lookup
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(3):
        assert lib.gsn_ntt_noalloc(f.fid, x.data_ptr(), 18, 0, stream) == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    big = torch.zeros((1 << 22) * f.limbs, dtype=torch.int32, device="cuda")
    rc = lib.gsn_ntt_noalloc(f.fid, big.data_ptr(), 22, 0, stream)
    assert rc == 3 and b"scratch" in lib.gsn_last_error()
    assert lib.gsn_ntt_noalloc(f.fid, x.data_ptr(), 18, 2, stream) == 1  # coset: not supported here
