"""Element formats: Montgomery conversion, limb-order conversion, and the
transform's independence of the representation (NTT(x R) = NTT(x) R)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("fname", ["p32", "bls12_381_fr", "mnt4753_fr"])
def test_montgomery_round_trip_and_values(gsn, cuda_device, fname):
    f = gsn.FIELDS[fname]
    x = f.random_array(1000, seed=77)
    d = gsn.to_device(x)
    gsn.convert(f, d, gsn.TO_MONTGOMERY)
    got = f.array_to_ints(gsn.to_host(d))
    assert got == [(v * f.R) % f.p for v in f.array_to_ints(x)]
    gsn.convert(f, d, gsn.FROM_MONTGOMERY)
    assert np.array_equal(gsn.to_host(d).reshape(x.shape), x)


@pytest.mark.parametrize("fname", ["bls12_381_fr", "mnt4753_fr"])
def test_reverse_limbs(gsn, cuda_device, fname):
    f = gsn.FIELDS[fname]
    x = f.random_array(300, seed=78)
    d = gsn.to_device(x)
    gsn.convert(f, d, gsn.REVERSE_LIMBS)
    assert np.array_equal(gsn.to_host(d).reshape(x.shape), x[:, ::-1])
    gsn.convert(f, d, gsn.REVERSE_LIMBS)
    assert np.array_equal(gsn.to_host(d).reshape(x.shape), x)


@pytest.mark.parametrize("fname,log_n", [("p32", 16), ("bls12_381_fr", 12), ("mnt4753_fr", 10)])
def test_ntt_is_representation_agnostic(gsn, cuda_device, fname, log_n):
    """Transforming Montgomery-form data gives the Montgomery form of the result."""
    f = gsn.FIELDS[fname]
    x = f.random_array(1 << log_n, seed=79)
    a = gsn.to_device(x)
    b = gsn.to_device(x)
    gsn.ntt(f, a)
    gsn.convert(f, a, gsn.TO_MONTGOMERY)      # NTT(x) R
    gsn.convert(f, b, gsn.TO_MONTGOMERY)
    gsn.ntt(f, b)                              # NTT(x R)
    assert np.array_equal(gsn.to_host(a), gsn.to_host(b))


def test_convert_errors(gsn, cuda_device):
    f = gsn.BLS12_381
    d = gsn.to_device(f.random_array(8, seed=1))
    lib = gsn.load()
    assert lib.gsn_convert(1, d.data_ptr(), 8, 7, None) == 1
    assert lib.gsn_convert(1, d.data_ptr() + 4, 7, 0, None) == 1
    assert lib.gsn_convert(5, d.data_ptr(), 8, 0, None) == 2
