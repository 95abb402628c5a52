"""The C++ drop-in (include/gsn_best_fft.h): a C++ program calls
best_fft<FieldT>(std::vector<FieldT>&, const FieldT&) exactly as the reference's
test/main.cpp:57 does, linked against the in-tree library; its output must
equal the oracle's."""
import pathlib
import shutil
import subprocess

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu
ROOT = pathlib.Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def dropin_exe(tmp_path_factory, gsn):
    if not shutil.which("g++"):
        pytest.skip("g++ not available")
    libdir = gsn.library_path().parent
    exe = tmp_path_factory.mktemp("cpp") / "best_fft_dropin"
    subprocess.run(["g++", "-std=c++17", "-O2", f"-I{ROOT / 'include'}", str(ROOT / "tests/cpp/best_fft_dropin.cpp"),
                    f"-L{libdir}", "-lgpusnarks_gb300", f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    return exe


@pytest.mark.parametrize("fid,log_n", [(0, 16), (1, 12), (2, 10)])
def test_cpp_best_fft(gsn, cuda_device, dropin_exe, tmp_path, fid, log_n):
    f = gsn.BY_ID[fid]
    x = f.random_array(1 << log_n, seed=0x5EED0700 + fid)
    w = f.to_limbs(gsn.root_of_unity(f, log_n))
    fin, fw, fout = tmp_path / "in.bin", tmp_path / "w.bin", tmp_path / "out.bin"
    x.tofile(fin)
    w.tofile(fw)
    r = subprocess.run([str(dropin_exe), str(fid), str(log_n), str(fin), str(fw), str(fout)],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    got = np.fromfile(fout, dtype=np.uint32).reshape(x.shape)
    assert np.array_equal(got, O.ntt(fid, x).reshape(x.shape))


@pytest.fixture(scope="module")
def multiexp_exe(tmp_path_factory, gsn):
    if not shutil.which("g++"):
        pytest.skip("g++ not available")
    libdir = gsn.library_path().parent
    exe = tmp_path_factory.mktemp("cpp") / "multiexp_dropin"
    subprocess.run(["g++", "-std=c++17", "-O2", f"-I{ROOT / 'include'}", str(ROOT / "tests/cpp/multiexp_dropin.cpp"),
                    f"-L{libdir}", "-lgpusnarks_gb300", f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    return exe


@pytest.mark.parametrize("fid,n", [(0, 1000), (1, 777), (2, 129)])
def test_cpp_multiexp(gsn, cuda_device, multiexp_exe, tmp_path, fid, n):
    """multiexp<FieldT, FieldMul>(a, mul) called as the reference's test/main.cpp:118 does: the Montgomery
    product of the stored words summed, and the canonical form, both equal to the oracle."""
    f = gsn.BY_ID[fid]
    a = f.random_array(n, seed=0x5EED0710 + fid)
    b = f.random_array(n, seed=0x5EED0720 + fid)
    fa, fb, fo = tmp_path / "a.bin", tmp_path / "b.bin", tmp_path / "out.bin"
    a.tofile(fa)
    b.tofile(fb)
    r = subprocess.run([str(multiexp_exe), str(fid), str(n), str(fa), str(fb), str(fo)],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    got = np.fromfile(fo, dtype=np.uint32).reshape(2, f.limbs)
    assert np.array_equal(got[0], O.multiexp(fid, a, b, O.MULTIEXP_MONTGOMERY))
    assert np.array_equal(got[1], O.multiexp(fid, a, b, O.MULTIEXP_CANONICAL))
