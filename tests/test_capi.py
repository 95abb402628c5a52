"""The C-ABI library loads and exports every function include/*.h declares.

CPU only: nothing here launches a kernel.  Host-side helpers that need no GPU
(field constants, default roots) are checked against the oracle's own
constants.
"""
import ctypes
import pathlib
import re

import numpy as np
import pytest

import oracle as O

ROOT = pathlib.Path(__file__).resolve().parent.parent
DECL = re.compile(r"^[A-Za-z_][\w\s\*]*?\b(gsn_\w+)\s*\(", re.M)


def declared_in_headers():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        text = h.read_text()
        # only C declarations inside extern "C" headers, not the C++ shim helpers
        for m in DECL.finditer(text):
            names.add(m.group(1))
    return sorted(names)


def test_headers_declare_entry_points():
    names = declared_in_headers()
    assert "gsn_ntt" in names and "gsn_ntt_host" in names


def test_library_exports_every_declared_symbol(gsn):
    lib = ctypes.CDLL(str(gsn.library_path()))
    missing = [n for n in declared_in_headers() if not hasattr(lib, n)]
    assert not missing, f"declared but not exported: {missing}"


def test_python_binding_covers_c_abi(gsn):
    bound = set(gsn.declared_symbols())
    missing = [n for n in declared_in_headers() if n not in bound and not n.startswith("gsn_server")
               and not n.startswith("gsn_batch") and not n.startswith("gsn_autotune")
               and not n.startswith("gsn_tuning")]
    assert not missing, f"no ctypes signature for: {missing}"


@pytest.mark.parametrize("fid,limbs,adic", [(0, 1, 30), (1, 8, 32), (2, 24, 30)])
def test_field_constants_match_oracle(gsn, fid, limbs, adic):
    lib = gsn.load()
    assert lib.gsn_field_limbs(fid) == limbs
    assert lib.gsn_field_two_adicity(fid) == adic
    out = np.zeros(limbs, dtype=np.uint32)
    assert lib.gsn_field_modulus(fid, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))) == 0
    assert O.from_limbs(out) == O.MODULI[fid]
    for k in (0, 1, 5, 16, min(adic, 28)):
        assert gsn.root_of_unity(fid, k) == O.root(fid, k)


def test_product_constants_independent_of_oracle(gsn):
    for fid in (0, 1, 2):
        f = gsn.BY_ID[fid]
        assert f.p == O.MODULI[fid]
        assert f.generator == O.GENERATORS[fid]


def test_bad_field_and_size_rejected_without_gpu(gsn):
    lib = gsn.load()
    assert lib.gsn_field_limbs(9) < 0
    out = np.zeros(24, dtype=np.uint32)
    p = out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))
    assert lib.gsn_root_of_unity(9, 4, p) == 2
    assert lib.gsn_root_of_unity(0, 31, p) == 3
    assert b"2-adicity" in lib.gsn_last_error()
