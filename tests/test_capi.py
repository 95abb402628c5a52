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


def test_entry_points_validate_before_touching_the_gpu(gsn):
    """Every entry point checks its arguments on the host first: with no GPU here, a bad
    argument must come back as its own error code, not as a CUDA failure."""
    lib = gsn.load()
    w = np.zeros(24, dtype=np.uint32)
    w[0] = 2  # not a root of unity of any order > 2
    wp = w.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32))
    fake = ctypes.c_void_p(0x10000)  # never dereferenced: every call below fails its checks first
    ARG, FIELD, SIZE, OMEGA = 1, 2, 3, 4
    cases = [
        (lambda: lib.gsn_ntt(1, None, 4, None, 0, None, None), ARG, b"null"),
        (lambda: lib.gsn_ntt(7, fake, 4, None, 0, None, None), FIELD, b"unknown field"),
        (lambda: lib.gsn_ntt(1, fake, 40, None, 0, None, None), SIZE, b"exceeds"),
        (lambda: lib.gsn_ntt(1, fake, 4, None, 9, None, None), ARG, b"direction"),
        (lambda: lib.gsn_ntt(1, fake, 4, wp, 0, None, None), OMEGA, b"primitive"),
        (lambda: lib.gsn_ntt(1, ctypes.c_void_p(0x10004), 4, None, 0, None, None), ARG, b"aligned"),
        (lambda: lib.gsn_ntt_host(1, None, 4, None, 0, None), ARG, b"null"),
        (lambda: lib.gsn_ntt_scratch(1, fake, 4, None, 0, None, None, None), ARG, b"scratch"),
        (lambda: lib.gsn_prepare(1, 40, None), SIZE, b"exceeds"),
        (lambda: lib.gsn_pointwise_mul(1, None, None, 16, None), ARG, b"null"),
        (lambda: lib.gsn_convert(1, fake, 16, 7, None), ARG, b"mode"),
        (lambda: lib.gsn_coset_quotient(1, None, None, None, 4, None, None), ARG, b"null"),
        (lambda: lib.gsn_qap_h(1, None, None, None, 4, None, None), ARG, b"null"),
        (lambda: lib.gsn_qap_h(1, fake, fake, ctypes.c_void_p(0x20000), 4, None, None), ARG, b"distinct"),
        (lambda: lib.gsn_fft_ref_compat(fake, 30, wp, 3, None), SIZE, b"2^24"),
        (lambda: lib.gsn_batch_create(1, None, 3, 0, None), ARG, b"null"),
        (lambda: lib.gsn_ntt_batch(1, None, 0, None), ARG, b"empty batch"),
        (lambda: lib.gsn_server_create(None, None), ARG, b"null"),
        (lambda: lib.gsn_server_submit(None, None, None), ARG, b"null"),
        (lambda: lib.gsn_fill_random(1, None, 16, 1, None), ARG, b"null"),
        (lambda: lib.gsn_autotune(9, 8, 10, 3), FIELD, b"unknown field"),
        (lambda: lib.gsn_tuning_load(b"/nonexistent/tuning.json"), ARG, b"cannot read"),
        (lambda: lib.gsn_plan_describe(1, 10, ctypes.create_string_buffer(4), 4), ARG, b"too small"),
        (lambda: lib.gsn_multiexp(9, fake, fake, 16, fake, 0, None), FIELD, b"unknown field"),
        (lambda: lib.gsn_multiexp(1, fake, fake, 16, fake, 5, None), ARG, b"mode"),
        (lambda: lib.gsn_multiexp(1, fake, fake, 16, None, 0, None), ARG, b"null output"),
        (lambda: lib.gsn_multiexp(1, None, fake, 16, fake, 0, None), ARG, b"null input"),
        (lambda: lib.gsn_multiexp(1, ctypes.c_void_p(0x10004), fake, 16, fake, 0, None), ARG, b"aligned"),
        (lambda: lib.gsn_multiexp(1, fake, fake, (1 << 40) + 1, fake, 0, None), SIZE, b"exceeds"),
        (lambda: lib.gsn_multiexp_host(1, None, None, 16, fake, 0), ARG, b"null input"),
    ]
    for i, (call, want, msg) in enumerate(cases):
        rc = call()
        assert rc == want and msg in lib.gsn_last_error(), (i, rc, lib.gsn_last_error())
    assert lib.gsn_ntt_host_batch(1, None, 0, 4, None, 0, None) == 0  # nothing to do


def test_server_config_rejects_unknown_policy(gsn):
    from gpusnarks_gb300.serve import ServerConfig
    lib = gsn.load()
    h = ctypes.c_void_p()
    cfg = ServerConfig(1 << 30, 2, 0, 0, 7, 0)
    assert lib.gsn_server_create(ctypes.byref(cfg), ctypes.byref(h)) == 1
    assert b"bad server config" in lib.gsn_last_error()


def test_tuning_table_save_load_round_trip(gsn, tmp_path):
    """The committed table loads without a GPU, and saving then reloading it keeps every plan and time."""
    import json
    lib = gsn.load()
    table = ROOT / "gpusnarks_gb300" / "tuning" / "gb300.json"
    assert lib.gsn_tuning_load(str(table).encode()) == 0
    buf = ctypes.create_string_buffer(512)

    def describe(fid, k):
        assert lib.gsn_plan_describe(fid, k, buf, 512) == 0
        d = json.loads(buf.value)
        d.pop("ms", None)
        return d

    before = {(fid, k): describe(fid, k) for fid in (0, 1, 2) for k in range(8, 21)}
    out = tmp_path / "saved.json"
    assert lib.gsn_tuning_save(str(out).encode()) == 0
    saved = json.loads(out.read_text())["plans"]
    orig = json.loads(table.read_text())["plans"]
    key = lambda p: (p["field"], p["mode"], p["log_n"])
    assert sorted(map(key, saved)) == sorted(map(key, orig))
    assert {key(p): p["ms"] for p in saved} == pytest.approx({key(p): p["ms"] for p in orig}, rel=1e-4)
    assert lib.gsn_tuning_clear() == 0
    assert lib.gsn_tuning_load(str(out).encode()) == 0
    assert {(fid, k): describe(fid, k) for fid in (0, 1, 2) for k in range(8, 21)} == before
    assert lib.gsn_tuning_load(str(table).encode()) == 0
