"""ctypes binding of the C ABI in include/gpusnarks_gb300.h.

The library is built in-tree (gpusnarks_gb300/_lib/libgpusnarks_gb300.so) by
gpusnarks_gb300.build.  Loading fails loudly when it is missing: there is no
CPU fallback for any operation.
"""
from __future__ import annotations

import ctypes
import pathlib

from . import build as _build

_u32p = ctypes.POINTER(ctypes.c_uint32)
_lib: ctypes.CDLL | None = None

GSN_OK = 0
ERRORS = {1: "GSN_ERR_ARG", 2: "GSN_ERR_FIELD", 3: "GSN_ERR_SIZE", 4: "GSN_ERR_OMEGA",
          5: "GSN_ERR_CUDA", 6: "GSN_ERR_NOMEM", 7: "GSN_ERR_BUSY", 8: "GSN_ERR_TIMEOUT",
          9: "GSN_ERR_STATE"}


class GsnError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


# (name, restype, argtypes) for every exported function.
_SIGNATURES = [
    ("gsn_last_error", ctypes.c_char_p, []),
    ("gsn_version", ctypes.c_int, []),
    ("gsn_field_limbs", ctypes.c_int, [ctypes.c_int]),
    ("gsn_field_two_adicity", ctypes.c_int, [ctypes.c_int]),
    ("gsn_field_max_log_n", ctypes.c_int, [ctypes.c_int]),
    ("gsn_field_modulus", ctypes.c_int, [ctypes.c_int, _u32p]),
    ("gsn_root_of_unity", ctypes.c_int, [ctypes.c_int, ctypes.c_uint32, _u32p]),
    ("gsn_ntt", ctypes.c_int, [ctypes.c_int, ctypes.c_void_p, ctypes.c_uint32, _u32p, ctypes.c_int, _u32p,
                               ctypes.c_void_p]),
    ("gsn_ntt_scratch", ctypes.c_int, [ctypes.c_int, ctypes.c_void_p, ctypes.c_uint32, _u32p, ctypes.c_int,
                                       _u32p, ctypes.c_void_p, ctypes.c_void_p]),
    ("gsn_ntt_host", ctypes.c_int, [ctypes.c_int, ctypes.c_void_p, ctypes.c_uint32, _u32p, ctypes.c_int, _u32p]),
    ("gsn_ntt_host_batch", ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_void_p), ctypes.c_size_t,
                                          ctypes.c_uint32, _u32p, ctypes.c_int, _u32p]),
    ("gsn_ntt_noalloc", ctypes.c_int, [ctypes.c_int, ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int,
                                       ctypes.c_void_p]),
    ("gsn_prepare", ctypes.c_int, [ctypes.c_int, ctypes.c_uint32, _u32p]),
    ("gsn_pointwise_mul", ctypes.c_int, [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64,
                                         ctypes.c_void_p]),
    ("gsn_coset_quotient", ctypes.c_int, [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_uint32, _u32p, ctypes.c_void_p]),
    ("gsn_qap_h", ctypes.c_int, [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint32,
                                 _u32p, ctypes.c_void_p]),
    ("gsn_multiexp", ctypes.c_int, [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p,
                                    ctypes.c_int, ctypes.c_void_p]),
    ("gsn_multiexp_host", ctypes.c_int, [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64,
                                         ctypes.c_void_p, ctypes.c_int]),
    ("gsn_fft_ref_compat", ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint32, _u32p, ctypes.c_int, ctypes.c_void_p]),
    ("gsn_convert", ctypes.c_int, [ctypes.c_int, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int, ctypes.c_void_p]),
    ("gsn_synchronize", ctypes.c_int, [ctypes.c_void_p]),
    ("gsn_host_alloc", ctypes.c_int, [ctypes.POINTER(ctypes.c_void_p), ctypes.c_size_t]),
    ("gsn_host_free", ctypes.c_int, [ctypes.c_void_p]),
    ("gsn_release_caches", ctypes.c_int, []),
    ("gsn_kernel_launch_count", ctypes.c_uint64, []),
    ("gsn_microbench_imad", ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_double),
                                           ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    ("gsn_microbench_imad_form", ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]),
    ("gsn_microbench_mont", ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                           ctypes.POINTER(ctypes.c_double)]),
    ("gsn_microbench_mont_coop", ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                ctypes.POINTER(ctypes.c_double)]),
    ("gsn_microbench_p32_butterfly", ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]),
    ("gsn_batch_create", ctypes.c_int, [ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int,
                                        ctypes.POINTER(ctypes.c_void_p)]),
    ("gsn_batch_launch", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    ("gsn_batch_launch_per_call", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    ("gsn_batch_status", ctypes.c_int, [ctypes.c_void_p]),
    ("gsn_batch_info", ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64),
                                      ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64),
                                      ctypes.POINTER(ctypes.c_uint64)]),
    ("gsn_batch_destroy", ctypes.c_int, [ctypes.c_void_p]),
    ("gsn_ntt_batch", ctypes.c_int, [ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    ("gsn_batch_selftest_wait", ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_uint32)]),
    ("gsn_fill_random", ctypes.c_int, [ctypes.c_int, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64,
                                       ctypes.c_void_p]),
    ("gsn_autotune", ctypes.c_int, [ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int]),
    ("gsn_autotune_batch", ctypes.c_int, [ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_int]),
    ("gsn_tuning_save", ctypes.c_int, [ctypes.c_char_p]),
    ("gsn_tuning_load", ctypes.c_int, [ctypes.c_char_p]),
    ("gsn_tuning_clear", ctypes.c_int, []),
    ("gsn_plan_describe", ctypes.c_int, [ctypes.c_int, ctypes.c_uint32, ctypes.c_char_p, ctypes.c_size_t]),
]

TUNING_FILE = pathlib.Path(__file__).resolve().parent / "tuning" / "gb300.json"


class BatchJob(ctypes.Structure):
    """Mirror of gsn_batch_job (include/gpusnarks_gb300.h)."""
    _fields_ = [("data", ctypes.c_void_p), ("log_n", ctypes.c_uint32), ("dir", ctypes.c_int32),
                ("omega", ctypes.c_void_p), ("shift", ctypes.c_void_p)]


def library_path() -> pathlib.Path:
    return _build.LIB


def load(build_if_missing: bool = False) -> ctypes.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if not path.exists():
        if not build_if_missing:
            raise RuntimeError(
                f"native library {path} is not built; run `python -c \"import __graft_entry__ as g; g.build()\"` "
                "(there is no CPU fallback)")
        _build.build()
    lib = ctypes.CDLL(str(path))
    for name, res, args in _SIGNATURES:
        fn = getattr(lib, name, None)
        if fn is None:
            continue  # symbol tests report missing exports explicitly
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    if TUNING_FILE.exists():  # plans measured on GB300 by gsn_autotune
        lib.gsn_tuning_load(str(TUNING_FILE).encode())
    return lib


def declared_symbols() -> list[str]:
    return [s[0] for s in _SIGNATURES]


def check(rc: int) -> None:
    if rc != GSN_OK:
        msg = load().gsn_last_error()
        raise GsnError(rc, msg.decode() if msg else "")


def u32p(arr):
    """ctypes uint32* for a contiguous numpy uint32 array (None passes through)."""
    if arr is None:
        return None
    return arr.ctypes.data_as(_u32p)
