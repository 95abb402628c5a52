"""gpusnarks_gb300: GB300-native finite-field NTT behind the reference's
``best_fft`` boundary (cuda/fft_kernel.h:24-25).

This module is the host-side mirror of that interface for Python callers.  All
work goes through the C ABI of the in-tree native library (include/
gpusnarks_gb300.h); there is no CPU fallback.

Element arrays use the reference layout: little-endian uint32 limbs per
element (cuda/device_field.h:75), numpy shape ``(n, limbs)`` (``(n,)`` for
the one-limb field) or the same bytes in a torch CUDA tensor of dtype int32.
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import GsnError, check, declared_symbols, library_path, load, u32p
from .fields import BLS12_381, BY_ID, FIELDS, MNT4_753, MNT4_753_Q, P32, Field

FORWARD, INVERSE, COSET_FORWARD, COSET_INVERSE = 0, 1, 2, 3
DIRECTIONS = {"forward": FORWARD, "inverse": INVERSE, "coset_forward": COSET_FORWARD,
              "coset_inverse": COSET_INVERSE}

__all__ = ["Field", "P32", "BLS12_381", "MNT4_753", "MNT4_753_Q", "FIELDS", "BY_ID", "GsnError",
           "FORWARD", "INVERSE", "COSET_FORWARD", "COSET_INVERSE", "load", "library_path",
           "declared_symbols", "best_fft", "ntt", "root_of_unity", "field_of", "pointwise_mul",
           "prepare", "launch_count", "multiexp", "multiexp_host", "MULTIEXP_CANONICAL",
           "MULTIEXP_MONTGOMERY"]


def field_of(f) -> Field:
    if isinstance(f, Field):
        return f
    if isinstance(f, str):
        return FIELDS[f]
    return BY_ID[int(f)]


def _limbs(f: Field, x) -> np.ndarray | None:
    if x is None:
        return None
    if isinstance(x, (int, np.integer)):
        return f.to_limbs(int(x))
    return np.ascontiguousarray(x, dtype=np.uint32).reshape(-1)[: f.limbs].copy()


def root_of_unity(field, log_n: int) -> int:
    f = field_of(field)
    out = np.zeros(f.limbs, dtype=np.uint32)
    check(load().gsn_root_of_unity(f.fid, log_n, u32p(out)))
    return f.from_limbs(out)


def prepare(field, log_n: int, omega=None) -> None:
    f = field_of(field)
    w = _limbs(f, omega)
    check(load().gsn_prepare(f.fid, log_n, u32p(w)))


def _log2_exact(n: int) -> int:
    if n <= 0 or n & (n - 1):
        raise ValueError(f"size {n} is not a power of two")
    return n.bit_length() - 1


def best_fft(a: np.ndarray, omg=None, *, field=None, direction=FORWARD, shift=None) -> np.ndarray:
    """In-place transform of a host array, like ``best_fft(std::vector<FieldT>&, const FieldT&)``.

    ``a``: numpy uint32 array of shape (n, limbs) (or (n,) for p32), modified in
    place and returned.  ``omg``: the forward root (int or limbs); None = the
    field's default root g^((p-1)/n).  ``field`` defaults from the limb count
    (1 -> p32, 8 -> BLS12-381 r, 24 -> MNT4-753 r).
    """
    if not isinstance(a, np.ndarray) or a.dtype != np.uint32 or not a.flags.c_contiguous:
        raise TypeError("best_fft expects a C-contiguous numpy uint32 array")
    if field is None:
        limbs = 1 if a.ndim == 1 else a.shape[1]
        field = {1: P32, 8: BLS12_381, 24: MNT4_753}[limbs]
    f = field_of(field)
    n = a.size // f.limbs
    log_n = _log2_exact(n)
    w = _limbs(f, omg)
    s = _limbs(f, shift)
    check(load().gsn_ntt_host(f.fid, a.ctypes.data, log_n, u32p(w), int(direction), u32p(s)))
    return a


def best_fft_many(arrays, omg=None, *, field=None, direction=FORWARD, shift=None):
    """``best_fft`` on several host arrays of one size, each in place, with the copies of neighbouring arrays
    overlapping each transform (gsn_ntt_host_batch).  ``arrays``: C-contiguous numpy uint32 arrays, or
    integer addresses of host buffers (e.g. from host_buffer) with ``field`` and the size given by ``log_n``
    through a (address, log_n) tuple.  Returns the list."""
    items = list(arrays)
    if not items:
        return items
    ptrs, sizes = [], set()
    for a in items:
        if isinstance(a, tuple):
            ptrs.append(int(a[0]))
            sizes.add(int(a[1]))
            continue
        if not isinstance(a, np.ndarray) or a.dtype != np.uint32 or not a.flags.c_contiguous:
            raise TypeError("best_fft_many expects C-contiguous numpy uint32 arrays")
        if field is None:
            field = {1: P32, 8: BLS12_381, 24: MNT4_753}[1 if a.ndim == 1 else a.shape[1]]
        ptrs.append(a.ctypes.data)
        sizes.add(_log2_exact(a.size // field_of(field).limbs))
    if field is None or len(sizes) != 1:
        raise ValueError("best_fft_many needs one field and one size for all arrays")
    f = field_of(field)
    arr = (ctypes.c_void_p * len(ptrs))(*ptrs)
    check(load().gsn_ntt_host_batch(f.fid, arr, len(ptrs), sizes.pop(), u32p(_limbs(f, omg)), int(direction),
                                    u32p(_limbs(f, shift))))
    return items


def _stream_handle(stream):
    if stream is None:
        import torch
        return torch.cuda.current_stream().cuda_stream
    if isinstance(stream, int):
        return stream
    return stream.cuda_stream


def ntt(field, data, *, direction=FORWARD, omega=None, shift=None, stream=None, scratch=None):
    """In-place transform of device data (a torch CUDA tensor, int32 storage).

    Asynchronous on ``stream`` (default: torch's current stream).
    """
    f = field_of(field)
    n = data.numel() // f.limbs
    log_n = _log2_exact(n)
    w = _limbs(f, omega)
    s = _limbs(f, shift)
    h = _stream_handle(stream)
    lib = load()
    if scratch is None:
        check(lib.gsn_ntt(f.fid, data.data_ptr(), log_n, u32p(w), int(direction), u32p(s), h))
    else:
        check(lib.gsn_ntt_scratch(f.fid, data.data_ptr(), log_n, u32p(w), int(direction), u32p(s),
                                  scratch.data_ptr(), h))
    return data


def pointwise_mul(field, a, b, *, stream=None):
    f = field_of(field)
    n = a.numel() // f.limbs
    check(load().gsn_pointwise_mul(f.fid, a.data_ptr(), b.data_ptr(), n, _stream_handle(stream)))
    return a


def coset_quotient(field, a, b, c, *, shift=None, stream=None):
    """In place on device tensors of coset evaluations: a = (a*b - c) / (shift^n - 1)."""
    f = field_of(field)
    log_n = _log2_exact(a.numel() // f.limbs)
    check(load().gsn_coset_quotient(f.fid, a.data_ptr(), b.data_ptr(), c.data_ptr(), log_n,
                                    u32p(_limbs(f, shift)), _stream_handle(stream)))
    return a


def qap_h(field, a, b, c, *, shift=None, stream=None):
    """H = (A*B - C) / Z from the evaluations of A, B, C on the domain (device tensors); the n
    coefficients of H land in ``a``; ``b`` and ``c`` are overwritten."""
    f = field_of(field)
    log_n = _log2_exact(a.numel() // f.limbs)
    check(load().gsn_qap_h(f.fid, a.data_ptr(), b.data_ptr(), c.data_ptr(), log_n, u32p(_limbs(f, shift)),
                           _stream_handle(stream)))
    return a


def fft_ref_compat(data, omega_limbs, log_cpus: int = 10, *, stream=None):
    """The reference's host FFT dataflow (test/fft_host.h:56-118) over its own 24-limb Scalar arithmetic,
    on the GPU, bit for bit (not a DFT).  ``data``: device tensor of n*24 raw limbs; ``omega_limbs``: 24
    raw limbs."""
    n = data.numel() // 24
    w = np.ascontiguousarray(omega_limbs, dtype=np.uint32).reshape(-1)[:24].copy()
    check(load().gsn_fft_ref_compat(data.data_ptr(), _log2_exact(n), u32p(w), int(log_cpus),
                                    _stream_handle(stream)))
    return data


MULTIEXP_CANONICAL, MULTIEXP_MONTGOMERY = 0, 1


def multiexp(field, a, b, out=None, *, mode=MULTIEXP_CANONICAL, stream=None):
    """sum_i a[i] * b[i] mod p on the GPU (the reference's multiexp over field elements,
    cuda/multi_exp.cu:104-137).  ``a``, ``b``: device tensors of n elements; ``out``: a device tensor of
    one element (allocated when None).  Asynchronous on ``stream``; returns ``out``."""
    import torch
    f = field_of(field)
    n = a.numel() // f.limbs
    if b.numel() != a.numel():
        raise ValueError("a and b must hold the same number of elements")
    if out is None:
        out = torch.empty(f.limbs, dtype=torch.int32, device=a.device)
    check(load().gsn_multiexp(f.fid, a.data_ptr(), b.data_ptr(), n, out.data_ptr(), int(mode),
                              _stream_handle(stream)))
    return out


def multiexp_host(a: np.ndarray, b: np.ndarray, *, field=None, mode=MULTIEXP_CANONICAL) -> np.ndarray:
    """The same from host arrays, like the reference's multiexp(std::vector&, std::vector&): returns the
    one result element as limbs."""
    a = np.ascontiguousarray(a, dtype=np.uint32)
    b = np.ascontiguousarray(b, dtype=np.uint32)
    if field is None:
        field = {1: P32, 8: BLS12_381, 24: MNT4_753}[1 if a.ndim == 1 else a.shape[1]]
    f = field_of(field)
    if a.size != b.size:
        raise ValueError("a and b must hold the same number of elements")
    out = np.zeros(f.limbs, dtype=np.uint32)
    check(load().gsn_multiexp_host(f.fid, a.ctypes.data, b.ctypes.data, a.size // f.limbs, out.ctypes.data,
                                   int(mode)))
    return out


TO_MONTGOMERY, FROM_MONTGOMERY, REVERSE_LIMBS = 0, 1, 2


def convert(field, data, mode: int, *, stream=None):
    """In place: enter / leave Montgomery form, or reverse each element's limb order."""
    f = field_of(field)
    n = data.numel() // f.limbs
    check(load().gsn_convert(f.fid, data.data_ptr(), n, int(mode), _stream_handle(stream)))
    return data


def autotune(field, lo: int, hi: int, reps: int = 5, *, batched: bool = False) -> None:
    """Time candidate plans for every log n in [lo, hi] and keep the fastest
    (for single transforms, or for the persistent batched kernel)."""
    fn = load().gsn_autotune_batch if batched else load().gsn_autotune
    check(fn(field_of(field).fid, lo, hi, reps))


def save_tuning(path) -> None:
    check(load().gsn_tuning_save(str(path).encode()))


def load_tuning(path) -> None:
    check(load().gsn_tuning_load(str(path).encode()))


def clear_tuning() -> None:
    check(load().gsn_tuning_clear())


def plan(field, log_n: int) -> dict:
    """The plan (passes, radices, tile widths, threads, kernel) a transform would use."""
    import json
    buf = ctypes.create_string_buffer(1024)
    check(load().gsn_plan_describe(field_of(field).fid, log_n, buf, len(buf)))
    return json.loads(buf.value.decode())


def launch_count() -> int:
    return int(load().gsn_kernel_launch_count())


def to_device(arr: np.ndarray, device="cuda"):
    """numpy uint32 limbs -> torch int32 CUDA tensor with the same bytes."""
    import torch
    return torch.from_numpy(np.ascontiguousarray(arr).view(np.int32)).to(device)


def to_host(t) -> np.ndarray:
    return t.cpu().numpy().view(np.uint32)


def host_buffer(nbytes: int):
    """Pinned host memory from the library (ctypes pointer, free with free_host_buffer)."""
    p = ctypes.c_void_p()
    check(load().gsn_host_alloc(ctypes.byref(p), nbytes))
    return p


def free_host_buffer(p) -> None:
    check(load().gsn_host_free(p))

