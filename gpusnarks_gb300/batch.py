"""Batched transforms: many independent NTTs in one persistent launch.

Thin wrapper over gsn_batch_* (include/gpusnarks_gb300.h).  The jobs' data
stays in caller-owned device memory and is transformed in place.
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import BatchJob, check, load


def _job_array(field, jobs):
    """(ctypes gsn_batch_job array, arrays it points into) for jobs of
    (device_ptr:int, log_n:int, direction:int, omega, shift)."""
    from . import _limbs  # late import: package init order

    keep = []
    arr = (BatchJob * len(jobs))()
    for i, (ptr, log_n, direction, omega, shift) in enumerate(jobs):
        w = _limbs(field, omega)
        s = _limbs(field, shift)
        keep += [w, s]
        arr[i].data = ptr
        arr[i].log_n = log_n
        arr[i].dir = direction
        arr[i].omega = None if w is None else w.ctypes.data
        arr[i].shift = None if s is None else s.ctypes.data
    return arr, keep


def ntt_batch(field, jobs, *, stream=None) -> None:
    """gsn_ntt_batch: transform every job in one persistent launch and wait for it."""
    from . import _stream_handle, field_of

    f = field_of(field)
    arr, _keep = _job_array(f, jobs)
    check(load().gsn_ntt_batch(f.fid, ctypes.cast(arr, ctypes.c_void_p), len(jobs), _stream_handle(stream)))


class Batch:
    GRAPH = 1

    def __init__(self, field, jobs, *, graph: bool = True):
        """jobs: iterable of (device_ptr:int, log_n:int, direction:int, omega, shift)."""
        from . import field_of  # late import: package init order

        self.field = field_of(field)
        arr, self._keep = _job_array(self.field, jobs)
        self._jobs = arr
        h = ctypes.c_void_p()
        check(load().gsn_batch_create(self.field.fid, ctypes.cast(arr, ctypes.c_void_p), len(jobs),
                                      self.GRAPH if graph else 0, ctypes.byref(h)))
        self._h = h

    def _stream(self, stream):
        from . import _stream_handle
        return _stream_handle(stream)

    def launch(self, stream=None) -> None:
        check(load().gsn_batch_launch(self._h, self._stream(stream)))

    def launch_per_call(self, stream=None) -> None:
        check(load().gsn_batch_launch_per_call(self._h, self._stream(stream)))

    def status(self) -> None:
        check(load().gsn_batch_status(self._h))

    def info(self) -> dict:
        vals = [ctypes.c_uint64() for _ in range(4)]
        check(load().gsn_batch_info(self._h, *[ctypes.byref(v) for v in vals]))
        return dict(zip(("jobs", "work_items", "elements", "device_bytes"), (v.value for v in vals)))

    def close(self) -> None:
        if self._h:
            check(load().gsn_batch_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def fill_random(field, data, seed: int, *, stream=None) -> None:
    """Device-side uniform elements of [0, p) (replicated on the host by Field.device_random)."""
    from . import _stream_handle, field_of
    f = field_of(field)
    n = data.numel() // f.limbs
    check(load().gsn_fill_random(f.fid, data.data_ptr(), n, seed, _stream_handle(stream)))


def job_sizes(count: int, lo: int, hi: int, seed: int) -> list[int]:
    """log2 sizes drawn uniformly from {lo..hi} (log-uniform sizes) with a seeded PRNG."""
    rng = np.random.default_rng(seed)
    return [int(k) for k in rng.integers(lo, hi + 1, size=count)]
