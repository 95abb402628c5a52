"""Serving: Python handle on the native request loop (gsn_server_*).

The scheduler, admission, batching and copies all run in the native library;
this module builds requests and traces and reads results.
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import check, load


class ServerConfig(ctypes.Structure):
    _fields_ = [("hbm_budget_bytes", ctypes.c_uint64), ("max_inflight", ctypes.c_int32),
                ("max_batch_jobs", ctypes.c_int32), ("max_launch_work", ctypes.c_uint64),
                ("policy", ctypes.c_int32), ("reserved", ctypes.c_int32)]


OLDEST_FIRST = 0       # GSN_SERVE_OLDEST_FIRST
LEAST_WORK_FIRST = 1   # GSN_SERVE_LEAST_WORK_FIRST


class Request(ctypes.Structure):
    _fields_ = [("field", ctypes.c_int32), ("log_n", ctypes.c_uint32), ("dir", ctypes.c_int32),
                ("shift", ctypes.c_void_p), ("host_in", ctypes.c_void_p), ("host_out", ctypes.c_void_p)]


class TraceEntry(ctypes.Structure):
    _fields_ = [("arrival_s", ctypes.c_double), ("req", Request)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("completed", ctypes.c_uint64), ("failed", ctypes.c_uint64),
                ("launches", ctypes.c_uint64), ("device_bytes_in_use", ctypes.c_uint64),
                ("device_bytes_peak", ctypes.c_uint64), ("busy_s", ctypes.c_double),
                ("step_max_s", ctypes.c_double * 5)]


_SIGS = [
    ("gsn_server_create", [ctypes.POINTER(ServerConfig), ctypes.POINTER(ctypes.c_void_p)]),
    ("gsn_server_warmup", [ctypes.c_void_p, ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32]),
    ("gsn_server_submit", [ctypes.c_void_p, ctypes.POINTER(Request), ctypes.POINTER(ctypes.c_uint64)]),
    ("gsn_server_wait", [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_double, ctypes.POINTER(ctypes.c_double)]),
    ("gsn_server_fetch", [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_void_p]),
    ("gsn_server_release", [ctypes.c_void_p, ctypes.c_uint64]),
    ("gsn_server_get_stats", [ctypes.c_void_p, ctypes.POINTER(ServerStats)]),
    ("gsn_server_destroy", [ctypes.c_void_p]),
    ("gsn_server_run_trace", [ctypes.c_void_p, ctypes.POINTER(TraceEntry), ctypes.c_size_t,
                              ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double)]),
    ("gsn_server_run_trace_phases", [ctypes.c_void_p, ctypes.POINTER(TraceEntry), ctypes.c_size_t,
                                     ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                                     ctypes.POINTER(ctypes.c_double)]),
]

PHASES = ("queue", "upload", "wait_launch", "compute", "download")


def _lib():
    lib = load()
    for name, args in _SIGS:
        fn = getattr(lib, name)
        fn.restype = ctypes.c_int
        fn.argtypes = args
    return lib


class Server:
    def __init__(self, hbm_budget_bytes: int, max_inflight: int = 4, max_batch_jobs: int = 0,
                 max_launch_work: int = 0, policy: int = OLDEST_FIRST):
        self.lib = _lib()
        cfg = ServerConfig(hbm_budget_bytes, max_inflight, max_batch_jobs, max_launch_work, policy, 0)
        h = ctypes.c_void_p()
        check(self.lib.gsn_server_create(ctypes.byref(cfg), ctypes.byref(h)))
        self.h = h
        self._keep = []

    def warmup(self, field, lo: int, hi: int) -> None:
        from . import field_of
        check(self.lib.gsn_server_warmup(self.h, field_of(field).fid, lo, hi))

    def submit(self, field, host_in: np.ndarray, direction: int = 0, shift=None, host_out: np.ndarray | None = None):
        from . import _limbs, field_of
        f = field_of(field)
        n = host_in.size // f.limbs
        s = _limbs(f, shift)
        self._keep += [host_in, host_out, s]
        req = Request(f.fid, n.bit_length() - 1, direction, None if s is None else s.ctypes.data,
                      host_in.ctypes.data, None if host_out is None else host_out.ctypes.data)
        rid = ctypes.c_uint64()
        check(self.lib.gsn_server_submit(self.h, ctypes.byref(req), ctypes.byref(rid)))
        return rid.value

    def wait(self, rid: int, timeout_s: float = 60.0) -> float:
        lat = ctypes.c_double()
        check(self.lib.gsn_server_wait(self.h, rid, timeout_s, ctypes.byref(lat)))
        return lat.value

    def fetch(self, rid: int, out: np.ndarray) -> np.ndarray:
        check(self.lib.gsn_server_fetch(self.h, rid, out.ctypes.data))
        return out

    def release(self, rid: int) -> None:
        check(self.lib.gsn_server_release(self.h, rid))

    def stats(self) -> dict:
        st = ServerStats()
        check(self.lib.gsn_server_get_stats(self.h, ctypes.byref(st)))
        out = {k: getattr(st, k) for k, _ in ServerStats._fields_}
        out["step_max_s"] = list(st.step_max_s)
        return out

    def run_trace(self, entries, phases: bool = False):
        """Replay (arrival, Request) entries.  Returns (latencies, makespan), and with phases=True also an
        (n, 5) array of seconds per request spent in PHASES."""
        arr = (TraceEntry * len(entries))(*entries)
        lat = (ctypes.c_double * len(entries))()
        mk = ctypes.c_double()
        if not phases:
            check(self.lib.gsn_server_run_trace(self.h, arr, len(entries), lat, ctypes.byref(mk)))
            return np.array(lat[:], dtype=np.float64), mk.value
        ph = (ctypes.c_double * (5 * len(entries)))()
        check(self.lib.gsn_server_run_trace_phases(self.h, arr, len(entries), lat, ph, ctypes.byref(mk)))
        return (np.array(lat[:], dtype=np.float64), mk.value,
                np.array(ph[:], dtype=np.float64).reshape(len(entries), 5))

    def close(self) -> None:
        if self.h:
            check(self.lib.gsn_server_destroy(self.h))
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def poisson_trace(count: int, rate: float, seed: int, fields=(1, 2), lo=12, hi=22, dirs=(0, 1, 2)):
    """Seeded Poisson arrivals (exponential gaps, mean 1/rate), field chosen
    uniformly from `fields`, log2 size uniform in [lo, hi], direction uniform."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, size=count)
    t = np.cumsum(gaps) - gaps[0]
    fs = rng.choice(np.array(fields), size=count)
    ks = rng.integers(lo, hi + 1, size=count)
    ds = rng.choice(np.array(dirs), size=count)
    return [(float(t[i]), int(fs[i]), int(ks[i]), int(ds[i])) for i in range(count)]


def verification_sample(trace, seed: int, count: int = 48, max_bytes: int = 2 << 30) -> list[int]:
    """Indices of a seeded sample of trace requests whose outputs are checked: the largest request of
    each field and one of each (field, direction) pair first, then random ones, at most `count` requests
    and `max_bytes` of output in total."""
    from . import BY_ID
    rng = np.random.default_rng(seed + 1)
    size = [(1 << k) * BY_ID[fid].limbs * 4 for _, fid, k, _ in trace]
    must: list[int] = []
    for fid in sorted({e[1] for e in trace}):
        idx = [i for i, e in enumerate(trace) if e[1] == fid]
        must.append(max(idx, key=lambda i: (trace[i][2], -i)))
        for d in sorted({trace[i][3] for i in idx}):
            cand = [i for i in idx if trace[i][3] == d]
            must.append(int(rng.choice(cand)))
    rest = [int(i) for i in rng.permutation(len(trace))]
    out: list[int] = []
    total = 0
    for i in must + rest:
        if i in out or len(out) >= count:
            continue
        if total + size[i] > max_bytes and i not in must:
            continue
        out.append(i)
        total += size[i]
    return sorted(out)


def bench_serving(g, torch, *, seconds: float = 1.0, rate: float = 2000.0, budget_gb: float = 120.0,
                  max_inflight: int = 4, seed: int = 0x5EED0005, policy: int = OLDEST_FIRST) -> dict:
    """The mixed serving stream: Poisson arrivals at `rate` req/s for `seconds`, BLS12-381 / MNT4-753
    50/50, sizes 2^12..2^22, forward / inverse / coset-forward; 120 GB budget."""
    from . import BY_ID
    trace = poisson_trace(max(1, int(rate * seconds)), rate, seed)
    # one pinned input and output buffer per (field, size): inputs are uniform
    # random elements; outputs of equal-shape requests overwrite each other,
    # except for a seeded sample of requests (below) that get their own output
    bufs = {}
    for _, fid, k, _ in trace:
        if (fid, k) not in bufs:
            f = BY_ID[fid]
            nbytes = (1 << k) * f.limbs * 4
            pin = g.host_buffer(nbytes)
            pout = g.host_buffer(nbytes)
            a = np.ctypeslib.as_array(ctypes.cast(pin, ctypes.POINTER(ctypes.c_uint32)), shape=((1 << k) * f.limbs,))
            a[:] = f.device_random(1 << k, seed + 97 * k + fid).reshape(-1)
            bufs[(fid, k)] = (pin, pout)
    own: dict[int, ctypes.c_void_p] = {}  # sampled requests' own output buffers
    srv = Server(int(budget_gb * (1 << 30)), max_inflight=max_inflight, policy=policy)
    try:
        for fid in (1, 2):
            srv.warmup(fid, 12, 22)
        # one untimed request per buffer pair first: the first DMA from or to a freshly allocated pinned
        # buffer runs far below the link rate, and a serving process reuses its buffers
        srv.run_trace([TraceEntry(0.0, Request(fid, k, 0, None, pin.value, pout.value))
                       for (fid, k), (pin, pout) in bufs.items()])
        sample = verification_sample(trace, seed)
        for i in sample:
            _, fid, k, _ = trace[i]
            own[i] = g.host_buffer((1 << k) * BY_ID[fid].limbs * 4)
        entries = []
        for i, (t, fid, k, d) in enumerate(trace):
            pin, pout = bufs[(fid, k)]
            out = own[i] if i in own else pout
            entries.append(TraceEntry(t, Request(fid, k, d, None, pin.value, out.value)))
        lat, makespan, ph = srv.run_trace(entries, phases=True)
        st = srv.stats()
        # every sampled output against the plain path (gsn_ntt on the same input, same direction)
        verified = True
        for i in sample:
            _, fid, k, d = trace[i]
            f = BY_ID[fid]
            shape = ((1 << k) * f.limbs,)
            pin, _ = bufs[(fid, k)]
            x = np.ctypeslib.as_array(ctypes.cast(pin, ctypes.POINTER(ctypes.c_uint32)), shape=shape).copy()
            got = np.ctypeslib.as_array(ctypes.cast(own[i], ctypes.POINTER(ctypes.c_uint32)), shape=shape)
            t = g.to_device(x)
            g.ntt(f, t, direction=d)
            verified = verified and bool(np.array_equal(g.to_host(t), got))
            del t
    finally:
        srv.close()
        for pin, pout in bufs.values():
            g.free_host_buffer(pin)
            g.free_host_buffer(pout)
        for b in own.values():
            g.free_host_buffer(b)
    elements = sum(1 << k for _, _, k, _ in trace)
    return {"requests": len(trace), "rate_req_s": rate, "arrival_window_s": round(trace[-1][0], 4),
            "p50_ms": round(float(np.percentile(lat, 50)) * 1e3, 3),
            "p99_ms": round(float(np.percentile(lat, 99)) * 1e3, 3),
            "mean_ms": round(float(lat.mean()) * 1e3, 3), "makespan_s": round(makespan, 4),
            "throughput_req_s": round(len(trace) / makespan, 1),
            "throughput_Melem_s": round(elements / makespan / 1e6, 2),
            "launches": st["launches"], "device_bytes_peak": st["device_bytes_peak"],
            "scheduler_step_max_ms": {k: round(v * 1e3, 3) for k, v in
                                      zip(("admit", "uploads", "retire", "downloads", "launch"), st["step_max_s"])},
            "phase_ms_p50": {k: round(float(np.percentile(ph[:, i], 50)) * 1e3, 3) for i, k in enumerate(PHASES)},
            "phase_ms_p99": {k: round(float(np.percentile(ph[:, i], 99)) * 1e3, 3) for i, k in enumerate(PHASES)},
            "p99_request_phases_ms": {k: round(float(ph[int(np.argsort(lat)[int(0.99 * (len(lat) - 1))]), i]) * 1e3, 3)
                                      for i, k in enumerate(PHASES)},
            "verified": verified, "verified_requests": len(sample),
            "verified_how": "a seeded sample (both fields, every direction, the largest size of each field) "
                            "with their own output buffers, bit-exact against gsn_ntt on the same input",
            "budget_bytes": int(budget_gb * (1 << 30)), "max_inflight": max_inflight,
            "policy": "least_work_first" if policy == LEAST_WORK_FIRST else "oldest_first"}
