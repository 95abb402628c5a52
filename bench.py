"""Benchmark: field NTT on one GB300 (per rank), one JSON line on rank 0.

Headline workload (``value``): forward NTT over the MNT4-753 scalar field r
(24 x 32-bit limbs), n = 2^18, seeded uniform inputs, data resident in HBM;
the input (25 MB) is smaller than L2, so L2 is flushed (256 MB write) before
every timed step and only the transform is timed, with CUDA events on the
launching stream.  ``e2e`` is the same transform through the C-ABI host entry
point gsn_ntt_host (the best_fft drop-in) on a pinned host buffer: the input
is copied in from and the result copied back to host memory inside the timed
region.  ``roofline`` compares the transform's algorithmic integer
multiply-adds (2352 per 24-limb Montgomery product, (n/2) log2 n products)
with the measured throughput of the same PTX carry-chain instructions
(gsn_microbench_imad) in the same process.

``extra`` carries the other configurations (32-bit sweep against the HBM
roofline, MNT4 2^20, the 4096-job BLS12-381 batch against per-call, serving
p50/p99) unless --headline-only.

--impl reference times the reference's host FFT algorithm (the oracle's
restatement of test/fft_host.h, fixed butterfly, OpenMP over all host cores)
on the same workload; it is the CPU arm the driver compares against.

Multi-GPU: the path shards by independent transforms (replicas); under
torchrun every rank runs the workload on its own GPU and rank 0 reports the
max time over ranks (weak scaling).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import pathlib
import shutil
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "field-NTT Melem/s & % roofline, batched vs per-call; serving p50/p99 latency"
HEADLINE_LOG_N = 18
SEED = 0x5EED0000
PEAKS = ROOT / "MEASURED_PEAKS.json"
PUBLISHED_REF_768_2_18_S = 21.42  # README.md:46, GTX 1060, the reference's own (non-DFT) dataflow
# MNT4-753 q, the modulus the reference's fields::Scalar compiles in (cuda/device_field.h:62-65)
REF_Q = int("41898490967918953402344214791240637128170709919953949071783502921025352812571106773058"
            "893763790338921418070971888253786114353726529584385201591605722013126468931404347949"
            "840543007986327743462853720628051692141265303114721689601")


# --------------------------------------------------------------------------- utils
def headline_config(ws: int) -> dict:
    """The workload's `config`, printed identically by both arms."""
    return {"workload": "forward NTT, MNT4-753 scalar field r (24 limbs), n=2^18, per GPU",
            "field": "mnt4753_fr", "log_n": HEADLINE_LOG_N, "elements_per_step": 1 << HEADLINE_LOG_N,
            "l2": "GPU arm: flushed (256 MB write) before each step; input 25 MB < L2",
            "parallelism": f"replicas x{ws}"}


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    return rank, local, ws


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, ws: int) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi samples during the timed region (SM clock, throttle reasons)."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        if shutil.which("nvidia-smi"):
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


class NvmlSampler:
    """Reads the SM clock and the clock-event (throttle) reasons through NVML every ~2 ms in a thread, so
    even a timed region of a few milliseconds is covered.  Read-only queries; raises on any NVML error so
    the caller can fall back to nvidia-smi."""

    SW_POWER_CAP, HW_SLOWDOWN, SW_THERMAL, HW_THERMAL = 0x4, 0x8, 0x20, 0x40

    def __init__(self, torch, index: int):
        self.lib = ctypes.CDLL("libnvidia-ml.so.1")
        self.samples: list[tuple[int, int]] = []
        self.stop = False
        if self.lib.nvmlInit_v2() != 0:
            raise RuntimeError("nvmlInit failed")
        try:
            self.h = ctypes.c_void_p()
            uuid = "GPU-" + str(torch.cuda.get_device_properties(index).uuid)
            if self.lib.nvmlDeviceGetHandleByUUID(uuid.encode(), ctypes.byref(self.h)) != 0:
                raise RuntimeError("no NVML handle for " + uuid)
            self.reasons_fn = getattr(self.lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
                self.lib.nvmlDeviceGetCurrentClocksThrottleReasons
            mx = ctypes.c_uint()
            if self.lib.nvmlDeviceGetMaxClockInfo(self.h, 1, ctypes.byref(mx)) != 0:  # 1 = NVML_CLOCK_SM
                raise RuntimeError("nvmlDeviceGetMaxClockInfo failed")
            self.max_mhz = mx.value
            self._sample()
            if not self.samples:
                raise RuntimeError("NVML clock query failed")
        except Exception:
            self.lib.nvmlShutdown()
            raise

    def _sample(self):
        clk, rs = ctypes.c_uint(), ctypes.c_ulonglong()
        if self.lib.nvmlDeviceGetClockInfo(self.h, 1, ctypes.byref(clk)) == 0 and \
                self.reasons_fn(self.h, ctypes.byref(rs)) == 0:
            self.samples.append((clk.value, rs.value))

    def _run(self):
        while not self.stop:
            self._sample()
            time.sleep(0.002)

    def __enter__(self):
        self.samples.clear()
        self.thread = threading.Thread(target=self._run, daemon=True)
        self.thread.start()
        return self

    def __exit__(self, *a):
        self.stop = True
        self.thread.join()
        self.lib.nvmlShutdown()

    def summary(self) -> dict:
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": self.max_mhz, "reasons": [], "samples": 0, "source": "nvml"}
        names = {self.SW_POWER_CAP: "sw_power_cap", self.HW_SLOWDOWN: "hw_slowdown",
                 self.SW_THERMAL: "sw_thermal_slowdown", self.HW_THERMAL: "hw_thermal_slowdown"}
        reasons = sorted({nm for _, r in self.samples for bit, nm in names.items() if r & bit})
        return {"sm_mhz": float(np.median([c for c, _ in self.samples])), "sm_max_mhz": float(self.max_mhz),
                "reasons": reasons, "samples": len(self.samples), "source": "nvml, every ~2 ms"}


def clock_sampler(torch, index: int):
    try:
        return NvmlSampler(torch, index)
    except Exception:
        return ClockSampler(index)


def peaks() -> dict:
    try:
        return json.loads(PEAKS.read_text())
    except Exception:
        return {}


# --------------------------------------------------------------------------- GPU arm
def imad_peak(g) -> dict:
    lib = g.load()
    a, b, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    g._lib.check(lib.gsn_microbench_imad(20000, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
    out = {"mads_per_s": a.value, "mads_per_clk_sm": b.value, "sm_mhz": c.value}
    # the carry-free forms beside it: instructions per second, and per SM per clock at the same clock
    sms = max(1, int(__import__("torch").cuda.get_device_properties(0).multi_processor_count))
    for form, name in ((1, "mad_wide"), (2, "mad_lo"), (3, "mad_hi"), (4, "add_chain")):
        v = ctypes.c_double()
        g._lib.check(lib.gsn_microbench_imad_form(form, 20000, ctypes.byref(v)))
        out[f"{name}_per_s"] = v.value
        out[f"{name}_per_clk_sm"] = v.value / sms / (c.value * 1e6) if c.value > 0 else None
    return out


def montgomery_schedules(g, iters: int = 2000) -> dict:
    """Montgomery products per second on the whole GPU for the one-thread schedules (0 row chains,
    1 even/odd accumulators merged every row, the kernels' default) and the 24-limb product split over
    2 or 4 cooperating lanes."""
    lib = g.load()
    out = {}
    for name, fid in (("bls12_381_fr", 1), ("mnt4753_fr", 2)):
        per = {}
        for sched in (0, 1):
            v = ctypes.c_double()
            g._lib.check(lib.gsn_microbench_mont(fid, sched, iters, ctypes.byref(v)))
            per[f"thread_schedule{sched}_G_per_s"] = round(v.value / 1e9, 3)
        if fid == 2:
            for lanes in (2, 4):
                v = ctypes.c_double()
                g._lib.check(lib.gsn_microbench_mont_coop(fid, lanes, iters, ctypes.byref(v)))
                per[f"coop_{lanes}_lanes_G_per_s"] = round(v.value / 1e9, 3)
        out[name] = per
    return out


def ref_compat_shipped_call(g, torch) -> dict:
    """The reference's shipped call (test/main.cpp:45-71: every input Scalar(1234), omega = the raw limbs
    of its modulus, log_cpus = 10) through gsn_fft_ref_compat on the GPU at n = 2^12 and 2^16.  The
    CPU restatement of the same dataflow is timed in cpu_baseline()."""
    q = np.array([(REF_Q >> (32 * i)) & 0xFFFFFFFF for i in range(24)], dtype=np.uint32)
    out = {"log_cpus": 10}
    for log_n in (12, 16):
        data = np.zeros((1 << log_n, 24), dtype=np.uint32)
        data[:, 0] = 1234
        d = g.to_device(data)
        g.fft_ref_compat(d, q, 10)  # warm
        torch.cuda.synchronize()
        d.copy_(g.to_device(data))
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        g.fft_ref_compat(d, q, 10)
        e.record()
        e.synchronize()
        out[f"gpu_ms_2^{log_n}"] = round(s.elapsed_time(e), 3)
    return out


def time_device_ntt(g, torch, f, log_n: int, steps: int, warmup: int, direction=0, flush=None):
    """Per-step CUDA-event time of one in-place transform (L2 flushed before each)."""
    n = 1 << log_n
    data = torch.empty(n * f.limbs, dtype=torch.int32, device="cuda")
    from gpusnarks_gb300.batch import fill_random
    fill_random(f, data, SEED + log_n)
    stream = torch.cuda.current_stream()
    for _ in range(warmup):
        g.ntt(f, data, direction=direction)
    torch.cuda.synchronize()
    times = []
    launches0 = g.launch_count()
    for _ in range(steps):
        if flush is not None:
            flush.zero_()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        g.ntt(f, data, direction=direction)
        e.record(stream)
        e.synchronize()
        times.append(s.elapsed_time(e) * 1e-3)
    launches = g.launch_count() - launches0
    del data
    return times, launches


def time_e2e_host(g, f, log_n: int, steps: int, warmup: int):
    """gsn_ntt_host on pinned host memory: H2D + transform + D2H per step."""
    n = 1 << log_n
    nbytes = n * f.limbs * 4
    buf = g.host_buffer(nbytes)
    arr = np.ctypeslib.as_array(ctypes.cast(buf, ctypes.POINTER(ctypes.c_uint32)), shape=(n * f.limbs,))
    arr[:] = f.device_random(n, SEED + log_n).reshape(-1)
    lib = g.load()
    for _ in range(warmup):
        g._lib.check(lib.gsn_ntt_host(f.fid, buf.value, log_n, None, 0, None))
    times = []
    for _ in range(steps):
        t0 = time.perf_counter()
        g._lib.check(lib.gsn_ntt_host(f.fid, buf.value, log_n, None, 0, None))
        times.append(time.perf_counter() - t0)
    g.free_host_buffer(buf)
    return times, nbytes


def time_e2e_pipelined(g, f, log_n: int, steps: int, warmup: int):
    """gsn_ntt_host_batch over `steps` pinned host buffers, one per step: every step's input is copied in
    from and its result copied back to host memory inside the timed call, with the copies of neighbouring
    steps overlapping each transform.  Returns the whole call's seconds."""
    n = 1 << log_n
    nbytes = n * f.limbs * 4
    bufs = [g.host_buffer(nbytes) for _ in range(steps)]
    try:
        for i, b in enumerate(bufs):
            a = np.ctypeslib.as_array(ctypes.cast(b, ctypes.POINTER(ctypes.c_uint32)), shape=(n * f.limbs,))
            a[:] = f.device_random(n, SEED + log_n + i).reshape(-1)
        lib = g.load()
        arr = (ctypes.c_void_p * steps)(*[b.value for b in bufs])
        # warm-up over every buffer: the first transfer to or from a freshly page-locked buffer costs
        # extra (about 2x a warm one here), as the single-call e2e's reused buffer does not
        for _ in range(max(1, warmup)):
            g._lib.check(lib.gsn_ntt_host_batch(f.fid, arr, steps, log_n, None, 0, None))
        t0 = time.perf_counter()
        g._lib.check(lib.gsn_ntt_host_batch(f.fid, arr, steps, log_n, None, 0, None))
        return time.perf_counter() - t0
    finally:
        for b in bufs:
            g.free_host_buffer(b)


def profiled_traffic(key: str):
    """DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) recorded from an ncu capture
    in profiles/traffic.txt (`<kernel> <size>: <bytes>` lines); None when absent."""
    path = ROOT / "profiles" / "traffic.txt"
    if not path.exists():
        return None
    for ln in path.read_text().splitlines():
        if ln.startswith(key + ":"):
            return int(ln.split(":", 1)[1].split()[0])
    return None


def profiled_pipe(key: str):
    """(fmaheavy-busy % per launch, durations us) recorded in profiles/traffic.txt as
    `pipe <kernel> <size>: a b c durations_us x y z` lines; None when absent."""
    path = ROOT / "profiles" / "traffic.txt"
    if not path.exists():
        return None
    for ln in path.read_text().splitlines():
        if ln.startswith("pipe " + key + ":"):
            body = ln.split(":", 1)[1].split()
            if "durations_us" in body:
                i = body.index("durations_us")
                return [float(v) for v in body[:i]], [float(v) for v in body[i + 1:]]
            return [float(v) for v in body], None
    return None


def imad_work(f, log_n: int) -> float:
    s = f.limbs
    per_mul = 2 * (2 * s * s + s)
    return per_mul * (2 ** (log_n - 1)) * log_n


def p32_sweep(g, torch, flush, hbm_gbs, steps=5):
    out = {}
    l2 = torch.cuda.get_device_properties(0).L2_cache_size
    for log_n in (20, 22, 24, 26, 28):
        n = 1 << log_n
        ts, _ = time_device_ntt(g, torch, g.P32, log_n, steps, 2, flush=flush)
        t = float(np.median(ts))
        pmin = 1 if 4 * n <= l2 / 2 else 2
        B = 2 * 4 * n * pmin
        out[f"2^{log_n}"] = {"ms": round(t * 1e3, 4), "Melem_s": round(n / t / 1e6, 1),
                             "hbm_frac": round(B / t / 1e9 / hbm_gbs, 4),
                             "single_pass_frac": round(8 * n / t / 1e9 / hbm_gbs, 4), "p_min": pmin}
    out["2^26"]["dram_bytes_per_launch"] = profiled_traffic("ntt_p32_fixed_kernel 2^26")
    # the CPU restatement beside the sizes it finishes in seconds (the reference's README times its CPU FFT
    # at 2^20 and 2^22 only and reports 2^25 and 2^28 as not finished)
    for log_n in (20, 22):
        out[f"2^{log_n}"]["cpu_port"] = cpu_port_rate(0, log_n, g.P32.device_random(1 << log_n, SEED + log_n))
    return out


def cpu_threads() -> tuple[int, int]:
    """(threads, log_cpus) for the CPU restatement: every host core, num_cpus = the largest power of two."""
    threads = os.cpu_count() or 1
    return threads, max(0, int(math.floor(math.log2(threads))))


def cpu_port_rate(fid: int, log_n: int, x, reps: int = 1) -> dict:
    """The oracle's restatement of the reference host FFT (fixed butterfly) on all host cores: median of
    `reps` full transforms of `x` (one untimed first)."""
    import oracle
    threads, log_cpus = cpu_threads()
    w = oracle.root(fid, log_n)
    oracle.fft(fid, x, w, log_cpus=log_cpus, nthreads=threads)
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        oracle.fft(fid, x, w, log_cpus=log_cpus, nthreads=threads)
        ts.append(time.perf_counter() - t0)
    t = float(np.median(ts))
    return {"ms": round(t * 1e3, 3), "Melem_s": round((1 << log_n) / t / 1e6, 4), "cores": threads,
            "log_cpus": log_cpus, "kind": "port"}


def config1_p32_2_16(g, torch, flush, hbm_gbs, steps=20):
    """Plain forward NTT over p32 at n = 2^16 (the reference's README row 'FFT 32-bit n=2^16'):
    device-resident time (L2 flushed before each step) against the HBM roofline with P_min = 1, the
    whole best_fft-style call from host memory (gsn_ntt_host), the output checked against the oracle, and
    the CPU restatement beside it."""
    import oracle
    f = g.P32
    log_n = 16
    n = 1 << log_n
    ts, _ = time_device_ntt(g, torch, f, log_n, steps, 3, flush=flush)
    t = float(np.median(ts))
    x = f.device_random(n, SEED + log_n)
    d = g.to_device(x)
    g.ntt(f, d)
    verified = bool(np.array_equal(g.to_host(d), oracle.ntt(0, x)))
    e2e, _ = time_e2e_host(g, f, log_n, steps, 3)
    te = float(np.median(e2e))
    B = 2 * 4 * n
    return {"ms": round(t * 1e3, 4), "Melem_s": round(n / t / 1e6, 1), "hbm_frac": round(B / t / 1e9 / hbm_gbs, 4),
            "p_min": 1, "host_call_ms": round(te * 1e3, 4), "host_call_Melem_s": round(n / te / 1e6, 1),
            "host_call_api": "gsn_ntt_host on pinned memory (copy in, transform, copy out)",
            "verified_vs_oracle": verified, "cpu_port": cpu_port_rate(0, log_n, x, reps=5),
            "published_reference_s": {"gpu": 0.32, "cpu": 0.21, "where": "README.md:30, GTX 1080 / Xeon"}}


def poly_product_2_21(g, torch, reps=5):
    """Config 3's companion: two seeded polynomials with 2^20 coefficients multiplied by forward NTTs of
    size 2^21, a pointwise product and an inverse NTT, device-resident (inputs > L2 in total: 2 x 8 MiB is
    not, so L2 is not flushed: this times the four launches back to back as a prover would run them).
    Checked against the oracle's NTT product; the CPU restatement of the same three transforms beside it."""
    import oracle
    f = g.P32
    P = f.p
    m = 1 << 20
    a = f.device_random(m, SEED + 3 * 100 + 1)
    b = f.device_random(m, SEED + 3 * 100 + 2)
    A = np.zeros(2 * m, dtype=np.uint32)
    B = np.zeros(2 * m, dtype=np.uint32)
    A[:m], B[:m] = a, b
    dA0, dB0 = g.to_device(A), g.to_device(B)
    dA, dB = dA0.clone(), dB0.clone()
    stream = torch.cuda.current_stream()

    def run():
        g.ntt(f, dA)
        g.ntt(f, dB)
        g.pointwise_mul(f, dA, dB)
        g.ntt(f, dA, direction=g.INVERSE)

    run()
    torch.cuda.synchronize()
    c = g.to_host(dA)
    ts = []
    for _ in range(reps):
        dA.copy_(dA0)
        dB.copy_(dB0)
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        run()
        e.record(stream)
        e.synchronize()
        ts.append(s.elapsed_time(e) * 1e-3)
    t = float(np.median(ts))
    # CPU: the restated host FFT for the three transforms, numpy for the pointwise product and n^-1
    threads, log_cpus = cpu_threads()
    w = oracle.root(0, 21)
    t0 = time.perf_counter()
    Ao = oracle.fft(0, A, w, log_cpus=log_cpus, nthreads=threads)
    Bo = oracle.fft(0, B, w, log_cpus=log_cpus, nthreads=threads)
    prod = ((Ao.astype(np.uint64) * Bo.astype(np.uint64)) % np.uint64(P)).astype(np.uint32)
    y = oracle.fft(0, prod, pow(w, P - 2, P), log_cpus=log_cpus, nthreads=threads)
    want = ((y.astype(np.uint64) * np.uint64(pow(2 * m, P - 2, P))) % np.uint64(P)).astype(np.uint32)
    t_cpu = time.perf_counter() - t0
    return {"ms": round(t * 1e3, 4), "transforms": 3, "pointwise": 1,
            "Melem_s": round(3 * 2 * m / t / 1e6, 1),
            "coefficients_per_s_M": round(2 * m / t / 1e6, 1),
            "verified_vs_oracle": bool(np.array_equal(c, want)),
            "cpu_port": {"ms": round(t_cpu * 1e3, 1), "cores": threads, "log_cpus": log_cpus, "kind": "port",
                         "what": "three restated host FFTs of 2^21 + numpy pointwise product and n^-1 scale"}}


def multiexp_bench(g, torch, hbm_gbs, imad_per_s, reps=10):
    """sum_i a[i] b[i] (the reference's multiexp for field elements) per field at a size well above L2:
    device-resident inputs, CUDA-event time of the two launches, elements/s against the HBM roofline (both
    arrays read once: 2 x 4N bytes per element) and against the multiply-add roofline (N^2 word products
    per element, 2 IMAD each); a 4097-element case checked against the oracle; the oracle's serial
    restatement of test/multiexp.h (as the reference runs it) timed on a subset beside it."""
    import oracle
    from gpusnarks_gb300.batch import fill_random
    out = {}
    stream = torch.cuda.current_stream()
    for f, log_n, cpu_n in ((g.P32, 26, 1 << 22), (g.BLS12_381, 24, 1 << 18), (g.MNT4_753, 21, 1 << 15)):
        n = 1 << log_n
        a = torch.empty(n * f.limbs, dtype=torch.int32, device="cuda")
        b = torch.empty(n * f.limbs, dtype=torch.int32, device="cuda")
        fill_random(f, a, SEED + 600 + f.fid)
        fill_random(f, b, SEED + 700 + f.fid)
        r = torch.empty(f.limbs, dtype=torch.int32, device="cuda")
        for _ in range(3):
            g.multiexp(f, a, b, r)
        torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            s0, e0 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s0.record(stream)
            g.multiexp(f, a, b, r)
            e0.record(stream)
            e0.synchronize()
            ts.append(s0.elapsed_time(e0) * 1e-3)
        t = float(np.median(ts))
        del a, b
        x = f.random_array(4097, seed=SEED + 800 + f.fid)
        y = f.random_array(4097, seed=SEED + 900 + f.fid)
        got = g.to_host(g.multiexp(f, g.to_device(x), g.to_device(y)))
        verified = bool(np.array_equal(got, oracle.multiexp(f.fid, x, y)))
        xc = f.device_random(cpu_n, SEED + 1000 + f.fid)
        yc = f.device_random(cpu_n, SEED + 1100 + f.fid)
        t0 = time.perf_counter()
        oracle.multiexp(f.fid, xc, yc)
        t_cpu = time.perf_counter() - t0
        nbytes = 2 * 4 * f.limbs * n
        imad = 2 * f.limbs * f.limbs * n
        out[f.name] = {"log_n": log_n, "ms": round(t * 1e3, 4), "Gelem_s": round(n / t / 1e9, 3),
                       "hbm_frac": round(nbytes / t / 1e9 / hbm_gbs, 4),
                       "imad_frac": round(imad / t / imad_per_s, 4), "launches": 2,
                       "verified_vs_oracle_4097": verified,
                       "cpu_port": {"Melem_s": round(cpu_n / t_cpu / 1e6, 3), "elements": cpu_n, "cores": 1,
                                    "kind": "port", "sample": "serial restatement of test/multiexp.h:3-13"}}
    return out


def batch_vs_per_call(g, torch, njobs=4096, lo=10, hi=20, reps=3):
    from gpusnarks_gb300.batch import Batch, fill_random, job_sizes
    f = g.BLS12_381
    sizes = job_sizes(njobs, lo, hi, SEED + 4)
    total = sum(1 << k for k in sizes)
    pool = torch.empty(total * f.limbs, dtype=torch.int32, device="cuda")
    fill_random(f, pool, SEED + 4)
    jobs, off = [], 0
    for k in sizes:
        jobs.append((pool.data_ptr() + off * f.limbs * 4, k, 0, None, None))
        off += 1 << k
    b = Batch(f, jobs, graph=True)
    stream = torch.cuda.current_stream()
    # a seeded sample of jobs is checked after the first batched launch against the plain per-call path
    # (gsn_ntt on a copy of the same input); every size class 2^lo..2^hi is in the sample
    rng = np.random.default_rng(SEED + 44)
    by_size: dict[int, list[int]] = {}
    for i, k in enumerate(sizes):
        by_size.setdefault(k, []).append(i)
    sample = sorted({int(rng.choice(v)) for v in by_size.values()} |
                    {int(i) for i in rng.choice(njobs, size=min(njobs, 32), replace=False)})
    offs = np.cumsum([0] + [1 << k for k in sizes])
    views = {i: pool[int(offs[i]) * f.limbs:int(offs[i + 1]) * f.limbs] for i in sample}
    want = {i: v.clone() for i, v in views.items()}
    for i, w in want.items():
        g.ntt(f, w)

    def timed(fn):
        ts = []
        for _ in range(reps):
            torch.cuda.synchronize()
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record(stream)
            fn()
            e.record(stream)
            e.synchronize()
            ts.append(s.elapsed_time(e) * 1e-3)
        return float(np.median(ts))

    b.launch()
    torch.cuda.synchronize()
    b.status()
    verified = all(torch.equal(views[i], want[i]) for i in sample)
    b.launch_per_call()
    torch.cuda.synchronize()
    t_batch = timed(lambda: b.launch())
    b.status()
    t_call = timed(lambda: b.launch_per_call())
    info = b.info()
    b.close()
    del pool
    torch.cuda.empty_cache()
    work = sum(imad_work(f, k) for k in sizes)
    # CPU restatement on a bounded subset: the sampled jobs up to 2^16 (every size class up to there)
    import oracle
    threads, log_cpus = cpu_threads()
    cpu_jobs = [i for i in sample if sizes[i] <= 16]
    cpu_el, t0 = 0, time.perf_counter()
    for i in cpu_jobs:
        x = f.device_random(1 << sizes[i], SEED + 4400 + i)
        oracle.fft(1, x, oracle.root(1, sizes[i]), log_cpus=min(log_cpus, sizes[i]), nthreads=threads)
        cpu_el += 1 << sizes[i]
    t_cpu = time.perf_counter() - t0
    return {"jobs": njobs, "elements": total, "log_n_range": [lo, hi],
            "verified": verified, "verified_jobs": len(sample),
            "verified_how": "seeded sample covering every size class, after the first batched launch, "
                            "bit-exact against gsn_ntt (the per-call path) on a copy of the same input",
            "cpu_port": {"Melem_s": round(cpu_el / t_cpu / 1e6, 4) if t_cpu > 0 else None, "jobs": len(cpu_jobs),
                         "elements": cpu_el, "cores": threads, "kind": "port",
                         "sample": "the verified jobs up to 2^16, restated host FFT each"},
            "batched_ms": round(t_batch * 1e3, 3), "per_call_ms": round(t_call * 1e3, 3),
            "batched_Melem_s": round(total / t_batch / 1e6, 1), "per_call_Melem_s": round(total / t_call / 1e6, 1),
            "speedup": round(t_call / t_batch, 3), "batched_imad_T_s": round(work / t_batch / 1e12, 3),
            "work_items": info["work_items"]}


def run_gpu(args, rank, local, ws):
    import torch

    import gpusnarks_gb300 as g
    torch.cuda.set_device(local)
    g.load()
    f = g.MNT4_753
    log_n = HEADLINE_LOG_N
    n = 1 << log_n
    flush = torch.empty(256 << 20, dtype=torch.int8, device="cuda")
    pk = peaks()
    hbm_gbs = float(pk.get("hbm_gbs", 6800.0))
    ip = imad_peak(g)

    # headline: device-resident transforms
    barrier(ws)
    torch.cuda.synchronize()
    with clock_sampler(torch, local) as clk:
        ts, launches = time_device_ntt(g, torch, f, log_n, args.steps, args.warmup, flush=flush)
    torch.cuda.synchronize()
    barrier(ws)
    t_total = max_over_ranks(sum(ts), ws)
    t_step = t_total / args.steps
    value = n * args.steps * ws / t_total / 1e6
    # One step is `per_step` launches of the pass kernel; per launch, the algorithmic work is the
    # step's work / per_step and the average duration the step time / per_step.
    per_step = max(1, int(launches) // args.steps)
    achieved = (imad_work(f, log_n) / per_step) / (t_step / per_step)

    # e2e through the host entry point
    e2e_ts, nbytes = time_e2e_host(g, f, log_n, args.steps, max(1, args.warmup // 2))
    e2e_single = max_over_ranks(float(np.mean(e2e_ts)), ws)
    e2e_t = max_over_ranks(time_e2e_pipelined(g, f, log_n, args.steps, max(1, args.warmup // 2)), ws) / args.steps

    line = {
        "metric": METRIC, "value": round(value, 3), "unit": "Melem/s", "n_gpus": ws, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(t_step * 1e3, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": headline_config(ws),
        "e2e": {"value": round(n * ws / e2e_t / 1e6, 3), "unit": "Melem/s", "h2d_bytes_per_step": nbytes,
                "d2h_bytes_per_step": nbytes,
                "api": "gsn_ntt_host_batch over one pinned host buffer per step: each step's input copied in "
                       "and result copied out inside the timed call, neighbouring steps' copies overlapping "
                       "each transform",
                "single_call_Melem_s": round(n * ws / e2e_single / 1e6, 3),
                "single_call_api": "gsn_ntt_host per step (copy in, transform, copy out, synchronous)"},
        "roofline": {"bound": "imad", "achieved": round(achieved / 1e12, 4),
                     "peak": round(ip["mads_per_s"] / 1e12, 4), "unit": "TIMAD/s",
                     "frac": round(achieved / ip["mads_per_s"], 4), "traffic": None,
                     "peak_source": "gsn_microbench_imad in this process (PTX mad.lo.cc/madc.hi.cc chains, "
                                    "all SMs, full occupancy)",
                     "algorithmic_work": "2352 IMAD per 24-limb Montgomery product x (n/2) log2 n",
                     "launches_per_step": per_step},
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
        "published_reference": {"what": "FFT 768-bit n=2^18, GTX 1060, reference dataflow (not a DFT)",
                                "seconds": PUBLISHED_REF_768_2_18_S,
                                "Melem_s": round(n / PUBLISHED_REF_768_2_18_S / 1e6, 5)},
    }
    line["roofline"]["traffic"] = profiled_traffic("ntt_pass_kernel<FieldMNT4_753> 2^18")
    # the same fraction read off the hardware: ncu's fmaheavy-pipe busy cycles of the headline passes,
    # duration-weighted, over those of the denominator kernel (profiles/imad_pipe_*.md)
    pp, pd = profiled_pipe("ntt_pass_kernel<FieldMNT4_753> 2^18") or (None, None), profiled_pipe("imad_chain_kernel")
    if pp and pp[0] and pd:
        busy = float(np.average(pp[0], weights=pp[1])) if pp[1] else float(np.mean(pp[0]))
        line["roofline"]["pipe_check"] = {
            "fmaheavy_busy_pct": round(busy, 2), "denominator_fmaheavy_busy_pct": pd[0][0],
            "frac_vs_pipe": round(busy / pd[0][0], 4),
            "source": "ncu sm__pipe_fmaheavy_cycles_active of the three passes (duration-weighted) and of "
                      "imad_chain_kernel, profiles/imad_pipe_multiply_forms_and_pass_kernels.md"}
    if rank == 0 and ws == 1:
        line["cpu_baseline"] = cpu_baseline(args)
    if not args.headline_only and rank == 0:
        extra = {}
        t20, _ = time_device_ntt(g, torch, f, 20, 3, 1, flush=flush)
        extra["mnt4753_fr_2^20"] = {"ms": round(float(np.median(t20)) * 1e3, 3),
                                    "imad_frac": round(imad_work(f, 20) / float(np.median(t20)) / ip["mads_per_s"], 4)}
        extra["mnt4753_fr_2^20"]["cpu_port"] = cpu_port_rate(2, 20, f.device_random(1 << 20, SEED + 20))
        extra["p32_2^16"] = config1_p32_2_16(g, torch, flush, hbm_gbs)
        extra["p32_sweep"] = p32_sweep(g, torch, flush, hbm_gbs)
        extra["poly_product_2^21"] = poly_product_2_21(g, torch)
        extra["multiexp"] = multiexp_bench(g, torch, hbm_gbs, ip["mads_per_s"])
        extra["hbm_peak_gbs"] = hbm_gbs
        extra["hbm_peak_source"] = ("measured: MEASURED_PEAKS.json hbm_gbs (STREAM-style copy on this pool's GB300)"
                                    if "hbm_gbs" in pk else "fallback: 6.8 TB/s, one earlier GB300 measurement")
        try:
            extra["bls12_381_batch_4096"] = batch_vs_per_call(g, torch)
        except Exception as exc:  # report, do not hide
            extra["bls12_381_batch_4096"] = {"error": str(exc)}
        try:
            from gpusnarks_gb300.serve import LEAST_WORK_FIRST, bench_serving
            # the configured stream (2000 req/s offers more work than one GPU
            # completes, so its latency is queueing) and a sustainable rate
            extra["serving"] = bench_serving(g, torch, seconds=args.serve_seconds)
            # the same stream, smallest transforms launched first
            extra["serving_least_work_first"] = bench_serving(g, torch, seconds=args.serve_seconds,
                                                              policy=LEAST_WORK_FIRST)
            # a sustainable rate; 3x the window so its p99 rests on ~12 requests rather than 4
            extra["serving_400_req_s"] = bench_serving(g, torch, seconds=3 * args.serve_seconds, rate=400.0)
        except Exception as exc:
            extra["serving"] = {"error": str(exc)}
        extra["imad_microbench"] = ip
        extra["montgomery_schedules"] = montgomery_schedules(g)
        try:
            extra["ref_compat_shipped_call"] = ref_compat_shipped_call(g, torch)
        except Exception as exc:  # report, do not hide
            extra["ref_compat_shipped_call"] = {"error": str(exc)}
        line["extra"] = extra
    return line


# --------------------------------------------------------------------------- CPU arm
def cpu_baseline(args) -> dict:
    """The oracle's restatement of the reference host FFT on this host's cores."""
    import oracle
    import gpusnarks_gb300.fields as fields
    f = fields.MNT4_753
    n = 1 << HEADLINE_LOG_N
    x = f.device_random(n, SEED + HEADLINE_LOG_N)
    threads = os.cpu_count() or 1
    log_cpus = max(0, int(math.floor(math.log2(threads))))
    w = oracle.root(2, HEADLINE_LOG_N)
    oracle.fft(2, x, w, log_cpus=log_cpus, nthreads=threads)  # warm
    reps, ts = 0, []
    t_start = time.perf_counter()
    while reps < args.cpu_reps or (time.perf_counter() - t_start < 10 and reps < 20):
        t0 = time.perf_counter()
        oracle.fft(2, x, w, log_cpus=log_cpus, nthreads=threads)
        ts.append(time.perf_counter() - t0)
        reps += 1
    t = float(np.median(ts))
    # the reference's shipped call (test/main.cpp:45-71) over its own Scalar arithmetic, at n = 2^12
    shipped = np.zeros((1 << 12, 24), dtype=np.uint32)
    shipped[:, 0] = 1234
    t0 = time.perf_counter()
    oracle.refscalar_fft(shipped, oracle.to_limbs(3, REF_Q), 10, nthreads=threads)
    shipped_ms = (time.perf_counter() - t0) * 1e3
    return {"value": round(n / t / 1e6, 5), "unit": "Melem/s", "cores": threads, "kind": "port",
            "sample": f"full n=2^18 MNT4-753 r transform x{reps} (median), num_cpus decomposition "
                      f"log_cpus={log_cpus}, {threads} OpenMP threads; oracle/oracle.cpp restating "
                      "test/fft_host.h with the fixed butterfly",
            "shipped_call_2^12_ms": round(shipped_ms, 1),
            "shipped_call": "test/main.cpp:45-71 at n=2^12 (inputs Scalar(1234), omega = Scalar(_mod), "
                            "log_cpus=10) over the restated reference Scalar, all threads; "
                            "extra.ref_compat_shipped_call times the same on the GPU"}


def run_reference(args, rank, ws):
    """The reference arm: W untimed and K timed steps, each one full forward transform of the headline
    workload through the oracle's restatement of the reference host FFT, on all host threads.  A step that
    would push the timed region past two minutes ends it early (the count is reported)."""
    if rank != 0:
        return None
    import oracle
    import gpusnarks_gb300.fields as fields
    f = fields.MNT4_753
    n = 1 << HEADLINE_LOG_N
    x = f.device_random(n, SEED + HEADLINE_LOG_N)
    threads = os.cpu_count() or 1
    log_cpus = max(0, int(math.floor(math.log2(threads))))
    w = oracle.root(2, HEADLINE_LOG_N)
    for _ in range(args.warmup):
        oracle.fft(2, x, w, log_cpus=log_cpus, nthreads=threads)
    ts = []
    t_start = time.perf_counter()
    for _ in range(args.steps):
        t0 = time.perf_counter()
        oracle.fft(2, x, w, log_cpus=log_cpus, nthreads=threads)
        ts.append(time.perf_counter() - t0)
        if time.perf_counter() - t_start + ts[-1] > 120.0:
            break
    t = float(np.median(ts))
    v = round(n / t / 1e6, 5)
    cb = {"value": v, "unit": "Melem/s", "cores": threads, "kind": "port",
          "sample": f"{len(ts)} timed steps (of {args.steps} asked) after {args.warmup} untimed, each a full "
                    f"n=2^18 MNT4-753 r forward transform, median; num_cpus decomposition log_cpus={log_cpus}, "
                    f"{threads} OpenMP threads; oracle/oracle.cpp restating test/fft_host.h with the fixed "
                    "butterfly"}
    return {"impl": "reference", "metric": METRIC, "value": v, "unit": "Melem/s", "n_gpus": ws,
            "steps": len(ts), "warmup": args.warmup, "ms_per_step": round(t * 1e3, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": headline_config(ws),
            "cpu_baseline": cb,
            "e2e": {"value": v, "unit": "Melem/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--headline-only", action="store_true")
    ap.add_argument("--cpu-reps", type=int, default=3)
    ap.add_argument("--serve-seconds", type=float, default=1.0)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    rank, local, ws = dist_init()
    if args.impl == "reference":
        line = run_reference(args, rank, ws)
    else:
        line = run_gpu(args, rank, local, ws)
    if rank == 0 and line is not None:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
