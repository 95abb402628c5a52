"""Run one transform configuration a few times, for profilers.

    python -m gpusnarks_gb300.profile_case --field p32 --log-n 24 --reps 3
    python -m gpusnarks_gb300.profile_case --field bls12_381_fr --batch 512 --batch-lo 10 --batch-hi 18
    python -m gpusnarks_gb300.profile_case --microbench imad --iters 2000
    python -m gpusnarks_gb300.profile_case --multiexp 24 --field bls12_381_fr --reps 1 --warmup 1

Fills the input on the device (gsn_fill_random), runs `warmup` untimed and
`reps` further transforms through the C ABI, prints the mean event time.
With --batch J it runs J jobs of seeded log-uniform sizes 2^lo..2^hi as one
persistent graph-captured launch (the batched path) instead.  It is the
command the committed ncu summaries under profiles/ were taken with.
"""
from __future__ import annotations

import argparse


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--field", default="p32", choices=["p32", "bls12_381_fr", "mnt4753_fr"])
    ap.add_argument("--log-n", type=int, default=20)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=1)
    ap.add_argument("--direction", type=int, default=0)
    ap.add_argument("--batch", type=int, default=0, help="jobs in one batched launch (0: one transform)")
    ap.add_argument("--batch-lo", type=int, default=10)
    ap.add_argument("--batch-hi", type=int, default=18)
    ap.add_argument("--microbench", default="", choices=["", "imad", "imad_wide", "imad_lo", "imad_hi", "add_chain"],
                    help="run one integer multiply-add microbenchmark instead (--iters steps per thread)")
    ap.add_argument("--iters", type=int, default=2000)
    ap.add_argument("--multiexp", type=int, default=0, help="log2 n: run gsn_multiexp on 2^n elements instead")
    args = ap.parse_args()

    import torch

    import gpusnarks_gb300 as g
    from gpusnarks_gb300.batch import fill_random

    if args.microbench:
        run_microbench(g, args)
        return
    if args.multiexp:
        run_multiexp(g, torch, args)
        return
    f = g.FIELDS[args.field]
    if args.batch:
        run_batch(g, torch, f, args)
        return
    n = 1 << args.log_n
    data = torch.empty(n * f.limbs, dtype=torch.int32, device="cuda")
    fill_random(f, data, 0x5EED0000 + args.log_n)
    for _ in range(args.warmup):
        g.ntt(f, data, direction=args.direction)
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    for _ in range(args.reps):
        g.ntt(f, data, direction=args.direction)
    e.record()
    torch.cuda.synchronize()
    ms = s.elapsed_time(e) / max(args.reps, 1)
    print(f"{args.field} 2^{args.log_n}: {ms:.4f} ms per transform, {n / ms / 1e3:.1f} Melem/s")



def run_multiexp(g, torch, args) -> None:
    """gsn_multiexp over 2^multiexp seeded elements (two launches per call)."""
    from gpusnarks_gb300.batch import fill_random
    f = g.FIELDS[args.field]
    n = 1 << args.multiexp
    a = torch.empty(n * f.limbs, dtype=torch.int32, device="cuda")
    b = torch.empty(n * f.limbs, dtype=torch.int32, device="cuda")
    fill_random(f, a, 0x5EED0600)
    fill_random(f, b, 0x5EED0700)
    out = torch.empty(f.limbs, dtype=torch.int32, device="cuda")
    for _ in range(args.warmup):
        g.multiexp(f, a, b, out)
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    for _ in range(args.reps):
        g.multiexp(f, a, b, out)
    e.record()
    torch.cuda.synchronize()
    ms = s.elapsed_time(e) / max(args.reps, 1)
    print(f"{args.field} multiexp 2^{args.multiexp}: {ms:.4f} ms, {n / ms / 1e6:.2f} G elements/s")


def run_microbench(g, args) -> None:
    """gsn_microbench_imad (carry chains: a warm-up launch, then the timed one) or one carry-free form of
    gsn_microbench_imad_form (the same two launches)."""
    import ctypes
    lib = g.load()
    if args.microbench == "imad":
        a, b, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        g._lib.check(lib.gsn_microbench_imad(args.iters, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        print(f"carry-chain multiply-adds: {a.value / 1e12:.3f} T/s, {b.value:.1f} per SM per clock at {c.value:.0f} MHz")
        return
    form = {"imad_wide": 1, "imad_lo": 2, "imad_hi": 3, "add_chain": 4}[args.microbench]
    v = ctypes.c_double()
    g._lib.check(lib.gsn_microbench_imad_form(form, args.iters, ctypes.byref(v)))
    print(f"{args.microbench}: {v.value / 1e12:.3f} T instructions/s")


def run_batch(g, torch, f, args) -> None:
    from gpusnarks_gb300.batch import Batch, fill_random, job_sizes

    sizes = job_sizes(args.batch, args.batch_lo, args.batch_hi, 0x5EED0004)
    total = sum(1 << k for k in sizes)
    pool = torch.empty(total * f.limbs, dtype=torch.int32, device="cuda")
    fill_random(f, pool, 0x5EED0004)
    jobs, off = [], 0
    for k in sizes:
        jobs.append((pool.data_ptr() + off * f.limbs * 4, k, args.direction, None, None))
        off += 1 << k
    b = Batch(f, jobs, graph=True)
    stream = torch.cuda.current_stream()
    try:
        for _ in range(args.warmup):
            b.launch(stream)
        torch.cuda.synchronize()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        for _ in range(args.reps):
            b.launch(stream)
        e.record()
        torch.cuda.synchronize()
        b.status()
    finally:
        b.close()
    ms = s.elapsed_time(e) / max(args.reps, 1)
    print(f"{args.field} batch of {args.batch} (2^{args.batch_lo}..2^{args.batch_hi}, {total} elements): "
          f"{ms:.4f} ms per launch, {total / ms / 1e3:.1f} Melem/s")


if __name__ == "__main__":
    main()
