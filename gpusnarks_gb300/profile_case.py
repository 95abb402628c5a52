"""Run one transform configuration a few times, for profilers.

    python -m gpusnarks_gb300.profile_case --field p32 --log-n 24 --reps 3

Fills the input on the device (gsn_fill_random), runs `warmup` untimed and
`reps` further transforms through the C ABI, prints the mean event time.  It
is the command the committed ncu summaries under profiles/ were taken with.
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
    args = ap.parse_args()

    import torch

    import gpusnarks_gb300 as g
    from gpusnarks_gb300.batch import fill_random

    f = g.FIELDS[args.field]
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


if __name__ == "__main__":
    main()
