"""Autotune plans on the current GPU and write the tuning table.

    python -m gpusnarks_gb300.tune --out gpusnarks_gb300/tuning/gb300.json

Times the candidate plans of gsn_autotune (single transforms) and
gsn_autotune_batch (inside the persistent batched kernel) for each field over
every supported size for single transforms (p32 2^8..2^28, BLS12-381
2^8..2^26, MNT4-753 2^6..2^24) and up to 2^22 inside the batched kernel, and
saves the fastest per (field, log n, mode).  gpusnarks_gb300 loads the
committed table at start-up.
"""
from __future__ import annotations

import argparse
import os
import time


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", required=True)
    ap.add_argument("--reps", type=int, default=4)
    ap.add_argument("--fields", default="p32,bls12_381_fr,mnt4753_fr")
    ap.add_argument("--modes", default="call,batch")
    args = ap.parse_args()
    os.environ.setdefault("GSN_TUNE_VERBOSE", "1")

    import gpusnarks_gb300 as g

    ranges = {"p32": (8, 28), "bls12_381_fr": (8, 26), "mnt4753_fr": (6, 24)}
    batch_ranges = {"p32": (8, 22), "bls12_381_fr": (8, 22), "mnt4753_fr": (6, 22)}
    g.load()
    g.clear_tuning()
    for mode in args.modes.split(","):
        for name in args.fields.split(","):
            lo, hi = (batch_ranges if mode == "batch" else ranges)[name]
            t0 = time.time()
            g.autotune(name, lo, hi, args.reps, batched=(mode == "batch"))
            print(f"{name} [{mode}]: tuned 2^{lo}..2^{hi} in {time.time() - t0:.1f} s", flush=True)
    g.save_tuning(args.out)
    print("wrote", args.out)


if __name__ == "__main__":
    main()
