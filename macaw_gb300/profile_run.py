"""Runs the lattice (or core, or k-eigenvalue) workload once for profiling (ncu).

  python -m macaw_gb300.profile_run --precision fp64 --hist 1000000 --batches 2
  python -m macaw_gb300.profile_run --workload eigen --hist 200000 --batches 2

One untimed batch (so the first launches of every kernel are warm), then
`--batches` batches of `--hist` histories through one pipelined call, with
fixed execution parameters (the autotuner's choices on this workload unless
overridden).  Prints the pipelined run's statistics as JSON, with the
untimed batch's under "warm".  The eigen workload runs one inactive
generation and then `--batches` active ones of `--hist` particles in one
call, and prints the per-generation records.
"""
from __future__ import annotations

import argparse
import json

from . import Tracker, problems
from ._lib import MC_PREC_FP64, MC_PREC_MIXED


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--precision", choices=["fp64", "mixed"], default="fp64")
    ap.add_argument("--hist", type=int, default=1_000_000)
    ap.add_argument("--batches", type=int, default=2)
    ap.add_argument("--pins", type=int, default=17, help="pin cells per lattice side")
    ap.add_argument("--block", type=int, default=0)
    ap.add_argument("--max-seg", type=int, default=0, help="0: 128 for mixed, 64 for fp64")
    ap.add_argument("--sort", type=int, default=9)
    ap.add_argument("--workload", choices=["lattice", "core", "eigen"], default="lattice")
    args = ap.parse_args()
    prec = MC_PREC_MIXED if args.precision == "mixed" else MC_PREC_FP64
    block = args.block or (64 if prec == MC_PREC_MIXED else 128)
    max_seg = args.max_seg or (128 if prec == MC_PREC_MIXED else 64)
    n = args.hist
    if args.workload == "eigen":
        p = problems.eigen_lattice_problem(nx=args.pins, ny=args.pins)
        with Tracker(0) as t:
            t.load(p)
            g = t.eigen(n, 1 + args.batches, 1, seed=1, precision=prec, bank_size=n, block_size=block,
                        max_seg=max_seg, sort_queue=args.sort, graph=True)
            print(json.dumps([{k: g[k][i].item() for k in g.dtype.names} for i in range(g.size)]))
        return
    p = problems.lattice_problem(nx=args.pins, ny=args.pins) if args.workload == "lattice" \
        else problems.core_problem()
    with Tracker(0) as t:
        t.load(p)
        kw = dict(bank_size=n, block_size=block, max_seg=max_seg, sort_queue=args.sort, precision=prec)
        warm = t.run(n, first=0, seed=1, accumulate=True, **kw).as_dict()
        st = t.run(n * args.batches, first=n, seed=1, accumulate=True, batch_sizes=[n] * args.batches, **kw)
        print(json.dumps(dict(st.as_dict(), warm=warm)))


if __name__ == "__main__":
    main()
