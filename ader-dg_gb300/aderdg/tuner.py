"""Autotuner of the FP32 modes' kernel shapes.

For each (system, N, precision) it times the candidates of three knobs on the
GPU and keeps the fastest:
  predictor       the FP32 space-time predictor's shape: cells per CTA
                  (default, twice, half), one more CTA per SM for the register
                  allocation, the middle Picard iterations unrolled,
                  per-node contractions instead of the row/column tiling, or
                  the row/column pass on the tensor cores (mma.sync, 3xTF32)
                  (predictor.cuh PredVariant);
  cells           the cell kernel's CTA size (default, twice, half);
  subcell_per_sm  the subcell re-solve's persistent CTAs per SM (0: as many
                  as fit).
The knobs are tuned one after the other, each with the others at their best
so far.  A candidate's time is its kernel's device time in eager steps with
CUDA events between the launches (aderdg_profile_step), the median over
`reps` rounds that interleave the candidates, on the system's base case at a
grid whose cell count is typical of the request mix.  A candidate replaces
the default only when it is at least MARGIN (2%) faster, so that timing noise
does not pick shapes (a candidate that does not apply to a system and degree,
e.g. the tensor-core pass below N = 3, runs the default and times alike).  The reference has no
counterpart: its shapes are compile-time parameters (Euler/ader_dg.f90:17-20).

    python -m aderdg.tuner [--out FILE] [--precisions fp32_mixed,fp32_wide]
                           [--systems 0,1,2] [--degrees 1,2,3,4,5] [--reps 5]
                           [--workload NAME --side S]

writes the table (default: the package's tuning_gb300.json, which aderdg.load
applies; ADERDG_TUNING names another file).  --workload / --side time the
candidates on another workload of the system (e.g. euler_vortex at 256^2)
instead of its base case.
"""
import argparse
import json
import os

import time

import numpy as np

from . import workloads
from .core import (FP32_MIXED, FP32_WIDE, SYS_ADVDIFF, SYS_BN, SYS_EULER, TUNING_FILE, Solver, load, set_tuning,
                   tuning_variants)

BASE = {SYS_ADVDIFF: "ad_sine", SYS_EULER: "euler_rp2d", SYS_BN: "bn_cylinder"}
SIDE = {1: 320, 2: 256, 3: 192, 4: 160, 5: 128}  # 40k-100k cells, as the larger requests of the mix
PHASE = {"predictor": "predictor", "cells": "cells", "subcell_per_sm": "subcell"}
MARGIN = 0.02


def tune_one(system, N, precision, reps=5, side=None, warm_steps=10, workload=None):
    """Tunes (system, N, precision) and sets the result in the library's
    table; returns {"predictor", "cells", "subcell_per_sm", "ms": {knob: {candidate: ms}}}."""
    n_pred, n_cells = tuning_variants()
    name = workload or BASE[system]
    if workloads.WORKLOADS[name]["system"] != system:
        raise ValueError("workload %s is not of system %d" % (name, system))
    cfg, ic, params, tend = workloads.make(name, side=side or SIDE[N], N=N, precision=precision)
    limiter = cfg.limiter and system != SYS_ADVDIFF
    s = Solver(cfg)
    s.initial_condition(ic, params)
    t, _ = s.run(0.0, tend, warm_steps)
    cur = dict(predictor=0, cells=0, subcell_per_sm=0)
    times = {}
    knobs = [("predictor", list(range(n_pred))), ("cells", list(range(n_cells)))]
    if limiter:
        knobs.append(("subcell_per_sm", [0, 1, 2, 3]))
    for knob, cands in knobs:
        samples = {c: [] for c in cands}
        for _ in range(reps):
            for c in cands:
                set_tuning(system, N, precision, **dict(cur, **{knob: c}))
                t, ph = s.profile_step(t, tend)
                samples[c].append(ph[PHASE[knob]])
        med = {c: float(np.median(v)) for c, v in samples.items()}
        best = min(med, key=lambda c: med[c])
        cur[knob] = best if med[best] < (1.0 - MARGIN) * med[cands[0]] else cands[0]
        times[knob] = med
    s.close()
    set_tuning(system, N, precision, **cur)
    return dict(cur, ms=times, workload=dict(name=name, side=cfg.imax, N=N))


def tune(systems=(SYS_ADVDIFF, SYS_EULER, SYS_BN), degrees=(1, 2, 3, 4, 5), precisions=(FP32_MIXED, FP32_WIDE),
         reps=5, log=None, workload=None, side=None):
    """Tunes every combination; returns the table {"entries": {...}, ...}."""
    entries = {}
    for prec in precisions:
        for system in systems:
            for N in degrees:
                t0 = time.perf_counter()
                r = tune_one(system, N, prec, reps=reps, workload=workload, side=side)
                entries["%d_%d_%d" % (system, N, prec)] = r
                if log:
                    log("system %d N %d precision %d: predictor %d cells %d subcell/SM %d (%.1f s); predictor ms %s"
                        % (system, N, prec, r["predictor"], r["cells"], r["subcell_per_sm"],
                           time.perf_counter() - t0,
                           " ".join("%d:%.4f" % (k, v) for k, v in sorted(r["ms"]["predictor"].items()))))
    return {"version": 1, "entries": entries,
            "what": "kernel shapes of the FP32 modes per '<system>_<N>_<precision>', picked by aderdg/tuner.py "
                    "from per-kernel device times (ms: median per candidate)"}


def main(argv=None):
    ap = argparse.ArgumentParser(prog="python -m aderdg.tuner")
    ap.add_argument("--out", default=TUNING_FILE)
    ap.add_argument("--precisions", default="fp32_mixed,fp32_wide")
    ap.add_argument("--systems", default="0,1,2")
    ap.add_argument("--degrees", default="1,2,3,4,5")
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--workload", default=None, help="time on this workload instead of the base case")
    ap.add_argument("--side", type=int, default=None)
    args = ap.parse_args(argv)
    os.environ["ADERDG_TUNING"] = ""  # start from the defaults, not from an earlier table
    load()
    names = {"fp32_mixed": FP32_MIXED, "fp32_wide": FP32_WIDE}
    table = tune(systems=[int(x) for x in args.systems.split(",")], degrees=[int(x) for x in args.degrees.split(",")],
                 precisions=[names[x] for x in args.precisions.split(",")], reps=args.reps,
                 log=lambda m: print(m, flush=True), workload=args.workload, side=args.side)
    with open(args.out, "w") as fh:
        json.dump(table, fh, indent=1, sort_keys=True)
    print("wrote", args.out)


if __name__ == "__main__":
    main()
