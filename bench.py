#!/usr/bin/env python
"""Benchmark of the GB300 ADER-DG time step.

One "step" is one complete ADER-DG time step (calc_time_step, predictor with
volume integral, Riemann problems, surface integral + element update + DMP,
subcell limiter) over the whole grid of the workload.  Default workload: the
Euler isentropic vortex, N=4, 256x256 periodic cells on [0,10]^2, limiter on,
FP64.  The metric is DOF-updates per second, one DOF-update being one
coefficient uh(v,i,j,cell) advanced by one step (nVar (N+1)^2 per cell).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Ours: `value` is device time (CUDA events on the library's stream, L2 flushed
before every timed step) with the state resident in HBM; `e2e` is the same
metric through aderdg_step_host with host buffers (host->device copy of uh,
one step, device->host copy of uh, wall clock); `roofline` is the FP64-pipe
roofline of the dominant kernel (the predictor).  The reference arm times the
FP64 CPU restatement of the reference (oracle/) on this machine's host cores.
Multi-GPU: requests are independent simulations, so N GPUs run N replicas
(weak scaling, no collective).
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "ader-dg_gb300"))

METRIC = "batched DOF-updates/s vs plain FP64 GPU path on 1 GB300; p50/p99 solve latency"
UNIT = "DOF-updates/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="euler_vortex")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp32"])
    ap.add_argument("--side", type=int, default=0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-variants", action="store_true")
    return ap.parse_args()


# ---------------------------------------------------------------- flop model
def predictor_flops_per_cell(system, N):
    """Floating-point operations the predictor kernel executes per cell
    (fused multiply-add = 2, division = 1), from the loop structure of
    predictor.cuh: the first Picard iteration evaluated once (constant in
    time), N-1 full iterations, the last iteration contracted to the time
    average, then the volume integral and the face extrapolation."""
    P = N + 1
    V = {0: 1, 1: 4, 2: 9}[system]
    cflux = {0: 6, 1: 19, 2: 60}[system]            # pointwise flux (+ its gradient for AD)
    extra = {0: 8 * P, 1: 0, 2: 8 * P + 12 + 2 * V}[system]  # AD/BN gradients, BN NCP and its update
    contract = 4 * P * V                              # one time level: 2P FMAs per variable
    it1 = cflux + contract + extra + 3 * P * V
    mid = P * (cflux + contract + extra) + P * V + 2 * P * P * V
    last = P * (cflux + 4 * V + contract + extra) + V + 2 * P * V
    vol = V * (4 * P + 3)
    per_node = it1 + max(N - 1, 0) * mid + last + vol
    faces = 4 * P * V * 2 * 2 * P
    return P * P * per_node + faces


def predictor_bytes_per_cell(system, N, rbytes):
    P = N + 1
    V = {0: 1, 1: 4, 2: 9}[system]
    bnd = 4 * P * V * rbytes * (3 if system == 0 else 2)
    return 8 * V * P * P * 2 + bnd  # read uh, write duh, write face states


# ---------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown," \
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown," \
             "clocks_event_reasons.sw_power_cap"

    def __init__(self, index=0):
        self.samples = []
        self.proc = None
        self.index = index

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if s[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for s in self.samples:
            for k, n in enumerate(names):
                if len(s) > 5 + k and s[5 + k].lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.samples)}


# ---------------------------------------------------------------- helpers
def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        lr = int(os.environ.get("LOCAL_RANK", "0"))
        torch.cuda.set_device(lr)
        dist.init_process_group("nccl")
        return dist, int(os.environ["RANK"]), ws, lr
    return None, 0, 1, 0


def barrier(dist):
    if dist is not None:
        dist.barrier()


def allmax(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def setup_solver(aderdg, name, side, prec):
    cfg, ic, params, tend = aderdg.workloads.make(name, side=side or None, precision=prec)
    uh, lh = aderdg.project_initial_condition(cfg, ic, params)
    s = aderdg.Solver(cfg)
    s.upload(uh)
    if cfg.limiter:
        s.init_limiter(lh)
    return s, cfg, uh, lh, tend


def cpu_oracle_rate(name, side, steps_budget_s=20.0, max_steps=5, threads=1):
    """FP64 CPU restatement of the reference timed on this host: the first
    `max_steps` steps of the workload (bounded to ~steps_budget_s)."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import aderdg
    import pyoracle as po
    cfg, ic, params, tend = aderdg.workloads.make(name, side=side or None)
    oc = po.make_config(cfg.system, cfg.N, cfg.imax, cfg.jmax, xl=cfg.xl, xr=cfg.xr, bc=cfg.bc, cfl=cfg.cfl,
                        gamma=cfg.gamma, gamma_s=cfg.gamma_s, gamma_g=cfg.gamma_g, pi_s=cfg.pi_s, pi_g=cfg.pi_g,
                        cx=cfg.cx, cy=cfg.cy, a=cfg.a, ad_flux_mode=cfg.ad_flux_mode, limiter=cfg.limiter)
    o = po.Oracle(oc)
    uh, lh = o.project_ic(ic, params)
    o.set(po.UH, uh)
    if cfg.limiter:
        o.init_limiter(lh)
    t, done, el = 0.0, 0, 0.0
    while done < max_steps and el < steps_budget_s:
        t0 = time.perf_counter()
        t, _, _ = o.step(t, tend)
        el += time.perf_counter() - t0
        done += 1
    return cfg.dofs * done / el, done, el, cfg


# ---------------------------------------------------------------- arms
def run_reference(args):
    dist, rank, ws, _ = dist_init()
    if rank != 0:
        return
    # each step is one full oracle step of a bounded patch of the workload
    # (same N and cell size; the per-DOF cost does not depend on the grid size)
    import aderdg
    cfg, _, _, _ = aderdg.workloads.make(args.workload, side=args.side or None)
    side = cfg.imax
    per_dof_s = 1.0 / 2.5e6
    budget = 150.0
    while side > 16 and (args.steps + args.warmup) * cfg.nvar * cfg.P ** 2 * side * side * per_dof_s > budget:
        side //= 2
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import pyoracle as po
    c2, ic, params, tend = aderdg.workloads.make(args.workload, side=side)
    scale = side / cfg.imax
    c2.xr = (c2.xl[0] + (cfg.xr[0] - cfg.xl[0]) * scale, c2.xl[1] + (cfg.xr[1] - cfg.xl[1]) * scale)
    oc = po.make_config(c2.system, c2.N, c2.imax, c2.jmax, xl=c2.xl, xr=c2.xr, bc=c2.bc, cfl=c2.cfl,
                        gamma=c2.gamma, gamma_s=c2.gamma_s, gamma_g=c2.gamma_g, pi_s=c2.pi_s, pi_g=c2.pi_g,
                        cx=c2.cx, cy=c2.cy, a=c2.a, ad_flux_mode=c2.ad_flux_mode, limiter=c2.limiter)
    o = po.Oracle(oc)
    uh, lh = o.project_ic(ic, params)
    o.set(po.UH, uh)
    if c2.limiter:
        o.init_limiter(lh)
    t = 0.0
    for _ in range(args.warmup):
        t, _, _ = o.step(t, tend)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        t, _, _ = o.step(t, tend)
    el = time.perf_counter() - t0
    val = c2.dofs * args.steps / el
    sample = "%d steps of a %dx%d patch (cell size of the %dx%d workload), single thread, FP64" % (
        args.steps, side, side, cfg.imax, cfg.jmax)
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": el / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic: projected initial field of the workload (deterministic)",
            "config": workload_config(cfg, args),
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": 1, "kind": "port", "sample": sample},
            "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def workload_config(cfg, args):
    names = {0: "advection-diffusion", 1: "euler", 2: "baer-nunziato"}
    return {"workload": args.workload, "system": names[cfg.system], "N": cfg.N, "grid": [cfg.imax, cfg.jmax],
            "precision": args.precision, "limiter": bool(cfg.limiter), "global_batch": 1,
            "l2": "flushed before every timed step", "parallelism": "replicas" if args.gpus > 1 else "single"}


def run_ours(args):
    dist, rank, ws, lr = dist_init()
    import aderdg
    aderdg.build()
    prec = aderdg.FP32_MIXED if args.precision == "fp32" else aderdg.FP64
    s, cfg, uh, lh, tend = setup_solver(aderdg, args.workload, args.side, prec)
    t = 0.0
    for _ in range(args.warmup):
        t, _, _ = s.step(t, tend)
    barrier(dist)
    with ClockSampler(lr) as clk:
        t, ms = s.time_steps(t, tend, args.steps, flush_l2=True)
    total_ms = allmax(dist, float(ms.sum()))
    barrier(dist)
    dofs_total = cfg.dofs * args.steps * ws
    value = dofs_total / (total_ms * 1e-3)
    # per-phase device times of one step (predictor = the dominant kernel)
    t, phases = s.profile_step(t, tend)
    launches = 7 if cfg.limiter else 5
    if rank != 0:
        return
    info = s.info()
    p50, p99 = float(np.percentile(ms, 50)), float(np.percentile(ms, 99))
    fp64_peak, fp32_peak = aderdg.probe_peaks()
    fpeak = fp32_peak if prec == aderdg.FP32_MIXED else fp64_peak
    flops = predictor_flops_per_cell(cfg.system, cfg.N) * cfg.cells
    pred_ms = phases["predictor"]
    achieved = flops / (pred_ms * 1e-3) / 1e9
    peaks = {}
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as fh:
            peaks = json.load(fh)
    except OSError:
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    rb = 4 if prec == aderdg.FP32_MIXED else 8
    pbytes = predictor_bytes_per_cell(cfg.system, cfg.N, rb) * cfg.cells
    roof = {"bound": "fp32" if prec == aderdg.FP32_MIXED else "fp64", "kernel": "k_predictor",
            "achieved": achieved, "peak": fpeak, "unit": "GFLOP/s", "frac": achieved / fpeak,
            "peak_source": "measured by aderdg_probe_peaks (dependent-FMA microkernel, this GPU); "
                           "MEASURED_PEAKS.json carries no FP64/FP32 non-tensor figure",
            "flops_per_launch": flops, "launch_ms": pred_ms, "traffic": None,
            "hbm": {"algorithmic_bytes": pbytes, "achieved_gbs": pbytes / (pred_ms * 1e-3) / 1e9,
                    "peak_gbs": hbm_peak, "frac": pbytes / (pred_ms * 1e-3) / 1e9 / hbm_peak,
                    "peak_source": "MEASURED_PEAKS.json hbm_gbs"}}
    try:
        with open(os.path.join(REPO, "profiles", "traffic.json")) as fh:
            tr = json.load(fh).get("%s_N%d_%s" % (args.workload, cfg.N, args.precision))
            if tr:
                roof["traffic"] = tr["bytes_per_cell"] * cfg.cells
    except (OSError, ValueError):
        pass
    # e2e: the drop-in step with host buffers (pinned via torch when available)
    host = np.empty(cfg.dofs, dtype=np.float64)
    try:
        import torch
        pinned = torch.empty(cfg.dofs, dtype=torch.float64).pin_memory()
        host = pinned.numpy()
    except Exception:
        pass
    s.download_into(host)
    e2e_steps = max(3, min(args.steps, 10))
    t_e = time.perf_counter()
    for _ in range(e2e_steps):
        t, _, _ = s.step_host(host, t, tend)
    e2e_s = time.perf_counter() - t_e
    e2e = {"value": cfg.dofs * e2e_steps / e2e_s, "unit": UNIT, "h2d_bytes_per_step": cfg.dofs * 8,
           "d2h_bytes_per_step": cfg.dofs * 8, "steps": e2e_steps, "api": "aderdg_step_host"}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64" if prec == aderdg.FP32_MIXED else "f64",
            "data": "synthetic: projected initial field of the workload (deterministic)",
            "config": workload_config(cfg, args),
            "latency_ms": {"p50": p50, "p99": p99, "what": "device time per time step"},
            "phase_ms": phases, "gpu_launches": launches * args.steps,
            "roofline": roof, "e2e": e2e, "clocks": clk.summary(),
            "limited_cells": info["n_limited"], "dt": info["dt"]}
    if cfg.limiter and tend > 0:
        line["time_to_solution_s_extrapolated"] = tend / info["dt"] * total_ms / args.steps * 1e-3
    if not args.no_variants and args.workload == "euler_vortex" and prec == aderdg.FP64:
        s2, c2, _, _, tend2 = setup_solver(aderdg, args.workload, args.side, aderdg.FP32_MIXED)
        t2 = 0.0
        for _ in range(args.warmup):
            t2, _, _ = s2.step(t2, tend2)
        t2, ms2 = s2.time_steps(t2, tend2, args.steps, flush_l2=True)
        line["fp32_mixed"] = {"value": c2.dofs * args.steps / (ms2.sum() * 1e-3), "unit": UNIT,
                              "ms_per_step": float(ms2.mean()), "speedup_vs_fp64": float(ms.sum() / ms2.sum())}
        s2.close()
    if not args.no_cpu_baseline:
        rate, done, el, _ = cpu_oracle_rate(args.workload, args.side, steps_budget_s=20.0, max_steps=3)
        line["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": 1, "kind": "port",
                                "sample": "first %d steps of the full %dx%d workload (%.1f s), FP64 oracle, "
                                          "one thread" % (done, cfg.imax, cfg.jmax, el)}
    print(json.dumps(line), flush=True)
    s.close()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
