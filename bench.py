#!/usr/bin/env python
"""Benchmark of the GB300 ADER-DG time step.

Metric: DOF-updates per second, one DOF-update being one coefficient
uh(v,i,j,cell) advanced by one ADER-DG time step (nVar (N+1)^2 per cell), plus
the p50/p99 time-to-solution of served requests.

Default workload ("mix"): the seeded request mix -- each request draws its
system uniformly from {advection-diffusion, Euler vortex, Euler 2D Riemann
problem, Baer-Nunziato cylinder}, N uniformly from {2,3,4,5}, a square grid
side log-uniformly from [32, 512] and initial-field parameters jittered by
+-10% (workloads.request_mix, seed 0); the first --requests of the 1024
requests, each advanced --steps steps (fixed K).  One bench "step" is one time
step of every request.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                    [--workload mix|euler_vortex|euler_rp2d|bn_cylinder|ad_sine]

Ours:
  value       batched FP32-mixed throughput, all requests resident in HBM in
              their (system, N) batches, the batches stepping concurrently on
              their own streams (wall clock between fully synchronised points;
              the state, ~tens of GB, is far larger than L2);
  plain_fp64  the plain single-instance FP64 GPU path on the same requests
              (one simulation at a time, CUDA events per step, L2 flushed);
  e2e         the served run through the public API with every request
              submitted at once: admission with the initial field evaluated on
              the device (the request's parameters copied host->device), the
              batched steps, each result copied device->host when its request
              ends; a second served run with Poisson arrivals at --rate req/s
              gives the p50/p99 time-to-solution (latency_s);
  roofline    the dominant kernel of the batched step (k_predictor) against
              the FP32 (mixed mode) or FP64 FMA peak, from its CUDA-event
              durations measured live and the flop model
              predictor_flops_per_cell; in the mixed mode it is bound by the
              shared-memory wavefronts of its contractions, not by the pipe;
  cpu_baseline the FP64 CPU restatement of the reference (oracle/), one thread,
              on a bounded sample of the same requests.
The reference arm times the same restatement on the host (the Fortran
reference cannot be built on these machines).  Multi-GPU: requests are
independent, so N GPUs serve N replicas of the mix (weak scaling).
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
NVAR = {0: 1, 1: 4, 2: 9}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="mix")
    ap.add_argument("--requests", type=int, default=128)
    ap.add_argument("--rate", type=float, default=100.0)
    ap.add_argument("--precision", default="fp32", choices=["fp64", "fp32"])
    ap.add_argument("--side", type=int, default=0)
    ap.add_argument("--hbm-budget-gb", type=float, default=160.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--host-setup", action="store_true", help="serve with host-projected initial fields")
    ap.add_argument("--to-tend", action="store_true",
                    help="single workload: also run it from t=0 to its end time (time-to-solution, exact-solution error)")
    return ap.parse_args()


# ---------------------------------------------------------------- work models
def predictor_flops_per_cell(system, N, ad_fused=True):
    """Floating-point operations of the predictor per cell from the loop
    structure of predictor.cuh: per node the operator rows (setup), the first
    Picard iteration once (state constant in time), N-1 middle iterations, the
    last one contracted to the time average and the volume integral; per cell
    the face extrapolation.  A fused multiply-add is 2, a division 1; an
    accumulation of n terms from zero is 2n - 1; Baer-Nunziato's structurally
    zero components (ninth flux component, two NCP components) cost nothing.
    Equal to the instrumented count of tests/test_flop_model.py.  ad_fused: the
    advection-diffusion flux includes the convective part."""
    P, V = N + 1, NVAR[system]
    P2 = P * P
    mids = max(N - 1, 0)
    dot = lambda n: 2 * n - 1  # noqa: E731  (n-term accumulation)
    if system == 0:
        flux = 2 * dot(P) + 2 + (4 if ad_fused else 0)  # gradient, -a grad, + c q
        contract = dot(2 * P)
        setup = 4 * P + 6             # Dx, Dy, Gx, Gy rows and scales, volume scales
        it1 = flux + contract + 3 * P  # q(l) = g u - ts b
        mid = P * (flux + 1 + contract + 2 * P)
        last = P * flux + 6 * dot(P) + contract + 2  # Fh, Gh, H; H contracted once
        vol = 2 * dot(P) + 3
        faces = 4 * P * 3 * dot(P)    # qbnd and the two gradQbnd components
    elif system == 1:
        cflux = 18                    # EulerSys::pflux
        contract = V * dot(2 * P)
        setup = 2 * P + 6
        it1 = cflux + contract + 3 * P * V
        mid = P * (cflux + contract + V + 2 * P * V)
        # last: Fh and H = sum_l tw_l F_l accumulated, H contracted once, qh = wg u - D H
        last = P * cflux + 4 * V * dot(P) + contract + 2 * V
        vol = V * (2 * dot(P) + 3)
        faces = 4 * P * V * 2 * dot(P)
    else:
        cflux = 42                    # BNSys::pflux
        VF, VN = 8, 7                 # non-zero flux / NCP components
        contract = VF * dot(2 * P)
        ncp = 2 * dot(P) + 9 + 2 * (VN - 1) + 1  # grad alpha, NCP, b += dt NCP
        setup = 4 * P + 6
        it1 = cflux + contract + ncp + 3 * P * V
        mid = P * (cflux + contract + ncp + V + 2 * P * V)
        # last: Fh and H, H contracted once, then per level the NCP term (grad alpha, NCP,
        # tw_l dt, qh -= tw_l dt NCP_l) and Sh
        last = (P * cflux + 4 * VF * dot(P) + contract + V + VF +
                P * (2 * dot(P) + 9 + 1 + 2 * VN) + VN * dot(P))
        vol = (VF - 2) * (2 * dot(P) + 5) + 2 * (2 * dot(P) + 3) + 1
        faces = 4 * P * (V + VF) * dot(P)
    return P2 * (setup + it1 + mids * mid + last + vol) + faces


# ---------------------------------------------------------------- clocks
class ClockSampler:
    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown," \
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown," \
             "clocks_event_reasons.sw_power_cap"

    def __init__(self, index=0):
        self.samples, self.proc, self.index = [], None, index

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
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

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [v for v in (num(s[1]) for s in self.samples) if v is not None]
        mx = [v for v in (num(s[2]) for s in self.samples) if v is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for s in self.samples for k, n in enumerate(names)
                          if len(s) > 5 + k and s[5 + k].lower().startswith("active")})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


# ---------------------------------------------------------------- helpers
def dist_init(backend="nccl"):
    """Replicas: one process per GPU (torchrun), no data exchange; the
    process group only carries the barrier and the max over ranks of the
    timings."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        lr = int(os.environ.get("LOCAL_RANK", "0"))
        if backend == "nccl":
            torch.cuda.set_device(lr)
        dist.init_process_group(backend)
        return dist, int(os.environ["RANK"]), ws, lr
    return None, 0, 1, 0


def barrier(dist):
    if dist is not None:
        dist.barrier()


def allmax(dist, x):
    if dist is None:
        return x
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def mix_specs(n):
    import aderdg
    return aderdg.workloads.request_mix(1024, seed=0)[:n]


def spec_config(aderdg, spec, precision):
    cfg, ic, _, _ = aderdg.workloads.make(spec["name"], side=spec["side"], N=spec["N"], precision=precision)
    return cfg, ic


def oracle_rate(specs, budget_s=20.0, side_cap=48, steps=1):
    """DOF-updates/s of the FP64 oracle, one thread, over `specs` with grid
    sides capped at side_cap (same N, system and cell count per side; the
    cost per DOF does not depend on the number of cells), bounded by budget_s."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import aderdg
    import pyoracle as po
    dofs, el, used = 0, 0.0, 0
    for spec in specs:
        if el > budget_s:
            break
        cfg, ic, _, _ = aderdg.workloads.make(spec["name"], side=min(spec["side"], side_cap), N=spec["N"])
        oc = po.make_config(cfg.system, cfg.N, cfg.imax, cfg.jmax, xl=cfg.xl, xr=cfg.xr, bc=cfg.bc, cfl=cfg.cfl,
                            gamma=cfg.gamma, gamma_s=cfg.gamma_s, gamma_g=cfg.gamma_g, pi_s=cfg.pi_s,
                            pi_g=cfg.pi_g, cx=cfg.cx, cy=cfg.cy, a=cfg.a, ad_flux_mode=cfg.ad_flux_mode,
                            limiter=cfg.limiter)
        o = po.Oracle(oc)
        uh, lh = o.project_ic(ic, spec["params"])
        o.set(po.UH, uh)
        if cfg.limiter and cfg.system != 0:
            o.init_limiter(lh)
        t = 0.0
        t0 = time.perf_counter()
        for _ in range(steps):
            t, _, _ = o.step(t, spec["tend"])
        el += time.perf_counter() - t0
        dofs += cfg.dofs * steps
        used += 1
    return dofs / el, used, el


# ---------------------------------------------------------------- arms
def _oracle_worker(job):
    """One process of the reference arm: oracle steps of one request."""
    spec, side_cap, steps = job
    rate, _, el = oracle_rate([spec], budget_s=1e9, side_cap=side_cap, steps=steps)
    return rate


def run_reference(args):
    """The FP64 CPU restatement on all host cores: one process per core, each
    stepping one request of the mix (requests are independent)."""
    import multiprocessing as mp
    dist, rank, ws, _ = dist_init()
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    with ctx.Pool(cores) as pool:
        if args.workload == "mix":
            specs = mix_specs(args.requests)
            jobs = lambda k: [(specs[(cores * k + q) % len(specs)], 40, 2) for q in range(cores)]  # noqa: E731
            sample = ("per step: two oracle steps of each of %d requests of the mix at once (one per core, rotating "
                      "through the first %d), grid sides capped at 40; FP64" % (cores, args.requests))
            cfg_desc = {"workload": "mix", "requests": args.requests, "steps_per_request": args.steps}
        else:
            import aderdg
            cfg, ic, params, tend = aderdg.workloads.make(args.workload, side=args.side or None)
            spec = dict(name=args.workload, N=cfg.N, side=cfg.imax, params=params, tend=tend)
            jobs = lambda k: [(spec, 64, 2)] * cores  # noqa: E731
            sample = "per step: two oracle steps of a 64x64 grid of the workload on each of %d cores; FP64" % cores
            cfg_desc = {"workload": args.workload, "N": cfg.N, "grid": [cfg.imax, cfg.jmax]}
        for k in range(args.warmup):
            pool.map(_oracle_worker, [(j[0], 16, 1) for j in jobs(k)])
        rates = []
        t0 = time.perf_counter()
        for k in range(args.steps):
            # cores step their requests at once: the aggregate rate is the sum of theirs
            rates.append(sum(pool.map(_oracle_worker, jobs(k))))
        el = time.perf_counter() - t0
    val = float(np.mean(rates))
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": el / max(args.steps, 1) * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic: projected initial fields of the seeded request mix (deterministic)",
            "config": cfg_desc,
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_mix(args, aderdg, dist, rank, ws, lr):
    prec = aderdg.FP32_MIXED if args.precision == "fp32" else aderdg.FP64
    specs = mix_specs(args.requests)
    K, W = args.steps, args.warmup
    # ---- batched, resident: every request admitted into its (system, N) batch
    groups, members = {}, []
    need = {}
    for spec in specs:
        cfg, ic = spec_config(aderdg, spec, prec)
        key = (cfg.system, cfg.N)
        need[key] = need.get(key, 0) + aderdg.Batch.units(cfg)
        members.append((spec, cfg, ic, key))
    for key, units in need.items():
        lim = 0 if key[0] == aderdg.SYS_ADVDIFF else 1
        groups[key] = aderdg.Batch(key[0], key[1], prec, lim, capacity_units=units + 16,
                                   max_instances=sum(1 for m in members if m[3] == key) + 1)
    total_dofs = 0
    bytes_in = 0
    slots = []
    for spec, cfg, ic, key in members:
        uh, lh = aderdg.project_initial_condition(cfg, ic, spec["params"])
        lim = cfg.limiter and cfg.system != aderdg.SYS_ADVDIFF
        slot = groups[key].admit(cfg, uh, lh if lim else None, spec["tend"], W + K + 1)
        assert slot is not None
        slots.append((key, slot, cfg.dofs))
        total_dofs += cfg.dofs
        bytes_in += uh.nbytes + (lh.nbytes if lim else 0)
    for g in groups.values():
        g.launch(W)
    for g in groups.values():
        g.sync()
    steps0 = [groups[key].query(slot)["steps"] for key, slot, _ in slots]
    barrier(dist)
    with ClockSampler(lr) as clk:
        # CUDA events on a timing stream that every group's stream waits for
        # and that waits for all of them (the groups run concurrently)
        batched_s = aderdg.Batch.run_timed(list(groups.values()), K) * 1e-3
    for g in groups.values():
        g.sync()
    batched_s = allmax(dist, batched_s)
    barrier(dist)
    # DOF-updates actually done in the timed region (a request that reaches its end time stops early)
    updates = sum(d * (groups[key].query(slot)["steps"] - s0) for (key, slot, d), s0 in zip(slots, steps0))
    value = updates * ws / batched_s
    # dominant kernel: per-launch device times of one more (eager) step of every group
    phase_tot = {}
    pred_flops = 0.0
    for key, g in groups.items():
        ph = g.profile()
        for k, v in ph.items():
            phase_tot[k] = phase_tot.get(k, 0.0) + v
    for spec, cfg, ic, key in members:
        pred_flops += predictor_flops_per_cell(cfg.system, cfg.N, ad_fused=cfg.ad_flux_mode != 0) * cfg.cells
    dev_bytes = sum(g.info()["device_bytes"] for g in groups.values())
    for g in groups.values():
        g.close()
    if rank != 0:
        return None
    fp64_peak, fp32_peak = aderdg.probe_peaks()
    mixed = prec == aderdg.FP32_MIXED
    peak = fp32_peak if mixed else fp64_peak
    pred_ms = phase_tot.get("predictor", 0.0)
    kern_ms = {k: v for k, v in phase_tot.items() if k not in ("begin", "end")}
    dominant = max(kern_ms, key=lambda k: kern_ms[k])
    ach = pred_flops / (pred_ms * 1e-3) / 1e9 if pred_ms > 0 else None
    roof = {"bound": "fp32" if mixed else "fp64", "kernel": "k_predictor (all (system, N) groups of the mix)",
            "achieved": ach, "peak": peak, "unit": "GFLOP/s", "frac": (ach / peak) if ach else None,
            "peak_source": "FMA throughput measured on this GPU by aderdg_probe_peaks (dependent-FMA "
                           "microkernel); MEASURED_PEAKS.json carries no non-tensor FP32/FP64 figure",
            "flops_per_launch": pred_flops, "flop_model": "bench.py predictor_flops_per_cell x cells",
            "launch_ms": pred_ms, "dominant_phase": dominant,
            "phase_share": {k: v / sum(kern_ms.values()) for k, v in kern_ms.items()},
            "phase_ms_one_step": phase_tot, "traffic": None,
            "limiter": ("FP32: shared-memory wavefronts of the flux contractions (79% of peak, FP32 pipe 46%, in the "
                        "ncu capture of profiles/k_predictor_k_cells_euler_vortex_256_N4.md); FP64: the FP64 pipe"
                        if mixed else "the FP64 pipe (90% busy in profiles/k_predictor_k_cells_euler_vortex_256_N4.md)")}
    try:
        with open(os.path.join(REPO, "profiles", "traffic.json")) as fh:
            tr = json.load(fh)
        per = tr.get("k_predictor_fp32mixed_bytes_per_dof" if mixed else "k_predictor_fp64_bytes_per_dof")
        if per:
            roof["traffic"] = per * total_dofs
            roof["traffic_note"] = ("DRAM bytes per DOF of k_predictor from one ncu capture (profiles/traffic.json), "
                                    "times the DOFs of the mix")
    except (OSError, ValueError):
        pass
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": K, "warmup": W,
            "ms_per_step": batched_s / K * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+f64" if prec == aderdg.FP32_MIXED else "f64",
            "data": "synthetic: seeded request mix (request_mix seed 0), projected initial fields; no dataset",
            "config": {"workload": "mix (served/batched request mix)", "requests": len(specs),
                       "steps_per_request": K, "dofs_per_step": total_dofs,
                       "dof_updates_timed": updates, "groups": len(groups),
                       "precision": args.precision, "l2": "state (%.1f GB on device) far larger than L2" %
                       (dev_bytes / 1e9), "parallelism": "replicas" if ws > 1 else "single",
                       "arrival_rate_per_s": args.rate},
            "roofline": roof, "clocks": clk.summary(),
            "gpu_launches": sum(7 if k[0] != 0 else 5 for k in groups) * K}
    return line


def run_plain_fp64(aderdg, specs, steps):
    """The plain single-instance FP64 path: one simulation at a time, CUDA
    events per step, L2 flushed before every timed step."""
    dofs, ms = 0, 0.0
    for spec in specs:
        cfg, ic = spec_config(aderdg, spec, aderdg.FP64)
        uh, lh = aderdg.project_initial_condition(cfg, ic, spec["params"])
        s = aderdg.Solver(cfg)
        s.upload(uh)
        if cfg.limiter and cfg.system != aderdg.SYS_ADVDIFF:
            s.init_limiter(lh)
        t, _, _ = s.step(0.0, spec["tend"])
        t, st = s.time_steps(t, spec["tend"], steps, flush_l2=True)
        dofs += cfg.dofs * steps
        ms += float(st.sum())
        s.close()
    return dofs / (ms * 1e-3), ms


def run_served(aderdg, args, specs, prec, rate):
    """Continuous batching of the mix: Poisson arrivals at `rate` requests/s
    (inf: all at once), initial fields evaluated on the device at admission
    (the request's parameters cross to the device), each result downloaded to
    the host when its request ends."""
    srv = aderdg.serving.Server(hbm_budget_bytes=args.hbm_budget_gb * 1e9, precision=prec, sync_every=4,
                                device_setup=not args.host_setup, download_results=True)
    rep = srv.run(specs, rate=rate, seed=0, max_steps=args.steps)
    rep.pop("requests_done")
    srv.close()
    return rep, rep["h2d_bytes"], rep["d2h_bytes"]


def run_single(args, aderdg, dist, rank, ws, lr):
    """A plain named workload on one simulation (not the headline)."""
    prec = aderdg.FP32_MIXED if args.precision == "fp32" else aderdg.FP64
    cfg, ic, params, tend = aderdg.workloads.make(args.workload, side=args.side or None, precision=prec)
    uh, lh = aderdg.project_initial_condition(cfg, ic, params)
    s = aderdg.Solver(cfg)
    s.upload(uh)
    if cfg.limiter and cfg.system != aderdg.SYS_ADVDIFF:
        s.init_limiter(lh)
    t = 0.0
    for _ in range(args.warmup):
        t, _, _ = s.step(t, tend)
    barrier(dist)
    with ClockSampler(lr) as clk:
        t, ms = s.time_steps(t, tend, args.steps, flush_l2=True)
    total_ms = allmax(dist, float(ms.sum()))
    t, phases = s.profile_step(t, tend)
    if rank != 0:
        return None
    fp64_peak, fp32_peak = aderdg.probe_peaks()
    fpeak = fp32_peak if prec == aderdg.FP32_MIXED else fp64_peak
    flops = predictor_flops_per_cell(cfg.system, cfg.N, ad_fused=cfg.ad_flux_mode != 0) * cfg.cells
    ach = flops / (phases["predictor"] * 1e-3) / 1e9
    host = np.empty(cfg.dofs, dtype=np.float64)
    s.download_into(host)
    n_e = max(3, min(args.steps, 10))
    t_e = time.perf_counter()
    for _ in range(n_e):
        t, _, _ = s.step_host(host, t, tend)
    e2e_s = time.perf_counter() - t_e
    info = s.info()
    s.close()
    to_tend = run_to_tend(aderdg, cfg, ic, params, tend) if args.to_tend else None
    return {"metric": METRIC, "value": cfg.dofs * args.steps * ws / (total_ms * 1e-3), "unit": UNIT, "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+f64" if prec == aderdg.FP32_MIXED else "f64",
            "data": "synthetic: projected initial field of the workload (deterministic)",
            "config": {"workload": args.workload, "N": cfg.N, "grid": [cfg.imax, cfg.jmax],
                       "precision": args.precision, "l2": "flushed before every timed step"},
            "latency_ms": {"p50": float(np.percentile(ms, 50)), "p99": float(np.percentile(ms, 99))},
            "phase_ms": phases, "gpu_launches": (7 if cfg.limiter else 5) * args.steps,
            "roofline": {"bound": "fp32" if prec == aderdg.FP32_MIXED else "fp64", "kernel": "k_predictor",
                         "achieved": ach, "peak": fpeak, "unit": "GFLOP/s", "frac": ach / fpeak, "traffic": None,
                         "peak_source": "aderdg_probe_peaks on this GPU"},
            "e2e": {"value": cfg.dofs * n_e / e2e_s, "unit": UNIT, "h2d_bytes_per_step": cfg.dofs * 8,
                    "d2h_bytes_per_step": cfg.dofs * 8, "api": "aderdg_step_host"},
            "clocks": clk.summary(), "limited_cells": info["n_limited"], "to_tend": to_tend}


def run_to_tend(aderdg, cfg, ic, params, tend):
    """The whole simulation, t = 0 to its end time, with the device-resident run
    loop (aderdg_run: graph replays, dt on the device, one host synchronisation
    every 64 steps): time-to-solution from the initial field to the final state,
    and for the fields with an exact solution (isentropic vortex, sine wave) the
    error norms of the final cell averages."""
    import torch
    s = aderdg.Solver(cfg)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    s.initial_condition(ic, params)
    t, n = s.run(0.0, tend, 10 ** 8, sync_every=64)
    torch.cuda.synchronize()
    tts = time.perf_counter() - t0
    out = {"tend": tend, "time_reached": t, "steps": n, "tts_s": tts, "dof_updates_per_s": cfg.dofs * n / tts,
           "limited_cells_at_end": s.info()["n_limited"]}
    if ic in (aderdg.IC_EULER_VORTEX, aderdg.IC_AD_SINE):
        e1, e2, ei = s.error_norms(ic, params)
        out["error_vs_exact"] = {"l1": e1, "l2": e2, "linf": ei, "variable": 0}
    s.close()
    return out


def run_ours(args):
    dist, rank, ws, lr = dist_init()
    import aderdg
    aderdg.build()
    if args.workload != "mix":
        line = run_single(args, aderdg, dist, rank, ws, lr)
        if line:
            print(json.dumps(line), flush=True)
        return
    line = run_mix(args, aderdg, dist, rank, ws, lr)
    if rank != 0:
        return
    prec = aderdg.FP32_MIXED if args.precision == "fp32" else aderdg.FP64
    specs = mix_specs(args.requests)
    if not args.no_serve:
        # e2e: every request submitted at once through the serving API (the
        # throughput of `value`, end to end); latency: Poisson arrivals at --rate
        api = ("aderdg_batch_admit_ic / launch / sync / download / release (continuous batching)"
               if not args.host_setup else
               "aderdg_batch_admit / launch / sync / download / release (continuous batching)")
        rep, h2d, d2h = run_served(aderdg, args, specs, prec, float("inf"))
        line["e2e"] = {"value": rep["dof_updates_per_s"], "unit": UNIT, "h2d_bytes_per_step": h2d / args.steps,
                       "d2h_bytes_per_step": d2h / args.steps, "api": api,
                       "arrivals": "all requests at t = 0", "makespan_s": rep["makespan_s"],
                       "tts_p50_s": rep["tts_p50_s"], "tts_p99_s": rep["tts_p99_s"], "requests": rep["requests"]}
        rp, _, _ = run_served(aderdg, args, specs, prec, args.rate)
        line["e2e"]["poisson"] = {"rate_per_s": args.rate, "value": rp["dof_updates_per_s"],
                                  "makespan_s": rp["makespan_s"]}
        line["latency_s"] = {"p50": rp["tts_p50_s"], "p99": rp["tts_p99_s"],
                             "what": "time to solution, arrival to result on the host, Poisson arrivals at %.0f/s"
                                     % args.rate}
    if not args.no_plain:
        plain_steps = min(args.steps, 10)
        rate, ms = run_plain_fp64(aderdg, specs, plain_steps)
        line["plain_fp64"] = {"value": rate, "unit": UNIT, "steps_per_request": plain_steps,
                              "what": "single-instance FP64 path, one request at a time, same requests"}
        line["batched_over_plain_fp64"] = line["value"] / rate
    if not args.no_cpu_baseline:
        rate, used, el = oracle_rate(specs, budget_s=20.0, side_cap=48)
        line["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": 1, "kind": "port",
                                "sample": "one FP64 oracle step of each of the first %d requests of the mix with grid "
                                          "sides capped at 48 (%.1f s), one thread" % (used, el)}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
