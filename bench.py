#!/usr/bin/env python
"""Benchmark of the GB300 ADER-DG time step.

Metric: DOF-updates per second, one DOF-update being one coefficient
uh(v,i,j,cell) advanced by one ADER-DG time step (nVar (N+1)^2 per cell), plus
the p50/p99 time-to-solution of served requests.

Default workload ("mix"): the seeded request mix -- each request draws its
system uniformly from {advection-diffusion, Euler vortex, Euler 2D Riemann
problem, Baer-Nunziato cylinder}, N uniformly from {2,3,4,5}, a square grid
side log-uniformly from [32, 512] and initial-field parameters jittered by
+-10% (workloads.request_mix, seed 0).  One bench "step" is one time step of
every request.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                    [--workload mix|euler_vortex|euler_rp2d|bn_cylinder|ad_sine]

Ours (FP32-mixed: the precision split of include/aderdg_gpu.h's
ADERDG_FP32_MIXED):
  value        batched throughput of the first --requests requests, all
               resident in HBM in their (system, N) batches, the batches
               stepping concurrently on their own streams; K steps timed on the
               device (the state, tens of GB, is far larger than L2);
  error_vs_fp64  every one of those requests against its own run on the plain
               FP64 path after the same W + K steps: relative L1 / L-infinity
               of uh and the limited-cell counts;
  fp32_wide    the same for the ADERDG_FP32_WIDE split, labelled separately;
  plain_fp64   the plain single-instance FP64 GPU path on the same requests
               (one simulation at a time, CUDA events per step, L2 flushed);
  e2e          the served run through the public API, --serve-requests (1024)
               requests of K steps submitted at once: admission with the
               initial field evaluated on the device (the request's parameters
               copied host->device), the batched steps, each result copied
               device->host when its request ends; e2e.rates / latency_s: the
               same requests arriving as Poisson processes at each --rates
               rate, with throughput and p50/p99 time-to-solution;
  roofline     the predictor (k_predictor) of the batched step against the
               FP32 FMA peak, from its CUDA-event duration measured live and
               the flop model predictor_flops_per_cell;
  cpu_baseline the reference arm's sample on one host core.
The reference arm (--impl reference) times the FP64 CPU restatement of the
reference (oracle/; the Fortran cannot be built on these machines) on all host
cores with one wall clock around the timed steps.  Multi-GPU: requests are
independent, so rank r serves requests r, r + N, ... (weak scaling; no
collective beyond the barrier and the timing reductions).
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
    ap.add_argument("--gpus", type=int, default=1, help="ranks (launch with torchrun for more than one)")
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="mix")
    ap.add_argument("--requests", type=int, default=128, help="resident requests per rank (value)")
    ap.add_argument("--serve-requests", type=int, default=1024, help="served requests in total (e2e, rates)")
    ap.add_argument("--rates", default="10,30,100,300,500", help="Poisson arrival rates swept, requests/s")
    ap.add_argument("--precision", default="fp32", choices=["fp64", "fp32"])
    ap.add_argument("--side", type=int, default=0)
    ap.add_argument("--N", type=int, default=0, help="single workload: degree (default: the workload's)")
    ap.add_argument("--hbm-budget-gb", type=float, default=160.0)
    ap.add_argument("--sync-every", type=int, default=4, help="served runs: steps per host round of a group")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--no-wide", action="store_true", help="skip the FP32-wide comparison run")
    ap.add_argument("--host-setup", action="store_true", help="serve with host-projected initial fields")
    ap.add_argument("--to-tend", action="store_true",
                    help="single workload: also run it from t=0 to its end time (time-to-solution, exact-solution error)")
    ap.add_argument("--study", default="",
                    help="single workload with an exact solution: grid sides (e.g. 32,64,128,256) each run from t=0 to "
                         "its end time; error against the exact solution and the observed order per refinement")
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


def subcell_flops_per_cell(system, N, dmp=True):
    """Floating-point operations of the subcell re-solve (k_subcell, FP64 in the
    FP32-mixed mode) per re-solved cell: what the new subcell data, the new
    polynomial, its DMP verdict (dmp: a recompute = 2 cell; a recompute = 1
    cell has none, Euler/limiter.f90:599-620) and its CFL denominators need.
    A fused multiply-add counts 2, a division or square root 1, as in
    predictor_flops_per_cell.

    Both systems equal the instrumented count of tests/test_subcell_flop_model.py.
    Euler
    -- the neighbourhood's subcell data the interior slopes read (the y pass
    of 3S + 2 neighbour rows, the x pass of the S^2 + 4S subcells), MUSCL-
    Hancock on the S^2 interior subcells (the halo subcells have zero slopes:
    their half-step flux differences vanish and their face states are their
    values), the Rusanov flux of every subgrid edge along its normal, the
    finite-volume update, put_subcell_data, the DMP (subcell and Gauss-Lobatto
    projections, thresholds, the pressure of every subcell) and the CFL
    denominator of every node.

    Baer-Nunziato: likewise equal to the instrumented count -- the neighbour
    subcells the slopes of the (S+2)^2 - 4 evolved subcells read (two rings:
    3S + 8 rows in the y pass, (S+2)^2 + 4S subcells in the x pass),
    MUSCL-Hancock with the NCP source on those subcells, per edge the Rusanov
    flux and the path-conservative fluctuation (3-point path integral), the
    finite-volume update with the fluctuations and the NCP source at the half
    step, put_subcell_data, the DMP (with the admissibility of every subcell)
    and the CFL denominators."""
    P, S, V = N + 1, 2 * N + 1, NVAR[system]
    H, NE = S + 2, (S + 1) * S
    dot = lambda n: 2 * n - 1  # noqa: E731
    if system != 2:
        flux, eig = 14, 4                      # flux along one axis with one reciprocal; |u_n| + c
        setup = 5                              # dx/S, dy/S, dt/(dx/S), dt/(dy/S), dt/2
        gather = (3 * S + 2) * V * P * dot(P) + (S * S + 4 * S) * V * dot(P)
        muscl = S * S * (20 * V + 4 * flux)    # slopes 4V, face states 6V, Qt 5V, half step 5V
        edges = 2 * NE * (2 * (flux + eig) + 1 + 5 * V)
        fv = S * S * 6 * V
        put = V * (P * S + P * P) * dot(S)
        dmp_work = (V * ((P * S + P * P) + (S * S + P * P)) * dot(P) + 7 * S * S + 4 * V) if dmp else 0
        cfl = P * P * 19
        return setup + gather + muscl + edges + fv + put + dmp_work + cfl
    # Baer-Nunziato: flux along one axis from one reciprocal of Q0 Q4 (35), the
    # sound speeds and maxval(abs(Lambda)) (12), the NCP source from p_g and u_n
    # (22: only the volume-fraction gradient enters), the Roe fluctuation (111:
    # PDEMatrixB has one non-zero column, so three path points of p_g, u_n
    # and p_g u_n times the jump of alpha)
    flux, eig, ncp, roe = 35, 12, 22, 111
    setup = 7                                  # dx/S, dy/S, dt/(dx/S), dt/(dy/S), dt/2 and their halves
    gather = (3 * S + 8) * V * P * dot(P) + (H * H + 4 * S) * V * dot(P)
    # the (S+2)^2 - 4 evolved subcells (the corners feed no edge): slopes 4V,
    # alpha gradient 2, source, face states 6V, 4 fluxes, Qt 5V + 1 (the
    # structural zeros of the source and of the ninth flux component), half step 5V
    muscl = (H * H - 4) * (4 * V + 2 + ncp + 6 * V + 4 * flux + 5 * V + 1 + 5 * V)
    # per edge: the jump, two fluxes and speeds, the Rusanov flux, the fluctuation
    edges = 2 * NE * (V + 2 * (flux + eig) + 4 * (V - 1) + 2 + roe)
    # per subcell: the half-step state, its source, flux differences 6V, the
    # five non-zero fluctuation components per direction, the seven of the source
    fv = S * S * (2 * V + ncp + 6 * V + 2 * 15 + 14)
    put = V * (P * S + P * P) * dot(S)
    dmp_work = (V * ((P * S + P * P) + (S * S + P * P)) * dot(P) + 4 * V + 27 * S * S) if dmp else 0
    cfl = P * P * 44
    return setup + gather + muscl + edges + fv + put + dmp_work + cfl


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


def mix_specs(n, rank=0, ws=1):
    """Rank `rank`'s shard of the first n * ws requests of the seeded mix
    (requests r, r + ws, ...): the ranks serve disjoint requests."""
    import aderdg
    total = n * ws
    return aderdg.workloads.request_mix(max(total, 1024), seed=0)[:total][rank::ws]


def spec_config(aderdg, spec, precision):
    cfg, ic, _, _ = aderdg.workloads.make(spec["name"], side=spec["side"], N=spec["N"], precision=precision)
    return cfg, ic


# ---------------------------------------------------------------- CPU arms
CPU_SIDE_CAP = 32  # grid side cap of the CPU samples (the cost per DOF does not depend on the cell count)


def _cpu_oracle(spec, side_cap):
    """An oracle on the projected initial field (and initial limiter) of one
    request with its grid side capped; returns (oracle, DOFs per step)."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import aderdg
    import pyoracle as po
    cfg, ic, _, _ = aderdg.workloads.make(spec["name"], side=min(spec["side"], side_cap), N=spec["N"])
    oc = po.make_config(cfg.system, cfg.N, cfg.imax, cfg.jmax, xl=cfg.xl, xr=cfg.xr, bc=cfg.bc, cfl=cfg.cfl,
                        gamma=cfg.gamma, gamma_s=cfg.gamma_s, gamma_g=cfg.gamma_g, pi_s=cfg.pi_s, pi_g=cfg.pi_g,
                        cx=cfg.cx, cy=cfg.cy, a=cfg.a, ad_flux_mode=cfg.ad_flux_mode, limiter=cfg.limiter)
    o = po.Oracle(oc)
    uh, lh = o.project_ic(ic, spec["params"])
    o.set(po.UH, uh)
    if cfg.limiter and cfg.system != 0:
        o.init_limiter(lh)
    return o, cfg.dofs


def _cpu_worker(job):
    """One host core of a CPU arm: set up its requests' oracles and take the
    warm-up steps (untimed), wait for the other cores, then take `steps` steps
    of each request; returns (start, end, DOF-updates) of the timed part.
    perf_counter is CLOCK_MONOTONIC, comparable across processes."""
    specs, side_cap, warmup, steps, barrier = job
    sims = [_cpu_oracle(s, side_cap) + (s["tend"],) for s in specs]
    t = [0.0] * len(sims)
    for k, (o, _, tend) in enumerate(sims):
        for _ in range(warmup):
            t[k], _, _ = o.step(t[k], tend)
    if barrier is not None:
        barrier.wait()
    t0 = time.perf_counter()
    dofs = 0
    for _ in range(steps):
        for k, (o, d, tend) in enumerate(sims):
            t[k], _, _ = o.step(t[k], tend)
            dofs += d
    t1 = time.perf_counter()
    if barrier is not None:
        barrier.wait()
    return t0, t1, dofs


CPU_SET = 8       # requests every core steps (the first of the mix)


def cpu_arm(specs, cores, side_cap, warmup, steps):
    """The FP64 CPU restatement of the reference (oracle/) on `cores` host
    cores, every core stepping its own copy of the requests `specs` (the same
    work on every core, so that no core idles while another finishes); one
    wall clock from the first core's start to the last core's end, after every
    core has built its oracles and taken its warm-up steps.  Returns
    (DOF-updates/s, wall seconds, DOF-updates)."""
    import multiprocessing as mp
    shards = [list(specs) for _ in range(cores)]
    if len(shards) == 1:
        t0, t1, dofs = _cpu_worker((shards[0], side_cap, warmup, steps, None))
        return dofs / (t1 - t0), t1 - t0, dofs
    ctx = mp.get_context("spawn")
    with ctx.Manager() as mgr:
        bar = mgr.Barrier(len(shards))
        with ctx.Pool(len(shards)) as pool:
            res = pool.map(_cpu_worker, [(sh, side_cap, warmup, steps, bar) for sh in shards])
    wall = max(r[1] for r in res) - min(r[0] for r in res)
    dofs = sum(r[2] for r in res)
    return dofs / wall, wall, dofs


# ---------------------------------------------------------------- arms
def run_reference(args):
    """The reference's CPU path: the FP64 restatement of the Fortran solvers
    (oracle/; the Fortran cannot be compiled on these machines) on all host
    cores, one request per core from the mix, grid sides capped at 32.  A bench
    step is one time step of every core's request; value = DOF-updates over the
    wall clock of the timed steps."""
    dist, rank, ws, _ = dist_init("gloo")
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    if args.workload == "mix":
        specs = mix_specs(CPU_SET)
        sample = ("on each of %d cores, the first %d requests of the mix (request_mix seed 0) with grid sides capped "
                  "at %d; %d untimed warm-up steps, then %d timed steps of every request; FP64"
                  % (cores, CPU_SET, CPU_SIDE_CAP, args.warmup, args.steps))
        cfg_desc = {"workload": "mix (served/batched request mix): the first %d requests, grid sides capped at %d, "
                                "on every host core" % (CPU_SET, CPU_SIDE_CAP), "requests": CPU_SET * cores}
    else:
        import aderdg
        cfg, ic, params, tend = aderdg.workloads.make(args.workload, side=args.side or None, N=args.N or None)
        specs = [dict(name=args.workload, N=cfg.N, side=cfg.imax, params=params, tend=tend)]
        sample = ("the workload on a %dx%d grid on each of %d cores; %d warm-up + %d timed steps; FP64"
                  % (CPU_SIDE_CAP, CPU_SIDE_CAP, cores, args.warmup, args.steps))
        cfg_desc = {"workload": args.workload, "N": cfg.N, "grid": [CPU_SIDE_CAP, CPU_SIDE_CAP]}
    val, wall, dofs = cpu_arm(specs, cores, CPU_SIDE_CAP, args.warmup, args.steps)
    line = {"impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": wall / max(args.steps, 1) * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic: projected initial fields of the seeded request mix (deterministic)",
            "config": cfg_desc, "dof_updates_per_step": dofs / max(args.steps, 1),
            "cpu_baseline": {"value": val, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def _resident(aderdg, specs, prec, W, K):
    """Every request of `specs` admitted into its (system, N) batch (initial
    field evaluated on the device), W untimed steps, then K steps of all the
    batches concurrently, timed on the device.  Returns (groups, slots,
    seconds, DOF-updates in the timed steps, DOFs per step)."""
    groups, members, need = {}, [], {}
    for spec in specs:
        cfg, ic = spec_config(aderdg, spec, prec)
        key = (cfg.system, cfg.N)
        need[key] = need.get(key, 0) + aderdg.Batch.units(cfg)
        members.append((spec, cfg, ic, key))
    for key, units in need.items():
        lim = 0 if key[0] == aderdg.SYS_ADVDIFF else 1
        groups[key] = aderdg.Batch(key[0], key[1], prec, lim, capacity_units=units + 16,
                                   max_instances=sum(1 for m in members if m[3] == key) + 1)
    slots, total_dofs = [], 0
    for spec, cfg, ic, key in members:
        # W + K steps, one more for the per-launch profile afterwards
        slot = groups[key].admit_ic(cfg, ic, spec["params"], spec["tend"], W + K + 1)
        assert slot is not None
        slots.append((key, slot, cfg))
        total_dofs += cfg.dofs
    for g in groups.values():
        g.launch(W)
    for g in groups.values():
        g.sync()
    steps0 = [groups[key].query(slot)["steps"] for key, slot, _ in slots]
    secs = aderdg.Batch.run_timed(list(groups.values()), K) * 1e-3
    for g in groups.values():
        g.sync()
    updates = sum(cfg.dofs * (groups[key].query(slot)["steps"] - s0) for (key, slot, cfg), s0 in zip(slots, steps0))
    return groups, slots, secs, updates, total_dofs


def _profile_groups(groups):
    """Per-launch device ms of one more (eager) step of every group, summed,
    and each group's re-solved cells in that step: (listed, troubled), the
    troubled ones being its recompute = 1 cells."""
    tot, listed = {}, {}
    for key, g in groups.items():
        for k, v in g.profile().items():
            tot[k] = tot.get(k, 0.0) + v
        c = g.counters()
        listed[key] = (c["n_listed"], c["n_recompute"])
    return tot, listed


def _launches_per_step(groups, prec, aderdg):
    """Kernel launches of one step of every group: control, predictor, faces,
    cells, [settle (FP32-mixed), mark, subcell,] control."""
    n = 0
    for key in groups:
        if key[0] == aderdg.SYS_ADVDIFF:
            n += 5
        else:
            n += 8 if prec == aderdg.FP32_MIXED else 7
    return n


def _err_stats(errs):
    """Summary of the per-request errors against the FP64 path."""
    l1 = np.array([e["rel_l1"] for e in errs])
    li = np.array([e["rel_linf"] for e in errs])
    lim64 = sum(e["limited_fp64"] for e in errs)
    dcount = sum(abs(e["limited"] - e["limited_fp64"]) for e in errs)
    return {"requests": len(errs), "max_l1": float(l1.max()), "p99_l1": float(np.percentile(l1, 99)),
            "median_l1": float(np.median(l1)), "max_linf": float(li.max()),
            "max_count_diff_pct": float(max(100.0 * abs(e["limited"] - e["limited_fp64"]) / max(e["limited_fp64"], 1)
                                            for e in errs)),
            "total_count_diff_pct": 100.0 * dcount / max(lim64, 1),
            "limited_cells_fp64": lim64, "mask_disagreements": sum(e["mask_diff"] for e in errs),
            "what": "per request, after the same steps from the same initial state: relative L1 (sum|u - u64| / "
                    "sum|u64|) and L-infinity (max|u - u64| / max|u64|) of uh against the plain FP64 GPU path; "
                    "limited cells (status != 0) against the FP64 path's"}


def run_plain_fp64(aderdg, specs, W, K, compare):
    """The plain single-instance FP64 path: one simulation at a time, W
    untimed steps, then K steps timed with CUDA events, L2 flushed before each.
    After them, each request's state is compared with its state in every
    batch run of `compare` ({label: (groups, slots)}, the same W + K steps)."""
    dofs, ms = 0, 0.0
    errs = {lab: [] for lab in compare}
    for k, spec in enumerate(specs):
        cfg, ic = spec_config(aderdg, spec, aderdg.FP64)
        s = aderdg.Solver(cfg)
        s.initial_condition(ic, spec["params"])
        t = 0.0
        for _ in range(W):
            t, _, _ = s.step(t, spec["tend"])
        t, st = s.time_steps(t, spec["tend"], K, flush_l2=True)
        dofs += cfg.dofs * K
        ms += float(st.sum())
        u64, s64 = s.download()
        s.close()
        n64 = int((s64 != 0).sum())
        for lab, (groups, slots) in compare.items():
            key, slot, _ = slots[k]
            u = groups[key].download(slot)
            stt = groups[key].download_status(slot)
            den1, deni = float(np.abs(u64).sum()), float(np.abs(u64).max())
            errs[lab].append({"rel_l1": float(np.abs(u - u64).sum()) / (den1 if den1 > 0 else 1.0),
                              "rel_linf": float(np.abs(u - u64).max()) / (deni if deni > 0 else 1.0),
                              "limited": int((stt != 0).sum()), "limited_fp64": n64,
                              "mask_diff": int(((stt != 0) != (s64 != 0)).sum())})
    return dofs / (ms * 1e-3), ms, errs





def run_served(aderdg, args, specs, prec, rate):
    """Continuous batching of `specs`: Poisson arrivals at `rate` requests/s
    (inf: all at once), initial fields evaluated on the device at admission
    (the request's parameters cross to the device), each result downloaded to
    the host when its request ends."""
    srv = aderdg.serving.Server(hbm_budget_bytes=args.hbm_budget_gb * 1e9, precision=prec, sync_every=args.sync_every,
                                device_setup=not args.host_setup, download_results=True)
    rep = srv.run(specs, rate=rate, seed=0, max_steps=args.steps)
    rep.pop("requests_done")
    srv.close()
    return rep


def run_single(args, aderdg, dist, rank, ws, lr):
    """A plain named workload on one simulation (not the headline)."""
    prec = aderdg.FP32_MIXED if args.precision == "fp32" else aderdg.FP64
    cfg, ic, params, tend = aderdg.workloads.make(args.workload, side=args.side or None, N=args.N or None,
                                                  precision=prec)
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
            "phase_ms": phases,
            "gpu_launches": ((8 if prec == aderdg.FP32_MIXED else 7)
                             if cfg.limiter and cfg.system != aderdg.SYS_ADVDIFF else 5) * args.steps,
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


def run_study(args, aderdg):
    """Convergence study of a workload with an exact solution (the isentropic
    vortex's configuration: N = 4, limiter on, grids 32 to 256, t = 10): each
    grid from its initial field to the end time through the device-resident
    loop; L1 / L2 / L-infinity error of the density (u for advection-diffusion)
    cell averages against the exact solution, as Euler/analyze_soln.f90:10-56
    measures it, and the order log2(e(h) / e(h/2)) between successive grids."""
    prec = aderdg.FP32_MIXED if args.precision == "fp32" else aderdg.FP64
    sides = [int(x) for x in args.study.split(",") if x]
    rows = []
    for side in sides:
        cfg, ic, params, tend = aderdg.workloads.make(args.workload, side=side, N=args.N or None, precision=prec)
        if ic not in (aderdg.IC_EULER_VORTEX, aderdg.IC_AD_SINE):
            raise SystemExit("--study needs a workload with an exact solution (euler_vortex, ad_sine)")
        r = run_to_tend(aderdg, cfg, ic, params, tend)
        err = r["error_vs_exact"]
        rows.append(dict(side=side, N=cfg.N, steps=r["steps"], tts_s=r["tts_s"],
                         limited_cells_at_end=r["limited_cells_at_end"], l1=err["l1"], l2=err["l2"], linf=err["linf"]))
    for a, b in zip(rows, rows[1:]):
        b["order_l1"] = float(np.log2(a["l1"] / b["l1"])) if b["l1"] > 0 else None
        b["order_linf"] = float(np.log2(a["linf"] / b["linf"])) if b["linf"] > 0 else None
    return {"study": args.workload, "precision": args.precision, "limiter": int(cfg.limiter), "tend": tend,
            "grids": rows, "what": "error of the final cell averages against the exact solution per grid; order "
                                   "between successive grids"}


def allsum(dist, x):
    if dist is None:
        return x
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def _traffic(units, kernel_key, mode_key):
    """DRAM bytes of one launch of a kernel over the groups, from the
    per-(system, N) captures in profiles/traffic.json (bytes per unit --
    DOF for k_predictor, re-solved cell for k_subcell -- times each group's
    units), and the limiter the captures name; None where a group has no
    capture."""
    try:
        with open(os.path.join(REPO, "profiles", "traffic.json")) as fh:
            tr = json.load(fh)
    except (OSError, ValueError):
        return None, None
    per = tr.get(kernel_key, {}).get(mode_key, {})
    tot, miss = 0.0, 0
    for key, n in units.items():
        b = per.get("%d_%d" % key)
        if b is None:
            miss += 1
        else:
            tot += b * n
    return (tot if miss == 0 else None), tr.get("limiter", {}).get(kernel_key, {}).get(mode_key)


def _tuning_desc(aderdg):
    """The tuner's table the run used (applied when the library loaded)."""
    import hashlib
    path = os.environ.get("ADERDG_TUNING", aderdg.core.TUNING_FILE)
    if not path or not os.path.exists(path):
        return {"table": None, "what": "default kernel shapes"}
    with open(path, "rb") as fh:
        digest = hashlib.sha256(fh.read()).hexdigest()[:16]
    return {"table": os.path.relpath(path, REPO), "sha256_16": digest,
            "what": "kernel shapes of the FP32 modes picked per (system, N, precision) by aderdg/tuner.py"}


def run_mix(args, aderdg, dist, rank, ws, lr):
    """The seeded request mix, resident: `value` (FP32-mixed), the FP32-wide
    split beside it, the plain FP64 path on the same requests, and every
    request's error against its FP64 run."""
    W, K = args.warmup, args.steps
    specs = mix_specs(args.requests, rank, ws)
    if args.precision == "fp64":
        modes = [("fp64", aderdg.FP64)]
    else:
        modes = [("fp32_mixed", aderdg.FP32_MIXED)] + ([] if args.no_wide else [("fp32_wide", aderdg.FP32_WIDE)])
    runs, clk_samples = {}, []
    for lab, prec in modes:
        barrier(dist)
        with ClockSampler(lr) as clk:
            groups, slots, secs, updates, total_dofs = _resident(aderdg, specs, prec, W, K)
        clk_samples += clk.samples
        secs = allmax(dist, secs)
        updates = allsum(dist, updates)
        runs[lab] = dict(prec=prec, groups=groups, slots=slots, secs=secs, updates=updates, dofs=total_dofs)
    barrier(dist)
    compare = {lab: (r["groups"], r["slots"]) for lab, r in runs.items() if r["prec"] != aderdg.FP64}
    plain = None
    if not args.no_plain:
        plain = run_plain_fp64(aderdg, specs, W, K, compare)
    for r in runs.values():
        r["phases"], r["listed"] = _profile_groups(r["groups"])
        r["group_dofs"] = {}
        for key, slot, cfg in r["slots"]:
            r["group_dofs"][key] = r["group_dofs"].get(key, 0) + cfg.dofs
        r["dev_bytes"] = sum(g.info()["device_bytes"] for g in r["groups"].values())
        r["launches"] = _launches_per_step(r["groups"], r["prec"], aderdg)
        for g in r["groups"].values():
            g.close()
        r["groups"] = None
    plain_rate = allsum(dist, plain[0]) if plain else None
    if rank != 0:
        return None
    head_lab = modes[0][0]
    head = runs[head_lab]
    clk = ClockSampler(lr)
    clk.samples = clk_samples
    fp64_peak, fp32_peak = aderdg.probe_peaks()
    mixed = head["prec"] != aderdg.FP64
    peak = fp32_peak if mixed else fp64_peak
    pred_flops = sum(predictor_flops_per_cell(cfg.system, cfg.N, ad_fused=cfg.ad_flux_mode != 0) * cfg.cells
                     for _, _, cfg in head["slots"])
    ph = head["phases"]
    kern_ms = {k: v for k, v in ph.items() if k not in ("begin", "end")}
    pred_ms = ph.get("predictor", 0.0)
    ach = pred_flops / (pred_ms * 1e-3) / 1e9 if pred_ms > 0 else None
    mode_key = "fp32" if mixed else "fp64"
    traffic, limiter = _traffic(head["group_dofs"], "k_predictor_bytes_per_dof", mode_key)
    listed = {k: n[0] for k, n in head["listed"].items() if k[0] != aderdg.SYS_ADVDIFF}
    sub_traffic, sub_limiter = _traffic(listed, "k_subcell_bytes_per_listed_cell", mode_key)
    dominant = max(kern_ms, key=lambda k: kern_ms[k])
    sub_ms = ph.get("subcell", 0.0)
    sub_flops = sum(subcell_flops_per_cell(key[0], key[1], dmp=False) * n1
                    + (subcell_flops_per_cell(key[0], key[1]) - subcell_flops_per_cell(key[0], key[1], dmp=False))
                    * (n1 - n2) for key, (n1, n2) in head["listed"].items())
    sub_ach = sub_flops / (sub_ms * 1e-3) / 1e9 if sub_ms > 0 else None
    roof_sub = {"bound": "fp64", "kernel": "k_subcell (the subcell re-solve, FP64, all groups with the limiter)",
                "achieved": sub_ach, "peak": fp64_peak, "unit": "GFLOP/s",
                "frac": (sub_ach / fp64_peak) if sub_ach else None,
                "peak_source": "FP64 FMA throughput measured on this GPU by aderdg_probe_peaks",
                "flops_per_launch": sub_flops, "listed_cells": int(sum(n[0] for n in head["listed"].values())),
                "troubled_cells": int(sum(n[1] for n in head["listed"].values())),
                "flop_model": "bench.py subcell_flops_per_cell x re-solved cells of the profiled step, "
                              "the DMP projections for its recompute = 2 cells only",
                "launch_ms": sub_ms, "dominant_phase": dominant,
                "phase_share": {k: v / sum(kern_ms.values()) for k, v in kern_ms.items()},
                "phase_ms_one_step": ph, "traffic": sub_traffic,
                "traffic_source": "profiles/traffic.json: DRAM bytes per re-solved cell of k_subcell per (system, N) "
                                  "group from one ncu capture of the batched mix, times each group's re-solved cells",
                "limiter": sub_limiter}
    roof = {"bound": "fp32" if mixed else "fp64", "kernel": "k_predictor (all (system, N) groups of the mix)",
            "achieved": ach, "peak": peak, "unit": "GFLOP/s", "frac": (ach / peak) if ach else None,
            "peak_source": "FMA throughput measured on this GPU by aderdg_probe_peaks (dependent-FMA "
                           "microkernel); MEASURED_PEAKS.json carries no non-tensor FP32/FP64 figure",
            "flops_per_launch": pred_flops, "flop_model": "bench.py predictor_flops_per_cell x cells",
            "launch_ms": pred_ms, "dominant_phase": dominant,
            "phase_share": {k: v / sum(kern_ms.values()) for k, v in kern_ms.items()},
            "phase_ms_one_step": ph, "traffic": traffic,
            "groups": {"%d_%d" % k: {"dofs": head["group_dofs"][k], "listed_cells": head["listed"].get(k, (0, 0))[0],
                                   "troubled_cells": head["listed"].get(k, (0, 0))[1]}
                       for k in head["group_dofs"]},
            "traffic_source": "profiles/traffic.json: DRAM bytes per DOF of k_predictor per (system, N) group from "
                              "one ncu capture of the batched mix, times each group's DOFs",
            "limiter": limiter}
    value = head["updates"] / head["secs"]
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": K, "warmup": W,
            "ms_per_step": head["secs"] / K * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+f64" if mixed else "f64",
            "data": "synthetic: seeded request mix (request_mix seed 0), initial fields evaluated on the device; "
                    "no dataset",
            "config": {"workload": "mix: the first %d of the 1024 seeded requests%s, all resident in HBM in their "
                                   "(system, N) batches, K steps each" % (args.requests * ws,
                                                                         " (sharded over the ranks)" if ws > 1 else ""),
                       "requests": args.requests * ws, "steps_per_request": K, "dofs_per_step": head["dofs"],
                       "dof_updates_timed": head["updates"], "groups": len(head["group_dofs"]),
                       "precision": head_lab, "l2": "state (%.1f GB on device) far larger than L2" %
                       (head["dev_bytes"] / 1e9), "parallelism": "request shards, no collective" if ws > 1 else
                       "single", "serving": "config 5: %d requests, Poisson rates %s req/s (e2e.rates)" %
                       (args.serve_requests, args.rates)},
            "roofline": roof_sub if (dominant == "subcell" and sub_ach) else roof,
            "roofline_predictor" if (dominant == "subcell" and sub_ach) else "roofline_subcell":
                roof if (dominant == "subcell" and sub_ach) else roof_sub,
            "clocks": clk.summary(), "gpu_launches": head["launches"] * K,
            "tuning": _tuning_desc(aderdg)}
    for lab, r in runs.items():
        if lab == head_lab:
            continue
        line[lab] = {"value": r["updates"] / r["secs"], "unit": UNIT, "ms_per_step": r["secs"] / K * 1e3,
                     "phase_ms_one_step": r["phases"],
                     "what": "the same resident mix with the Baer-Nunziato face flux and the subcell re-solve in "
                             "FP32 and uncertified FP32 DMP comparisons (ADERDG_FP32_WIDE)"}
    if plain:
        rate, ms, errs = plain
        line["plain_fp64"] = {"value": plain_rate, "unit": UNIT, "steps_per_request": K,
                              "what": "single-instance FP64 path, one request at a time, same requests, L2 flushed"}
        line["batched_over_plain_fp64"] = value / plain_rate
        for lab, e in errs.items():
            tgt = line if lab == head_lab else line[lab]
            tgt["error_vs_fp64"] = _err_stats(e)
            if lab != head_lab:
                tgt["over_plain_fp64"] = tgt["value"] / plain_rate
    return line


def run_ours(args):
    dist, rank, ws, lr = dist_init()
    if args.gpus != ws:
        print("bench.py --gpus %d: launch it with torchrun --nproc-per-node %d (WORLD_SIZE is %d)"
              % (args.gpus, args.gpus, ws), file=sys.stderr, flush=True)
        sys.exit(2)
    import aderdg
    aderdg.build()
    if args.study:
        if rank == 0:
            print(json.dumps(run_study(args, aderdg)), flush=True)
        return
    if args.workload != "mix":
        line = run_single(args, aderdg, dist, rank, ws, lr)
        if line:
            print(json.dumps(line), flush=True)
        return
    line = run_mix(args, aderdg, dist, rank, ws, lr)
    prec = aderdg.FP64 if args.precision == "fp64" else aderdg.FP32_MIXED
    serve = mix_specs(args.serve_requests // ws, rank, ws) if args.serve_requests >= ws else []
    served = {}
    if not args.no_serve and serve:
        # e2e: the served requests all submitted at once through the serving
        # API; then Poisson arrivals at each rate of the sweep (each rank takes
        # its share of the arrival stream)
        rates = [float(x) for x in args.rates.split(",") if x]
        for rate in [float("inf")] + rates:
            barrier(dist)
            rep = run_served(aderdg, args, serve, prec, rate / ws)
            makespan = allmax(dist, rep["makespan_s"])
            served[rate] = dict(rep, makespan_s=makespan,
                                dof_updates_per_s=allsum(dist, rep["dof_updates"]) / makespan)
    if rank != 0:
        return
    if served:
        api = ("aderdg_batch_admit_ic / launch / sync / download / release (continuous batching)"
               if not args.host_setup else
               "aderdg_batch_admit / launch / sync / download / release (continuous batching)")
        burst = served[float("inf")]
        line["e2e"] = {"value": burst["dof_updates_per_s"], "unit": UNIT,
                       "h2d_bytes_per_step": burst["h2d_bytes"] / args.steps,
                       "d2h_bytes_per_step": burst["d2h_bytes"] / args.steps, "api": api,
                       "arrivals": "all %d requests at t = 0" % args.serve_requests,
                       "makespan_s": burst["makespan_s"], "tts_p50_s": burst["tts_p50_s"],
                       "tts_p99_s": burst["tts_p99_s"], "requests": burst["requests"], "failed": burst["failed"],
                       "steps_per_request": args.steps,
                       "rates": [{"rate_per_s": r, "dof_updates_per_s": v["dof_updates_per_s"],
                                  "tts_p50_s": v["tts_p50_s"], "tts_p99_s": v["tts_p99_s"],
                                  "makespan_s": v["makespan_s"], "requests": v["requests"], "failed": v["failed"]}
                                 for r, v in served.items() if np.isfinite(r)]}
        mid = [v for r, v in served.items() if np.isfinite(r)]
        line["latency_s"] = {"per_rate": {"%g" % r: {"p50": v["tts_p50_s"], "p99": v["tts_p99_s"]}
                                          for r, v in served.items() if np.isfinite(r)},
                             "what": "time to solution, arrival to result on the host, %d requests of %d steps, "
                                     "Poisson arrivals" % (args.serve_requests, args.steps)}
        if mid:
            line["latency_s"].update(p50=float(np.median([v["tts_p50_s"] for v in mid])),
                                     p99=float(max(v["tts_p99_s"] for v in mid)))
    if not args.no_cpu_baseline:
        rate, wall, dofs = cpu_arm(mix_specs(CPU_SET), 1, CPU_SIDE_CAP, args.warmup, args.steps)
        line["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": 1, "kind": "port",
                                "sample": "the reference arm's per-core sample on one host core: the first %d "
                                          "requests of the mix, grid sides capped at %d, %d warm-up + %d timed steps "
                                          "each (%.1f s); FP64" % (CPU_SET, CPU_SIDE_CAP, args.warmup, args.steps,
                                                                   wall)}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
