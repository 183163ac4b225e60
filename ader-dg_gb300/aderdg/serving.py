"""Continuous-batching request server for ADER-DG simulations.

Requests (independent simulations: system, N, grid, initial-field parameters,
end time) arrive over time.  Each is admitted, as soon as it has arrived and
its group has room, into the batch of its (system, N) group; a batch steps all
its simulations with one set of launches, each simulation with its own CFL
time step, and groups run concurrently on their own CUDA streams.  Finished
simulations are downloaded and released, freeing room for waiting requests
while the others keep running on the GPU.  Initial fields are evaluated on
the device at admission (device_setup=True, only the request's parameters
cross to the device), or projected on a host thread pool and copied in.

Reported per run: aggregate DOF-updates/s over the makespan and the p50/p99
time-to-solution (arrival to result on the host) of the requests.  A request
whose time step became non-finite (the batch reports ADERDG_ENONFINITE for it;
its neighbours in the batch are unaffected) is released and reported failed:
it counts neither towards the throughput nor the time-to-solution
percentiles.
"""
import collections
import concurrent.futures
import math
import time

import numpy as np

from . import workloads
from .core import FP64, SYS_ADVDIFF, Batch, PinnedArray, project_initial_condition

ENONFINITE = -5  # aderdg_status: the simulation's time step became non-finite


class Request:
    __slots__ = ("rid", "name", "N", "side", "params", "tend", "max_steps", "arrival", "cfg", "ic", "prepared",
                 "admitted", "finished", "steps", "dofs", "group", "slot", "result", "time", "failed", "uh",
                 "lh")

    def __init__(self, rid, spec, arrival, precision, max_steps):
        self.rid = rid
        self.name, self.N, self.side = spec["name"], spec["N"], spec["side"]
        self.params, self.tend = spec["params"], spec["tend"]
        self.max_steps = max_steps
        self.arrival = arrival
        self.cfg, self.ic, _, _ = workloads.make(self.name, side=self.side, N=self.N, precision=precision)
        self.prepared = None
        self.admitted = self.finished = None
        self.steps = 0
        self.dofs = self.cfg.dofs
        self.group = (self.cfg.system, self.N)
        self.slot = None
        self.result = None
        self.time = 0.0
        self.failed = False
        # optional host initial state (admitted as given instead of the initial field)
        self.uh = spec.get("uh")
        self.lh = spec.get("lh")


def poisson_arrivals(n, rate, seed):
    """Arrival times of a Poisson process of `rate` requests/s; an infinite
    (or non-positive) rate is a burst: every request arrives at t = 0."""
    if not np.isfinite(rate) or rate <= 0:
        return np.zeros(n)
    rng = np.random.default_rng(seed + 1000)
    return np.cumsum(rng.exponential(1.0 / rate, size=n))


class Server:
    """Admits requests into per-(system, N) batches under an HBM budget."""

    def __init__(self, hbm_budget_bytes, precision=FP64, max_instances=256, sync_every=4, workers=8,
                 keep_results=False, device_setup=True, download_results=True, share="equal", backfill_window=16,
                 backfill_s=1.0):
        self.budget = int(hbm_budget_bytes)
        # admission: up to backfill_window waiting requests of a group are tried
        # per round (1: strict arrival order), while its oldest waiting request
        # has waited at most backfill_s seconds
        self.backfill_window = max(1, int(backfill_window))
        self.backfill_s = backfill_s
        # how the budget is split over the (system, N) groups: "equal" in
        # equal parts, "demand" in proportion to the device bytes their
        # requests need in total (each group then holds about the same
        # fraction of its requests at once); never less than a group's
        # largest request.  Measured on the 1024-request mix at 160 GB:
        # "demand" serves 2% more DOF-updates/s but the large groups' requests
        # then hold the memory and the median time-to-solution grows 2-3x.
        self.share = share
        self.precision = precision
        self.max_instances = max_instances
        self.sync_every = sync_every
        self.keep_results = keep_results
        self.download_results = download_results or keep_results
        self.device_setup = device_setup
        self.h2d_bytes = 0
        self.d2h_bytes = 0
        self.groups = {}
        self.pool = concurrent.futures.ThreadPoolExecutor(max_workers=workers)

    @staticmethod
    def split_budget(budget, demand, need, unit_bytes, share="equal"):
        """Units of each group's batch: its share of `budget` bytes ("equal":
        budget / groups; "demand": in proportion to demand[g], the bytes its
        requests need in total), in units of unit_bytes[g], and never fewer
        than need[g], its largest request."""
        total = sum(demand.values())
        out = {}
        for g in need:
            frac = 1.0 / len(need) if (share == "equal" or total <= 0) else demand[g] / total
            out[g] = max(int(budget * frac / unit_bytes[g]), need[g])
        return out

    def _group(self, req, units):
        g = self.groups.get(req.group)
        if g is None:
            system, N = req.group
            lim = 0 if system == SYS_ADVDIFF else 1
            g = Batch(system, N, self.precision, lim, capacity_units=units, max_instances=self.max_instances)
            self.groups[req.group] = g
        return g

    @staticmethod
    def _prepare(req):
        if req.uh is not None:
            return req.uh, req.lh
        uh, lh = project_initial_condition(req.cfg, req.ic, req.params)
        return uh, (lh if req.cfg.limiter and req.cfg.system != SYS_ADVDIFF else None)

    def run(self, specs, rate=100.0, seed=0, max_steps=0):
        """Serve `specs` (workloads.request_mix entries) arriving as a Poisson
        process of `rate` requests/s; each runs to its end time or max_steps."""
        arrivals = poisson_arrivals(len(specs), rate, seed)
        reqs = [Request(k, s, float(a), self.precision, max_steps) for k, (s, a) in enumerate(zip(specs, arrivals))]
        need = collections.defaultdict(int)
        demand = collections.defaultdict(float)
        ubytes = {}
        for r in reqs:
            u = Batch.units(r.cfg)
            need[r.group] = max(need[r.group], u)
            lim = 0 if r.cfg.system == SYS_ADVDIFF else 1
            ubytes[r.group] = Batch.unit_bytes(r.cfg.system, r.N, self.precision, lim)
            demand[r.group] += u * ubytes[r.group]
        units = self.split_budget(self.budget, demand, need, ubytes, self.share)
        for r in reqs:  # all batches exist before the clock starts
            self._group(r, units[r.group])
        # results that are not kept land in one page-locked buffer (full-rate
        # device-to-host copies, no first-touch page faults)
        stage = PinnedArray(max(r.dofs for r in reqs)) if (self.download_results and not self.keep_results
                                                           and reqs) else None
        pending = collections.deque(reqs)
        waiting = {g: collections.deque() for g in self.groups}
        running = {g: {} for g in self.groups}
        inflight = {g: False for g in self.groups}  # a round of steps queued and not yet synced
        done = []
        t0 = time.perf_counter()
        clock = lambda: time.perf_counter() - t0  # noqa: E731
        futures = {}
        total_steps_dofs = 0
        while pending or any(waiting.values()) or any(running.values()):
            now = clock()
            while pending and pending[0].arrival <= now:
                r = pending.popleft()
                if not self.device_setup or r.uh is not None:
                    futures[r.rid] = self.pool.submit(self._prepare, r)
                waiting[r.group].append(r)
            # admit in arrival order per group while there is room, and start the
            # group's steps before admitting into the next group, so that its
            # kernels overlap the next admissions
            for g, q in waiting.items():
                b = self.groups[g]
                # in arrival order; a request that does not fit yet does not
                # block the smaller ones behind it (backfill, within a window),
                # unless it has waited longer than backfill_s: then the room
                # that frees up is kept for it
                k = 0
                now = clock()
                while k < len(q):
                    r = q[k]
                    slot = None
                    if self.device_setup and r.uh is None:
                        slot = b.admit_ic(r.cfg, r.ic, r.params, r.tend, r.max_steps)
                        if slot is not None:
                            self.h2d_bytes += 32 * 8
                    else:
                        f = futures[r.rid]
                        if f.done():
                            uh, lh = f.result()
                            slot = b.admit(r.cfg, uh, lh, r.tend, r.max_steps)
                            if slot is not None:
                                del futures[r.rid]
                                self.h2d_bytes += uh.nbytes + (lh.nbytes if lh is not None else 0)
                    if slot is None:
                        if (k + 1 >= self.backfill_window or now - q[0].arrival > self.backfill_s
                                or len(running[g]) >= self.max_instances):
                            break
                        k += 1
                        continue
                    del q[k]
                    r.slot, r.admitted = slot, clock()
                    running[g][slot] = r
                if running[g] and not inflight[g]:
                    b.launch(self.sync_every)
                    inflight[g] = True
            active = [g for g in self.groups if inflight[g]]
            if not active:
                if pending:
                    time.sleep(max(0.0, min(pending[0].arrival - clock(), 0.01)))
                else:
                    time.sleep(0.0005)
                continue
            # the groups whose round has completed, in completion order: a
            # group's next round is queued as soon as its own round ends,
            # without waiting behind another group's longer round
            ready = [g for g in active if self.groups[g].ready()]
            if not ready:
                if not (pending and pending[0].arrival <= clock()):
                    time.sleep(0.0002)
                continue
            for g in ready:
                b = self.groups[g]
                b.sync()
                inflight[g] = False
                for slot in list(running[g]):
                    r = running[g][slot]
                    q = b.query(slot)
                    if q["done"]:
                        r.failed = q["status"] == ENONFINITE
                        if self.download_results and not r.failed:
                            res = b.download(slot, out=None if stage is None else stage.array)
                            self.d2h_bytes += res.nbytes
                            if self.keep_results:
                                r.result = res
                        r.steps, r.time, r.finished = q["steps"], q["time"], clock()
                        if not r.failed:
                            total_steps_dofs += r.steps * r.dofs
                        b.release(slot)
                        del running[g][slot]
                        done.append(r)
                # the group's next round right away (the GPU does not wait for the
                # host's turn over the other groups), unless requests wait to join it
                if running[g] and not waiting[g] and not (pending and pending[0].arrival <= clock()):
                    b.launch(self.sync_every)
                    inflight[g] = True
        makespan = clock()
        ok = [r for r in done if not r.failed]
        tts = np.array([r.finished - r.arrival for r in ok]) if ok else np.array([math.nan])
        return {
            "requests": len(ok),
            "failed": len(done) - len(ok),
            "failed_ids": [r.rid for r in done if r.failed],
            "dof_updates": int(total_steps_dofs),
            "makespan_s": makespan,
            "dof_updates_per_s": total_steps_dofs / makespan if makespan > 0 else math.nan,
            "tts_p50_s": float(np.percentile(tts, 50)),
            "tts_p99_s": float(np.percentile(tts, 99)),
            "groups": len(self.groups),
            "h2d_bytes": self.h2d_bytes,
            "d2h_bytes": self.d2h_bytes,
            "requests_done": done,
        }

    def close(self):
        for b in self.groups.values():
            b.close()
        self.groups.clear()
        self.pool.shutdown(wait=False)


def main(argv=None):
    """Serve the seeded request mix at one or more Poisson arrival rates and
    print one JSON line per rate: throughput and time-to-solution percentiles.

        python -m aderdg.serving --requests 1024 --steps 50 --rates 10,30,100,300,500
    """
    import argparse
    import json

    from .core import FP32_MIXED, FP64

    ap = argparse.ArgumentParser(prog="python -m aderdg.serving")
    ap.add_argument("--requests", type=int, default=256)
    ap.add_argument("--seed", type=int, default=0, help="request_mix seed")
    ap.add_argument("--rates", default="100", help="comma-separated arrival rates, requests/s")
    ap.add_argument("--steps", type=int, default=50, help="steps per request (0: to its end time)")
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    ap.add_argument("--budget-gb", type=float, default=160.0, help="HBM budget of the batches")
    ap.add_argument("--host-setup", action="store_true", help="project initial fields on the host")
    args = ap.parse_args(argv)
    prec = FP32_MIXED if args.precision == "fp32" else FP64
    specs = workloads.request_mix(max(args.requests, 1024), seed=args.seed)[:args.requests]
    for rate in [float(x) for x in args.rates.split(",")]:
        srv = Server(hbm_budget_bytes=args.budget_gb * 1e9, precision=prec, device_setup=not args.host_setup)
        rep = srv.run(specs, rate=rate, seed=args.seed, max_steps=args.steps)
        rep.pop("requests_done")
        srv.close()
        rep.update(rate=rate, seed=args.seed, steps=args.steps, precision=args.precision)
        print(json.dumps(rep), flush=True)


if __name__ == "__main__":
    main()
