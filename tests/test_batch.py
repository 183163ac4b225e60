"""Batched simulations: one launch steps many simulations of one (system, N),
each with its own grid, boundary conditions, CFL time step and end time.
Every simulation's result in the batch must equal its result alone (bit for
bit: the arithmetic per cell does not depend on the batch), including when
others are admitted or released while it runs."""
import numpy as np
import pytest

import aderdg

pytestmark = pytest.mark.gpu


def _alone(cfg, ic, params, steps, tend):
    uh, lh = aderdg.project_initial_condition(cfg, ic, params)
    s = aderdg.Solver(cfg)
    s.upload(uh)
    if cfg.limiter and cfg.system != aderdg.SYS_ADVDIFF:
        s.init_limiter(lh)
    t = 0.0
    for _ in range(steps):
        t, _, _ = s.step(t, tend)
    out, _ = s.download()
    s.close()
    return out, t


def _admit(b, cfg, ic, params, tend, max_steps=0):
    uh, lh = aderdg.project_initial_condition(cfg, ic, params)
    return b.admit(cfg, uh, lh if cfg.limiter and cfg.system != aderdg.SYS_ADVDIFF else None, tend, max_steps)


MEMBERS = {
    aderdg.SYS_EULER: [("euler_rp2d", 20, {}), ("euler_vortex", 24, {}), ("euler_rp2d", 13, {"xr": (1.0, 0.7)})],
    aderdg.SYS_BN: [("bn_cylinder", 16, {}), ("bn_cylinder", 11, {})],
    aderdg.SYS_ADVDIFF: [("ad_sine", 12, {}), ("ad_sine", 9, {"cx": 0.3})],
}


@pytest.mark.parametrize("system,N,prec", [(aderdg.SYS_EULER, 3, aderdg.FP64), (aderdg.SYS_EULER, 3, aderdg.FP32_MIXED),
                                           (aderdg.SYS_BN, 2, aderdg.FP64), (aderdg.SYS_BN, 3, aderdg.FP32_MIXED),
                                           (aderdg.SYS_ADVDIFF, 4, aderdg.FP64), (aderdg.SYS_ADVDIFF, 3, aderdg.FP32_MIXED)])
def test_batch_results_equal_alone(gpu_lib, system, N, prec):
    members = []
    for name, side, over in MEMBERS[system]:
        cfg, ic, params, tend = aderdg.workloads.make(name, side=side, N=N, precision=prec, **over)
        members.append((cfg, ic, params, tend))
    lim = members[0][0].limiter
    b = aderdg.Batch(system, N, prec, lim, capacity_units=4096, max_instances=8)
    slots = [_admit(b, *m) for m in members]
    assert all(s is not None for s in slots)
    steps = 4
    b.launch(steps)
    b.sync()
    for slot, (cfg, ic, params, tend) in zip(slots, members):
        q = b.query(slot)
        ref, t = _alone(cfg, ic, params, steps, tend)
        assert q["steps"] == steps and q["time"] == t
        assert np.array_equal(b.download(slot), ref)
    b.close()


def test_batch_admit_and_release_while_running(gpu_lib):
    N = 3
    A = aderdg.workloads.make("euler_rp2d", side=18, N=N)
    B = aderdg.workloads.make("euler_vortex", side=14, N=N)
    C = aderdg.workloads.make("euler_rp2d", side=10, N=N)
    b = aderdg.Batch(aderdg.SYS_EULER, N, aderdg.FP64, 1, capacity_units=19 * 19 + 15 * 15 + 10, max_instances=4)
    sa = _admit(b, *A)
    b.launch(3)
    b.sync()
    sb = _admit(b, *B)
    assert _admit(b, *C) is None  # no room until A leaves
    b.launch(2)
    b.sync()
    ref_a, ta = _alone(*A[:3], 5, A[3])
    assert np.array_equal(b.download(sa), ref_a) and b.query(sa)["time"] == ta
    b.release(sa)
    sc = _admit(b, *C)
    assert sc is not None
    b.launch(3)
    b.sync()
    ref_b, tb = _alone(*B[:3], 5, B[3])
    ref_c, tc = _alone(*C[:3], 3, C[3])
    assert np.array_equal(b.download(sb), ref_b) and b.query(sb)["time"] == tb
    assert np.array_equal(b.download(sc), ref_c) and b.query(sc)["time"] == tc
    b.close()


def test_batch_step_budget_and_end_time(gpu_lib):
    N = 2
    cfg, ic, params, tend = aderdg.workloads.make("ad_sine", side=8, N=N)
    b = aderdg.Batch(aderdg.SYS_ADVDIFF, N, aderdg.FP64, 0, capacity_units=512, max_instances=4)
    s1 = _admit(b, cfg, ic, params, tend, max_steps=3)
    s2 = _admit(b, cfg, ic, params, 0.01, max_steps=0)
    b.launch(50)
    assert b.sync() == 0
    q1, q2 = b.query(s1), b.query(s2)
    assert q1["steps"] == 3 and q1["done"]
    assert q2["time"] == 0.01 and q2["done"]
    b.close()


def test_two_groups_run_concurrently(gpu_lib):
    ga = aderdg.workloads.make("euler_rp2d", side=16, N=2)
    gb = aderdg.workloads.make("bn_cylinder", side=12, N=3)
    ba = aderdg.Batch(aderdg.SYS_EULER, 2, aderdg.FP64, 1, capacity_units=1024, max_instances=2)
    bb = aderdg.Batch(aderdg.SYS_BN, 3, aderdg.FP64, 1, capacity_units=1024, max_instances=2)
    sa, sb = _admit(ba, *ga), _admit(bb, *gb)
    for _ in range(2):
        ba.launch(2)
        bb.launch(2)
        ba.sync()
        bb.sync()
    assert np.array_equal(ba.download(sa), _alone(*ga[:3], 4, ga[3])[0])
    assert np.array_equal(bb.download(sb), _alone(*gb[:3], 4, gb[3])[0])
    ba.close()
    bb.close()


def test_batch_rejects_mismatched_config(gpu_lib):
    b = aderdg.Batch(aderdg.SYS_EULER, 3, aderdg.FP64, 1, capacity_units=256, max_instances=2)
    cfg, ic, params, tend = aderdg.workloads.make("euler_rp2d", side=8, N=2)
    with pytest.raises(aderdg.AderdgError):
        _admit(b, cfg, ic, params, tend)
    b.close()


def test_download_into_pinned_buffer(gpu_lib):
    """aderdg_host_alloc memory as the target of a batch download: the same
    values as a download into ordinary memory."""
    cfg, ic, params, tend = aderdg.workloads.make("euler_rp2d", side=14, N=2, precision=aderdg.FP32_MIXED)
    b = aderdg.Batch(cfg.system, cfg.N, aderdg.FP32_MIXED, 1, capacity_units=400, max_instances=4)
    slot = b.admit_ic(cfg, ic, params, tend, 3)
    b.launch(3)
    b.sync()
    plain = b.download(slot)
    pin = aderdg.PinnedArray(cfg.dofs + 7)
    got = b.download(slot, out=pin.array)
    assert got.size == cfg.dofs and np.array_equal(got, plain)
    b.close()


def test_admissions_queue_without_waiting(gpu_lib):
    """Admissions and releases edit the device table in stream order without
    waiting for the GPU: many admissions straight after the batch is created,
    then K steps; every simulation has made exactly K steps and equals its run
    alone."""
    members = [("euler_rp2d", 10 + k % 5, {}) for k in range(10)]
    cfgs = []
    b = aderdg.Batch(aderdg.SYS_EULER, 2, aderdg.FP64, 1, capacity_units=3000, max_instances=16)
    slots = []
    for name, side, over in members:
        cfg, ic, params, tend = aderdg.workloads.make(name, side=side, N=2, **over)
        slots.append(b.admit_ic(cfg, ic, params, tend, 4))
        cfgs.append((cfg, ic, params, tend))
    b.release(slots[3])  # a release in the middle of the queued admissions
    b.launch(6)
    b.sync()
    for k, slot in enumerate(slots):
        if k == 3:
            continue
        q = b.query(slot)
        assert q["steps"] == 4 and q["done"] and q["status"] == 0, (k, q)
    for k in (0, 9):
        cfg, ic, params, tend = cfgs[k]
        s = aderdg.Solver(cfg)
        s.initial_condition(ic, params)
        t = 0.0
        for _ in range(4):
            t, _, _ = s.step(t, tend)
        alone, _ = s.download()
        s.close()
        assert np.array_equal(b.download(slots[k]), alone)
    b.close()


def test_ready_reports_completion_without_waiting(gpu_lib):
    """aderdg_batch_ready: true once everything queued on the batch's stream
    has completed (then sync does not wait), and never blocks."""
    import time
    cfg, ic, params, tend = aderdg.workloads.make("euler_rp2d", side=96, N=3)
    b = aderdg.Batch(aderdg.SYS_EULER, 3, aderdg.FP64, 1, capacity_units=97 * 97, max_instances=1)
    slot = _admit(b, cfg, ic, params, tend)
    b.sync()
    assert b.ready()
    b.launch(40)
    t0 = time.perf_counter()
    first = b.ready()                       # returns at once, whatever the answer
    assert time.perf_counter() - t0 < 0.05
    b.sync()
    assert b.ready()
    assert b.query(slot)["steps"] == 40
    print("ready right after queueing 40 steps: %s" % first)
    b.close()
