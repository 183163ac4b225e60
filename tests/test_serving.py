"""Continuous batching: requests that arrive while others run are admitted as
room frees up, their work overlaps on the GPU, and every request's result in
the mix equals its result alone (bit for bit).  A request whose state becomes
non-finite fails alone: it is reported failed and its batch neighbours'
results are unchanged (the reference has no such path; its NaN check is
commented out, Euler/limiter.f90:234-239)."""
import numpy as np
import pytest

import aderdg

pytestmark = pytest.mark.gpu


def _small_mix(n, seed):
    mix = aderdg.workloads.request_mix(n, seed=seed)
    for k, m in enumerate(mix):
        m["side"] = 8 + (m["side"] % 17)  # keep the test small: sides 8..24
        m["N"] = 2 + (k % 3)
    return mix


def _alone(r, device_setup, steps):
    s = aderdg.Solver(r.cfg)
    if device_setup:
        s.initial_condition(r.ic, r.params)
    else:
        uh, lh = aderdg.project_initial_condition(r.cfg, r.ic, r.params)
        s.upload(uh)
        if r.cfg.limiter and r.cfg.system != aderdg.SYS_ADVDIFF:
            s.init_limiter(lh)
    t = 0.0
    for _ in range(steps):
        t, _, _ = s.step(t, r.tend)
    ref, _ = s.download()
    s.close()
    return ref, t


@pytest.mark.parametrize("device_setup,precision,share", [(True, aderdg.FP64, "equal"), (False, aderdg.FP64, "equal"),
                                                          (True, aderdg.FP32_MIXED, "equal"),
                                                          (True, aderdg.FP32_MIXED, "demand")])
def test_served_results_equal_alone(gpu_lib, device_setup, precision, share):
    mix = _small_mix(16, seed=3)
    # a budget below every group's largest request: each group's batch then
    # holds exactly its largest request, so no two requests of a group run at
    # once; every request arrives at t = 0 and the 16 requests fall into at
    # most 12 (system, N) groups, so some wait for room while the groups run
    # side by side
    srv = aderdg.serving.Server(hbm_budget_bytes=1 << 20, precision=precision, sync_every=2, keep_results=True,
                                device_setup=device_setup, share=share)
    rep = srv.run(mix, rate=float("inf"), seed=3, max_steps=5)
    srv.close()
    done = rep["requests_done"]
    assert rep["requests"] == 16 and rep["failed"] == 0
    assert rep["tts_p99_s"] >= rep["tts_p50_s"] > 0
    # requests waited for room: admitted after an earlier request of their group finished
    waited = [r for r in done if any(q.group == r.group and q.finished <= r.admitted for q in done if q is not r)]
    assert len(waited) >= 1
    # work overlapped: two requests ran (admitted .. finished) at the same time
    assert any(a.admitted < b.finished and b.admitted < a.finished for a in done for b in done if a is not b)
    for r in done:
        assert r.steps == 5
        ref, t = _alone(r, device_setup, 5)
        assert t == r.time
        assert np.array_equal(r.result, ref), (r.name, r.N, r.side)


@pytest.mark.parametrize("precision", [aderdg.FP64, aderdg.FP32_MIXED])
def test_nonfinite_request_fails_alone(gpu_lib, precision):
    """Three Euler N=3 requests in one batch; the second one's initial state
    carries a NaN, injected on the host.  It is reported failed; the other two
    give their results alone, bit for bit."""
    specs = []
    for k, side in enumerate((12, 10, 14)):
        cfg, ic, params, tend = aderdg.workloads.make("euler_rp2d", side=side, N=3)
        spec = dict(name="euler_rp2d", N=3, side=side, params=params, tend=tend)
        if k == 1:
            uh, lh = aderdg.project_initial_condition(cfg, ic, params)
            uh[7] = np.nan
            spec.update(uh=uh, lh=lh)
        specs.append(spec)
    srv = aderdg.serving.Server(hbm_budget_bytes=1 << 30, precision=precision, sync_every=2, keep_results=True)
    rep = srv.run(specs, rate=float("inf"), seed=0, max_steps=4)
    srv.close()
    assert rep["failed"] == 1 and rep["failed_ids"] == [1]
    assert rep["requests"] == 2
    for r in rep["requests_done"]:
        if r.failed:
            continue
        ref, t = _alone(r, True, 4)
        assert r.steps == 4 and t == r.time
        assert np.array_equal(r.result, ref)
