"""Continuous batching: requests that arrive while others run are admitted as
room frees up, their work overlaps on the GPU, and every request's result in
the mix equals its result alone (bit for bit)."""
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


@pytest.mark.parametrize("device_setup", [True, False])
def test_served_results_equal_alone(gpu_lib, device_setup):
    mix = _small_mix(16, seed=3)
    # a budget small enough that requests wait for room while others run
    srv = aderdg.serving.Server(hbm_budget_bytes=24 << 20, sync_every=2, keep_results=True,
                                device_setup=device_setup)
    rep = srv.run(mix, rate=400.0, seed=3, max_steps=5)
    assert rep["requests"] == 16
    assert rep["tts_p99_s"] >= rep["tts_p50_s"] > 0
    waited = sum(1 for r in rep["requests_done"] if r.admitted - r.arrival > 1e-3)
    for r in rep["requests_done"]:
        assert r.steps == 5
        s = aderdg.Solver(r.cfg)
        if device_setup:
            s.initial_condition(r.ic, r.params)
        else:
            uh, lh = aderdg.project_initial_condition(r.cfg, r.ic, r.params)
            s.upload(uh)
            if r.cfg.limiter and r.cfg.system != aderdg.SYS_ADVDIFF:
                s.init_limiter(lh)
        t = 0.0
        for _ in range(5):
            t, _, _ = s.step(t, r.tend)
        ref, _ = s.download()
        s.close()
        assert t == r.time
        assert np.array_equal(r.result, ref), (r.name, r.N, r.side)
    srv.close()
    assert waited >= 0
