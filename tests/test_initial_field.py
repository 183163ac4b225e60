"""On-device set-up: the initial field at the Gauss-Legendre nodes and the
initial limiter computed on the GPU agree with the host set-up (bit for bit
where the field has no transcendental function, to the math libraries'
rounding otherwise), and admission from it behaves like admission from host
arrays."""
import numpy as np
import pytest

import aderdg
from helpers import rel_linf

pytestmark = pytest.mark.gpu

CASES = [("euler_rp2d", 20, 3, True), ("bn_cylinder", 16, 2, True), ("euler_vortex", 18, 4, False),
         ("ad_sine", 12, 3, False)]


@pytest.mark.parametrize("name,side,N,exact", CASES)
def test_device_initial_field_matches_host(gpu_lib, name, side, N, exact):
    cfg, ic, params, tend = aderdg.workloads.make(name, side=side, N=N)
    uh, lh = aderdg.project_initial_condition(cfg, ic, params)
    lim = cfg.limiter and cfg.system != aderdg.SYS_ADVDIFF
    a = aderdg.Solver(cfg)
    a.upload(uh)
    na = a.init_limiter(lh) if lim else 0
    b = aderdg.Solver(cfg)
    nb = b.initial_condition(ic, params)
    ua, sa = a.download()
    ub, sb = b.download()
    if exact:
        assert np.array_equal(ua, ub)
    else:
        assert rel_linf(ub, ua) <= 1e-14
    assert na == nb
    if lim:
        assert np.array_equal(sa, sb)
    t = 0.0
    for _ in range(3):
        ta, _, _ = a.step(t, tend)
        tb, _, _ = b.step(t, tend)
        t = ta
    ua, _ = a.download()
    ub, _ = b.download()
    if exact:
        assert ta == tb and np.array_equal(ua, ub)
    else:
        assert rel_linf(ub, ua) <= 1e-12
    a.close()
    b.close()


def test_batch_admit_ic_equals_admit(gpu_lib):
    cfg, ic, params, tend = aderdg.workloads.make("euler_rp2d", side=14, N=3)
    uh, lh = aderdg.project_initial_condition(cfg, ic, params)
    b = aderdg.Batch(cfg.system, cfg.N, cfg.precision, 1, capacity_units=1024, max_instances=4)
    s1 = b.admit(cfg, uh, lh, tend, 0)
    s2 = b.admit_ic(cfg, ic, params, tend, 0)
    assert np.array_equal(b.download(s1), b.download(s2))
    b.launch(4)
    b.sync()
    assert b.query(s1)["time"] == b.query(s2)["time"]
    assert np.array_equal(b.download(s1), b.download(s2))
    b.close()


def test_unknown_initial_field_rejected(gpu_lib):
    cfg, ic, params, tend = aderdg.workloads.make("euler_rp2d", side=8, N=2)
    s = aderdg.Solver(cfg)
    with pytest.raises(aderdg.AderdgError):
        s.initial_condition(aderdg.IC_BN_CYLINDER, params)  # a Baer-Nunziato field on an Euler grid
    s.close()
    b = aderdg.Batch(cfg.system, cfg.N, cfg.precision, 1, capacity_units=256, max_instances=2)
    with pytest.raises(aderdg.AderdgError):
        b.admit_ic(cfg, 99, params, tend, 0)
    assert b.info()["instances"] == 0
    b.close()
