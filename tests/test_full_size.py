"""The four base cases at their full sizes (AD 64^2 N=3, Euler vortex 256^2
N=4, Euler 2D Riemann problem 512^2 N=3, Baer-Nunziato cylinder 400^2 N=3).

- One FP64 step against the oracle: relative L1 / L-infinity of uh <= 1e-11,
  the same time step and the same troubled-cell mask.
- Size-independent properties over several steps: conservation of the totals
  on the periodic vortex (FP64 and FP32-mixed) and free-stream preservation
  of a uniform flow on the vortex grid.
"""
import numpy as np
import pytest

import aderdg
import pyoracle as po

from helpers import rel_l1, rel_linf, setup_pair

pytestmark = pytest.mark.gpu

FULL = [("ad_sine", 3, 64), ("euler_vortex", 4, 256), ("euler_rp2d", 3, 512), ("bn_cylinder", 3, 400)]


@pytest.mark.parametrize("name,N,side", FULL)
def test_full_size_step_parity_fp64(gpu_lib, name, N, side):
    cfg, ic, params, tend = aderdg.workloads.make(name, side=side, N=N)
    o, g, uh, lh = setup_pair(cfg, ic, params)
    t_o, dt_o, n_o = o.step(0.0, tend)
    t_g, dt_g, n_g = g.step(0.0, tend)
    assert dt_g == dt_o, (dt_g, dt_o)
    assert n_g == n_o
    ug, _ = g.download()
    uo = o.get(po.UH)
    e1, ei = rel_l1(ug, uo), rel_linf(ug, uo)
    assert e1 <= 1e-11 and ei <= 1e-11, (e1, ei)
    if cfg.limiter and cfg.system != aderdg.SYS_ADVDIFF:
        assert np.array_equal(g.get(aderdg.A_RECOMPUTE), o.get_int(po.RECOMPUTE))
    g.close()


def _totals(cfg, uh):
    """Integral of every conserved variable over the domain (Gauss-Legendre)."""
    P, V = cfg.N + 1, cfg.nvar
    w = aderdg.operator(cfg.N, aderdg.OP_W)
    W = np.outer(w, w).ravel()  # node i + P j
    dx = (cfg.xr[0] - cfg.xl[0]) / cfg.imax
    dy = (cfg.xr[1] - cfg.xl[1]) / cfg.jmax
    u = uh.reshape(cfg.cells, P * P, V)
    return np.einsum("n,cnv->v", W, u) * dx * dy


@pytest.mark.parametrize("precision,tol", [(aderdg.FP64, 1e-13), (aderdg.FP32_MIXED, 1e-8)])
def test_full_size_conservation_vortex(gpu_lib, precision, tol):
    cfg, ic, params, tend = aderdg.workloads.make("euler_vortex", precision=precision)
    s = aderdg.Solver(cfg)
    s.initial_condition(ic, params)
    u0, _ = s.download()
    before = _totals(cfg, u0)
    t, n = s.run(0.0, tend, 5)
    assert n == 5
    u1, _ = s.download()
    after = _totals(cfg, u1)
    s.close()
    # mass and energy are O(100) on the 10x10 domain; the momenta are too (u = v = 1)
    assert np.all(np.abs(after - before) <= tol * np.abs(before)), (before, after)


@pytest.mark.parametrize("precision,tol", [(aderdg.FP64, 1e-13), (aderdg.FP32_MIXED, 1e-6)])
def test_full_size_free_stream(gpu_lib, precision, tol):
    cfg, ic, params, tend = aderdg.workloads.make("euler_vortex", precision=precision)
    params = (0.0,) + tuple(params[1:])  # vortex strength 0: the uniform free stream
    s = aderdg.Solver(cfg)
    s.initial_condition(ic, params)
    u0, _ = s.download()
    t, n = s.run(0.0, tend, 3)
    assert n == 3
    u1, st = s.download()
    s.close()
    assert rel_linf(u1, u0) <= tol, rel_linf(u1, u0)
    assert not st.any()  # nothing limited


@pytest.mark.parametrize("name", ["euler_rp2d", "bn_cylinder"])
def test_full_size_fp32_mixed_troubled_cells(gpu_lib, name):
    """FP32-mixed against the FP64 path on the limiter-heavy cases at full size,
    10 steps: troubled-cell counts within 0.1% every step, the masks counted
    cell by cell, and relative L1 of uh <= 1e-5."""
    cfg64, ic, params, tend = aderdg.workloads.make(name)
    cfg32, _, _, _ = aderdg.workloads.make(name, precision=aderdg.FP32_MIXED)
    a, b = aderdg.Solver(cfg64), aderdg.Solver(cfg32)
    na0, nb0 = a.initial_condition(ic, params), b.initial_condition(ic, params)
    assert na0 == nb0
    ta = tb = 0.0
    differ = []
    for _ in range(10):
        ta, _, na = a.step(ta, tend)
        tb, _, nb = b.step(tb, tend)
        assert abs(na - nb) <= max(1, 0.001 * na), (na, nb)
        differ.append(int((a.get(aderdg.A_RECOMPUTE) != b.get(aderdg.A_RECOMPUTE)).sum()))
    assert max(differ) <= 0.001 * cfg64.cells, differ
    ua, _ = a.download()
    ub, _ = b.download()
    a.close()
    b.close()
    assert rel_l1(ub, ua) <= 1e-5, rel_l1(ub, ua)


def test_fp32_mixed_decisions_on_developed_shock_state(gpu_lib):
    """From an FP64 state 400 steps into the 2D Riemann problem (shocks, contacts
    and their troubled cells developed), both precisions restart from the same
    uh, status and Lh: the first step marks the same troubled cells and takes
    the same dt to 1e-6, and the counts stay within 0.1% for 3 steps."""
    cfg64, ic, params, tend = aderdg.workloads.make("euler_rp2d")
    cfg32, _, _, _ = aderdg.workloads.make("euler_rp2d", precision=aderdg.FP32_MIXED)
    base = aderdg.Solver(cfg64)
    base.initial_condition(ic, params)
    t0, n = base.run(0.0, tend, 400)
    assert n == 400
    uh, st = base.download()
    lh = base.get(aderdg.A_LH)
    base.close()
    a, b = aderdg.Solver(cfg64), aderdg.Solver(cfg32)
    for s in (a, b):
        s.upload(uh)
        s.upload_limiter(st, lh)
    ta = tb = t0
    for k in range(3):
        ta, da, na = a.step(ta, tend)
        tb, db, nb = b.step(tb, tend)
        assert abs(db - da) <= 1e-6 * da, (k, da, db)
        assert na > 1000 and abs(na - nb) <= 0.001 * na, (k, na, nb)
        if k == 0:
            assert np.array_equal(a.get(aderdg.A_RECOMPUTE), b.get(aderdg.A_RECOMPUTE))
    ua, _ = a.download()
    ub, _ = b.download()
    a.close()
    b.close()
    assert rel_l1(ub, ua) <= 1e-6, rel_l1(ub, ua)
