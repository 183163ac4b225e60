"""GPU parity against the CPU oracle, through the C ABI.

Tolerances (FP64 path): relative L1 and L-infinity of uh <= 1e-11 per step,
time step and troubled-cell mask identical on the first step.  The face,
update, DMP, limiter and time-step kernels follow the reference's FP64
operation order without contraction, so fed identical inputs they agree with
the oracle bit for bit (the phase tests below inject the oracle's inputs to
check exactly that); only the predictor's fused multiply-adds differ by
rounding.  Troubled-mask and status disagreements are counted on every step
and must be zero.  FP32 modes: relative L1 <= 1e-5 against the FP64 oracle
and the oracle's troubled-cell counts (test_mixed_precision.py checks that the
FP32-mixed mode's limiter decisions are exactly the FP64 ones).
"""
import numpy as np
import pytest

import aderdg
import pyoracle as po

from helpers import rel_l1, rel_linf, setup_pair

pytestmark = pytest.mark.gpu

TOL = 1e-11

CASES = [
    ("ad_sine", 1, 8), ("ad_sine", 2, 8), ("ad_sine", 3, 10), ("ad_sine", 4, 8), ("ad_sine", 5, 6),
    ("euler_vortex", 1, 10), ("euler_vortex", 2, 8), ("euler_vortex", 3, 10), ("euler_vortex", 4, 8),
    ("euler_vortex", 5, 6),
    ("euler_rp2d", 2, 12), ("euler_rp2d", 3, 16), ("euler_rp2d", 4, 10),
    ("bn_cylinder", 2, 12), ("bn_cylinder", 3, 14), ("bn_cylinder", 4, 8), ("bn_cylinder", 5, 6),
]


@pytest.mark.parametrize("name,N,side", CASES)
def test_step_parity_fp64(gpu_lib, name, N, side):
    cfg, ic, params, tend = aderdg.workloads.make(name, side=side, N=N)
    o, g, uh, lh = setup_pair(cfg, ic, params)
    lim = cfg.limiter and cfg.system != aderdg.SYS_ADVDIFF
    t_o = t_g = 0.0
    mask_diff = []  # troubled-mask and status disagreements per step
    for step in range(3):
        t_o, dt_o, n_o = o.step(t_o, tend)
        t_g, dt_g, n_g = g.step(t_g, tend)
        uo = o.get(po.UH)
        ug, st = g.download()
        if step == 0:
            assert dt_g == dt_o, (dt_g, dt_o)
            assert n_g == n_o
        else:
            assert abs(dt_g - dt_o) <= 1e-12 * dt_o
        e1, ei = rel_l1(ug, uo), rel_linf(ug, uo)
        assert e1 <= TOL and ei <= TOL, (step, e1, ei)
        if lim:
            mask_diff.append((int((g.get(aderdg.A_RECOMPUTE) != o.get_int(po.RECOMPUTE)).sum()),
                              int((st != o.get_int(po.STATUS)).sum()), n_g - n_o))
    # the states agree to 1e-11, far inside the DMP's tolerances: no cell
    # is decided differently on any step (counted per step, first step included)
    if lim:
        assert all(d == (0, 0, 0) for d in mask_diff), mask_diff


@pytest.mark.parametrize("ictype,N", [(3, 4), (1, 2), (2, 3), (7, 2)])
def test_bn_shock_tubes_as_shipped(gpu_lib, ictype, N):
    """Baer-Nunziato/baer_nunziato_params.ini (ICType 3, N=4; here 40x4) and
    the other shock tubes of Baer-Nunziato/initialize.f90:302-407."""
    cfg = aderdg.Config(system=aderdg.SYS_BN, N=N, imax=40, jmax=4, xl=(-0.5, -0.05), xr=(0.5, 0.05),
                        bc=(1, 1, 1, 1))
    o, g, uh, lh = setup_pair(cfg, aderdg.IC_BN_RP1D, (float(ictype), 0.0))
    t_o = t_g = 0.0
    for step in range(3):
        t_o, dt_o, n_o = o.step(t_o, 0.1)
        t_g, dt_g, n_g = g.step(t_g, 0.1)
        if step == 0:
            assert dt_g == dt_o and n_g == n_o
            assert np.array_equal(g.get(aderdg.A_RECOMPUTE), o.get_int(po.RECOMPUTE))
        ug, _ = g.download()
        uo = o.get(po.UH)
        assert rel_l1(ug, uo) <= TOL and rel_linf(ug, uo) <= TOL, (step, rel_l1(ug, uo), rel_linf(ug, uo))


def test_dmr_as_shipped(gpu_lib):
    """Euler/params.ini as shipped: N=1 double Mach reflection (here 48x12)."""
    cfg = aderdg.Config(system=aderdg.SYS_EULER, N=1, imax=48, jmax=12, xr=(4.0, 1.0), bc=(1, 1, 1, 1), bc_mode=1)
    o, g, uh, lh = setup_pair(cfg, aderdg.IC_EULER_DMR, ())
    t_o = t_g = 0.0
    for step in range(3):
        t_o, dt_o, n_o = o.step(t_o, 0.2)
        t_g, dt_g, n_g = g.step(t_g, 0.2)
        if step == 0:
            assert dt_g == dt_o and n_g == n_o
        ug, _ = g.download()
        assert rel_l1(ug, o.get(po.UH)) <= TOL and rel_linf(ug, o.get(po.UH)) <= TOL


def _phase_run(cfg, ic, params, tend=1.0):
    """Run one step phase by phase on both sides, feeding every GPU phase the
    oracle's inputs, and return the per-phase comparisons."""
    o, g, uh, lh = setup_pair(cfg, ic, params)
    lim = cfg.limiter and cfg.system != aderdg.SYS_ADVDIFF
    res = {}
    dt_o = o.calc_time_step(0.0, tend)
    dt_g = g.calc_time_step(0.0, tend)
    res["dt"] = dt_g == dt_o
    if lim:
        o.get_min_max()
        o.set_int(po.RECOMPUTE, np.zeros(cfg.cells, dtype=np.int32))
        o.save_olduh()
        g.limiter_prepare()
    o.predictor()
    g.space_time_predictor()
    res["qbnd"] = rel_linf(g.get(aderdg.A_QBND), o.get(po.QBND))
    if cfg.system == aderdg.SYS_ADVDIFF:
        res["fbnd"] = rel_linf(g.get(aderdg.A_GRADQBND), o.get(po.GRADQBND))
    else:
        res["fbnd"] = rel_linf(g.get(aderdg.A_FBND), o.get(po.FBND))
    res["fhi"] = rel_linf(g.get(aderdg.A_FHI), o.get(po.FHI))
    # feed the oracle's predictor outputs to the GPU from here on
    g.set(aderdg.A_FHI, o.get(po.FHI))
    if cfg.system == aderdg.SYS_BN:
        g.set(aderdg.A_SHI, o.get(po.SHI))
    g.set(aderdg.A_QBND, o.get(po.QBND))
    if cfg.system == aderdg.SYS_ADVDIFF:
        g.set(aderdg.A_GRADQBND, o.get(po.GRADQBND))
    else:
        g.set(aderdg.A_FBND, o.get(po.FBND))
    o.volume_integral()
    g.volume_integral()
    res["volume"] = np.array_equal(g.get(aderdg.A_DUH), o.get(po.DUH))
    o.riemann()
    g.riemann_problem()
    if cfg.system == aderdg.SYS_BN:
        res["faces"] = all(np.array_equal(g.get(a), o.get(b)) for a, b in
                           ((aderdg.A_FU, po.FM), (aderdg.A_FP, po.FP), (aderdg.A_GU, po.GM), (aderdg.A_GP, po.GP)))
    else:
        res["faces"] = np.array_equal(g.get(aderdg.A_FU), o.get(po.FU)) and np.array_equal(g.get(aderdg.A_GU),
                                                                                            o.get(po.GU))
    o.surface_integral()
    g.surface_integral()
    res["surface"] = np.array_equal(g.get(aderdg.A_DUH), o.get(po.DUH))
    n_o = o.element_update()
    n_g = g.element_update()
    res["update"] = np.array_equal(g.get(aderdg.A_UH), o.get(po.UH))
    res["nrec"] = (n_g, n_o)
    if lim:
        res["lmin"] = np.array_equal(g.get(aderdg.A_LMIN), o.get(po.LMIN))
        res["lmax"] = np.array_equal(g.get(aderdg.A_LMAX), o.get(po.LMAX))
        o.limiter()
        g.limiter()
        res["recompute"] = np.array_equal(g.get(aderdg.A_RECOMPUTE), o.get_int(po.RECOMPUTE))
        res["status"] = np.array_equal(g.get(aderdg.A_STATUS), o.get_int(po.STATUS))
        ug = g.get(aderdg.A_UH)
        res["limited_uh"] = np.array_equal(ug, o.get(po.UH))
        st = o.get_int(po.STATUS).astype(bool)
        S, V = cfg.S, cfg.nvar
        lg = g.get(aderdg.A_LH).reshape(cfg.cells, S * S * V)[st]
        lo = o.get(po.LH).reshape(cfg.cells, S * S * V)[st]
        res["lh"] = np.array_equal(lg, lo)
    return res


PHASE_CASES = [("ad_sine", 3, 8), ("euler_vortex", 4, 8), ("euler_rp2d", 3, 12), ("euler_rp2d", 5, 8),
               ("bn_cylinder", 3, 10), ("bn_cylinder", 2, 12)]


@pytest.mark.parametrize("name,N,side", PHASE_CASES)
def test_phases_bit_exact_given_oracle_inputs(gpu_lib, name, N, side):
    cfg, ic, params, tend = aderdg.workloads.make(name, side=side, N=N)
    res = _phase_run(cfg, ic, params, tend)
    assert res["dt"]
    for k in ("qbnd", "fbnd", "fhi"):
        assert res[k] <= 1e-12, (k, res[k])
    for k in ("volume", "faces", "surface", "update"):
        assert res[k], k
    assert res["nrec"][0] == res["nrec"][1]
    if "lh" in res:
        for k in ("lmin", "lmax", "recompute", "status", "limited_uh", "lh"):
            assert res[k], k


def test_dmr_phases_bit_exact(gpu_lib):
    cfg = aderdg.Config(system=aderdg.SYS_EULER, N=2, imax=24, jmax=6, xr=(4.0, 1.0), bc=(1, 1, 1, 1), bc_mode=1)
    res = _phase_run(cfg, aderdg.IC_EULER_DMR, (), 0.2)
    for k in ("dt", "volume", "faces", "surface", "update", "lmin", "lmax", "recompute", "status", "limited_uh", "lh"):
        assert res[k], k


def test_run_equals_repeated_steps(gpu_lib):
    cfg, ic, params, tend = aderdg.workloads.make("euler_rp2d", side=16, N=3)
    uh, lh = aderdg.project_initial_condition(cfg, ic, params)
    a, b = aderdg.Solver(cfg), aderdg.Solver(cfg)
    for s in (a, b):
        s.upload(uh)
        s.init_limiter(lh)
    t = 0.0
    for _ in range(5):
        t, _, _ = a.step(t, tend)
    t2, n = b.run(0.0, tend, 5, sync_every=2)
    assert n == 5 and t2 == t
    ua, sa = a.download()
    ub, sb = b.download()
    assert np.array_equal(ua, ub) and np.array_equal(sa, sb)


def test_run_stops_at_tend(gpu_lib):
    cfg, ic, params, _ = aderdg.workloads.make("ad_sine", side=8, N=2)
    uh, _ = aderdg.project_initial_condition(cfg, ic, params)
    s = aderdg.Solver(cfg)
    s.upload(uh)
    t, n = s.run(0.0, 0.02, 10000, sync_every=8)
    assert t == 0.02 and 0 < n < 10000


@pytest.mark.parametrize("precision", [aderdg.FP32_MIXED, aderdg.FP32_WIDE])
@pytest.mark.parametrize("name,N,side", [("euler_vortex", 3, 12), ("euler_rp2d", 3, 16), ("bn_cylinder", 3, 12),
                                         ("ad_sine", 3, 12)])
def test_fp32_mixed_error_vs_fp64_oracle(gpu_lib, name, N, side, precision):
    """Both FP32 modes within 1e-5 relative L1 of the FP64 oracle after 5
    steps, with the oracle's troubled-cell count on every step (the counts
    here are tens of cells: within 0.1% means equal)."""
    cfg, ic, params, tend = aderdg.workloads.make(name, side=side, N=N, precision=precision)
    o, g, uh, lh = setup_pair(cfg, ic, params)
    t_o = t_g = 0.0
    for _ in range(5):
        t_o, _, n_o = o.step(t_o, tend)
        t_g, _, n_g = g.step(t_g, tend)
        assert n_g == n_o
    ug, _ = g.download()
    assert rel_l1(ug, o.get(po.UH)) <= 1e-5


@pytest.mark.parametrize("precision", [aderdg.FP32_MIXED, aderdg.FP32_WIDE])
def test_fp32_mixed_large_magnitudes(gpu_lib, precision):
    """States of magnitude ~1e3 (the 2D Riemann problem with density and
    pressure scaled by 1000): FP32 projection errors would exceed the DMP's
    absolute tolerance 1e-4 there, so the mixed mode must take its FP64
    projections for those cells and still agree with the FP64 oracle."""
    cfg, ic, params, tend = aderdg.workloads.make("euler_rp2d", side=16, N=3, precision=precision)
    p = list(params)
    for q in range(4):
        p[2 + 4 * q] *= 1000.0
        p[5 + 4 * q] *= 1000.0
    o, g, uh, lh = setup_pair(cfg, ic, tuple(p))
    t_o = t_g = 0.0
    for _ in range(5):
        t_o, _, n_o = o.step(t_o, tend)
        t_g, _, n_g = g.step(t_g, tend)
    ug, _ = g.download()
    assert rel_l1(ug, o.get(po.UH)) <= 1e-5


def test_nonfinite_state_reported(gpu_lib):
    cfg = aderdg.Config(system=aderdg.SYS_EULER, N=2, imax=4, jmax=4, bc=(3, 3, 3, 3), limiter=0)
    uh = np.tile(np.array([1.0, 0.0, 0.0, 2.5]), cfg.cells * 9)
    uh[5] = np.nan  # host-side injected NaN in the input state
    s = aderdg.Solver(cfg)
    s.upload(uh)
    with pytest.raises(aderdg.AderdgError) as e:
        s.step(0.0, 1.0)
    assert e.value.code == -5
