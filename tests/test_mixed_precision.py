"""The FP32-mixed mode's limiter decisions are the FP64 ones.

The FP32-mixed mode computes the DMP's subcell and Gauss-Lobatto projections
in FP32 with a bound on their error, and the neighbourhood bounds it folds may
carry such a bound too.  A comparison is decided from those values only when
it holds by more than the bounds; otherwise the cell is settled from FP64
reference-order values (its own projections and its neighbours' recomputed
min/max).  The subcell re-solve, the positivity tests and the Baer-Nunziato
path-conservative face flux are FP64.  So, given the same state, the
FP32-mixed step must mark exactly the cells the FP64 DMP of the reference
marks (Euler/limiter.f90:179-245) and limit exactly those its limiter limits.
The re-solved cells carry the FP64 subcell re-solve's values
(Euler/limiter.f90:411-647, Baer-Nunziato/limiter.f90:416-596) to rounding:
the mixed mode forms them with fused multiply-adds and shared reciprocals
(relative max difference <= 1e-12); every other cell is equal bit for bit.

How it is checked: the FP32-mixed solver takes a step from state u0 (with its
limiter status and Lh); a second FP32-mixed solver without the limiter takes
the same step from the same u0 with the same dt and gives the updated state
u1 of every cell (the limiter only replaces the listed cells afterwards).  The
oracle then runs the reference's get_min_max on u0, the DMP of element_update
on u1 (dt = 0 and duh = 0, so that u1 stays as it is) and the reference's
limiter with the step's dt.  Its troubled mask and status must equal the
GPU's exactly, and its final state as stated above.
"""
import dataclasses

import numpy as np
import pytest

import aderdg
import pyoracle as po

from helpers import oracle_config

pytestmark = pytest.mark.gpu

CASES = [("euler_rp2d", 3, 24), ("euler_rp2d", 2, 32), ("bn_cylinder", 3, 20), ("bn_cylinder", 2, 24),
         ("euler_vortex", 4, 12)]


def _oracle_step_on(o, cfg, t, dt, u0, st0, lh0, u1):
    """Reference DMP and limiter of one step whose start state is (u0, st0,
    lh0) and whose updated state is u1; returns (nRecompute, recompute,
    status, uh)."""
    o.set(po.UH, u0)
    o.set_int(po.STATUS, st0)
    o.set_int(po.OLDSTATUS, st0)
    o.set(po.LH, lh0)
    o.set_time(t)
    o.get_min_max()
    o.set_int(po.RECOMPUTE, np.zeros(cfg.cells, dtype=np.int32))
    o.save_olduh()
    o.set(po.UH, u1)
    o.set(po.DUH, np.zeros_like(u1))
    o.set_dt(0.0)
    n = o.element_update()
    o.set_dt(dt)
    o.limiter()
    return n, o.get_int(po.RECOMPUTE), o.get_int(po.STATUS), o.get(po.UH)


def _compare_steps(name, N, side, precision, steps=6, warm=3):
    cfg, ic, params, tend = aderdg.workloads.make(name, side=side, N=N, precision=precision)
    uh, lh = aderdg.project_initial_condition(cfg, ic, params)
    a = aderdg.Solver(cfg)
    a.upload(uh)
    a.init_limiter(lh)
    b = aderdg.Solver(dataclasses.replace(cfg, limiter=0))
    o = po.Oracle(oracle_config(cfg))
    t, dt = 0.0, 0.0
    for _ in range(warm):  # a developed state with limited cells
        t, dt, _ = a.step(t, tend)
    diffs, troubled = [], 0
    for _ in range(steps):
        u0, _ = a.download()
        st0, lh0 = a.download_limiter()
        te = t + 0.5 * dt  # both solvers take dt = te - t exactly
        b.upload(u0)
        _, dtb, _ = b.step(t, te)
        u1, _ = b.download()
        t1, dta, na = a.step(t, te)
        assert dta == dtb == te - t
        ua, sta = a.download()
        rec_a = a.get(aderdg.A_RECOMPUTE)
        n_o, rec_o, st_o, u_o = _oracle_step_on(o, cfg, t, dta, u0, st0, lh0, u1)
        listed = np.repeat(rec_o > 0, cfg.P * cfg.P * cfg.nvar)
        rel = float(np.abs(ua - u_o)[listed].max() / np.abs(u_o).max()) if listed.any() else 0.0
        diffs.append((na - n_o, int((rec_a != rec_o).sum()), int((sta != st_o).sum()),
                      int((ua != u_o)[~listed].sum()), rel <= 1e-12))
        troubled += n_o
        t, dt = t1, dta
    for s in (a, b):
        s.close()
    return diffs, troubled


@pytest.mark.parametrize("name,N,side", CASES)
def test_mixed_limiter_is_fp64_on_same_state(gpu_lib, name, N, side):
    diffs, troubled = _compare_steps(name, N, side, aderdg.FP32_MIXED)
    # per step: count, recompute-mask, status and unlisted-uh disagreements,
    # and the listed cells within 1e-12
    assert all(d == (0, 0, 0, 0, True) for d in diffs), diffs
    if name != "euler_vortex":
        assert troubled > 0  # the case exercises the limiter


def _near_threshold_field(cfg, spread):
    """Euler cells whose initial DMP (argmax 0.1 against the cell's own nodal
    min/max, Euler/initialize.f90:287-307) sits within a relative `spread` of
    its threshold: energy E = 10 + A_c phi with a fixed nodal pattern phi whose
    projections undershoot its nodal minimum by c, and A_c = (0.1 / c)(1 + d_c),
    d_c spaced evenly over [-spread, spread]; density 1, momenta 0."""
    P, S = cfg.P, cfg.S
    lim = aderdg.operator(cfg.N, aderdg.OP_UH2LIM).reshape(P, S).T  # (s, k)
    lob = aderdg.operator(cfg.N, aderdg.OP_UH2LOB).reshape(P, P).T  # (q, k)
    rng = np.random.default_rng(7)
    phi = rng.uniform(-1.0, 1.0, (P, P))  # phi[j, i]
    sub = lim @ phi @ lim.T
    lbt = lob @ phi @ lob.T
    lo = min(sub.min(), lbt.min(), phi.min())
    hi = max(sub.max(), lbt.max(), phi.max())
    c = max(phi.min() - lo, hi - phi.max())
    assert c > 0.05
    n = cfg.cells
    A = (0.1 / c) * (1.0 + np.linspace(-spread, spread, n))
    uh = np.zeros((n, P, P, 4))
    uh[..., 0] = 1.0
    uh[..., 3] = 10.0 + A[:, None, None] * phi[None, :, :]
    return uh.ravel()


def test_initial_limiter_near_thresholds(gpu_lib):
    """Cells placed at their initial DMP threshold to within the FP32
    projections' error bound: the FP32-mixed initial limiter marks exactly
    the cells the FP64 path and the oracle mark."""
    base = aderdg.Config(system=aderdg.SYS_EULER, N=3, imax=32, jmax=32, bc=(3, 3, 3, 3))
    uh = _near_threshold_field(base, 3e-4)
    lh = np.zeros(base.cells * base.S * base.S * 4)
    o = po.Oracle(oracle_config(base))
    o.set(po.UH, uh)
    n_o = o.init_limiter(lh)
    st_o = o.get_int(po.STATUS)
    assert 0 < n_o < base.cells
    res = {}
    for prec in (aderdg.FP64, aderdg.FP32_MIXED, aderdg.FP32_WIDE):
        s = aderdg.Solver(dataclasses.replace(base, precision=prec))
        s.upload(uh)
        n = s.init_limiter(lh)
        st, _ = s.download_limiter()
        res[prec] = (n, int((st != st_o).sum()))
        s.close()
    assert res[aderdg.FP64] == (n_o, 0), res
    assert res[aderdg.FP32_MIXED] == (n_o, 0), res
    print("initial limiter near thresholds: oracle %d cells, FP32-wide mode %d cells (%d differ)"
          % (n_o, res[aderdg.FP32_WIDE][0], res[aderdg.FP32_WIDE][1]))


def test_refined_reciprocal_and_sqrt_within_2ulp(gpu_lib):
    """The FP32-mixed mode's FP64 reciprocal and square root (hardware
    approximations refined by a third-order Newton step, physics.cuh mrcp /
    msqrt) against the correctly rounded operations on the same device:
    within 2 ulp on normal inputs over the whole exponent range, and the
    correctly rounded result on zeros, denormals, infinities and NaNs."""
    rng = np.random.default_rng(7)
    e = rng.uniform(-1000, 1000, 200000)
    x = np.concatenate([np.ldexp(rng.uniform(1.0, 2.0, e.size), e.astype(int)),
                        rng.uniform(1e-3, 1e3, 100000),
                        -rng.uniform(1e-3, 1e3, 1000)])
    x = x[np.isfinite(x) & (np.abs(x) >= np.finfo(np.float64).tiny)]
    out = aderdg.core.probe_math(x)

    def ulps(a, b):
        ia, ib = a.view(np.int64), b.view(np.int64)
        return np.abs(ia - ib)

    d_rcp = ulps(out[:, 0], out[:, 1])
    pos = x > 0
    d_sqrt = ulps(out[pos, 2], out[pos, 3])
    print("refined rcp: max %d ulp (%.1f%% exact); sqrt: max %d ulp (%.1f%% exact)"
          % (d_rcp.max(), 100 * np.mean(d_rcp == 0), d_sqrt.max(), 100 * np.mean(d_sqrt == 0)))
    assert d_rcp.max() <= 2 and d_sqrt.max() <= 2
    assert np.all(np.isnan(out[~pos, 2]))
    special = np.array([0.0, -0.0, 5e-324, 1e-310, -1e-310, np.inf, -np.inf, np.nan])
    o = aderdg.core.probe_math(special)
    for k in (0, 2):
        a, b = o[:, k], o[:, k + 1]
        assert np.array_equal(np.isnan(a), np.isnan(b)) and np.array_equal(a[~np.isnan(a)], b[~np.isnan(b)]), (k, o)
