"""Order of accuracy of the GPU path on the smooth cases.

The isentropic vortex (Euler, periodic, exact solution = the initial vortex
carried by the free stream) and the advected, diffused sine wave (AD with the
fused flux, exact solution translated and damped) are run on two grids; the
L1 error of the cell averages (aderdg_error_norms, analyze_soln's measure
against the exact solution at the final time) must fall with order close to
N+1.  The limiter is off: an a posteriori limiter flags cells of a coarse,
under-resolved grid (the reference's behaviour), which is not what an order
test measures -- except in the study of the vortex's own configuration (N = 4,
limiter on, grids 32 to 128), where the resolved grids must flag no cell.
The FP64 errors are also compared with the oracle's on the same grids.
"""
import numpy as np
import pytest

import aderdg
import pyoracle as po

pytestmark = pytest.mark.gpu


def _gpu_error(name, side, N, tend, precision, limited=None, **over):
    over.setdefault("limiter", 0)
    cfg, ic, params, _ = aderdg.workloads.make(name, side=side, N=N, precision=precision, **over)
    s = aderdg.Solver(cfg)
    s.initial_condition(ic, params)
    t, _ = s.run(0.0, tend, 1000000)
    assert t == tend
    e = s.error_norms(ic, params)[0]
    if limited is not None:
        limited.append(s.info()["n_limited"])
    s.close()
    return e


def _oracle_vortex_error(side, N, tend):
    w = aderdg.workloads.WORKLOADS["euler_vortex"]
    cfg = po.make_config(po.SYS_EULER, N, side, side, xl=w["xl"], xr=w["xr"], bc=(3, 3, 3, 3), limiter=0)
    o = po.Oracle(cfg)
    uh, _ = o.project_ic(w["ic"], w["params"])
    o.set(po.UH, uh)
    t = 0.0
    while t < tend:
        t, _, _ = o.step(t, tend)
    P = N + 1
    xi, wq = o.operator(po.OP_XI), o.operator(po.OP_W)
    L = w["xr"][0] - w["xl"][0]
    h = L / side
    ii, jj = np.meshgrid(np.arange(side), np.arange(side), indexing="xy")
    X = np.mod((ii[:, :, None, None] + xi[None, None, None, :]) * h - w["params"][4] * t, L)
    Y = np.mod((jj[:, :, None, None] + xi[None, None, :, None]) * h - w["params"][5] * t, L)
    X, Y = np.broadcast_arrays(X, Y)
    ex = np.array([po.initial_field(cfg, w["ic"], w["params"], float(x), float(y))[0]
                   for x, y in zip(X.ravel(), Y.ravel())]).reshape(side * side, P * P)
    u = o.get(po.UH).reshape(side * side, P * P, 4)[:, :, 0]
    W = np.outer(wq, wq).ravel()
    return np.abs((u - ex) @ W).mean()


@pytest.mark.parametrize("N", [2, 3])
def test_vortex_order_fp64(N, gpu_lib):
    e1 = _gpu_error("euler_vortex", 16, N, 1.0, aderdg.FP64)
    e2 = _gpu_error("euler_vortex", 32, N, 1.0, aderdg.FP64)
    order = np.log2(e1 / e2)
    assert order > N + 1 - 0.3, (e1, e2, order)
    # the same errors as the oracle's (the FP64 path agrees with it to rounding)
    o1 = _oracle_vortex_error(16, N, 1.0)
    assert abs(e1 - o1) <= 1e-6 * o1, (e1, o1)


def test_vortex_order_fp32_mixed(gpu_lib):
    N = 2
    e1 = _gpu_error("euler_vortex", 16, N, 1.0, aderdg.FP32_MIXED)
    e2 = _gpu_error("euler_vortex", 32, N, 1.0, aderdg.FP32_MIXED)
    order = np.log2(e1 / e2)
    assert order > N + 1 - 0.4, (e1, e2, order)


@pytest.mark.parametrize("N", [2, 3])
def test_ad_sine_order(N, gpu_lib):
    e1 = _gpu_error("ad_sine", 8, N, 0.05, aderdg.FP64, ad_flux_mode=1)
    e2 = _gpu_error("ad_sine", 16, N, 0.05, aderdg.FP64, ad_flux_mode=1)
    order = np.log2(e1 / e2)
    assert order > N + 1 - 0.6, (e1, e2, order)


def test_vortex_study_n4_limiter_on(gpu_lib):
    """The vortex's configuration (Euler, N = 4, limiter on, periodic
    [0,10]^2) on grids 32, 64 and 128 to t = 1, FP64: L1 error of the density
    cell averages against the exact solution (Euler/analyze_soln.f90:10-56's
    measure) and no limited cell.  Order N + 1 = 5 from 32 to 64 (measured
    4.7); from 64 to 128 the error (measured 1.3e-11) meets the floor of the
    test itself: the isolated vortex is not periodic on [0,10]^2 (its velocity
    perturbation at the domain edges is about 2e-5), so its periodic
    extension has a kink there that the scheme resolves at lower order
    (measured order 4.3)."""
    errs, limited = [], []
    for side in (32, 64, 128):
        errs.append(_gpu_error("euler_vortex", side, 4, 1.0, aderdg.FP64, limited=limited, limiter=1))
    orders = [float(np.log2(errs[k] / errs[k + 1])) for k in range(2)]
    print("vortex N=4, limiter on: L1 %s, orders %s, limited cells %s" % (errs, orders, limited))
    assert orders[0] > 5 - 0.35, (errs, orders)
    assert orders[1] > 5 - 1.0, (errs, orders)
    assert limited == [0, 0, 0], limited
