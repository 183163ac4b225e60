"""Order of accuracy of the GPU path on the smooth cases.

The isentropic vortex (Euler, periodic, exact solution = the initial vortex
carried by the free stream) and the advected, diffused sine wave (AD with the
fused flux, exact solution translated and damped) are run on two grids; the
L1 error of the cell averages (aderdg_error_norms, analyze_soln's measure
against the exact solution at the final time) must fall with order close to
N+1.  The limiter is off: an a posteriori limiter flags cells of a coarse,
under-resolved grid (the reference's behaviour), which is not what an order
test measures.  The FP64 errors are also compared with the oracle's on the
same grids.
"""
import numpy as np
import pytest

import aderdg
import pyoracle as po

pytestmark = pytest.mark.gpu


def _gpu_error(name, side, N, tend, precision, **over):
    cfg, ic, params, _ = aderdg.workloads.make(name, side=side, N=N, precision=precision, limiter=0, **over)
    s = aderdg.Solver(cfg)
    s.initial_condition(ic, params)
    t, _ = s.run(0.0, tend, 1000000)
    assert t == tend
    e = s.error_norms(ic, params)[0]
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
