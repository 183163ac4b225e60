"""Helpers shared by the parity tests: oracle/GPU set-up side by side and the
error norms the tolerances are stated in."""
import numpy as np

import aderdg
import pyoracle as po


def oracle_config(cfg):
    return po.make_config(cfg.system, cfg.N, cfg.imax, cfg.jmax, xl=cfg.xl, xr=cfg.xr, bc=cfg.bc,
                          bc_mode=cfg.bc_mode, cfl=cfg.cfl, gamma=cfg.gamma, gamma_s=cfg.gamma_s,
                          gamma_g=cfg.gamma_g, pi_s=cfg.pi_s, pi_g=cfg.pi_g, cx=cfg.cx, cy=cfg.cy, a=cfg.a,
                          ad_flux_mode=cfg.ad_flux_mode, limiter=cfg.limiter)


def setup_pair(cfg, ic, params, with_gpu=True):
    """Oracle and GPU solver on the same projected initial field and initial limiter."""
    o = po.Oracle(oracle_config(cfg))
    uh, lh = o.project_ic(ic, params)
    o.set(po.UH, uh)
    nlim = o.init_limiter(lh) if cfg.limiter and cfg.system != aderdg.SYS_ADVDIFF else 0
    g = None
    if with_gpu:
        g = aderdg.Solver(cfg)
        g.upload(uh)
        ng = g.init_limiter(lh) if cfg.limiter and cfg.system != aderdg.SYS_ADVDIFF else 0
        assert ng == nlim, (ng, nlim)
    return o, g, uh, lh


def rel_l1(a, b):
    """sum |a - b| / sum |b|"""
    den = np.abs(b).sum()
    return float(np.abs(a - b).sum() / (den if den > 0 else 1.0))


def rel_linf(a, b):
    """max |a - b| / max |b|"""
    den = np.abs(b).max()
    return float(np.abs(a - b).max() / (den if den > 0 else 1.0))


def per_var(arr, V):
    return arr.reshape(-1, V)
