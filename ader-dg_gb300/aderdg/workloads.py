"""Named workloads: the four plain configurations and the seeded request mix.

Each plain workload returns (Config, initial-field id, parameters, end time).
The sizes are those of the configurations the reference is measured on; a
smaller `side` gives the same problem on a coarser grid for parity tests.
"""
import math

import numpy as np

from .core import (FP64, IC_AD_SINE, IC_BN_CYLINDER, IC_EULER_RP2D, IC_EULER_VORTEX, SYS_ADVDIFF, SYS_BN,
                   SYS_EULER, Config)

# scalar advection-diffusion, N=3, 64x64 periodic on [0,1]^2, c=(1,1), a=1e-3, u0 = sin(2 pi x) sin(2 pi y), t=1
AD_SINE = dict(system=SYS_ADVDIFF, N=3, side=64, xl=(0.0, 0.0), xr=(1.0, 1.0), bc=(3, 3, 3, 3), cx=1.0, cy=1.0,
               a=1e-3, limiter=0, ic=IC_AD_SINE, params=(1.0,), tend=1.0)
# Euler isentropic vortex, N=4, 256x256 periodic on [0,10]^2, eps=5 centred at (5,5), rho=u=v=p=1, t=10
EULER_VORTEX = dict(system=SYS_EULER, N=4, side=256, xl=(0.0, 0.0), xr=(10.0, 10.0), bc=(3, 3, 3, 3), limiter=1,
                    ic=IC_EULER_VORTEX, params=(5.0, 5.0, 5.0, 1.0, 1.0, 1.0, 1.0), tend=10.0)
# Euler four-quadrant 2D Riemann problem, N=3, 512x512 transmissive on [0,1]^2, split at (0.5,0.5), t=0.25
EULER_RP2D = dict(system=SYS_EULER, N=3, side=512, xl=(0.0, 0.0), xr=(1.0, 1.0), bc=(1, 1, 1, 1), limiter=1,
                  ic=IC_EULER_RP2D,
                  params=(0.5, 0.5, 1.5, 0.0, 0.0, 1.5, 0.5323, 1.206, 0.0, 0.3, 0.138, 1.206, 1.206, 0.029,
                          0.5323, 0.0, 1.206, 0.3),
                  tend=0.25)
# Baer-Nunziato cylindrical two-phase Riemann problem, N=3, 400x400 on [-0.5,0.5]^2, R=0.25, t=0.15
BN_CYLINDER = dict(system=SYS_BN, N=3, side=400, xl=(-0.5, -0.5), xr=(0.5, 0.5), bc=(1, 1, 1, 1), limiter=1,
                   gamma_s=1.4, gamma_g=1.4, pi_s=0.0, pi_g=0.0, ic=IC_BN_CYLINDER,
                   params=(0.0, 0.0, 0.25, 0.8, 1.0, 1.0, 0.5, 1.0, 0.3, 2.0, 2.0, 1.5, 2.0), tend=0.15)

WORKLOADS = {"ad_sine": AD_SINE, "euler_vortex": EULER_VORTEX, "euler_rp2d": EULER_RP2D, "bn_cylinder": BN_CYLINDER}


def make(name, side=None, N=None, precision=FP64, **over):
    """(Config, ic, params, tend) for a named workload."""
    w = dict(WORKLOADS[name])
    w.update(over)
    n = side or w["side"]
    cfg = Config(system=w["system"], N=N or w["N"], imax=n, jmax=n, xl=w["xl"], xr=w["xr"], bc=w["bc"],
                 limiter=w.get("limiter", 1), precision=precision, cx=w.get("cx", 1.0), cy=w.get("cy", 1.0),
                 a=w.get("a", 1e-3), gamma=w.get("gamma", 1.4), gamma_s=w.get("gamma_s", 1.4),
                 gamma_g=w.get("gamma_g", 1.4), pi_s=w.get("pi_s", 0.0), pi_g=w.get("pi_g", 0.0),
                 ad_flux_mode=w.get("ad_flux_mode", 0))
    return cfg, w["ic"], tuple(w["params"]), w["tend"]


def request_mix(n=1024, seed=0):
    """Seeded request mix: system uniform over the four base cases, N uniform in
    {2,3,4,5}, square grid side log-uniform in [32,512], every initial-field
    scalar jittered by U[0.9,1.1]; end time of the base case."""
    rng = np.random.default_rng(seed)
    names = list(WORKLOADS)
    out = []
    for _ in range(n):
        name = names[rng.integers(len(names))]
        N = int(rng.integers(2, 6))
        side = int(round(math.exp(rng.uniform(math.log(32), math.log(512)))))
        w = WORKLOADS[name]
        jit = rng.uniform(0.9, 1.1, size=len(w["params"]))
        params = tuple(float(p * j) for p, j in zip(w["params"], jit))
        out.append(dict(name=name, N=N, side=side, params=params, tend=w["tend"]))
    return out
