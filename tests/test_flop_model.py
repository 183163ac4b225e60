"""The predictor's flop model against an instrumented operation count.

`bench.predictor_flops_per_cell` gives the roofline's algorithmic flops of the
space-time predictor kernel (k_predictor).  Here the kernel's loop structure
(predictor.cuh: the per-node operator rows, the first Picard iteration with the
state constant in time, the middle iterations, the last one contracted to the
time average, the volume integral and the face extrapolation) is restated for
one cell in Python on a counting scalar.  Convention: every +, -, *, / on data
is one flop (a fused multiply-add counts 2, a division 1); constant zeros are
folded as a compiler folds them: an accumulation of n terms that starts from 0
is 2n - 1 flops, and the structurally zero components (Baer-Nunziato's ninth
flux component and the zero components of its non-conservative product) cost
nothing.  The restatement's outputs are checked against the oracle's
ader_space_time_predictor + volume_integral (Euler/space_time_predictor.f90:8-123,
Baer-Nunziato/space_time_predictor.f90:8-143,
Advection-Diffusion/space_time_predictor.f90:10-155, */volume_integral.f90), so
the count is that of a computation producing the reference's result, and the
model must equal it exactly.
"""
import numpy as np
import pytest

import bench
import pyoracle as po
from aderdg import workloads


class Z(float):
    """A structural (compile-time) zero: operations with it cost nothing."""

    def __add__(self, o): return o
    def __radd__(self, o): return o
    def __sub__(self, o): return -o
    def __rsub__(self, o): return o
    def __mul__(self, o): return ZERO
    def __rmul__(self, o): return ZERO
    def __neg__(self): return ZERO


ZERO = Z(0.0)


class Cnt:
    """A float that counts the arithmetic done on it."""
    n = 0
    __slots__ = ("x",)

    def __init__(self, x):
        self.x = float(x)

    @staticmethod
    def _v(o):
        return o.x if isinstance(o, Cnt) else float(o)

    def _op(self, r):
        Cnt.n += 1
        return Cnt(r)

    def __add__(self, o): return self if isinstance(o, Z) else self._op(self.x + Cnt._v(o))
    def __radd__(self, o): return self if isinstance(o, Z) else self._op(Cnt._v(o) + self.x)
    def __sub__(self, o): return self if isinstance(o, Z) else self._op(self.x - Cnt._v(o))
    def __rsub__(self, o): return -self if isinstance(o, Z) else self._op(Cnt._v(o) - self.x)
    def __mul__(self, o): return ZERO if isinstance(o, Z) else self._op(self.x * Cnt._v(o))
    def __rmul__(self, o): return ZERO if isinstance(o, Z) else self._op(Cnt._v(o) * self.x)
    def __truediv__(self, o): return self._op(self.x / Cnt._v(o))
    def __rtruediv__(self, o): return ZERO if isinstance(o, Z) else self._op(Cnt._v(o) / self.x)
    def __neg__(self): return Cnt(-self.x)


def fma(a, b, c):
    if isinstance(a, Z) or isinstance(b, Z):
        return c
    return a * b + c


def euler_pflux(pc, Q):
    """EulerSys::pflux (physics.cuh)."""
    ir = 1.0 / Q[0]
    u, v = Q[1] * ir, Q[2] * ir
    p = pc["gm1"] * (Q[3] - 0.5 * (Q[1] * u + Q[2] * v))
    e = Q[3] + p
    Fx = [Q[1], Q[1] * u + p, Q[2] * u, e * u]
    Fy = [Q[2], Q[1] * v, Q[2] * v + p, e * v]
    return Fx, Fy, None


def bn_pflux(pc, Q):
    """BNSys::pflux (physics.cuh): fluxes and the NCP scalars p_g, u_s, v_s."""
    a, b = Q[8], 1.0 - Q[8]
    irs, irg = 1.0 / Q[0], 1.0 / Q[4]
    us, vs = Q[1] * irs, Q[2] * irs
    ug, vg = Q[5] * irg, Q[6] * irg
    Ps = pc["gs1"] * (Q[3] - 0.5 * (Q[1] * us + Q[2] * vs)) - a * pc["gsps"]
    Pg = pc["gg1"] * (Q[7] - 0.5 * (Q[5] * ug + Q[6] * vg)) - b * pc["ggpg"]
    p_g = Pg / b
    es, eg = Q[3] + Ps, Q[7] + Pg
    Fx = [Q[1], Q[1] * us + Ps, Q[2] * us, es * us, Q[5], Q[5] * ug + Pg, Q[6] * ug, eg * ug, ZERO]
    Fy = [Q[2], Q[1] * vs, Q[2] * vs + Ps, es * vs, Q[6], Q[5] * vg, Q[6] * vg + Pg, eg * vg, ZERO]
    return Fx, Fy, (p_g, us, vs)


def bn_pncp(p_g, us, vs, ax, ay):
    """BNSys::pncp: NCP(q) . grad(alpha)."""
    un = us * ax + vs * ay
    return [ZERO, -p_g * ax, -p_g * ay, -p_g * un, ZERO, p_g * ax, p_g * ay, p_g * un, un]


def predictor_cell(ops, system, N, u_nodes, dt, dx, dy, pc, fused):
    """One cell of k_predictor.  u_nodes[node][v] (node = i + P j); returns the
    outputs qhi[node][v], Fhi[d][node][v], duh[node][v], qbnd[f][l][v],
    fbnd[f][l][v] (AD: gradQbnd[f][l][d]) and the flop count."""
    P, V = N + 1, po.NVAR[system]
    P2 = P * P
    Kxi, dudx, w, FL, FR = ops["Kxi"], ops["dudx"], ops["w"], ops["FL"], ops["FR"]
    T, g, ts, tw, wg = ops["T"], ops["g"], ops["ts"], ops["tw"], ops["wg"]
    dtc, dxc, dyc = Cnt(dt), Cnt(dx), Cnt(dy)
    Cnt.n = 0
    AD, BN = system == po.SYS_ADVDIFF, system == po.SYS_BN
    # per-node operator rows
    rows = []
    for node in range(P2):
        i, j = node % P, node // P
        cxw = (dtc / dxc) / w[i]
        cyw = (dtc / dyc) / w[j]
        Dx = [Kxi[k + P * i] * cxw for k in range(P)]
        Dy = [Kxi[k + P * j] * cyw for k in range(P)]
        Gx = Gy = None
        if AD or BN:
            Gx = [dudx[i + P * k] / dxc for k in range(P)]
            Gy = [dudx[j + P * k] / dyc for k in range(P)]
        rows.append((Dx, Dy, Gx, Gy))
    u = [[Cnt(x) for x in u_nodes[n]] for n in range(P2)]

    def contract(F, l, node):
        """b[v] = sum_k Dx(i,k) Fx(k,j,l) + sum_k Dy(j,k) Fy(i,k,l)."""
        i, j = node % P, node // P
        Dx, Dy = rows[node][0], rows[node][1]
        b = [ZERO] * V
        for k in range(P):
            for v in range(V):
                b[v] = fma(Dx[k], F[l][0][k + P * j][v], b[v])
        for k in range(P):
            for v in range(V):
                b[v] = fma(Dy[k], F[l][1][i + P * k][v], b[v])
        return b

    def grad(A, l, node):
        i, j = node % P, node // P
        Gx, Gy = rows[node][2], rows[node][3]
        gx, gy = ZERO, ZERO
        for k in range(P):
            gx = fma(Gx[k], A[l][k + P * j], gx)
            gy = fma(Gy[k], A[l][i + P * k], gy)
        return gx, gy

    F = [[[None] * P2, [None] * P2] for _ in range(P)]  # F[l][d][node] = V fluxes
    A = [[None] * P2 for _ in range(P)]                 # AD state / BN volume fraction [l][node]
    Fh = [[None] * P2, [None] * P2]                  # time-averaged fluxes [d][node]
    qh, Sh, Gh = [None] * P2, [None] * P2, [None] * P2
    q = [None] * P2
    if AD:
        ca, ccx, ccy = pc["a"], pc["cx"], pc["cy"]

        def ad_flux(l, node, qv):
            gx, gy = grad(A, l, node)
            fx, fy = -ca * gx, -ca * gy
            if fused:
                fx, fy = fma(ccx, qv, fx), fma(ccy, qv, fy)
            return gx, gy, fx, fy
        for node in range(P2):
            A[0][node] = u[node][0]
        for node in range(P2):
            _, _, fx, fy = ad_flux(0, node, u[node][0])
            F[0][0][node], F[0][1][node] = [fx], [fy]
        for node in range(P2):
            b = contract(F, 0, node)
            q[node] = [[g[l] * u[node][0] - ts[l] * b[0]] for l in range(P)]
        for it in range(2, P + 1):
            last = it == P
            for node in range(P2):
                for l in range(P):
                    A[l][node] = q[node][l][0]
            H = [None] * P2
            for node in range(P2):
                fh = [ZERO, ZERO]
                gh = [ZERO, ZERO]
                hh = [ZERO, ZERO]
                for l in range(P):
                    gx, gy, fx, fy = ad_flux(l, node, q[node][l][0])
                    F[l][0][node], F[l][1][node] = [fx], [fy]
                    if last:
                        fh = [fma(w[l], fx, fh[0]), fma(w[l], fy, fh[1])]
                        gh = [fma(w[l], gx, gh[0]), fma(w[l], gy, gh[1])]
                        hh = [fma(tw[l], fx, hh[0]), fma(tw[l], fy, hh[1])]
                if last:
                    Fh[0][node], Fh[1][node], Gh[node] = [fh[0]], [fh[1]], gh
                    H[node] = hh
            if last:  # the combined flux H = sum_l tw_l F_l, contracted once
                for node in range(P2):
                    F[0][0][node], F[0][1][node] = [H[node][0]], [H[node][1]]
            for node in range(P2):
                if not last:
                    qn = [[g[l] * u[node][0]] for l in range(P)]
                    for l in range(P):
                        b = contract(F, l, node)
                        for lp in range(P):
                            qn[lp][0] = fma(-T[lp + P * l], b[0], qn[lp][0])
                    q[node] = qn
                else:
                    b = contract(F, 0, node)
                    qh[node] = [wg * u[node][0] - b[0]]
    else:
        flux = bn_pflux if BN else euler_pflux
        ncp = [[None] * P2 for _ in range(P)]
        for node in range(P2):
            Fx, Fy, s = flux(pc, u[node])
            F[0][0][node], F[0][1][node] = Fx, Fy
            if BN:
                ncp[0][node] = s
                A[0][node] = u[node][8]
        for node in range(P2):
            b = contract(F, 0, node)
            if BN:
                ax, ay = grad(A, 0, node)
                n = bn_pncp(*ncp[0][node], ax, ay)
                b = [fma(dtc, n[v], b[v]) for v in range(V)]
            q[node] = [[g[l] * u[node][v] - ts[l] * b[v] for v in range(V)] for l in range(P)]
        for it in range(2, P + 1):
            last = it == P
            H = [None] * P2
            for node in range(P2):
                fh = [[ZERO] * V, [ZERO] * V]
                hh = [[ZERO] * V, [ZERO] * V]
                for l in range(P):
                    Fx, Fy, s = flux(pc, q[node][l])
                    F[l][0][node], F[l][1][node] = Fx, Fy
                    if BN:
                        ncp[l][node] = s
                        A[l][node] = q[node][l][8]
                    if last:
                        fh = [[fma(w[l], Fx[v], fh[0][v]) for v in range(V)],
                              [fma(w[l], Fy[v], fh[1][v]) for v in range(V)]]
                        hh = [[fma(tw[l], Fx[v], hh[0][v]) for v in range(V)],
                              [fma(tw[l], Fy[v], hh[1][v]) for v in range(V)]]
                if last:
                    Fh[0][node], Fh[1][node] = fh
                    H[node] = hh
            if last:
                # the last iteration contracts the combined flux H = sum_l tw_l F_l once
                for node in range(P2):
                    F[0][0][node], F[0][1][node] = H[node]
            for node in range(P2):
                if not last:
                    qn = [[g[l] * u[node][v] for v in range(V)] for l in range(P)]
                    for l in range(P):
                        b = contract(F, l, node)
                        if BN:
                            ax, ay = grad(A, l, node)
                            n = bn_pncp(*ncp[l][node], ax, ay)
                            b = [fma(dtc, n[v], b[v]) for v in range(V)]
                        for lp in range(P):
                            qn[lp] = [fma(-T[lp + P * l], b[v], qn[lp][v]) for v in range(V)]
                else:
                    acc = [wg * u[node][v] for v in range(V)]
                    sh = [ZERO] * V
                    b = contract(F, 0, node)
                    acc = [acc[v] - b[v] for v in range(V)]
                    if BN:
                        for l in range(P):
                            ax, ay = grad(A, l, node)
                            n = bn_pncp(*ncp[l][node], ax, ay)
                            c = tw[l] * dtc
                            sh = [fma(-w[l], n[v], sh[v]) for v in range(V)]
                            acc = [fma(-c, n[v], acc[v]) for v in range(V)]
                if not last:
                    q[node] = qn
                else:
                    qh[node] = acc
                    Sh[node] = sh
    # epilogue: volume integral (predictor_outputs, kVolume) and face extrapolation
    duh = [None] * P2
    for node in range(P2):
        i, j = node % P, node // P
        vx, vy = w[j] / dxc, w[i] / dyc
        d = []
        for v in range(V):
            sx, sy = ZERO, ZERO
            for k in range(P):
                sx = fma(Kxi[i + P * k], Fh[0][k + P * j][v], sx)
                sy = fma(Kxi[j + P * k], Fh[1][i + P * k][v], sy)
            dv = sx * vx + sy * vy
            if BN:
                dv = fma(w[i] * w[j], Sh[node][v], dv)
            d.append(dv)
        duh[node] = d
    qb = [[None] * P for _ in range(4)]
    fb = [[None] * P for _ in range(4)]
    for f in range(4):
        c = FL if f in (0, 2) else FR
        xdir = f < 2
        for l in range(P):
            nds = [(m + P * l) if xdir else (l + P * m) for m in range(P)]
            sq, sf = [], []
            for v in range(V):
                a, b2 = ZERO, ZERO
                for m in range(P):
                    a = fma(c[m], qh[nds[m]][v], a)
                    if not AD:
                        b2 = fma(c[m], Fh[0 if xdir else 1][nds[m]][v], b2)
                sq.append(a)
                sf.append(b2)
            if AD:
                sf = []
                for dd in range(2):
                    a = ZERO
                    for m in range(P):
                        a = fma(c[m], Gh[nds[m]][dd], a)
                    sf.append(a)
            qb[f][l], fb[f][l] = sq, sf
    return dict(qhi=qh, Fhi=Fh, duh=duh, qbnd=qb, fbnd=fb, flops=Cnt.n)


CASES = [(po.SYS_EULER, 1, False), (po.SYS_EULER, 2, False), (po.SYS_EULER, 4, False), (po.SYS_EULER, 5, False),
         (po.SYS_BN, 2, False), (po.SYS_BN, 3, False), (po.SYS_BN, 5, False),
         (po.SYS_ADVDIFF, 2, True), (po.SYS_ADVDIFF, 3, True), (po.SYS_ADVDIFF, 3, False), (po.SYS_ADVDIFF, 5, True)]


def _setup(system, N, fused):
    # a 3x3 patch of the base case's domain around its centre (vortex, cylinder, sine wave)
    w = workloads.WORKLOADS[{po.SYS_EULER: "euler_vortex", po.SYS_BN: "bn_cylinder",
                             po.SYS_ADVDIFF: "ad_sine"}[system]]
    cx, cy = [(a + b) / 2 for a, b in zip(w["xl"], w["xr"])]
    h = 0.15 * (w["xr"][0] - w["xl"][0])
    cfg = po.make_config(system, N, 3, 3, xl=(cx - 1.5 * h, cy - 1.5 * h), xr=(cx + 1.5 * h, cy + 1.5 * h),
                         bc=(3, 3, 3, 3), ad_flux_mode=1 if fused else 0)
    o = po.Oracle(cfg)
    uh, _ = o.project_ic(w["ic"], w["params"])
    # a generic smooth perturbation so that no term vanishes by symmetry
    rng = np.random.default_rng(system * 10 + N)
    V = po.NVAR[system]
    uh = uh.reshape(-1, V)
    if system == po.SYS_ADVDIFF:
        uh = uh + 0.1 * rng.standard_normal(uh.shape)
    else:
        uh = uh * (1.0 + 0.02 * rng.standard_normal(uh.shape))
        if system == po.SYS_BN:
            uh[:, 8] = np.clip(uh[:, 8], 0.05, 0.95)
    uh = uh.ravel()
    o.set(po.UH, uh)
    return cfg, o, uh


def _ops(o, P):
    Kxi, dudx, w = o.operator(po.OP_KXI), o.operator(po.OP_DUDX), o.operator(po.OP_W)
    FL, FR, iK1, F0 = o.operator(po.OP_FL), o.operator(po.OP_FR), o.operator(po.OP_IK1), o.operator(po.OP_F0)
    T = [0.0] * (P * P)  # T(l', l) = iK1(l', l) w_l at T[l' + P l]
    g, ts = [0.0] * P, [0.0] * P
    for lp in range(P):
        for l in range(P):
            T[lp + P * l] = iK1[lp + P * l] * w[l]
            g[lp] += iK1[lp + P * l] * F0[l]
            ts[lp] += T[lp + P * l]
    tw = [sum(w[lp] * T[lp + P * l] for lp in range(P)) for l in range(P)]
    wg = sum(w[lp] * g[lp] for lp in range(P))
    return dict(Kxi=list(Kxi), dudx=list(dudx), w=list(w), FL=list(FL), FR=list(FR), T=T, g=g, ts=ts, tw=tw, wg=wg)


@pytest.mark.parametrize("system,N,fused", CASES)
def test_flop_model_equals_instrumented_count(system, N, fused):
    cfg, o, uh = _setup(system, N, fused)
    P, V = N + 1, po.NVAR[system]
    P2 = P * P
    dt = 0.5 * o.calc_time_step(0.0, 1.0e9) if system != po.SYS_ADVDIFF else 1.0e-3
    o.set_dt(dt)
    o.predictor()
    o.volume_integral()
    pc = dict(gm1=cfg.gamma - 1.0, gs1=cfg.gamma_s - 1.0, gg1=cfg.gamma_g - 1.0, gsps=cfg.gamma_s * cfg.pi_s,
              ggpg=cfg.gamma_g * cfg.pi_g, a=cfg.a, cx=cfg.cx, cy=cfg.cy)
    dx = (cfg.xr[0] - cfg.xl[0]) / cfg.imax
    dy = (cfg.xr[1] - cfg.xl[1]) / cfg.jmax
    cell = 4  # the centre of the 3x3 grid
    un = uh.reshape(-1, P2, V)[cell]
    r = predictor_cell(_ops(o, P), system, N, un, dt, dx, dy, pc, fused)
    assert r["flops"] == bench.predictor_flops_per_cell(system, N, ad_fused=fused)

    def val(x):
        return x.x if isinstance(x, Cnt) else float(x)
    qhi = o.get(po.QHI).reshape(-1, P2, V)[cell]
    duh = o.get(po.DUH).reshape(-1, P2, V)[cell]
    fhi = o.get(po.FHI).reshape(-1, P2, 2, V)[cell]
    got_q = np.array([[val(x) for x in r["qhi"][n]] for n in range(P2)])
    got_d = np.array([[val(x) for x in r["duh"][n]] for n in range(P2)])
    got_f = np.array([[[val(x) for x in r["Fhi"][d][n]] for d in range(2)] for n in range(P2)])
    scale = lambda a: np.abs(a).max() + 1e-300  # noqa: E731
    assert np.abs(qhi).max() > 0.0 and np.abs(fhi).max() > 0.0 and np.abs(duh).max() > 0.0
    assert np.abs(got_q - qhi).max() <= 1e-12 * scale(qhi)
    assert np.abs(got_f - fhi).max() <= 1e-12 * scale(fhi)
    assert np.abs(got_d - duh).max() <= 1e-11 * scale(duh)
    # face extrapolation: qbnd(v, f, l), fbnd(v, f, l) (AD: gradQbnd(v, d, f, l))
    qb = o.get(po.QBND).reshape(-1, P, 4, V)[cell]
    got_qb = np.array([[[val(x) for x in r["qbnd"][f][l]] for f in range(4)] for l in range(P)])
    assert np.abs(got_qb - qb).max() <= 1e-12 * scale(qb)
    if system == po.SYS_ADVDIFF:
        gb = o.get(po.GRADQBND).reshape(-1, P, 4, 2, V)[cell][..., 0]
        got = np.array([[[val(x) for x in r["fbnd"][f][l]] for f in range(4)] for l in range(P)])
        assert np.abs(got - gb).max() <= 1e-11 * scale(gb)
    else:
        fb = o.get(po.FBND).reshape(-1, P, 4, V)[cell]
        got = np.array([[[val(x) for x in r["fbnd"][f][l]] for f in range(4)] for l in range(P)])
        assert np.abs(got - fb).max() <= 1e-12 * scale(fb)
