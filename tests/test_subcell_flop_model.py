"""The subcell re-solve's flop model against an instrumented count.

`bench.subcell_flops_per_cell` gives the roofline's algorithmic flops of the
subcell re-solve kernel (k_subcell), the dominant kernel of the FP32-mixed
step.  Here the re-solve of one cell is restated in Python on the counting
scalar of test_flop_model (every +, -, *, /, sqrt on data is one
flop, a fused multiply-add 2, an accumulation of n terms from zero 2n - 1;
compares, min/max, |x| and sign tests are free), computing exactly what the
result needs:

- the subcell data of the neighbourhood that the reconstruction reads: the
  interior subcells and the four strips beside them (Euler's slopes are
  formed on the interior only, Euler/limiter.f90:529-536), by the y and then
  the x contraction of get_subcell_data (Euler/limiter.f90:12-37);
- MUSCL-Hancock on the interior subcells (Euler/limiter.f90:538-566): the halo
  subcells have zero slopes, so their half-step flux differences vanish and
  their face states are their values;
- the Rusanov fluxes of the subgrid edges (Euler/limiter.f90:568-588, 361-378)
  with the flux along the edge normal only, the finite-volume update
  (:590-597) and put_subcell_data (:74-98);
- for a recompute = 2 cell, the DMP of the new polynomial (:179-245: subcell
  and Gauss-Lobatto projections, thresholds, the pressure of every subcell);
- the CFL denominator of every node of the new polynomial
  (Euler/calc_time_step.f90:9-52).

Baer-Nunziato (resolve_cell_bn) adds the slopes, the NCP source and the half
step on the halo subcells (two rings of neighbour subcells; the ring's
corners feed no edge), the path-conservative fluctuation of every edge and
the NCP source at the half step in the finite-volume update.

The restatement's results are checked against the oracle's limiter step on a
5 x 5 grid (the isentropic vortex; a smooth two-phase state for
Baer-Nunziato) whose centre cell is forced troubled (recompute = 1; its edge
neighbours become recompute = 2): the new subcell data, the new polynomial
and the DMP verdict of a recompute = 2 neighbour.  The model must equal the
count exactly.
"""
import math

import numpy as np
import pytest

import bench
import pyoracle as po
from aderdg import workloads
from helpers import oracle_config
from test_flop_model import Cnt, ZERO


def csqrt(a):
    Cnt.n += 1
    return Cnt(math.sqrt(a.x))


def cabs(a):
    return Cnt(abs(a.x))


def cmax(a, b):
    return a if a.x >= b.x else b


def minmod(a, b):
    """Euler/limiter.f90:384-405 (the sign test is not arithmetic)."""
    if a.x * b.x <= 0.0:
        return Cnt(0.0)
    return a if abs(a.x) < abs(b.x) else b


def flux_dir(Q, d, gm1, gamma, eig=False):
    """The flux along axis d (Euler/pde.f90:46-69, one direction) with one
    reciprocal of the density, and maxval(abs(Lambda)) along d
    (Euler/pde.f90:75-91) as |u_n| + c."""
    irho = 1.0 / Q[0]
    u, v = Q[1] * irho, Q[2] * irho
    p = gm1 * (Q[3] - 0.5 * (Q[1] * u + Q[2] * v))
    un = u if d == 0 else v
    F = [Q[1] if d == 0 else Q[2],
         Q[1] * un + p if d == 0 else Q[1] * un,
         Q[2] * un if d == 0 else Q[2] * un + p,
         un * (Q[3] + p)]
    if not eig:
        return F, None
    c = csqrt(gamma * p * irho)
    return F, cabs(un) + c


def pressure(Q, gm1):
    return gm1 * (Q[3] - 0.5 * (Q[1] * Q[1] + Q[2] * Q[2]) / Q[0])


def resolve_cell(nb, rec, ops, N, dt, dx, dy, gamma, lmin=None, lmax=None):
    """Re-solve of one Euler cell.  nb[(bi, bj)] = the start-of-step uh of the
    neighbour (bi, bj) as [v][kx + P ky] (all neighbours unlimited); returns
    the new subcell data sub1[v][a + S b], the new polynomial un[v][kx + P ky],
    the DMP verdict (recompute = 2; None otherwise), the CFL denominators and
    the flop count."""
    P, S, V = N + 1, 2 * N + 1, 4
    uh2lim, lim2uh, uh2lob = ops["uh2lim"], ops["lim2uh"], ops["uh2lob"]
    gm1 = gamma - 1.0
    Cnt.n = 0
    dtc, dxc, dyc = Cnt(dt), Cnt(dx), Cnt(dy)
    nbc = {k: [[Cnt(x) for x in row] for row in u] for k, u in nb.items()}
    ldx, ldy = dxc / S, dyc / S
    dtx, dty, hdt = dtc / ldx, dtc / ldy, 0.5 * dtc

    # ---- gather: y contraction of each neighbour's rows, cached, then x
    LY = {}

    def ly(bi, bj, v, kk, sb):
        key = (bi, bj, v, kk, sb)
        if key not in LY:
            acc = ZERO
            for m in range(P):
                acc = acc + nbc[(bi, bj)][v][kk + P * m] * uh2lim[sb + S * m]
            LY[key] = acc
        return LY[key]

    need = [(ii, jj) for jj in range(1, S + 1) for ii in range(1, S + 1)]
    need += [(ii, jj) for jj in range(1, S + 1) for ii in (0, S + 1)]
    need += [(ii, jj) for jj in (0, S + 1) for ii in range(1, S + 1)]
    SU = {}
    for ii, jj in need:
        bi = -1 if ii < 1 else (1 if ii > S else 0)
        bj = -1 if jj < 1 else (1 if jj > S else 0)
        sa, sb = ii - 1 - bi * S, jj - 1 - bj * S
        for v in range(V):
            acc = ZERO
            for kk in range(P):
                acc = acc + ly(bi, bj, v, kk, sb) * uh2lim[sa + S * kk]
            SU[(v, ii, jj)] = acc

    # ---- MUSCL-Hancock: interior subcells; halo face states are the values
    wLx, wRx, wLy, wRy = {}, {}, {}, {}
    for ii, jj in need:
        if 1 <= ii <= S and 1 <= jj <= S:
            continue
        for v in range(V):
            wLx[(v, ii, jj)] = wRx[(v, ii, jj)] = wLy[(v, ii, jj)] = wRy[(v, ii, jj)] = SU[(v, ii, jj)]
    for jj in range(1, S + 1):
        for ii in range(1, S + 1):
            q0 = [SU[(v, ii, jj)] for v in range(V)]
            sx = [minmod(SU[(v, ii + 1, jj)] - q0[v], q0[v] - SU[(v, ii - 1, jj)]) for v in range(V)]
            sy = [minmod(SU[(v, ii, jj + 1)] - q0[v], q0[v] - SU[(v, ii, jj - 1)]) for v in range(V)]
            hx_ = [0.5 * sx[v] for v in range(V)]
            hy_ = [0.5 * sy[v] for v in range(V)]
            wlx = [q0[v] - hx_[v] for v in range(V)]
            wrx = [q0[v] + hx_[v] for v in range(V)]
            wly = [q0[v] - hy_[v] for v in range(V)]
            wry = [q0[v] + hy_[v] for v in range(V)]
            FLx, _ = flux_dir(wlx, 0, gm1, gamma)
            FRx, _ = flux_dir(wrx, 0, gm1, gamma)
            FLy, _ = flux_dir(wly, 1, gm1, gamma)
            FRy, _ = flux_dir(wry, 1, gm1, gamma)
            for v in range(V):
                qt = -((FRx[v] - FLx[v]) / ldx)
                qt = qt - (FRy[v] - FLy[v]) / ldy
                g = hdt * qt
                wLx[(v, ii, jj)] = wlx[v] + g
                wRx[(v, ii, jj)] = wrx[v] + g
                wLy[(v, ii, jj)] = wly[v] + g
                wRy[(v, ii, jj)] = wry[v] + g

    # ---- Rusanov fluxes of the subgrid edges
    def rusanov(QL, QR, d):
        FL, eL = flux_dir(QL, d, gm1, gamma, eig=True)
        FR, eR = flux_dir(QR, d, gm1, gamma, eig=True)
        hs = 0.5 * cmax(eL, eR)
        return [0.5 * (FL[v] + FR[v]) - hs * (QR[v] - QL[v]) for v in range(V)]

    Fx = {(ii, jj): rusanov([wRx[(v, ii - 1, jj)] for v in range(V)], [wLx[(v, ii, jj)] for v in range(V)], 0)
          for jj in range(1, S + 1) for ii in range(1, S + 2)}
    Fy = {(ii, jj): rusanov([wRy[(v, ii, jj - 1)] for v in range(V)], [wLy[(v, ii, jj)] for v in range(V)], 1)
          for jj in range(1, S + 2) for ii in range(1, S + 1)}

    # ---- finite-volume update
    sub1 = [[None] * (S * S) for _ in range(V)]
    for jj in range(1, S + 1):
        for ii in range(1, S + 1):
            for v in range(V):
                sub1[v][(ii - 1) + S * (jj - 1)] = (SU[(v, ii, jj)] - dtx * (Fx[(ii + 1, jj)][v] - Fx[(ii, jj)][v])
                                                    - dty * (Fy[(ii, jj + 1)][v] - Fy[(ii, jj)][v]))

    # ---- put_subcell_data
    luhy = [[[None] * V for _ in range(S)] for _ in range(P)]
    for iii in range(S):
        for s in range(P):
            for v in range(V):
                acc = ZERO
                for k in range(S):
                    acc = acc + sub1[v][iii + S * k] * lim2uh[s + P * k]
                luhy[s][iii][v] = acc
    un = [[None] * (P * P) for _ in range(V)]
    for jjj in range(P):
        for s in range(P):
            for v in range(V):
                acc = ZERO
                for k in range(S):
                    acc = acc + luhy[jjj][k][v] * lim2uh[s + P * k]
                un[v][s + P * jjj] = acc

    # ---- DMP of the new polynomial (recompute = 2)
    verdict = None
    if rec == 2:
        def project(op, n_out):
            y = [[[None] * V for _ in range(P)] for _ in range(n_out)]
            for iii in range(P):
                for s in range(n_out):
                    for v in range(V):
                        acc = ZERO
                        for k in range(P):
                            acc = acc + un[v][iii + P * k] * op[s + n_out * k]
                        y[s][iii][v] = acc
            out = [[None] * (n_out * n_out) for _ in range(V)]
            for jjj in range(n_out):
                for s in range(n_out):
                    for v in range(V):
                        acc = ZERO
                        for k in range(P):
                            acc = acc + y[jjj][k][v] * op[s + n_out * k]
                        out[v][s + n_out * jjj] = acc
            return out
        lim = project(uh2lim, S)
        lob = project(uh2lob, P)
        verdict = True
        for v in range(V):
            vals = [x.x for x in un[v] + lim[v] + lob[v]]
            lo, hi = Cnt(lmin[v]), Cnt(lmax[v])
            ldiff = max(1.0e-4, (1.0e-3 * (hi - lo)).x)
            if min(vals) < (lo - ldiff).x or max(vals) > (hi + ldiff).x:
                verdict = False
        for k in range(S * S):
            Q = [lim[v][k] for v in range(V)]
            if Q[0].x <= 1.0e-12 or pressure(Q, gm1).x <= 1.0e-12:
                verdict = False

    # ---- CFL denominators of the new polynomial's nodes
    den = []
    for k in range(P * P):
        Q = [un[v][k] for v in range(V)]
        p = pressure(Q, gm1)
        c = csqrt(gamma * p / Q[0])
        u, w = Q[1] / Q[0], Q[2] / Q[0]
        ex = cmax(cmax(cabs(u - c), cabs(u)), cabs(u + c))
        ey = cmax(cmax(cabs(w - c), cabs(w)), cabs(w + c))
        den.append(ex / dxc + ey / dyc)
    return sub1, un, verdict, den, Cnt.n


def _oracle_step(N, workload="euler_vortex", V=4):
    """The oracle's phases of one step on a 5 x 5 isentropic-vortex grid, the
    centre cell forced troubled; the start-of-step state and the limiter's
    results."""
    I = J = 5
    wcfg, ic, params, _ = workloads.make(workload, side=I, N=N)
    cfg = oracle_config(wcfg)
    o = po.Oracle(cfg)
    uh, _ = o.project_ic(ic, params)
    if V == 9:
        uh = _smooth_bn(cfg, N, I, J)
    o.set(po.UH, uh)
    dt = o.calc_time_step(0.0, 1.0)
    o.set_dt(dt)
    o.get_min_max()
    lmin, lmax = o.get(po.LMIN).copy(), o.get(po.LMAX).copy()
    o.save_olduh()
    old = o.get(po.OLDUH).copy()
    o.predictor()
    o.volume_integral()
    o.riemann()
    o.surface_integral()
    o.element_update()
    rec = np.zeros(I * J, dtype=np.int32)
    rec[2 + I * 2] = 1
    o.set_int(po.RECOMPUTE, rec)
    o.limiter()
    P, S = N + 1, 2 * N + 1
    ops = {"uh2lim": o.operator(po.OP_UH2LIM), "lim2uh": o.operator(po.OP_LIM2UH), "uh2lob": o.operator(po.OP_UH2LOB)}
    return dict(I=I, cfg=cfg, dt=dt, dx=(cfg.xr[0] - cfg.xl[0]) / I, dy=(cfg.xr[1] - cfg.xl[1]) / J,
                gamma=cfg.gamma, ops=ops, old=old.reshape(J, I, P * P, V), uh=o.get(po.UH).reshape(J, I, P * P, V),
                newlh=o.get(po.NEWLH).reshape(J, I, S * S, V), status=o.get_int(po.STATUS).reshape(J, I),
                lmin=lmin.reshape(J, I, V), lmax=lmax.reshape(J, I, V))


def _smooth_bn(cfg, N, I, J):
    """A smooth two-phase state (perturbations of about 10% around a uniform
    one) as the nodal values of every cell: a cylinder on a 5 x 5 grid is too
    coarse for its reconstruction to stay admissible."""
    P = N + 1
    gs, gg, ps, pg = cfg.gamma_s, cfg.gamma_g, cfg.pi_s, cfg.pi_g
    uh = np.empty((J, I, P * P, 9))
    for j in range(J):
        for i in range(I):
            for node in range(P * P):
                x, y = i + 0.37 * (node % P), j + 0.41 * (node // P)
                a = 0.5 + 0.1 * math.sin(0.9 * x + 0.4 * y)
                rs, us, vs, p_s = 1.0 + 0.1 * math.cos(0.7 * x), 0.2 * math.sin(0.5 * y), 0.1 * math.cos(0.6 * x), 1.0
                rg, ug, vg, p_g = 0.5 + 0.05 * math.sin(0.8 * y), 0.1 * math.cos(0.4 * x), 0.2, 1.0 + 0.1 * math.sin(x)
                q0, q4 = a * rs, (1.0 - a) * rg
                es = 0.5 * (us * us + vs * vs) + (p_s + gs * ps) / (rs * (gs - 1.0))
                eg = 0.5 * (ug * ug + vg * vg) + (p_g + gg * pg) / (rg * (gg - 1.0))
                uh[j, i, node] = [q0, q0 * us, q0 * vs, q0 * es, q4, q4 * ug, q4 * vg, q4 * eg, a]
    return uh.ravel()


def _neighbourhood(r, i, j):
    return {(bi, bj): [list(r["old"][j + bj, i + bi, :, v]) for v in range(r["old"].shape[-1])]
            for bj in (-1, 0, 1) for bi in (-1, 0, 1)}


def _vals(a):
    return np.array([[x.x for x in row] for row in a])


@pytest.mark.parametrize("N", [1, 2, 3, 4, 5])
def test_euler_subcell_flop_model_equals_instrumented_count(N):
    r = _oracle_step(N)
    args = (r["ops"], N, r["dt"], r["dx"], r["dy"], r["gamma"])
    # the troubled centre cell (recompute = 1)
    sub1, un, verdict, _, n1 = resolve_cell(_neighbourhood(r, 2, 2), 1, *args)
    ref = r["newlh"][2, 2].T
    assert np.abs(_vals(sub1) - ref).max() <= 1e-12 * np.abs(ref).max(), N
    ref = r["uh"][2, 2].T
    assert np.abs(_vals(un) - ref).max() <= 1e-12 * np.abs(ref).max(), N
    assert verdict is None
    # its right neighbour (recompute = 2): new polynomial and DMP verdict
    sub2, un2, verdict2, den, n2 = resolve_cell(_neighbourhood(r, 3, 2), 2, *args,
                                                lmin=r["lmin"][2, 3], lmax=r["lmax"][2, 3])
    ref = r["uh"][2, 3].T
    assert np.abs(_vals(un2) - ref).max() <= 1e-12 * np.abs(ref).max(), N
    assert verdict2 == (r["status"][2, 3] == 0), (N, verdict2, r["status"][2, 3])
    assert all(d.x > 0 for d in den)
    # the model equals the count
    assert bench.subcell_flops_per_cell(po.SYS_EULER, N, dmp=False) == n1, (N, n1)
    assert bench.subcell_flops_per_cell(po.SYS_EULER, N) == n2, (N, n2)


# ------------------------------------------------------------ Baer-Nunziato
def bn_flux_dir(Q, d, pc, eig=False):
    """The flux along axis d (Baer-Nunziato/pde.f90:74-119, one direction)
    from one reciprocal of Q0 Q4, and maxval(abs(Lambda)) along d (:125-144)
    as max(|u_g| + a_g, |u_s| + a_s)."""
    r = 1.0 / (Q[0] * Q[4])
    i0, i4 = Q[4] * r, Q[0] * r
    us_, vs_, ug_, vg_ = Q[1] * i0, Q[2] * i0, Q[5] * i4, Q[6] * i4
    phg = 1.0 - Q[8]
    pps = pc["gs1"] * (Q[3] - 0.5 * (Q[1] * us_ + Q[2] * vs_)) - pc["gsps"] * Q[8]
    ppg = pc["gg1"] * (Q[7] - 0.5 * (Q[5] * ug_ + Q[6] * vg_)) - pc["ggpg"] * phg
    us, ug = (us_, ug_) if d == 0 else (vs_, vg_)
    F = [Q[1] if d == 0 else Q[2],
         Q[1] * us + pps if d == 0 else Q[1] * us,
         Q[2] * us if d == 0 else Q[2] * us + pps,
         us * (Q[3] + pps),
         Q[5] if d == 0 else Q[6],
         Q[5] * ug + ppg if d == 0 else Q[5] * ug,
         Q[6] * ug if d == 0 else Q[6] * ug + ppg,
         ug * (Q[7] + ppg),
         ZERO]
    if not eig:
        return F, None
    a_s = csqrt(pc["gs"] * (pps + pc["ps"] * Q[8]) * i0)
    a_g = csqrt(pc["gg"] * (ppg + pc["pg"] * phg) * i4)
    return F, cmax(cabs(ug) + a_g, cabs(us) + a_s)


def bn_pg_un(Q, qn, pc):
    """p_g and u_n = qn / Q0 from one reciprocal of Q0 Q4 (1 - Q8)."""
    b = Q[4] * (1.0 - Q[8])
    r = 1.0 / (b * Q[0])
    p_g = pc["gg1"] * (Q[7] * Q[4] - 0.5 * (Q[5] * Q[5] + Q[6] * Q[6])) * (Q[0] * r) - pc["ggpg"]
    return p_g, qn * (b * r)


def bn_ncp(Q, ax, ay, pc):
    """PDEFusedSrcNCP (Baer-Nunziato/pde.f90:192-231, 277-290): only the
    volume-fraction gradient (ax, ay) enters."""
    p_g, un = bn_pg_un(Q, Q[1] * ax + Q[2] * ay, pc)
    s1, s2, s3 = p_g * ax, p_g * ay, p_g * un
    return [ZERO, s1, s2, s3, ZERO, -s1, -s2, -s3, -un]


def bn_roe_jump(QL, dQ, d, pc):
    """RoeMatrix(QL, QR) (QR - QL) (Baer-Nunziato/pde.f90:296-320, 150-186):
    PDEMatrixB has one non-zero column, the volume fraction's, so only the
    path integrals of p_g, u_n and p_g u_n and the jump of Q8 enter."""
    sq = math.sqrt(15.0) / 10.0
    sGP, wGP = (0.5 - sq, 0.5, 0.5 + sq), (5.0 / 18.0, 8.0 / 18.0, 5.0 / 18.0)
    bp = bu = bpu = ZERO
    for g in range(3):
        Q = {v: QL[v] + sGP[g] * dQ[v] for v in (0, 1 if d == 0 else 2, 4, 5, 6, 7, 8)}
        p, un = bn_pg_un(Q, Q[1] if d == 0 else Q[2], pc)
        bp = bp + wGP[g] * p
        bu = bu + wGP[g] * un
        bpu = bpu + wGP[g] * (p * un)
    m1, m3, m8 = bp * dQ[8], bpu * dQ[8], bu * dQ[8]
    return [ZERO, -m1 if d == 0 else ZERO, -m1 if d == 1 else ZERO, -m3,
            ZERO, m1 if d == 0 else ZERO, m1 if d == 1 else ZERO, m3, m8]


def bn_prim(Q, pc):
    """cons2prim (Baer-Nunziato/pde.f90:8-43): rho_s, u_s, v_s, p_s, rho_g, u_g, v_g, p_g."""
    phg = 1.0 - Q[8]
    rs, rg = Q[0] / Q[8], Q[4] / phg
    us, vs, ug, vg = Q[1] / Q[0], Q[2] / Q[0], Q[5] / Q[4], Q[6] / Q[4]
    Es, Eg = Q[3] / Q[8], Q[7] / phg
    ps_ = pc["gs1"] * (Es - 0.5 * rs * (us * us + vs * vs)) - pc["gsps"]
    pg_ = pc["gg1"] * (Eg - 0.5 * rg * (ug * ug + vg * vg)) - pc["ggpg"]
    return rs, us, vs, ps_, rg, ug, vg, pg_


def resolve_cell_bn(nb, rec, ops, N, dt, dx, dy, pc, lmin=None, lmax=None):
    """Re-solve of one Baer-Nunziato cell (Baer-Nunziato/limiter.f90:416-596):
    as resolve_cell, with the slopes, the NCP source and the half step on the
    halo subcells too (two rings of neighbour subcells), the path-conservative
    fluctuations of every edge and the NCP source at the half step in the
    finite-volume update."""
    P, S, V = N + 1, 2 * N + 1, 9
    uh2lim, lim2uh, uh2lob = ops["uh2lim"], ops["lim2uh"], ops["uh2lob"]
    Cnt.n = 0
    dtc, dxc, dyc = Cnt(dt), Cnt(dx), Cnt(dy)
    nbc = {k: [[Cnt(x) for x in row] for row in u] for k, u in nb.items()}
    ldx, ldy = dxc / S, dyc / S
    dtx, dty, hdt = dtc / ldx, dtc / ldy, 0.5 * dtc
    hdtx, hdty = 0.5 * dtx, 0.5 * dty
    H = S + 2

    # ---- gather: the values the slopes of the (S+2)^2 - 4 evolved subcells read
    LY = {}

    def ly(bi, bj, v, kk, sb):
        key = (bi, bj, v, kk, sb)
        if key not in LY:
            acc = ZERO
            for m in range(P):
                acc = acc + nbc[(bi, bj)][v][kk + P * m] * uh2lim[sb + S * m]
            LY[key] = acc
        return LY[key]

    corner = lambda ii, jj: ii in (0, H - 1) and jj in (0, H - 1)  # noqa: E731
    states = [(ii, jj) for jj in range(H) for ii in range(H) if not corner(ii, jj)]
    need = set((ii, jj) for jj in range(H) for ii in range(H))
    need |= set((ii, jj) for jj in range(1, S + 1) for ii in (-1, S + 2))
    need |= set((ii, jj) for jj in (-1, S + 2) for ii in range(1, S + 1))
    SU = {}
    for ii, jj in sorted(need):
        bi = -1 if ii < 1 else (1 if ii > S else 0)
        bj = -1 if jj < 1 else (1 if jj > S else 0)
        sa, sb = ii - 1 - bi * S, jj - 1 - bj * S
        for v in range(V):
            acc = ZERO
            for kk in range(P):
                acc = acc + ly(bi, bj, v, kk, sb) * uh2lim[sa + S * kk]
            SU[(v, ii, jj)] = acc

    # ---- MUSCL-Hancock with the NCP source (Baer-Nunziato/limiter.f90:486-524)
    wLx, wRx, wLy, wRy, slt, ga = {}, {}, {}, {}, {}, {}
    for ii, jj in states:
        q0 = [SU[(v, ii, jj)] for v in range(V)]
        sx = [minmod(SU[(v, ii + 1, jj)] - q0[v], q0[v] - SU[(v, ii - 1, jj)]) for v in range(V)]
        sy = [minmod(SU[(v, ii, jj + 1)] - q0[v], q0[v] - SU[(v, ii, jj - 1)]) for v in range(V)]
        gx, gy = sx[8] / ldx, sy[8] / ldy
        ga[(ii, jj)] = (gx, gy)
        src = bn_ncp(q0, gx, gy, pc)
        hx_ = [0.5 * sx[v] for v in range(V)]
        hy_ = [0.5 * sy[v] for v in range(V)]
        wlx = [q0[v] - hx_[v] for v in range(V)]
        wrx = [q0[v] + hx_[v] for v in range(V)]
        wly = [q0[v] - hy_[v] for v in range(V)]
        wry = [q0[v] + hy_[v] for v in range(V)]
        FLx, _ = bn_flux_dir(wlx, 0, pc)
        FRx, _ = bn_flux_dir(wrx, 0, pc)
        FLy, _ = bn_flux_dir(wly, 1, pc)
        FRy, _ = bn_flux_dir(wry, 1, pc)
        for v in range(V):
            qt = src[v] - (FRx[v] - FLx[v]) / ldx
            qt = qt - (FRy[v] - FLy[v]) / ldy
            slt[(v, ii, jj)] = qt
            g = hdt * qt
            wLx[(v, ii, jj)] = wlx[v] + g
            wRx[(v, ii, jj)] = wrx[v] + g
            wLy[(v, ii, jj)] = wly[v] + g
            wRy[(v, ii, jj)] = wry[v] + g

    # ---- edge fluxes and fluctuations, once per edge (:526-545)
    def edge(QL, QR, d):
        dQ = [QR[v] - QL[v] for v in range(V)]
        FL, eL = bn_flux_dir(QL, d, pc, eig=True)
        FR, eR = bn_flux_dir(QR, d, pc, eig=True)
        hs = 0.5 * cmax(eL, eR)
        F = [0.5 * (FL[v] + FR[v]) - hs * dQ[v] for v in range(V)]
        return F, bn_roe_jump(QL, dQ, d, pc)

    Ex = {(ii, jj): edge([wRx[(v, ii - 1, jj)] for v in range(V)], [wLx[(v, ii, jj)] for v in range(V)], 0)
          for jj in range(1, S + 1) for ii in range(1, S + 2)}
    Ey = {(ii, jj): edge([wRy[(v, ii, jj - 1)] for v in range(V)], [wLy[(v, ii, jj)] for v in range(V)], 1)
          for jj in range(1, S + 2) for ii in range(1, S + 1)}

    # ---- finite-volume update with the fluctuations and the NCP source at the half step
    sub1 = [[None] * (S * S) for _ in range(V)]
    for jj in range(1, S + 1):
        for ii in range(1, S + 1):
            qh = [SU[(v, ii, jj)] + hdt * slt[(v, ii, jj)] for v in range(V)]
            src = bn_ncp(qh, ga[(ii, jj)][0], ga[(ii, jj)][1], pc)
            (fp, Dp), (fm, Dm) = Ex[(ii + 1, jj)], Ex[(ii, jj)]
            (gp, Gp), (gm, Gm) = Ey[(ii, jj + 1)], Ey[(ii, jj)]
            for v in range(V):
                sub1[v][(ii - 1) + S * (jj - 1)] = (SU[(v, ii, jj)] - dtx * (fp[v] - fm[v]) - dty * (gp[v] - gm[v])
                                                    - hdtx * (Dp[v] + Dm[v]) - hdty * (Gp[v] + Gm[v])
                                                    + dtc * src[v])

    # ---- put_subcell_data
    luhy = [[[None] * V for _ in range(S)] for _ in range(P)]
    for iii in range(S):
        for s in range(P):
            for v in range(V):
                acc = ZERO
                for k in range(S):
                    acc = acc + sub1[v][iii + S * k] * lim2uh[s + P * k]
                luhy[s][iii][v] = acc
    un = [[None] * (P * P) for _ in range(V)]
    for jjj in range(P):
        for s in range(P):
            for v in range(V):
                acc = ZERO
                for k in range(S):
                    acc = acc + luhy[jjj][k][v] * lim2uh[s + P * k]
                un[v][s + P * jjj] = acc

    verdict = None
    if rec == 2:
        lim = _project(un, uh2lim, S, P, V)
        lob = _project(un, uh2lob, P, P, V)
        verdict = True
        for v in range(V):
            vals = [x.x for x in un[v] + lim[v] + lob[v]]
            lo, hi = Cnt(lmin[v]), Cnt(lmax[v])
            ldiff = max(1.0e-4, (1.0e-3 * (hi - lo)).x)
            if min(vals) < (lo - ldiff).x or max(vals) > (hi + ldiff).x:
                verdict = False
        for k in range(S * S):
            Q = [lim[v][k] for v in range(V)]
            rs, _, _, ps_, rg, _, _, pg_ = bn_prim(Q, pc)
            if (rs.x <= 1e-12 or rg.x <= 1e-12 or (ps_ + pc["ps"]).x <= 1e-12 or (pg_ + pc["pg"]).x <= 1e-12
                    or not 0.0 < Q[8].x < 1.0):
                verdict = False

    den = []
    for k in range(P * P):
        Q = [un[v][k] for v in range(V)]
        rs, us, vs, ps_, rg, ug, vg, pg_ = bn_prim(Q, pc)
        a_s = csqrt(pc["gs"] * (ps_ + pc["ps"]) / rs)
        a_g = csqrt(pc["gg"] * (pg_ + pc["pg"]) / rg)
        e = []
        for u_s, u_g in ((us, ug), (vs, vg)):
            m = cabs(u_g - a_g)
            for x in (cabs(u_g + a_g), cabs(u_s - a_s), cabs(u_s + a_s), cabs(u_g), cabs(u_s)):
                m = cmax(m, x)
            e.append(m)
        den.append(e[0] / dxc + e[1] / dyc)
    return sub1, un, verdict, den, Cnt.n


def _project(un, op, n_out, P, V):
    """get_subcell_data / get_lobatto_data (Euler/limiter.f90:12-68) of un."""
    y = [[[None] * V for _ in range(P)] for _ in range(n_out)]
    for iii in range(P):
        for s in range(n_out):
            for v in range(V):
                acc = ZERO
                for k in range(P):
                    acc = acc + un[v][iii + P * k] * op[s + n_out * k]
                y[s][iii][v] = acc
    out = [[None] * (n_out * n_out) for _ in range(V)]
    for jjj in range(n_out):
        for s in range(n_out):
            for v in range(V):
                acc = ZERO
                for k in range(P):
                    acc = acc + y[jjj][k][v] * op[s + n_out * k]
                out[v][s + n_out * jjj] = acc
    return out


@pytest.mark.parametrize("N", [1, 2, 3, 4, 5])
def test_bn_subcell_flop_model_equals_instrumented_count(N):
    r = _oracle_step(N, "bn_cylinder", 9)
    gs, gg, ps, pg = r["cfg"].gamma_s, r["cfg"].gamma_g, r["cfg"].pi_s, r["cfg"].pi_g
    pc = dict(gs=gs, gg=gg, ps=ps, pg=pg, gs1=gs - 1.0, gg1=gg - 1.0, gsps=gs * ps, ggpg=gg * pg)
    args = (r["ops"], N, r["dt"], r["dx"], r["dy"], pc)
    sub1, un, verdict, _, n1 = resolve_cell_bn(_neighbourhood(r, 2, 2), 1, *args)
    ref = r["newlh"][2, 2].T
    assert np.abs(_vals(sub1) - ref).max() <= 1e-12 * np.abs(ref).max(), N
    ref = r["uh"][2, 2].T
    assert np.abs(_vals(un) - ref).max() <= 1e-12 * np.abs(ref).max(), N
    sub2, un2, verdict2, den, n2 = resolve_cell_bn(_neighbourhood(r, 3, 2), 2, *args,
                                                   lmin=r["lmin"][2, 3], lmax=r["lmax"][2, 3])
    ref = r["uh"][2, 3].T
    assert np.abs(_vals(un2) - ref).max() <= 1e-12 * np.abs(ref).max(), N
    assert verdict2 == (r["status"][2, 3] == 0), (N, verdict2, r["status"][2, 3])
    assert all(d.x > 0 for d in den)
    assert bench.subcell_flops_per_cell(po.SYS_BN, N, dmp=False) == n1, (N, n1)
    assert bench.subcell_flops_per_cell(po.SYS_BN, N) == n2, (N, n2)
