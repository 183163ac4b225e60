// physics.cuh -- pointwise physics of the three PDE systems on the device.
//
// Two flavours per system:
//   * reference-order FP64 functions (flux, max_eig, positivity, Rusanov
//     pieces) used by the face, update, limiter and time-step kernels.  The
//     translation units that use them are compiled with --fmad=false, so each
//     expression rounds exactly like the reference's FP64 evaluation of the
//     same expression (Euler/pde.f90, Baer-Nunziato/pde.f90,
//     Advection-Diffusion/pde.f90).
//   * predictor fluxes (pflux) templated on the compute precision, written for
//     fused multiply-adds and reciprocals instead of repeated divisions.  They
//     are algebraically equal to the reference expressions and used only by
//     the space-time predictor.
#pragma once

#include "common.cuh"

namespace aderdg {

// ---------------------------------------------------------------------------
struct EulerSys {
  static constexpr int V = 4;
  static constexpr int ID = kSysEuler;

  // Euler/pde.f90:46-69; F[d*V + v]
  __device__ static void flux(const Phys& ph, const double* Q, double* F) {
    double irho = 1.0 / Q[0];
    double p = (ph.gamma - 1.0) * (Q[3] - 0.5 * (Q[1] * Q[1] + Q[2] * Q[2]) * irho);
    F[0] = Q[1];
    F[1] = irho * Q[1] * Q[1] + p;
    F[2] = irho * Q[1] * Q[2];
    F[3] = irho * Q[1] * (Q[3] + p);
    F[4] = Q[2];
    F[5] = irho * Q[2] * Q[1];
    F[6] = irho * Q[2] * Q[2] + p;
    F[7] = irho * Q[2] * (Q[3] + p);
  }
  // maxval(abs(Lambda)) of Euler/pde.f90:75-91 for the unit normal of axis d
  __device__ static double max_eig(const Phys& ph, const double* Q, int d) {
    double u = (d == 0 ? Q[1] : Q[2]) / Q[0];
    double p = (ph.gamma - 1.0) * (Q[3] - 0.5 * (Q[1] * Q[1] + Q[2] * Q[2]) / Q[0]);
    double c = sqrt(ph.gamma * p / Q[0]);
    return fmax(fmax(fabs(u - c), fabs(u)), fabs(u + c));
  }
  // both axes at once: the pressure and sound speed do not depend on the
  // normal, so they are formed once (same expressions, same rounding)
  __device__ static void max_eig2(const Phys& ph, const double* Q, double& ex, double& ey) {
    double p = (ph.gamma - 1.0) * (Q[3] - 0.5 * (Q[1] * Q[1] + Q[2] * Q[2]) / Q[0]);
    double c = sqrt(ph.gamma * p / Q[0]);
    double u = Q[1] / Q[0], v = Q[2] / Q[0];
    ex = fmax(fmax(fabs(u - c), fabs(u)), fabs(u + c));
    ey = fmax(fmax(fabs(v - c), fabs(v)), fabs(v + c));
  }
  // FP32 eigenvalues for the mixed-precision CFL (the max reduction stays FP64)
  __device__ static void max_eig2_f32(const Phys& ph, const double* Qd, double& ex, double& ey) {
    const float q0 = (float)Qd[0], q1 = (float)Qd[1], q2 = (float)Qd[2], q3 = (float)Qd[3];
    const float iq = 1.0f / q0;
    const float p = (float)(ph.gamma - 1.0) * (q3 - 0.5f * (q1 * q1 + q2 * q2) * iq);
    const float c = sqrtf((float)ph.gamma * p * iq);
    const float u = q1 * iq, v = q2 * iq;
    ex = (double)(fabsf(u) + c);
    ey = (double)(fabsf(v) + c);
  }
  // Euler/pde.f90:29-40
  __device__ static void prim2cons(const Phys& ph, const double* Vp, double* Q) {
    Q[0] = Vp[0];
    Q[1] = Vp[0] * Vp[1];
    Q[2] = Vp[0] * Vp[2];
    Q[3] = Vp[3] / (ph.gamma - 1) + 0.5 * Vp[0] * (Vp[1] * Vp[1] + Vp[2] * Vp[2]);
  }
  // Euler/pde.f90:120-145: true when admissible
  __device__ static bool positive(const Phys& ph, const double* Q) {
    double irho = 1.0 / Q[0];
    double p = (ph.gamma - 1) * (Q[3] - 0.5 * (Q[1] * Q[1] + Q[2] * Q[2]) * irho);
    return !(Q[0] <= 1.0e-12) && !(p <= 1.0e-12);
  }
  // Same answer as positive(): an FP32 evaluation with a margin 20x its
  // rounding error settles the clearly admissible states, the exact FP64
  // expression decides the rest.
  __device__ static bool positive_fast(const Phys& ph, const double* Q) {
    if (Q[0] <= 1.0e-12) return false;
    const float q0 = (float)Q[0], q1 = (float)Q[1], q2 = (float)Q[2], q3 = (float)Q[3];
    const float ke = 0.5f * (q1 * q1 + q2 * q2) / q0;
    const float g1 = (float)(ph.gamma - 1.0);
    const float pf = g1 * (q3 - ke);
    const float margin = g1 * 1.0e-5f * (fabsf(q3) + ke);
    if (q0 > 1.0e-30f && q0 < 1.0e30f && pf - margin > 2.0e-12f && margin < 1.0e30f) return true;
    return positive(ph, Q);
  }

  // physical constants of the predictor flux in its compute precision
  template <class R>
  struct PConst {
    R gm1;
    __device__ explicit PConst(const Phys& ph) : gm1(R(ph.gamma - 1.0)) {}
  };
  // predictor flux: Fx, Fy of the same state
  template <class R>
  __device__ __forceinline__ static void pflux(const PConst<R>& pc, const R* Q, R* Fx, R* Fy) {
    const R ir = R(1) / Q[0];
    const R u = Q[1] * ir, v = Q[2] * ir;
    const R p = pc.gm1 * (Q[3] - R(0.5) * (Q[1] * u + Q[2] * v));
    const R e = Q[3] + p;
    Fx[0] = Q[1];
    Fx[1] = Q[1] * u + p;
    Fx[2] = Q[2] * u;
    Fx[3] = e * u;
    Fy[0] = Q[2];
    Fy[1] = Q[1] * v;
    Fy[2] = Q[2] * v + p;
    Fy[3] = e * v;
  }
};

// ---------------------------------------------------------------------------
struct BNSys {
  static constexpr int V = 9;
  static constexpr int ID = kSysBN;

  // Baer-Nunziato/pde.f90:8-43
  __device__ static void cons2prim(const Phys& ph, const double* Q, double* Vp) {
    double phi_s = Q[8], phi_g = 1.0 - Q[8];
    double rho_s = Q[0] / phi_s, rho_g = Q[4] / phi_g;
    double u_s = Q[1] / Q[0], v_s = Q[2] / Q[0];
    double u_g = Q[5] / Q[4], v_g = Q[6] / Q[4];
    double E_s = Q[3] / phi_s, E_g = Q[7] / phi_g;
    double p_s = (ph.gs - 1.0) * (E_s - 0.5 * rho_s * (u_s * u_s + v_s * v_s)) - ph.gs * ph.ps;
    double p_g = (ph.gg - 1.0) * (E_g - 0.5 * rho_g * (u_g * u_g + v_g * v_g)) - ph.gg * ph.pg;
    Vp[0] = rho_s; Vp[1] = u_s; Vp[2] = v_s; Vp[3] = p_s;
    Vp[4] = rho_g; Vp[5] = u_g; Vp[6] = v_g; Vp[7] = p_g; Vp[8] = phi_s;
  }
  // Baer-Nunziato/pde.f90:74-119
  __device__ static void flux(const Phys& ph, const double* Q, double* F) {
    double phi_s = Q[8], phi_g = 1.0 - Q[8];
    double rho_s = Q[0] / phi_s, rho_g = Q[4] / phi_g;
    double u_s = Q[1] / Q[0], v_s = Q[2] / Q[0];
    double u_g = Q[5] / Q[4], v_g = Q[6] / Q[4];
    double E_s = Q[3] / phi_s, E_g = Q[7] / phi_g;
    double p_s = (ph.gs - 1.0) * (E_s - 0.5 * rho_s * (u_s * u_s + v_s * v_s)) - ph.gs * ph.ps;
    double p_g = (ph.gg - 1.0) * (E_g - 0.5 * rho_g * (u_g * u_g + v_g * v_g)) - ph.gg * ph.pg;
    F[0] = phi_s * rho_s * u_s;
    F[1] = phi_s * (rho_s * u_s * u_s + p_s);
    F[2] = phi_s * rho_s * u_s * v_s;
    F[3] = phi_s * u_s * (E_s + p_s);
    F[4] = phi_g * rho_g * u_g;
    F[5] = phi_g * (rho_g * u_g * u_g + p_g);
    F[6] = phi_g * rho_g * u_g * v_g;
    F[7] = phi_g * u_g * (E_g + p_g);
    F[8] = 0.0;
    F[9] = phi_s * rho_s * v_s;
    F[10] = phi_s * rho_s * u_s * v_s;
    F[11] = phi_s * (rho_s * v_s * v_s + p_s);
    F[12] = phi_s * v_s * (E_s + p_s);
    F[13] = phi_g * rho_g * v_g;
    F[14] = phi_g * rho_g * u_g * v_g;
    F[15] = phi_g * (rho_g * v_g * v_g + p_g);
    F[16] = phi_g * v_g * (E_g + p_g);
    F[17] = 0.0;
  }
  // Baer-Nunziato/pde.f90:125-144
  __device__ static double max_eig(const Phys& ph, const double* Q, int d) {
    double Vp[9];
    cons2prim(ph, Q, Vp);
    double u_s = (d == 0) ? Vp[1] * 1.0 + Vp[2] * 0.0 : Vp[1] * 0.0 + Vp[2] * 1.0;
    double u_g = (d == 0) ? Vp[5] * 1.0 + Vp[6] * 0.0 : Vp[5] * 0.0 + Vp[6] * 1.0;
    double a_s = sqrt(ph.gs * (Vp[3] + ph.ps) / Vp[0]);
    double a_g = sqrt(ph.gg * (Vp[7] + ph.pg) / Vp[4]);
    double m = fabs(u_g - a_g);
    m = fmax(m, fabs(u_g + a_g));
    m = fmax(m, fabs(u_s - a_s));
    m = fmax(m, fabs(u_s + a_s));
    m = fmax(m, fabs(u_g));
    m = fmax(m, fabs(u_s));
    return m;
  }
  __device__ static void max_eig2(const Phys& ph, const double* Q, double& ex, double& ey) {
    double Vp[9];
    cons2prim(ph, Q, Vp);
    double a_s = sqrt(ph.gs * (Vp[3] + ph.ps) / Vp[0]);
    double a_g = sqrt(ph.gg * (Vp[7] + ph.pg) / Vp[4]);
    for (int d = 0; d < 2; ++d) {
      double u_s = (d == 0) ? Vp[1] * 1.0 + Vp[2] * 0.0 : Vp[1] * 0.0 + Vp[2] * 1.0;
      double u_g = (d == 0) ? Vp[5] * 1.0 + Vp[6] * 0.0 : Vp[5] * 0.0 + Vp[6] * 1.0;
      double m = fabs(u_g - a_g);
      m = fmax(m, fabs(u_g + a_g));
      m = fmax(m, fabs(u_s - a_s));
      m = fmax(m, fabs(u_s + a_s));
      m = fmax(m, fabs(u_g));
      m = fmax(m, fabs(u_s));
      (d == 0 ? ex : ey) = m;
    }
  }
  __device__ static void max_eig2_f32(const Phys& ph, const double* Qd, double& ex, double& ey) {
    float q[9];
    for (int v = 0; v < 9; ++v) q[v] = (float)Qd[v];
    const float a = q[8], b = 1.0f - q[8];
    const float irs = 1.0f / q[0], irg = 1.0f / q[4];
    const float us = q[1] * irs, vs = q[2] * irs, ug = q[5] * irg, vg = q[6] * irg;
    const float rs = q[0] / a, rg = q[4] / b;
    const float ps = (float)(ph.gs - 1.0) * (q[3] / a - 0.5f * rs * (us * us + vs * vs)) - (float)(ph.gs * ph.ps);
    const float pg = (float)(ph.gg - 1.0) * (q[7] / b - 0.5f * rg * (ug * ug + vg * vg)) - (float)(ph.gg * ph.pg);
    const float as = sqrtf((float)ph.gs * (ps + (float)ph.ps) / rs), ag = sqrtf((float)ph.gg * (pg + (float)ph.pg) / rg);
    ex = (double)fmaxf(fabsf(ug) + ag, fabsf(us) + as);
    ey = (double)fmaxf(fabsf(vg) + ag, fabsf(vs) + as);
  }
  // column 9 of PDEMatrixB (Baer-Nunziato/pde.f90:150-186); the other columns are zero
  __device__ static void matrixB_col9(const Phys& ph, const double* Q, int d, double* b) {
    const double nv0 = d == 0 ? 1.0 : 0.0, nv1 = d == 0 ? 0.0 : 1.0;
    double phi_g = 1.0 - Q[8];
    double rho_g = Q[4] / phi_g;
    double u_s = Q[1] / Q[0], v_s = Q[2] / Q[0];
    double u_n = nv0 * u_s + nv1 * v_s;
    double u_g = Q[5] / Q[4], v_g = Q[6] / Q[4];
    double E_g = Q[7] / phi_g;
    double p_g = (ph.gg - 1.0) * (E_g - 0.5 * rho_g * (u_g * u_g + v_g * v_g)) - ph.gg * ph.pg;
    b[0] = 0.0;
    b[1] = -(nv0 * p_g);
    b[2] = -(nv1 * p_g);
    b[3] = -(p_g * u_n);
    b[4] = 0.0;
    b[5] = nv0 * p_g;
    b[6] = nv1 * p_g;
    b[7] = p_g * u_n;
    b[8] = u_n;
  }
  // D = RoeMatrix(QL,QR) * (QR - QL): 3-point Gauss-Legendre path integral,
  // Baer-Nunziato/pde.f90:296-320 and the matmul of :348
  __device__ static void roe_times_jump(const Phys& ph, const double* QL, const double* QR, int d, double* D) {
    const double sq = sqrt(15.0) / 10.;
    const double sGP[3] = {0.5 - sq, 0.5, 0.5 + sq};
    const double wGP[3] = {5. / 18.0, 8. / 18., 5. / 18.};
    double broe[9], b[9], Q[9];
    for (int v = 0; v < 9; ++v) broe[v] = 0.0;
    for (int g = 0; g < 3; ++g) {
      for (int v = 0; v < 9; ++v) Q[v] = QL[v] + sGP[g] * (QR[v] - QL[v]);
      matrixB_col9(ph, Q, d, b);
      for (int v = 0; v < 9; ++v) broe[v] = broe[v] + wGP[g] * b[v];
    }
    const double dq9 = QR[8] - QL[8];
    for (int v = 0; v < 9; ++v) D[v] = broe[v] * dq9;
  }
  // -NCP, Baer-Nunziato/pde.f90:192-231 and :277-290; only the volume-fraction gradient enters
  __device__ static void src_ncp(const Phys& ph, const double* Q, double ax, double ay, double* S) {
    double phi_g = 1.0 - Q[8];
    double rho_g = Q[4] / phi_g;
    double u_s = Q[1] / Q[0], v_s = Q[2] / Q[0];
    double u_g = Q[5] / Q[4], v_g = Q[6] / Q[4];
    double E_g = Q[7] / phi_g;
    double p_g = (ph.gg - 1.0) * (E_g - 0.5 * rho_g * (u_g * u_g + v_g * v_g)) - ph.gg * ph.pg;
    double un = u_s * ax + v_s * ay;
    S[0] = -0.0;
    S[1] = -(-p_g * ax);
    S[2] = -(-p_g * ay);
    S[3] = -(-p_g * un);
    S[4] = -0.0;
    S[5] = -(p_g * ax);
    S[6] = -(p_g * ay);
    S[7] = -(p_g * un);
    S[8] = -un;
  }
  // Baer-Nunziato/pde.f90:49-68
  __device__ static void prim2cons(const Phys& ph, const double* Vp, double* Q) {
    Q[0] = Vp[8] * Vp[0];
    Q[1] = Q[0] * Vp[1];
    Q[2] = Q[0] * Vp[2];
    Q[3] = Q[0] * (0.5 * (Vp[1] * Vp[1] + Vp[2] * Vp[2]) + (Vp[3] + ph.gs * ph.ps) / (Vp[0] * (ph.gs - 1.0)));
    Q[4] = (1.0 - Vp[8]) * Vp[4];
    Q[5] = Q[4] * Vp[5];
    Q[6] = Q[4] * Vp[6];
    Q[7] = Q[4] * (0.5 * (Vp[5] * Vp[5] + Vp[6] * Vp[6]) + (Vp[7] + ph.gg * ph.pg) / (Vp[4] * (ph.gg - 1.0)));
    Q[8] = Vp[8];
  }
  // Baer-Nunziato/pde.f90:237-266
  __device__ static bool positive(const Phys& ph, const double* Q) {
    double Vp[9];
    cons2prim(ph, Q, Vp);
    bool bad = (Vp[0] <= 1.0e-12 || Vp[4] <= 1.0e-12);
    bad = bad || ((Vp[3] + ph.ps) <= 1.0e-12 || (Vp[7] + ph.pg) <= 1.0e-12);
    bad = bad || (Vp[8] <= 0.0 || Vp[8] >= 1.0);
    return !bad;
  }
  // Same answer as positive(), with an FP32 pre-check (margin 20x its
  // rounding error) that settles clearly admissible states.
  __device__ static bool positive_fast(const Phys& ph, const double* Q) {
    if (!(Q[8] > 0.0) || !(Q[8] < 1.0)) return positive(ph, Q);
    float q[9];
    for (int v = 0; v < 9; ++v) {
      q[v] = (float)Q[v];
      const float aq = fabsf(q[v]);
      if (!(aq < 1.0e30f) || (aq != 0.0f && aq < 1.0e-30f)) return positive(ph, Q);
    }
    const float a = q[8], b = 1.0f - q[8];
    if (!(a > 1.0e-6f) || !(b > 1.0e-6f)) return positive(ph, Q);
    const float rs = q[0] / a, rg = q[4] / b;
    const float kes = 0.5f * (q[1] * q[1] + q[2] * q[2]) / q[0];  // 0.5 rho_s |u_s|^2 * phi_s
    const float keg = 0.5f * (q[5] * q[5] + q[6] * q[6]) / q[4];
    const float es = q[3] / a, eg = q[7] / b;
    const float gs1 = (float)(ph.gs - 1.0), gg1 = (float)(ph.gg - 1.0);
    const float ps = gs1 * (es - kes / a) - (float)(ph.gs * ph.ps) + (float)ph.ps;  // p_s + pi_s
    const float pg = gg1 * (eg - keg / b) - (float)(ph.gg * ph.pg) + (float)ph.pg;  // p_g + pi_g
    const float ms = 1.0e-5f * (gs1 * (fabsf(es) + kes / a) + (float)fabs(ph.gs * ph.ps) + (float)fabs(ph.ps));
    const float mg = 1.0e-5f * (gg1 * (fabsf(eg) + keg / b) + (float)fabs(ph.gg * ph.pg) + (float)fabs(ph.pg));
    const bool clear = rs > 2.0e-12f * (1.0f + 1.0e-5f) + 1.0e-5f * rs && rg > 2.0e-12f + 1.0e-5f * rg &&
                       ps - ms > 2.0e-12f && pg - mg > 2.0e-12f && ms < 1.0e30f && mg < 1.0e30f;
    return clear ? true : positive(ph, Q);
  }

  template <class R>
  struct PConst {
    R gs1, gg1, gsps, ggpg;
    __device__ explicit PConst(const Phys& ph)
        : gs1(R(ph.gs - 1.0)), gg1(R(ph.gg - 1.0)), gsps(R(ph.gs * ph.ps)), ggpg(R(ph.gg * ph.pg)) {}
  };
  // predictor flux plus the three scalars the NCP needs (p_g, u_s, v_s)
  template <class R>
  __device__ __forceinline__ static void pflux(const PConst<R>& pc, const R* Q, R* Fx, R* Fy, R& p_g, R& u_s, R& v_s) {
    const R a = Q[8], b = R(1) - Q[8];
    const R irs = R(1) / Q[0], irg = R(1) / Q[4];
    u_s = Q[1] * irs;
    v_s = Q[2] * irs;
    const R u_g = Q[5] * irg, v_g = Q[6] * irg;
    const R Ps = pc.gs1 * (Q[3] - R(0.5) * (Q[1] * u_s + Q[2] * v_s)) - a * pc.gsps;  // phi_s p_s
    const R Pg = pc.gg1 * (Q[7] - R(0.5) * (Q[5] * u_g + Q[6] * v_g)) - b * pc.ggpg;  // phi_g p_g
    p_g = Pg / b;
    const R es = Q[3] + Ps, eg = Q[7] + Pg;
    Fx[0] = Q[1];
    Fx[1] = Q[1] * u_s + Ps;
    Fx[2] = Q[2] * u_s;
    Fx[3] = es * u_s;
    Fx[4] = Q[5];
    Fx[5] = Q[5] * u_g + Pg;
    Fx[6] = Q[6] * u_g;
    Fx[7] = eg * u_g;
    Fx[8] = R(0);
    Fy[0] = Q[2];
    Fy[1] = Q[1] * v_s;
    Fy[2] = Q[2] * v_s + Ps;
    Fy[3] = es * v_s;
    Fy[4] = Q[6];
    Fy[5] = Q[5] * v_g;
    Fy[6] = Q[6] * v_g + Pg;
    Fy[7] = eg * v_g;
    Fy[8] = R(0);
  }
  // NCP(q) . grad(alpha) added to the predictor's flux contraction (= -lSh)
  template <class R>
  __device__ __forceinline__ static void pncp(R p_g, R u_s, R v_s, R ax, R ay, R* n) {
    const R un = u_s * ax + v_s * ay;
    n[0] = R(0);
    n[1] = -p_g * ax;
    n[2] = -p_g * ay;
    n[3] = -p_g * un;
    n[4] = R(0);
    n[5] = p_g * ax;
    n[6] = p_g * ay;
    n[7] = p_g * un;
    n[8] = un;
  }
};

// ---------------------------------------------------------------------------
struct ADSys {
  static constexpr int V = 1;
  static constexpr int ID = kSysAD;
  template <class R>
  struct PConst {
    __device__ explicit PConst(const Phys&) {}
  };
  // Advection-Diffusion/pde.f90:70-80 (|cx nv1 + cy nv2|)
  __device__ static double max_eig_c(const Phys& ph, int d) {
    return fabs(d == 0 ? ph.cx * 1.0 + ph.cy * 0.0 : ph.cx * 0.0 + ph.cy * 1.0);
  }
};

}  // namespace aderdg
