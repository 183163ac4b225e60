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

// Physical constants in the compute type T, formed once from Phys with the
// same FP64 expressions the reference writes inline (gamma - 1, gamma_s *
// pi_s, ...): for T = double every function below rounds exactly like the
// reference expression; T = float serves the FP32-wide subcell re-solve.
template <class T>
struct PhysC {
  T gamma, gm1;                    // Euler
  T gs, gg, ps, pg, gs1, gg1, gsps, ggpg;  // Baer-Nunziato
  __device__ explicit PhysC(const Phys& ph)
      : gamma(T(ph.gamma)), gm1(T(ph.gamma - 1.0)), gs(T(ph.gs)), gg(T(ph.gg)), ps(T(ph.ps)), pg(T(ph.pg)),
        gs1(T(ph.gs - 1.0)), gg1(T(ph.gg - 1.0)), gsps(T(ph.gs * ph.ps)), ggpg(T(ph.gg * ph.pg)) {}
};
template <class T> __device__ __forceinline__ T tabs(T x) {
  if constexpr (sizeof(T) == 4) return fabsf(x); else return fabs(x);
}
template <class T> __device__ __forceinline__ T tmax(T a, T b) {
  if constexpr (sizeof(T) == 4) return fmaxf(a, b); else return fmax(a, b);
}
template <class T> __device__ __forceinline__ T tmin(T a, T b) {
  if constexpr (sizeof(T) == 4) return fminf(a, b); else return fmin(a, b);
}
template <class T> __device__ __forceinline__ T tsqrt(T x) {
  if constexpr (sizeof(T) == 4) return sqrtf(x); else return sqrt(x);
}
// Reciprocal and square root of the FP32-mixed mode's FP64 arithmetic (the
// reciprocal-sharing physics *_r; the FP64 mode keeps the correctly rounded
// operations and the reference's divisions).  The hardware's approximations
// (rcp.approx.ftz.f64, rsqrt.approx.ftz.f64) are refined by one third-order
// Newton step, derived from the series of the exact quotients:
//   1/x:     e = 1 - x r0,        1/x     = r0 / (1 - e)    ~ r0 (1 + e + e^2)
//   sqrt(a): s0 = a y0, h = 1 - s0 y0, sqrt(a) = s0 (1 - h)^(-1/2) ~ s0 (1 + h/2 + 3 h^2 / 8)
// (the neglected terms are e^3 and 5 h^3 / 16 relative).  Within 2 ulp of the
// correctly rounded results for normal finite inputs (checked against them on
// the device by aderdg_probe_math); zeros, denormals, infinities and NaNs (the
// exponent field all zeros or all ones, an integer test) take the correctly
// rounded operation.  FP32: the correctly rounded operations.
// FP32 -> FP64, exact, on the integer pipe (sign, exponent rebias, mantissa
// shift) for zeros and normal values; infinities, NaNs and denormals take the
// hardware conversion.  The FP64-bound kernels of the FP32-mixed mode read
// FP32 inputs (the Baer-Nunziato face states): their conversions then leave
// the FP64 pipe.
__device__ __forceinline__ double widen_bits(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned e = (u >> 23) & 0xffu, m = u & 0x7fffffu;
  if (e == 0xffu || (e == 0u && m != 0u)) return (double)f;
  unsigned long long d = (unsigned long long)(u & 0x80000000u) << 32;
  if (e) d |= ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)m << 29);
  return __longlong_as_double((long long)d);
}
template <class T, class R> __device__ __forceinline__ T widen(R x) {
  if constexpr (sizeof(T) == 8 && sizeof(R) == 4) return widen_bits(x);
  else return (T)x;
}
__device__ __forceinline__ bool m_special(double x) {
  const unsigned long long ex = (unsigned long long)__double_as_longlong(x) & 0x7ff0000000000000ull;
  return ex == 0ull || ex == 0x7ff0000000000000ull;
}
template <class T> __device__ __forceinline__ T mrcp(T x) {
  if constexpr (sizeof(T) == 4) {
    return T(1) / x;
  } else {
    if (m_special(x)) return 1.0 / x;
    double r;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(r) : "d"(x));
    const double e = fma(-x, r, 1.0);
    return fma(fma(e, e, e), r, r);
  }
}
template <class T> __device__ __forceinline__ T msqrt(T a) {
  if constexpr (sizeof(T) == 4) {
    return sqrtf(a);
  } else {
    if (m_special(a) || __double_as_longlong(a) < 0) return sqrt(a);
    double y;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(a));
    const double s = a * y;
    const double h = fma(-s, y, 1.0);
    return fma(s * h, fma(h, 0.375, 0.5), s);
  }
}

// ---------------------------------------------------------------------------
struct EulerSys {
  static constexpr int V = 4;
  static constexpr int ID = kSysEuler;

  // Euler/pde.f90:46-69; F[d*V + v]
  template <class T>
  __device__ static void flux(const PhysC<T>& pc, const T* Q, T* F) {
    T irho = T(1) / Q[0];
    T p = pc.gm1 * (Q[3] - T(0.5) * (Q[1] * Q[1] + Q[2] * Q[2]) * irho);
    F[0] = Q[1];
    F[1] = irho * Q[1] * Q[1] + p;
    F[2] = irho * Q[1] * Q[2];
    F[3] = irho * Q[1] * (Q[3] + p);
    F[4] = Q[2];
    F[5] = irho * Q[2] * Q[1];
    F[6] = irho * Q[2] * Q[2] + p;
    F[7] = irho * Q[2] * (Q[3] + p);
  }
  __device__ static void flux(const Phys& ph, const double* Q, double* F) { flux<double>(PhysC<double>(ph), Q, F); }
  // maxval(abs(Lambda)) of Euler/pde.f90:75-91 for the unit normal of axis d
  template <class T>
  __device__ static T max_eig(const PhysC<T>& pc, const T* Q, int d) {
    T u = (d == 0 ? Q[1] : Q[2]) / Q[0];
    T p = pc.gm1 * (Q[3] - T(0.5) * (Q[1] * Q[1] + Q[2] * Q[2]) / Q[0]);
    T c = tsqrt(pc.gamma * p / Q[0]);
    return tmax(tmax(tabs(u - c), tabs(u)), tabs(u + c));
  }
  __device__ static double max_eig(const Phys& ph, const double* Q, int d) { return max_eig<double>(PhysC<double>(ph), Q, d); }
  // both axes at once: the pressure and sound speed do not depend on the
  // normal, so they are formed once (same expressions, same rounding)
  __device__ static void max_eig2(const Phys& ph, const double* Q, double& ex, double& ey) {
    double p = (ph.gamma - 1.0) * (Q[3] - 0.5 * (Q[1] * Q[1] + Q[2] * Q[2]) / Q[0]);
    double c = sqrt(ph.gamma * p / Q[0]);
    double u = Q[1] / Q[0], v = Q[2] / Q[0];
    ex = fmax(fmax(fabs(u - c), fabs(u)), fabs(u + c));
    ey = fmax(fmax(fabs(v - c), fabs(v)), fabs(v + c));
  }
  // Flux F[d*V + v] and maxval(abs(Lambda)) along axis d of one state with a
  // single reciprocal of the density: algebraically Euler/pde.f90:46-91, used
  // by the FP32-mixed mode's FP64 subcell re-solve (compiled with fused
  // multiply-adds; its values agree with the reference order to rounding).
  template <class T>
  __device__ static void flux_eig_r(const PhysC<T>& pc, const T* Q, int d, T* F, T& eig) {
    const T irho = mrcp<T>(Q[0]);
    const T u = Q[1] * irho, v = Q[2] * irho;
    const T p = pc.gm1 * (Q[3] - T(0.5) * (Q[1] * u + Q[2] * v));
    if (F) {
      F[0] = Q[1];
      F[1] = Q[1] * u + p;
      F[2] = Q[1] * v;
      F[3] = u * (Q[3] + p);
      F[4] = Q[2];
      F[5] = Q[2] * u;
      F[6] = Q[2] * v + p;
      F[7] = v * (Q[3] + p);
    }
    const T un = d == 0 ? u : v;
    const T c = msqrt<T>(pc.gamma * p * irho);
    eig = tabs(un) + c;  // = max(|un - c|, |un + c|) exactly, c >= 0
  }
  template <class T>
  __device__ static void flux_r(const PhysC<T>& pc, const T* Q, T* F) {
    T e;
    flux_eig_r(pc, Q, 0, F, e);
  }
  template <class T>
  __device__ static T max_eig_r(const PhysC<T>& pc, const T* Q, int d) {
    T e;
    flux_eig_r<T>(pc, Q, d, nullptr, e);
    return e;
  }
  // The flux along axis d only, F[v] (Fx = F[0..3], Fy = F[4..7] of
  // flux_eig_r; Q1 v = Q2 u), and maxval(abs(Lambda)) along d
  template <class T>
  __device__ static void flux_dir_eig_r(const PhysC<T>& pc, const T* Q, int d, T* F, T& eig) {
    const T irho = mrcp<T>(Q[0]);
    const T u = Q[1] * irho, v = Q[2] * irho;
    const T p = pc.gm1 * (Q[3] - T(0.5) * (Q[1] * u + Q[2] * v));
    const T un = d == 0 ? u : v;
    F[0] = d == 0 ? Q[1] : Q[2];
    F[1] = Q[1] * un + (d == 0 ? p : T(0));
    F[2] = Q[2] * un + (d == 1 ? p : T(0));
    F[3] = un * (Q[3] + p);
    const T c = msqrt<T>(pc.gamma * p * irho);
    eig = tabs(un) + c;  // = max(|un - c|, |un + c|) exactly, c >= 0
  }
  // Constants of the FP32-mixed cell kernel (CFL eigenvalues, admissibility pre-test).
  struct FConst {
    float gm1, gamma;
    __device__ explicit FConst(const Phys& ph) : gm1(ph.f32c[0]), gamma(ph.f32c[1]) {}
  };
  // FP32 eigenvalues for the mixed-precision CFL
  // False when the FP32 pressure is not settled (within 1e-4 of the energy
  // terms it cancels, or not positive): the caller evaluates in FP64.
  __device__ static bool max_eig2_f32(const FConst& fc, const float* q, float& ex, float& ey) {
    const float iq = 1.0f / q[0];
    const float ke = 0.5f * (q[1] * q[1] + q[2] * q[2]) * iq;
    const float p = fc.gm1 * (q[3] - ke);
    if (!(p > 1.0e-4f * fc.gm1 * (fabsf(q[3]) + ke)) || !(q[0] > 0.0f)) return false;
    const float c = sqrtf(fc.gamma * p * iq);
    ex = fabsf(q[1] * iq) + c;
    ey = fabsf(q[2] * iq) + c;
    return ex < 1.0e30f && ey < 1.0e30f;
  }
  // True when every state within e (componentwise) of the FP32 state q passes
  // positive()'s test, with a margin for this evaluation's own rounding.  False
  // means "not settled": the caller re-evaluates the state in FP64.
  // With rho >= r_lo and kinetic energy <= K / r_lo (K from the largest
  // momenta), p >= (gamma - 1) (E_lo - K / r_lo); the test is written times
  // r_lo, without a division.
  __device__ static bool admissible_box_f32(const FConst& fc, const float* q, const float* e) {
    const float r_lo = q[0] - e[0];
    if (!(r_lo > 2.0e-12f) || !(fc.gm1 > 0.0f)) return false;
    const float m1 = fabsf(q[1]) + e[1], m2 = fabsf(q[2]) + e[2];
    const float K = 0.5f * (m1 * m1 + m2 * m2);
    const float mag = (fabsf(q[3]) + e[3]) * r_lo + K;
    const float lhs = fc.gm1 * (((q[3] - e[3]) * r_lo - K) - 1.0e-5f * mag);
    return lhs > 2.0e-12f * r_lo && mag < 1.0e30f;
  }
  // Euler/pde.f90:29-40
  template <class T>
  __device__ static void prim2cons(const PhysC<T>& pc, const T* Vp, T* Q) {
    Q[0] = Vp[0];
    Q[1] = Vp[0] * Vp[1];
    Q[2] = Vp[0] * Vp[2];
    Q[3] = Vp[3] / pc.gm1 + T(0.5) * Vp[0] * (Vp[1] * Vp[1] + Vp[2] * Vp[2]);
  }
  __device__ static void prim2cons(const Phys& ph, const double* Vp, double* Q) { prim2cons<double>(PhysC<double>(ph), Vp, Q); }
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
  template <class T>
  __device__ static void cons2prim(const PhysC<T>& pc, const T* Q, T* Vp) {
    T phi_s = Q[8], phi_g = T(1) - Q[8];
    T rho_s = Q[0] / phi_s, rho_g = Q[4] / phi_g;
    T u_s = Q[1] / Q[0], v_s = Q[2] / Q[0];
    T u_g = Q[5] / Q[4], v_g = Q[6] / Q[4];
    T E_s = Q[3] / phi_s, E_g = Q[7] / phi_g;
    T p_s = pc.gs1 * (E_s - T(0.5) * rho_s * (u_s * u_s + v_s * v_s)) - pc.gsps;
    T p_g = pc.gg1 * (E_g - T(0.5) * rho_g * (u_g * u_g + v_g * v_g)) - pc.ggpg;
    Vp[0] = rho_s; Vp[1] = u_s; Vp[2] = v_s; Vp[3] = p_s;
    Vp[4] = rho_g; Vp[5] = u_g; Vp[6] = v_g; Vp[7] = p_g; Vp[8] = phi_s;
  }
  __device__ static void cons2prim(const Phys& ph, const double* Q, double* Vp) { cons2prim<double>(PhysC<double>(ph), Q, Vp); }
  // Baer-Nunziato/pde.f90:74-119
  template <class T>
  __device__ static void flux(const PhysC<T>& pc, const T* Q, T* F) {
    T phi_s = Q[8], phi_g = T(1) - Q[8];
    T rho_s = Q[0] / phi_s, rho_g = Q[4] / phi_g;
    T u_s = Q[1] / Q[0], v_s = Q[2] / Q[0];
    T u_g = Q[5] / Q[4], v_g = Q[6] / Q[4];
    T E_s = Q[3] / phi_s, E_g = Q[7] / phi_g;
    T p_s = pc.gs1 * (E_s - T(0.5) * rho_s * (u_s * u_s + v_s * v_s)) - pc.gsps;
    T p_g = pc.gg1 * (E_g - T(0.5) * rho_g * (u_g * u_g + v_g * v_g)) - pc.ggpg;
    F[0] = phi_s * rho_s * u_s;
    F[1] = phi_s * (rho_s * u_s * u_s + p_s);
    F[2] = phi_s * rho_s * u_s * v_s;
    F[3] = phi_s * u_s * (E_s + p_s);
    F[4] = phi_g * rho_g * u_g;
    F[5] = phi_g * (rho_g * u_g * u_g + p_g);
    F[6] = phi_g * rho_g * u_g * v_g;
    F[7] = phi_g * u_g * (E_g + p_g);
    F[8] = T(0);
    F[9] = phi_s * rho_s * v_s;
    F[10] = phi_s * rho_s * u_s * v_s;
    F[11] = phi_s * (rho_s * v_s * v_s + p_s);
    F[12] = phi_s * v_s * (E_s + p_s);
    F[13] = phi_g * rho_g * v_g;
    F[14] = phi_g * rho_g * u_g * v_g;
    F[15] = phi_g * (rho_g * v_g * v_g + p_g);
    F[16] = phi_g * v_g * (E_g + p_g);
    F[17] = T(0);
  }
  __device__ static void flux(const Phys& ph, const double* Q, double* F) { flux<double>(PhysC<double>(ph), Q, F); }
  // Baer-Nunziato/pde.f90:125-144
  template <class T>
  __device__ static T max_eig(const PhysC<T>& pc, const T* Q, int d) {
    T Vp[9];
    cons2prim(pc, Q, Vp);
    T u_s = (d == 0) ? Vp[1] * T(1) + Vp[2] * T(0) : Vp[1] * T(0) + Vp[2] * T(1);
    T u_g = (d == 0) ? Vp[5] * T(1) + Vp[6] * T(0) : Vp[5] * T(0) + Vp[6] * T(1);
    T a_s = tsqrt(pc.gs * (Vp[3] + pc.ps) / Vp[0]);
    T a_g = tsqrt(pc.gg * (Vp[7] + pc.pg) / Vp[4]);
    T m = tabs(u_g - a_g);
    m = tmax(m, tabs(u_g + a_g));
    m = tmax(m, tabs(u_s - a_s));
    m = tmax(m, tabs(u_s + a_s));
    m = tmax(m, tabs(u_g));
    m = tmax(m, tabs(u_s));
    return m;
  }
  __device__ static double max_eig(const Phys& ph, const double* Q, int d) { return max_eig<double>(PhysC<double>(ph), Q, d); }
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
  struct FConst {
    float gs, gg, gs1, gg1, gsps, ggpg, ps, pg;
    __device__ explicit FConst(const Phys& ph)
        : gs(ph.f32c[0]), gg(ph.f32c[1]), gs1(ph.f32c[2]), gg1(ph.f32c[3]), gsps(ph.f32c[4]), ggpg(ph.f32c[5]),
          ps(ph.f32c[6]), pg(ph.f32c[7]) {}
  };
  // False when an FP32 pressure p + pi is not settled (within 1e-4 of the
  // terms it cancels, or not positive) or a fraction is out of (0.01, 0.99):
  // the caller evaluates in FP64.
  __device__ static bool max_eig2_f32(const FConst& fc, const float* q, float& ex, float& ey) {
    const float a = q[8], b = 1.0f - q[8];
    if (!(a > 0.01f) || !(b > 0.01f) || !(q[0] > 0.0f) || !(q[4] > 0.0f)) return false;
    const float irs = 1.0f / q[0], irg = 1.0f / q[4];
    const float us = q[1] * irs, vs = q[2] * irs, ug = q[5] * irg, vg = q[6] * irg;
    const float rs = q[0] / a, rg = q[4] / b;
    const float es = q[3] / a, kes = 0.5f * rs * (us * us + vs * vs);
    const float eg = q[7] / b, keg = 0.5f * rg * (ug * ug + vg * vg);
    const float pps = fc.gs1 * (es - kes) - fc.gsps + fc.ps;  // p_s + pi_s
    const float ppg = fc.gg1 * (eg - keg) - fc.ggpg + fc.pg;  // p_g + pi_g
    if (!(pps > 1.0e-4f * (fc.gs1 * (fabsf(es) + kes) + fabsf(fc.gsps) + fabsf(fc.ps))) ||
        !(ppg > 1.0e-4f * (fc.gg1 * (fabsf(eg) + keg) + fabsf(fc.ggpg) + fabsf(fc.pg))))
      return false;
    const float as = sqrtf(fc.gs * pps / rs), ag = sqrtf(fc.gg * ppg / rg);
    ex = fmaxf(fabsf(ug) + ag, fabsf(us) + as);
    ey = fmaxf(fabsf(vg) + ag, fabsf(vs) + as);
    return ex < 1.0e30f && ey < 1.0e30f;
  }
  // True when every state within e (componentwise) of the FP32 state q passes
  // positive()'s test (rho_s, rho_g, p_s + pi_s, p_g + pi_g above 1e-12 and
  // 0 < phi_s < 1), with a margin for this evaluation's own rounding.  With
  // phi in [a_lo, a_hi]: p_s + pi_s = (gamma_s - 1) ((Q3 - ke_s) / phi - pi_s),
  // ke_s = (Q1^2 + Q2^2) / (2 Q0), smallest at the X_lo / a end that makes it
  // smallest.  False means "not settled": the caller re-evaluates in FP64.
  __device__ static bool admissible_box_f32(const FConst& fc, const float* q, const float* e) {
    const float a_lo = q[8] - e[8], a_hi = q[8] + e[8];
    const float b_lo = 1.0f - a_hi, b_hi = 1.0f - a_lo;
    if (!(a_lo > 1.0e-2f) || !(b_lo > 1.0e-2f) || !(fc.gs1 > 0.0f) || !(fc.gg1 > 0.0f)) return false;
    const float q0 = q[0] - e[0], q4 = q[4] - e[4];
    if (!(q0 > 0.0f) || !(q4 > 0.0f) || !(q0 > 4.0e-12f * a_hi) || !(q4 > 4.0e-12f * b_hi)) return false;
    const float s1 = fabsf(q[1]) + e[1], s2 = fabsf(q[2]) + e[2];
    const float g1 = fabsf(q[5]) + e[5], g2 = fabsf(q[6]) + e[6];
    const float kes = 0.5f * (s1 * s1 + s2 * s2) / q0, keg = 0.5f * (g1 * g1 + g2 * g2) / q4;
    const float xs = (q[3] - e[3]) - kes, xg = (q[7] - e[7]) - keg;
    const float ys = xs / (xs >= 0.0f ? a_hi : a_lo) - fc.ps, yg = xg / (xg >= 0.0f ? b_hi : b_lo) - fc.pg;
    const float ms = 1.0e-5f * ((fabsf(q[3]) + e[3] + kes) / a_lo + fabsf(fc.ps));
    const float mg = 1.0e-5f * ((fabsf(q[7]) + e[7] + keg) / b_lo + fabsf(fc.pg));
    return fc.gs1 * (ys - ms) > 2.0e-12f && fc.gg1 * (yg - mg) > 2.0e-12f && ms < 1.0e30f && mg < 1.0e30f;
  }
  // column 9 of PDEMatrixB (Baer-Nunziato/pde.f90:150-186); the other columns are zero
  template <class T>
  __device__ static void matrixB_col9(const PhysC<T>& pc, const T* Q, int d, T* b) {
    const T nv0 = d == 0 ? T(1) : T(0), nv1 = d == 0 ? T(0) : T(1);
    T phi_g = T(1) - Q[8];
    T rho_g = Q[4] / phi_g;
    T u_s = Q[1] / Q[0], v_s = Q[2] / Q[0];
    T u_n = nv0 * u_s + nv1 * v_s;
    T u_g = Q[5] / Q[4], v_g = Q[6] / Q[4];
    T E_g = Q[7] / phi_g;
    T p_g = pc.gg1 * (E_g - T(0.5) * rho_g * (u_g * u_g + v_g * v_g)) - pc.ggpg;
    b[0] = T(0);
    b[1] = -(nv0 * p_g);
    b[2] = -(nv1 * p_g);
    b[3] = -(p_g * u_n);
    b[4] = T(0);
    b[5] = nv0 * p_g;
    b[6] = nv1 * p_g;
    b[7] = p_g * u_n;
    b[8] = u_n;
  }
  // D = RoeMatrix(QL,QR) * (QR - QL): 3-point Gauss-Legendre path integral,
  // Baer-Nunziato/pde.f90:296-320 and the matmul of :348
  template <class T>
  __device__ static void roe_times_jump(const PhysC<T>& pc, const T* QL, const T* QR, int d, T* D) {
    const double sq = sqrt(15.0) / 10.;
    const T sGP[3] = {T(0.5 - sq), T(0.5), T(0.5 + sq)};
    const T wGP[3] = {T(5. / 18.0), T(8. / 18.), T(5. / 18.)};
    T broe[9], b[9], Q[9];
    for (int v = 0; v < 9; ++v) broe[v] = T(0);
    for (int g = 0; g < 3; ++g) {
      for (int v = 0; v < 9; ++v) Q[v] = QL[v] + sGP[g] * (QR[v] - QL[v]);
      matrixB_col9(pc, Q, d, b);
      for (int v = 0; v < 9; ++v) broe[v] = broe[v] + wGP[g] * b[v];
    }
    const T dq9 = QR[8] - QL[8];
    for (int v = 0; v < 9; ++v) D[v] = broe[v] * dq9;
  }
  __device__ static void roe_times_jump(const Phys& ph, const double* QL, const double* QR, int d, double* D) {
    roe_times_jump<double>(PhysC<double>(ph), QL, QR, d, D);
  }
  // Reciprocal-sharing forms for the FP32-mixed mode's FP64 face flux and
  // subcell re-solve (compiled with fused multiply-adds; values agree with the
  // reference order to rounding).  Algebraically the reference expressions of
  // Baer-Nunziato/pde.f90 with phi = alpha_s (Q8), phi_g = 1 - phi:
  //   phi p_s = (gamma_s - 1) (Q3 - (Q1^2 + Q2^2) / (2 Q0)) - gamma_s pi_s phi,
  //   phi rho_s u_s = Q1, (p_s + pi_s) / rho_s = (phi p_s + pi_s phi) / Q0,
  // and likewise for the gas with Q4..Q7 and phi_g; so a state needs 1/Q0
  // and 1/Q4 only, both from one reciprocal of Q0 Q4.
  // Flux F[d*V + v] (pde.f90:74-119) and maxval(abs(Lambda)) along axis d (:125-144).
  template <class T>
  __device__ static void flux_eig_r(const PhysC<T>& pc, const T* Q, int d, T* F, T& eig) {
    const T r = mrcp<T>(Q[0] * Q[4]);
    const T i0 = Q[4] * r, i4 = Q[0] * r;
    const T u_s = Q[1] * i0, v_s = Q[2] * i0, u_g = Q[5] * i4, v_g = Q[6] * i4;
    const T phi_s = Q[8], phi_g = T(1) - Q[8];
    const T pps = pc.gs1 * (Q[3] - T(0.5) * (Q[1] * u_s + Q[2] * v_s)) - pc.gsps * phi_s;  // phi p_s
    const T ppg = pc.gg1 * (Q[7] - T(0.5) * (Q[5] * u_g + Q[6] * v_g)) - pc.ggpg * phi_g;  // phi_g p_g
    if (F) {
      F[0] = Q[1]; F[1] = Q[1] * u_s + pps; F[2] = Q[1] * v_s; F[3] = u_s * (Q[3] + pps);
      F[4] = Q[5]; F[5] = Q[5] * u_g + ppg; F[6] = Q[5] * v_g; F[7] = u_g * (Q[7] + ppg); F[8] = T(0);
      F[9] = Q[2]; F[10] = Q[2] * u_s; F[11] = Q[2] * v_s + pps; F[12] = v_s * (Q[3] + pps);
      F[13] = Q[6]; F[14] = Q[6] * u_g; F[15] = Q[6] * v_g + ppg; F[16] = v_g * (Q[7] + ppg); F[17] = T(0);
    }
    const T a_s = msqrt<T>(pc.gs * (pps + pc.ps * phi_s) * i0);
    const T a_g = msqrt<T>(pc.gg * (ppg + pc.pg * phi_g) * i4);
    const T us = d == 0 ? u_s : v_s, ug = d == 0 ? u_g : v_g;
    // max(|u - a|, |u + a|) = |u| + a exactly for a >= 0 (a NaN propagates alike)
    eig = tmax(tabs(ug) + a_g, tabs(us) + a_s);
  }
  template <class T>
  __device__ static void flux_r(const PhysC<T>& pc, const T* Q, T* F) {
    T e;
    flux_eig_r(pc, Q, 0, F, e);
  }
  template <class T>
  __device__ static T max_eig_r(const PhysC<T>& pc, const T* Q, int d) {
    T e;
    flux_eig_r<T>(pc, Q, d, nullptr, e);
    return e;
  }
  // The flux along axis d only, F[v] (the d-th half of flux_eig_r's F; Q1 v_s
  // = Q2 u_s), and maxval(abs(Lambda)) along d
  template <class T>
  __device__ static void flux_dir_eig_r(const PhysC<T>& pc, const T* Q, int d, T* F, T& eig) {
    const T r = mrcp<T>(Q[0] * Q[4]);
    const T i0 = Q[4] * r, i4 = Q[0] * r;
    const T u_s = Q[1] * i0, v_s = Q[2] * i0, u_g = Q[5] * i4, v_g = Q[6] * i4;
    const T phi_s = Q[8], phi_g = T(1) - Q[8];
    const T pps = pc.gs1 * (Q[3] - T(0.5) * (Q[1] * u_s + Q[2] * v_s)) - pc.gsps * phi_s;  // phi p_s
    const T ppg = pc.gg1 * (Q[7] - T(0.5) * (Q[5] * u_g + Q[6] * v_g)) - pc.ggpg * phi_g;  // phi_g p_g
    const T us = d == 0 ? u_s : v_s, ug = d == 0 ? u_g : v_g;
    F[0] = d == 0 ? Q[1] : Q[2];
    F[1] = Q[1] * us + (d == 0 ? pps : T(0));
    F[2] = Q[2] * us + (d == 1 ? pps : T(0));
    F[3] = us * (Q[3] + pps);
    F[4] = d == 0 ? Q[5] : Q[6];
    F[5] = Q[5] * ug + (d == 0 ? ppg : T(0));
    F[6] = Q[6] * ug + (d == 1 ? ppg : T(0));
    F[7] = ug * (Q[7] + ppg);
    F[8] = T(0);
    const T a_s = msqrt<T>(pc.gs * (pps + pc.ps * phi_s) * i0);
    const T a_g = msqrt<T>(pc.gg * (ppg + pc.pg * phi_g) * i4);
    // max(|u - a|, |u + a|) = |u| + a exactly for a >= 0 (a NaN propagates alike)
    eig = tmax(tabs(ug) + a_g, tabs(us) + a_s);
  }
  // p_g = (gamma_g - 1) (Q7 Q4 - (Q5^2 + Q6^2) / 2) / (Q4 phi_g) - gamma_g pi_g
  // and u_n = qn / Q0 (qn = n . (Q1, Q2)) from one reciprocal of Q0 Q4 phi_g
  template <class T>
  __device__ static void p_gas_un_r(const PhysC<T>& pc, const T* Q, T qn, T& p_g, T& un) {
    const T b = Q[4] * (T(1) - Q[8]);
    const T r = mrcp<T>(b * Q[0]);
    p_g = pc.gg1 * (Q[7] * Q[4] - T(0.5) * (Q[5] * Q[5] + Q[6] * Q[6])) * (Q[0] * r) - pc.ggpg;
    un = qn * (b * r);
  }
  // roe_times_jump with column 9 of B from p_g and u_n of p_gas_un_r
  template <class T>
  __device__ static void roe_times_jump_r(const PhysC<T>& pc, const T* QL, const T* QR, int d, T* D) {
    const double sq = sqrt(15.0) / 10.;
    const T sGP[3] = {T(0.5 - sq), T(0.5), T(0.5 + sq)};
    const T wGP[3] = {T(5. / 18.0), T(8. / 18.), T(5. / 18.)};
    T bp = T(0), bu = T(0), bpu = T(0);  // path integrals of p_g, u_n and p_g u_n
#pragma unroll
    for (int g = 0; g < 3; ++g) {
      T Q[9];
#pragma unroll
      for (int v = 0; v < 9; ++v) Q[v] = QL[v] + sGP[g] * (QR[v] - QL[v]);
      T p, un;
      p_gas_un_r(pc, Q, d == 0 ? Q[1] : Q[2], p, un);
      bp = bp + wGP[g] * p;
      bu = bu + wGP[g] * un;
      bpu = bpu + wGP[g] * (p * un);
    }
    const T dq9 = QR[8] - QL[8];
    D[0] = T(0);
    D[1] = d == 0 ? -bp * dq9 : T(0);
    D[2] = d == 1 ? -bp * dq9 : T(0);
    D[3] = -bpu * dq9;
    D[4] = T(0);
    D[5] = d == 0 ? bp * dq9 : T(0);
    D[6] = d == 1 ? bp * dq9 : T(0);
    D[7] = bpu * dq9;
    D[8] = bu * dq9;
  }
  template <class T>
  __device__ static void src_ncp_r(const PhysC<T>& pc, const T* Q, T ax, T ay, T* S) {
    T p_g, un;
    p_gas_un_r(pc, Q, Q[1] * ax + Q[2] * ay, p_g, un);
    S[0] = T(0);
    S[1] = p_g * ax;
    S[2] = p_g * ay;
    S[3] = p_g * un;
    S[4] = T(0);
    S[5] = -(p_g * ax);
    S[6] = -(p_g * ay);
    S[7] = -(p_g * un);
    S[8] = -un;
  }
  // -NCP, Baer-Nunziato/pde.f90:192-231 and :277-290; only the volume-fraction gradient enters
  template <class T>
  __device__ static void src_ncp(const PhysC<T>& pc, const T* Q, T ax, T ay, T* S) {
    T phi_g = T(1) - Q[8];
    T rho_g = Q[4] / phi_g;
    T u_s = Q[1] / Q[0], v_s = Q[2] / Q[0];
    T u_g = Q[5] / Q[4], v_g = Q[6] / Q[4];
    T E_g = Q[7] / phi_g;
    T p_g = pc.gg1 * (E_g - T(0.5) * rho_g * (u_g * u_g + v_g * v_g)) - pc.ggpg;
    T un = u_s * ax + v_s * ay;
    S[0] = -T(0);
    S[1] = -(-p_g * ax);
    S[2] = -(-p_g * ay);
    S[3] = -(-p_g * un);
    S[4] = -T(0);
    S[5] = -(p_g * ax);
    S[6] = -(p_g * ay);
    S[7] = -(p_g * un);
    S[8] = -un;
  }
  __device__ static void src_ncp(const Phys& ph, const double* Q, double ax, double ay, double* S) {
    src_ncp<double>(PhysC<double>(ph), Q, ax, ay, S);
  }
  // Baer-Nunziato/pde.f90:49-68
  template <class T>
  __device__ static void prim2cons(const PhysC<T>& pc, const T* Vp, T* Q) {
    Q[0] = Vp[8] * Vp[0];
    Q[1] = Q[0] * Vp[1];
    Q[2] = Q[0] * Vp[2];
    Q[3] = Q[0] * (T(0.5) * (Vp[1] * Vp[1] + Vp[2] * Vp[2]) + (Vp[3] + pc.gsps) / (Vp[0] * pc.gs1));
    Q[4] = (T(1) - Vp[8]) * Vp[4];
    Q[5] = Q[4] * Vp[5];
    Q[6] = Q[4] * Vp[6];
    Q[7] = Q[4] * (T(0.5) * (Vp[5] * Vp[5] + Vp[6] * Vp[6]) + (Vp[7] + pc.ggpg) / (Vp[4] * pc.gg1));
    Q[8] = Vp[8];
  }
  __device__ static void prim2cons(const Phys& ph, const double* Vp, double* Q) { prim2cons<double>(PhysC<double>(ph), Vp, Q); }
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
  struct FConst {
    __device__ explicit FConst(const Phys&) {}
  };
  // Advection-Diffusion/pde.f90:70-80 (|cx nv1 + cy nv2|)
  __device__ static double max_eig_c(const Phys& ph, int d) {
    return fabs(d == 0 ? ph.cx * 1.0 + ph.cy * 0.0 : ph.cx * 0.0 + ph.cy * 1.0);
  }
};

}  // namespace aderdg
