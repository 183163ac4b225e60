// ic_eval.h -- pointwise initial fields, shared by the host set-up
// (setup.cpp, aderdg_project_initial_condition) and the on-device set-up
// (initial.cu).  The same expressions on both sides; transcendental
// functions come from the host libm or the CUDA math library respectively.
//
// The double Mach reflection (Euler/initialize.f90:311-341), the zero field
// (Advection-Diffusion/initialize.f90:148-164) and the 1D Baer-Nunziato
// Riemann problems (Baer-Nunziato/initialize.f90:302-407) are the
// reference's; the isentropic vortex, the 2D four-quadrant Riemann problem,
// the two-phase cylinder and the sine wave are set-up extensions with the
// parameters listed in aderdg_gpu.h.
#pragma once

#include <math.h>

#include "../../include/aderdg_gpu.h"

#if defined(__CUDACC__)
#define ADERDG_HD __host__ __device__
#else
#define ADERDG_HD
#endif

namespace aderdg {

ADERDG_HD inline void ic_euler_prim2cons(double g, const double* V, double* Q) {  // Euler/pde.f90:29-40
  Q[0] = V[0];
  Q[1] = V[0] * V[1];
  Q[2] = V[0] * V[2];
  Q[3] = V[3] / (g - 1) + 0.5 * V[0] * (V[1] * V[1] + V[2] * V[2]);
}

ADERDG_HD inline void ic_bn_prim2cons(const aderdg_config& c, const double* V, double* Q) {  // Baer-Nunziato/pde.f90:49-68
  const double gs = c.gamma_s, gg = c.gamma_g, ps = c.pi_s, pg = c.pi_g;
  Q[0] = V[8] * V[0];
  Q[1] = Q[0] * V[1];
  Q[2] = Q[0] * V[2];
  Q[3] = Q[0] * (0.5 * (V[1] * V[1] + V[2] * V[2]) + (V[3] + gs * ps) / (V[0] * (gs - 1.0)));
  Q[4] = (1.0 - V[8]) * V[4];
  Q[5] = Q[4] * V[5];
  Q[6] = Q[4] * V[6];
  Q[7] = Q[4] * (0.5 * (V[5] * V[5] + V[6] * V[6]) + (V[7] + gg * pg) / (V[4] * (gg - 1.0)));
  Q[8] = V[8];
}

// Row of the Baer-Nunziato 1D Riemann problem table for ICType t, or -1.
ADERDG_HD inline int ic_bn_rp1d_row(double t) {
  const int k = (int)t;
  return k == 1 ? 0 : k == 2 ? 1 : k == 3 ? 2 : k == 7 ? 3 : -1;
}

// True when (system, ic, params) name a field this function can evaluate.
ADERDG_HD inline bool ic_valid(int system, int ic, const double* p) {
  switch (ic) {
    case ADERDG_IC_AD_ZERO:
    case ADERDG_IC_AD_SINE: return system == ADERDG_SYS_ADVDIFF;
    case ADERDG_IC_EULER_DMR:
    case ADERDG_IC_EULER_VORTEX:
    case ADERDG_IC_EULER_RP2D: return system == ADERDG_SYS_EULER;
    case ADERDG_IC_BN_RP1D: return system == ADERDG_SYS_BN && ic_bn_rp1d_row(p[0]) >= 0;
    case ADERDG_IC_BN_CYLINDER: return system == ADERDG_SYS_BN;
  }
  return false;
}

// Conservative state u at (x, y); pi = 4 atan(1) as the caller computes it.
// Returns -1 for an unknown field.
ADERDG_HD inline int eval_ic(const aderdg_config& c, int ic, const double* p, double pi, double x, double y, double* u) {
  double V[9];
  switch (ic) {
    case ADERDG_IC_AD_ZERO:
      u[0] = 0.0;
      return 0;
    case ADERDG_IC_AD_SINE:
      u[0] = p[0] * sin(2.0 * pi * x) * sin(2.0 * pi * y);
      return 0;
    case ADERDG_IC_EULER_DMR:
      if (x <= 1.0 / 6.0 + y / tan(pi / 3.0)) {
        V[0] = 8.0;
        V[1] = 8.25 * cos(pi / 6.0);
        V[2] = -8.25 * sin(pi / 6.0);
        V[3] = 116.5;
      } else {
        V[0] = 1.4;
        V[1] = 0.0;
        V[2] = 0.0;
        V[3] = 1.0;
      }
      ic_euler_prim2cons(c.gamma, V, u);
      return 0;
    case ADERDG_IC_EULER_VORTEX: {
      const double g = c.gamma, eps = p[0];
      const double dx = x - p[1], dy = y - p[2], r2 = dx * dx + dy * dy;
      const double amp = eps / (2.0 * pi) * exp(0.5 * (1.0 - r2));
      const double T0 = p[6] / p[3];
      const double T = T0 + -(g - 1.0) * eps * eps / (8.0 * g * pi * pi) * exp(1.0 - r2);
      const double rho = p[3] * pow(T / T0, 1.0 / (g - 1.0));
      V[0] = rho;
      V[1] = p[4] - amp * dy;
      V[2] = p[5] + amp * dx;
      V[3] = rho * T;
      ic_euler_prim2cons(g, V, u);
      return 0;
    }
    case ADERDG_IC_EULER_RP2D: {
      const int q = (y >= p[1]) ? (x >= p[0] ? 0 : 1) : (x < p[0] ? 2 : 3);
      for (int k = 0; k < 4; ++k) V[k] = p[2 + 4 * q + k];
      ic_euler_prim2cons(c.gamma, V, u);
      return 0;
    }
    case ADERDG_IC_BN_RP1D: {
      const double left[4][9] = {{1.0, 0.0, 0.0, 1.0, 0.5, 0.0, 0.0, 1.0, 0.4},
                                 {800.0, 0.0, 0.0, 500.0, 1.5, 0.0, 0.0, 2.0, 0.4},
                                 {1.0, 0.9, 0.0, 2.5, 1.0, 0.0, 0.0, 1.0, 0.9},
                                 {800.0, 1.0, 0.0, 1.0, 2.0, 1.0, 0.0, 1.0, 0.99}};
      const double right[4][9] = {{2.0, 0.0, 0.0, 2.0, 1.5, 0.0, 0.0, 2.0, 0.8},
                                  {1000.0, 0.0, 0.0, 600.0, 1.0, 0.0, 0.0, 1.0, 0.3},
                                  {1.0, 0.0, 0.0, 1.0, 1.2, 1.0, 0.0, 2.0, 0.2},
                                  {1000.0, 1.0, 0.0, 1.0, 1.0, 1.0, 0.0, 1.0, 0.01}};
      const int row = ic_bn_rp1d_row(p[0]);
      if (row < 0) return -1;
      const double* s = (x <= p[1]) ? left[row] : right[row];
      for (int k = 0; k < 9; ++k) V[k] = s[k];
      ic_bn_prim2cons(c, V, u);
      return 0;
    }
    case ADERDG_IC_BN_CYLINDER: {
      const double dx = x - p[0], dy = y - p[1];
      const double* s = (dx * dx + dy * dy < p[2] * p[2]) ? p + 3 : p + 8;
      V[0] = s[1];
      V[1] = 0.0;
      V[2] = 0.0;
      V[3] = s[2];
      V[4] = s[3];
      V[5] = 0.0;
      V[6] = 0.0;
      V[7] = s[4];
      V[8] = s[0];
      ic_bn_prim2cons(c, V, u);
      return 0;
    }
  }
  return -1;
}

}  // namespace aderdg
