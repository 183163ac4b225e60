// output.cu -- on-device output and error analysis of a simulation.
//
// k_cell_averages: the cell averages of uh and their primitive variables,
// the field the reference writes to its VTK files (Euler/write_data.f90:17-33,
// Baer-Nunziato/write_data.f90, Advection-Diffusion/write_data.f90), with the
// reference's summation order; one thread per cell.
//
// k_error_norms: the error of the cell averages of one variable against an
// exact field evaluated at the cells' Gauss-Legendre nodes (analyze_soln,
// Euler/analyze_soln.f90:10-56, which compares with the initial field; here
// also with the translated vortex and the translated, damped sine wave at the
// current time).  Sums in FP64 atomics, so the L1/L2 norms are reproducible to
// rounding, the L-infinity norm exactly.
//
// Compiled with --fmad=false (reference operation order).
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <string>

#include "ic_eval.h"
#include "setup.h"

namespace aderdg {

struct OutArgs {
  int P, V, imax, jmax, system, primitive;
  double w[10];
  double gamma, gs, gg, ps, pg;  // Euler / Baer-Nunziato constants
};

// PDECons2Prim of the three systems (Euler/pde.f90:8-23, Baer-Nunziato/pde.f90:8-43;
// advection-diffusion: the state itself)
__device__ void cons2prim_out(const OutArgs& g, const double* Q, double* Vp) {
  if (g.system == ADERDG_SYS_EULER) {
    const double p = (g.gamma - 1.0) * (Q[3] - 0.5 * (Q[1] * Q[1] + Q[2] * Q[2]) / Q[0]);
    Vp[0] = Q[0];
    Vp[1] = Q[1] / Q[0];
    Vp[2] = Q[2] / Q[0];
    Vp[3] = p;
  } else if (g.system == ADERDG_SYS_BN) {
    const double phi_s = Q[8], phi_g = 1.0 - Q[8];
    const double rho_s = Q[0] / phi_s, rho_g = Q[4] / phi_g;
    const double u_s = Q[1] / Q[0], v_s = Q[2] / Q[0];
    const double u_g = Q[5] / Q[4], v_g = Q[6] / Q[4];
    const double E_s = Q[3] / phi_s, E_g = Q[7] / phi_g;
    Vp[0] = rho_s;
    Vp[1] = u_s;
    Vp[2] = v_s;
    Vp[3] = (g.gs - 1.0) * (E_s - 0.5 * rho_s * (u_s * u_s + v_s * v_s)) - g.gs * g.ps;
    Vp[4] = rho_g;
    Vp[5] = u_g;
    Vp[6] = v_g;
    Vp[7] = (g.gg - 1.0) * (E_g - 0.5 * rho_g * (u_g * u_g + v_g * v_g)) - g.gg * g.pg;
    Vp[8] = phi_s;
  } else {
    Vp[0] = Q[0];
  }
}

__global__ void __launch_bounds__(256) k_cell_averages(OutArgs g, const double* uh, double* out) {
  const long long cell = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (cell >= (long long)g.imax * g.jmax) return;
  const int P = g.P, V = g.V;
  const double* u = uh + (size_t)cell * P * P * V;
  double Q[9];
  // Euler/write_data.f90:21-29: Q(iVar) += wGPN(ii) * wGPN(jj) * uh(iVar, ii, jj)
  for (int v = 0; v < V; ++v) {
    double q = 0.0;
    for (int jj = 0; jj < P; ++jj)
      for (int ii = 0; ii < P; ++ii) q = q + g.w[ii] * g.w[jj] * u[(ii + P * jj) * V + v];
    Q[v] = q;
  }
  double* o = out + (size_t)cell * V;
  if (g.primitive) {
    double Vp[9];
    cons2prim_out(g, Q, Vp);
    for (int v = 0; v < V; ++v) o[v] = Vp[v];
  } else {
    for (int v = 0; v < V; ++v) o[v] = Q[v];
  }
}

struct ErrArgs {
  OutArgs o;
  aderdg_config cfg;
  int ic, var;
  double p[32];
  double pi, xi[10];
  double dx, dy;
  double shift_x, shift_y, damp;  // exact field = damp * IC(x - shift_x, y - shift_y), wrapped periodically
};

__global__ void __launch_bounds__(256) k_error_norms(ErrArgs g, const double* uh, double* sums /* [2]: sum|e|, sum e^2 */,
                                                     unsigned long long* emax) {
  const long long cell = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const bool in = cell < (long long)g.o.imax * g.o.jmax;
  double e = 0.0;
  if (in) {
    const int P = g.o.P, V = g.o.V;
    const int i = (int)(cell % g.o.imax), j = (int)(cell / g.o.imax);
    // corner = centre - dx/2 (Euler/analyze_soln.f90:24)
    const double x0 = (g.cfg.xl[0] + ((double)i + 0.5) * g.dx) - 0.5 * g.dx;
    const double y0 = (g.cfg.xl[1] + ((double)j + 0.5) * g.dy) - 0.5 * g.dy;
    const double Lx = g.cfg.xr[0] - g.cfg.xl[0], Ly = g.cfg.xr[1] - g.cfg.xl[1];
    const double* u = uh + (size_t)cell * P * P * V;
    double ex = 0.0, num = 0.0, u0[9];
    // Euler/analyze_soln.f90:40-46: l (y) outer, k (x) inner
    for (int l = 0; l < P; ++l)
      for (int k = 0; k < P; ++k) {
        double x = x0 + g.xi[k] * g.dx - g.shift_x, y = y0 + g.xi[l] * g.dy - g.shift_y;
        if (g.shift_x != 0.0) x = g.cfg.xl[0] + (x - g.cfg.xl[0]) - floor((x - g.cfg.xl[0]) / Lx) * Lx;
        if (g.shift_y != 0.0) y = g.cfg.xl[1] + (y - g.cfg.xl[1]) - floor((y - g.cfg.xl[1]) / Ly) * Ly;
        eval_ic(g.cfg, g.ic, g.p, g.pi, x, y, u0);
        ex = ex + g.o.w[l] * g.o.w[k] * (g.damp * u0[g.var]);
        num = num + g.o.w[l] * g.o.w[k] * u[(k + P * l) * V + g.var];
      }
    e = fabs(ex - num);
  }
  // block sums, one atomic per block
  __shared__ double s1[8], s2[8];
  __shared__ unsigned long long sm[8];
  double a1 = e, a2 = e * e;
  unsigned long long m = (unsigned long long)__double_as_longlong(e);
  for (int o = 16; o > 0; o >>= 1) {
    a1 += __shfl_down_sync(0xffffffffu, a1, o);
    a2 += __shfl_down_sync(0xffffffffu, a2, o);
    const unsigned long long mo = __shfl_down_sync(0xffffffffu, m, o);
    m = m > mo ? m : mo;
  }
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    s1[w] = a1;
    s2[w] = a2;
    sm[w] = m;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double b1 = 0.0, b2 = 0.0;
    unsigned long long bm = 0ull;
    for (int q = 0; q < (int)(blockDim.x >> 5); ++q) {
      b1 += s1[q];
      b2 += s2[q];
      bm = bm > sm[q] ? bm : sm[q];
    }
    atomicAdd(&sums[0], b1);
    atomicAdd(&sums[1], b2);
    atomicMax(emax, bm);
  }
}

namespace {

bool out_args(const aderdg_config& cfg, OutArgs& g, std::string* why) {
  HostOps ops;
  if (!build_ops(cfg.N, ops, why)) return false;
  std::memset(&g, 0, sizeof(g));
  g.P = ops.P;
  g.V = cfg.system == ADERDG_SYS_ADVDIFF ? 1 : cfg.system == ADERDG_SYS_EULER ? 4 : 9;
  g.imax = cfg.imax;
  g.jmax = cfg.jmax;
  g.system = cfg.system;
  for (int k = 0; k < ops.P; ++k) g.w[k] = ops.w[k];
  g.gamma = cfg.gamma;
  g.gs = cfg.gamma_s;
  g.gg = cfg.gamma_g;
  g.ps = cfg.pi_s;
  g.pg = cfg.pi_g;
  return true;
}

}  // namespace

cudaError_t launch_cell_averages(const aderdg_config& cfg, const double* uh, int primitive, double* out,
                                 cudaStream_t s, std::string* why) {
  OutArgs g;
  if (!out_args(cfg, g, why)) return cudaErrorInvalidValue;
  g.primitive = primitive;
  const long long n = (long long)cfg.imax * cfg.jmax;
  k_cell_averages<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(g, uh, out);
  return cudaGetLastError();
}

cudaError_t launch_error_norms(const aderdg_config& cfg, const double* uh, int ic, const double* params, int var,
                               double time, double* sums_dev, unsigned long long* max_dev, cudaStream_t s,
                               std::string* why) {
  ErrArgs g;
  std::memset(&g, 0, sizeof(g));
  if (!out_args(cfg, g.o, why)) return cudaErrorInvalidValue;
  if (var < 0 || var >= g.o.V) {
    if (why) *why = "variable index out of range";
    return cudaErrorInvalidValue;
  }
  g.cfg = cfg;
  g.ic = ic;
  g.var = var;
  if (params) std::memcpy(g.p, params, sizeof(g.p));
  if (!ic_valid(cfg.system, ic, g.p)) {
    if (why) *why = "initial field " + std::to_string(ic) + " is not defined for this system / parameters";
    return cudaErrorInvalidValue;
  }
  HostOps ops;
  build_ops(cfg.N, ops, why);
  for (int k = 0; k < ops.P; ++k) g.xi[k] = ops.xi[k];
  g.pi = pi_value();
  g.dx = (cfg.xr[0] - cfg.xl[0]) / cfg.imax;
  g.dy = (cfg.xr[1] - cfg.xl[1]) / cfg.jmax;
  g.damp = 1.0;
  // exact solutions that move: the isentropic vortex travels with the free
  // stream (p[4], p[5]); the sine wave travels with (cx, cy) and decays by
  // exp(-8 pi^2 a t) (periodic domains)
  if (ic == ADERDG_IC_EULER_VORTEX) {
    g.shift_x = g.p[4] * time;
    g.shift_y = g.p[5] * time;
  } else if (ic == ADERDG_IC_AD_SINE) {
    g.shift_x = cfg.cx * time;
    g.shift_y = cfg.cy * time;
    g.damp = std::exp(-8.0 * g.pi * g.pi * cfg.a * time);
  }
  const long long n = (long long)cfg.imax * cfg.jmax;
  k_error_norms<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(g, uh, sums_dev, max_dev);
  return cudaGetLastError();
}

}  // namespace aderdg
