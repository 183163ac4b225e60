// initial.cu -- on-device set-up of a simulation: the initial field at the
// Gauss-Legendre nodes of every cell (uh) and at its subcell barycentres (the
// initial-limiter candidates), as initialize does on the host
// (Euler/initialize.f90:262-307).  Same expressions as the host set-up
// (ic_eval.h); compiled with --fmad=false, so the values differ from the
// host's only where the device and host math libraries round a
// transcendental function differently.  One thread per (cell, point).
#include <cuda_runtime.h>

#include <cstring>
#include <string>

#include "ic_eval.h"
#include "setup.h"

namespace aderdg {

struct IcArgs {
  aderdg_config cfg;
  int ic;
  double p[32];
  double pi;
  double xi[10];
  double xlb[19];
  int P, S, V;
  double dx, dy;
  long long ncells;
  int with_lh;
};

__global__ void __launch_bounds__(256) k_initial_field(IcArgs g, double* uh, double* lh) {
  const int P2 = g.P * g.P, S2 = g.S * g.S;
  const int npts = P2 + (g.with_lh ? S2 : 0);
  const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= g.ncells * npts) return;
  const long long cell = gid / npts;
  const int pt = (int)(gid - cell * npts);
  const int i = (int)(cell % g.cfg.imax), j = (int)(cell / g.cfg.imax);
  // cell corner = centre - dx/2 (Euler/initialize.f90:264-266)
  const double x0 = (g.cfg.xl[0] + ((double)i + 0.5) * g.dx) - 0.5 * g.dx;
  const double y0 = (g.cfg.xl[1] + ((double)j + 0.5) * g.dy) - 0.5 * g.dy;
  double u[9];
  if (pt < P2) {
    const int k = pt % g.P, l = pt / g.P;
    eval_ic(g.cfg, g.ic, g.p, g.pi, x0 + g.xi[k] * g.dx, y0 + g.xi[l] * g.dy, u);
    double* dst = uh + ((size_t)cell * P2 + k + g.P * l) * g.V;
    for (int v = 0; v < g.V; ++v) dst[v] = u[v];
  } else {
    const int q = pt - P2, a = q % g.S, b = q / g.S;
    eval_ic(g.cfg, g.ic, g.p, g.pi, x0 + g.xlb[a] * g.dx, y0 + g.xlb[b] * g.dy, u);
    double* dst = lh + ((size_t)cell * S2 + a + g.S * b) * g.V;
    for (int v = 0; v < g.V; ++v) dst[v] = u[v];
  }
}

// The initial-limiter candidates of the cells the initial DMP limited
// (status != 0): the initial field at their subcell barycentres, written to
// both Lh buffers, as the initial DMP's copy of the candidates does
// (Euler/initialize.f90:296-317).  Evaluated for those cells only, with the
// expressions of k_initial_field (same values).
__global__ void __launch_bounds__(256) k_initial_lh(IcArgs g, const int* status, double* lh0, double* lh1) {
  const int S2 = g.S * g.S;
  const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= g.ncells * S2) return;
  const long long cell = gid / S2;
  if (status[cell] == 0) return;
  const int q = (int)(gid - cell * S2), a = q % g.S, b = q / g.S;
  const int i = (int)(cell % g.cfg.imax), j = (int)(cell / g.cfg.imax);
  const double x0 = (g.cfg.xl[0] + ((double)i + 0.5) * g.dx) - 0.5 * g.dx;
  const double y0 = (g.cfg.xl[1] + ((double)j + 0.5) * g.dy) - 0.5 * g.dy;
  double u[9];
  eval_ic(g.cfg, g.ic, g.p, g.pi, x0 + g.xlb[a] * g.dx, y0 + g.xlb[b] * g.dy, u);
  const size_t o = ((size_t)cell * S2 + a + g.S * b) * g.V;
  for (int v = 0; v < g.V; ++v) {
    lh0[o + v] = u[v];
    lh1[o + v] = u[v];
  }
}

namespace {

bool ic_args(const aderdg_config& cfg, int ic, const double* params, IcArgs& g, std::string* why) {
  HostOps ops;
  if (!build_ops(cfg.N, ops, why)) return false;
  std::memset(&g, 0, sizeof(g));
  g.cfg = cfg;
  g.ic = ic;
  if (params) std::memcpy(g.p, params, sizeof(g.p));
  if (!ic_valid(cfg.system, ic, g.p)) {
    if (why) *why = "initial field " + std::to_string(ic) + " is not defined for this system / parameters";
    return false;
  }
  g.pi = pi_value();
  for (int k = 0; k < ops.P; ++k) g.xi[k] = ops.xi[k];
  for (int k = 0; k < ops.S; ++k) g.xlb[k] = ops.xilimbary[k];
  g.P = ops.P;
  g.S = ops.S;
  g.V = cfg.system == ADERDG_SYS_ADVDIFF ? 1 : cfg.system == ADERDG_SYS_EULER ? 4 : 9;
  g.dx = (cfg.xr[0] - cfg.xl[0]) / cfg.imax;
  g.dy = (cfg.xr[1] - cfg.xl[1]) / cfg.jmax;
  g.ncells = (long long)cfg.imax * cfg.jmax;
  return true;
}

}  // namespace

// Fills uh (and lh when non-null) of one simulation laid out from cell 0 of
// the given pointers; the caller validated cfg.  Returns a CUDA error.
cudaError_t launch_initial_field(const aderdg_config& cfg, int ic, const double* params, double* uh, double* lh,
                                 cudaStream_t s, std::string* why) {
  IcArgs g;
  if (!ic_args(cfg, ic, params, g, why)) return cudaErrorInvalidValue;
  g.with_lh = lh != nullptr;
  const long long n = g.ncells * (g.P * g.P + (lh ? g.S * g.S : 0));
  k_initial_field<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(g, uh, lh);
  return cudaGetLastError();
}

// The subcell candidates of the limited cells (status != 0) into lh0 and lh1,
// all laid out from cell 0 of the given pointers.
cudaError_t launch_initial_lh(const aderdg_config& cfg, int ic, const double* params, const int* status, double* lh0,
                              double* lh1, cudaStream_t s, std::string* why) {
  IcArgs g;
  if (!ic_args(cfg, ic, params, g, why)) return cudaErrorInvalidValue;
  const long long n = g.ncells * g.S * g.S;
  if (n > 0) k_initial_lh<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(g, status, lh0, lh1);
  return cudaGetLastError();
}

}  // namespace aderdg
