// predictor_tu.cu -- instantiates the space-time predictor (K1) for one
// (system, N), selected by -DADERDG_SYS=<0|1|2> -DADERDG_N=<1..5>.
// Compiled with fused multiply-adds (the predictor's contractions are FMA
// chains; its results agree with the reference to rounding, not bit for bit).
#include <cmath>

#include "faces.cuh"
#include "limiter.cuh"
#include "predictor.cuh"
#include "tables.h"

#ifndef ADERDG_SYS
#error "ADERDG_SYS must be defined"
#endif
#ifndef ADERDG_N
#error "ADERDG_N must be defined"
#endif

namespace aderdg {
namespace {

#if ADERDG_SYS == 0
using Sys = ADSys;
#elif ADERDG_SYS == 1
using Sys = EulerSys;
#else
using Sys = BNSys;
#endif
constexpr int N = ADERDG_N;

template <class R>
void make_ops(const HostOps& h, void* out) {
  constexpr int P = N + 1, S = 2 * N + 1;
  DevOps<N, R> o;
  for (int a = 0; a < P; ++a) {
    o.w[a] = (R)h.w[a];
    o.FL[a] = (R)h.FL[a];
    o.FR[a] = (R)h.FR[a];
    o.wd[a] = h.w[a];
    o.FLd[a] = h.FL[a];
    o.FRd[a] = h.FR[a];
    o.xid[a] = h.xi[a];
  }
  for (int a = 0; a < P; ++a) {
    o.wf[a] = (float)h.w[a];
    o.FLf[a] = (float)h.FL[a];
    o.FRf[a] = (float)h.FR[a];
  }
  for (int j = 0; j < P; ++j)
    for (int i = 0; i < P; ++i) o.iwwf[i + P * j] = (float)(1.0 / (h.w[i] * h.w[j]));
  for (int k = 0; k < P * P; ++k) {
    o.Kxi[k] = (R)h.Kxi[k];
    o.dudx[k] = (R)h.dudx[k];
  }
  // derived time operators (FP64, no contraction: identical on every host)
  double T[P][P];
  for (int lp = 0; lp < P; ++lp)
    for (int l = 0; l < P; ++l) T[lp][l] = h.iK1[lp + P * l] * h.w[l];
  double wg = 0.0;
  for (int lp = 0; lp < P; ++lp) {
    double g = 0.0, ts = 0.0;
    for (int l = 0; l < P; ++l) {
      g += h.iK1[lp + P * l] * h.F0[l];
      ts += T[lp][l];
      o.T[lp + P * l] = (R)T[lp][l];
    }
    o.g[lp] = (R)g;
    o.ts[lp] = (R)ts;
    wg += h.w[lp] * g;
  }
  for (int l = 0; l < P; ++l) {
    double tw = 0.0;
    for (int lp = 0; lp < P; ++lp) tw += h.w[lp] * T[lp][l];
    o.tw[l] = (R)tw;
  }
  o.wg = (R)wg;
  for (int k = 0; k < S * P; ++k) {
    o.uh2lim[k] = h.uh2lim[k];
    o.lim2uh[k] = h.lim2uh[k];
  }
  for (int k = 0; k < P * P; ++k) o.uh2lob[k] = h.uh2lob[k];
  for (int k = 0; k < S * P; ++k) o.uh2limf[k] = (float)h.uh2lim[k];
  for (int k = 0; k < P * P; ++k) o.uh2lobf[k] = (float)h.uh2lob[k];
  // Error of a two-pass FP32 projection (inputs and operators rounded to
  // FP32, P-term accumulations in each pass): at most (2P + 4) u Lambda^2 max|uh|,
  // u = 2^-24, Lambda = the larger of the operators' max row sums of |entries|;
  // taken with a factor 4 of safety.
  double lam = 0.0;
  for (int s = 0; s < S; ++s) {
    double r = 0.0;
    for (int k = 0; k < P; ++k) r += std::fabs(h.uh2lim[s + S * k]);
    lam = r > lam ? r : lam;
  }
  for (int q = 0; q < P; ++q) {
    double r = 0.0;
    for (int k = 0; k < P; ++k) r += std::fabs(h.uh2lob[q + P * k]);
    lam = r > lam ? r : lam;
  }
  o.perr = (float)(4.0 * (2 * P + 4) * std::ldexp(1.0, -24) * lam * lam);
  // a rounding of 2^-24 (|uh| + |d|) per node, through the two passes; factor 2 of safety
  o.pdev = (float)(2.0 * std::ldexp(1.0, -24) * lam * lam);
  *reinterpret_cast<DevOps<N, R>*>(out) = o;
}

template <class R, bool kPhase>
cudaError_t launch_pred(const BatchArgs& a, const void* ops, cudaStream_t s) {
  using C = PredCfg<Sys, N, R>;
  auto kern = k_predictor<Sys, N, R, kPhase>;
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM_BYTES);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  const long long grid = (a.ncells - a.cell0 + C::CPB - 1) / C::CPB;
  if (grid <= 0) return cudaSuccess;
  kern<<<(unsigned)grid, C::THREADS, C::SMEM_BYTES, s>>>(a, *reinterpret_cast<const DevOps<N, R>*>(ops));
  return cudaGetLastError();
}

cudaError_t predictor(const BatchArgs& a, const void* ops, int fp32, bool phase, cudaStream_t s) {
  if (fp32) return phase ? cudaErrorNotSupported : launch_pred<float, false>(a, ops, s);
  return phase ? launch_pred<double, true>(a, ops, s) : launch_pred<double, false>(a, ops, s);
}

#if ADERDG_SYS != 0
// FP32-mixed subcell re-solve: FP64 with the reciprocal-sharing physics forms,
// compiled here with fused multiply-adds (k_subcell's DMP projections keep
// the reference order through rounded intrinsics)
using SubMixed = SubCfg<Sys, N, double>;
int subcell_grid_mixed(int num_sms) {
  int per_sm = 0;
  cudaFuncSetAttribute(k_subcell<Sys, N, double, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                       SubMixed::SMEM_BYTES);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_subcell<Sys, N, double, true>, SubMixed::THREADS,
                                                    SubMixed::SMEM_BYTES) != cudaSuccess)
    per_sm = 1;
  return (per_sm < 1 ? 1 : per_sm) * num_sms;
}
cudaError_t subcell_mixed(const BatchArgs& a, const void* ops, const FaceConst& fc, int grid, cudaStream_t s) {
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_subcell<Sys, N, double, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         SubMixed::SMEM_BYTES);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  k_subcell<Sys, N, double, true><<<grid, SubMixed::THREADS, SubMixed::SMEM_BYTES, s>>>(
      a, *reinterpret_cast<const DevOps<N, double>*>(ops), fc);
  return cudaGetLastError();
}
#endif

#if ADERDG_SYS == 2
// FP32-mixed faces of Baer-Nunziato: FP32 face states and fluxes, the
// path-conservative Rusanov flux and its Roe-matrix path integral in FP64
// (compiled here, with fused multiply-adds, not in the reference-order unit)
cudaError_t faces_mixed(const BatchArgs& a, const FaceConst& fc, cudaStream_t s) {
  const long long n = (a.nfx + a.nfy) * (N + 1);
  if (n <= 0) return cudaSuccess;
  k_faces<Sys, N, float, double><<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a, fc);
  return cudaGetLastError();
}
#endif

}  // namespace

#define ADERDG_CAT2(a, b, c) a##b##_##c
#define ADERDG_CAT(a, b, c) ADERDG_CAT2(a, b, c)
void ADERDG_CAT(register_predictor_, ADERDG_SYS, ADERDG_N)(KernelTable& t) {
  t.sys = ADERDG_SYS;
  t.N = N;
  t.ops64_size = sizeof(DevOps<N, double>);
  t.ops32_size = sizeof(DevOps<N, float>);
  t.make_ops64 = &make_ops<double>;
  t.make_ops32 = &make_ops<float>;
  t.predictor = &predictor;
  t.pred_cells_per_cta[0] = PredCfg<Sys, N, double>::CPB;
  t.pred_cells_per_cta[1] = PredCfg<Sys, N, float>::CPB;
  t.pred_threads[0] = PredCfg<Sys, N, double>::THREADS;
  t.pred_threads[1] = PredCfg<Sys, N, float>::THREADS;
#if ADERDG_SYS == 2
  t.faces_mixed = &faces_mixed;
#endif
#if ADERDG_SYS != 0
  t.subcell_mixed = &subcell_mixed;
  t.subcell_grid_mixed = &subcell_grid_mixed;
#endif
}

}  // namespace aderdg
