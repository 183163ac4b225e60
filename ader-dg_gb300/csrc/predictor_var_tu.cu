// predictor_var_tu.cu -- one tuner candidate of the FP32 space-time predictor
// (K1) for one (system, N): -DADERDG_SYS, -DADERDG_N and -DADERDG_VAR (1..6,
// PredVariant in predictor.cuh; variant 0 is predictor_tu.cu's default).
// Compiled with fused multiply-adds, as predictor_tu.cu.
#include "predictor.cuh"
#include "tables.h"

#if !defined(ADERDG_SYS) || !defined(ADERDG_N) || !defined(ADERDG_VAR)
#error "ADERDG_SYS, ADERDG_N and ADERDG_VAR must be defined"
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
using Tune = PredVariant<ADERDG_VAR>;

// the tensor-core row/column pass (variant 6) exists where the row/column
// pass does (FP32 Euler / Baer-Nunziato, N >= 3); elsewhere the variant is
// not built and the default runs in its place
constexpr bool kBuilt = ADERDG_VAR != 6 || PredCfg<Sys, N, float, Tune>::MMA;

template <class T>
cudaError_t predictor_var(const BatchArgs& a, const void* ops, cudaStream_t s) {
  using C = PredCfg<Sys, N, float, T>;
  auto kern = k_predictor<Sys, N, float, false, T>;
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM_BYTES);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  const long long grid = (a.ncells - a.cell0 + C::CPB - 1) / C::CPB;
  if (grid <= 0) return cudaSuccess;
  kern<<<(unsigned)grid, C::THREADS, C::SMEM_BYTES, s>>>(a, *reinterpret_cast<const DevOps<N, float>*>(ops));
  return cudaGetLastError();
}

}  // namespace

#define ADERDG_CAT2(a, b, c, d) a##b##_##c##_##d
#define ADERDG_CAT(a, b, c, d) ADERDG_CAT2(a, b, c, d)
void ADERDG_CAT(register_predvar_, ADERDG_SYS, ADERDG_N, ADERDG_VAR)(KernelTable& t) {
  if constexpr (kBuilt) {
    t.predictor_var[ADERDG_VAR] = &predictor_var<Tune>;
    t.pred_var_cpb[ADERDG_VAR] = PredCfg<Sys, N, float, Tune>::CPB;
    t.pred_var_threads[ADERDG_VAR] = PredCfg<Sys, N, float, Tune>::THREADS;
  }
}

}  // namespace aderdg
