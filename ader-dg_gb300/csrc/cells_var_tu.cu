// cells_var_tu.cu -- the tuner's CTA-size candidates of the FP32-mode cell
// kernel (K3) for one (system, N), selected by -DADERDG_SYS and -DADERDG_N
// (CellCfg's VAR 1 and 2; VAR 0 is exact_tu.cu's default).  Compiled with
// --fmad=false, as exact_tu.cu.
#include "cells.cuh"
#include "tables.h"

#if !defined(ADERDG_SYS) || !defined(ADERDG_N)
#error "ADERDG_SYS and ADERDG_N must be defined"
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

template <int VAR>
cudaError_t cells_var(const BatchArgs& a, const void* ops, cudaStream_t s) {
  using C = CellCfg<Sys, N, VAR>;
  static bool attr = false;
  if (!attr) {
    cudaError_t e =
        cudaFuncSetAttribute(k_cells<Sys, N, true, VAR>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM_BYTES);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  const long long grid = (a.ncells - a.cell0 + C::CPB - 1) / C::CPB;
  if (grid <= 0) return cudaSuccess;
  k_cells<Sys, N, true, VAR><<<(unsigned)grid, C::THREADS, C::SMEM_BYTES, s>>>(
      a, *reinterpret_cast<const DevOps<N, double>*>(ops));
  return cudaGetLastError();
}

}  // namespace

#define ADERDG_CAT2(a, b, c) a##b##_##c
#define ADERDG_CAT(a, b, c) ADERDG_CAT2(a, b, c)
void ADERDG_CAT(register_cellsvar_, ADERDG_SYS, ADERDG_N)(KernelTable& t) {
  t.cells_var[1] = &cells_var<1>;
  t.cells_var[2] = &cells_var<2>;
  t.cells_var_threads[0] = CellCfg<Sys, N, 0>::THREADS;
  t.cells_var_threads[1] = CellCfg<Sys, N, 1>::THREADS;
  t.cells_var_threads[2] = CellCfg<Sys, N, 2>::THREADS;
}

}  // namespace aderdg
