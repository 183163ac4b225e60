// exact_tu.cu -- instantiates the FP64 reference-order kernels (faces K2,
// cell update K3, volume integral, limiter K4) for one (system, N), selected
// by -DADERDG_SYS and -DADERDG_N.  Compiled with --fmad=false.
#include "cells.cuh"
#include "faces.cuh"
#include "limiter.cuh"
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
constexpr int P = N + 1, P2 = P * P, V = Sys::V;

// volume_integral.f90 (Euler :8-36, BN :8-44) from the phase outputs Fhi/Shi
__global__ void __launch_bounds__(256) k_volume(BatchArgs a, DevOps<N, double> op) {
  const long long gid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (gid >= a.ncells * P2) return;
  const long long cell = gid / P2;
  const int node = (int)(gid - cell * P2);
  const int i = node % P, j = node / P;
  const int k = find_inst_cell(a.inst, a.ninst, cell);
  if (k < 0) return;
  const InstDesc& in = a.inst[k];
  if (!a.st[k].active) return;
  const double* F = a.fhi + (size_t)cell * P2 * 2 * V;  // Fhi(v,d,i,j)
  for (int v = 0; v < V; ++v) {
    double d = 0.0;
    double s = 0.0;
    for (int kk = 0; kk < P; ++kk) s = s + F[((kk + P * j) * 2 + 0) * V + v] * op.Kxi[i + P * kk];
    d = d + s * op.wd[j] / in.dx;
    s = 0.0;
    for (int kk = 0; kk < P; ++kk) s = s + F[((i + P * kk) * 2 + 1) * V + v] * op.Kxi[j + P * kk];
    d = d + s * op.wd[i] / in.dy;
    if constexpr (Sys::ID == kSysBN) d = d + op.wd[i] * op.wd[j] * a.shi[((size_t)cell * P2 + node) * V + v];
    a.duh[((size_t)cell * P2 + node) * V + v] = d;
  }
}

// fp32 = 1: FP32 storage and FP32 arithmetic; 0: FP64 in reference order
cudaError_t faces(const BatchArgs& a, const FaceConst& fc, int fp32, cudaStream_t s) {
  const long long n = (a.nfx + a.nfy) * P;
  if (n <= 0) return cudaSuccess;
  const unsigned grid = (unsigned)((n + 255) / 256);
  if (fp32)
    k_faces<Sys, N, float, float><<<grid, 256, 0, s>>>(a, fc);
  else
    k_faces<Sys, N, double, double><<<grid, 256, 0, s>>>(a, fc);
  return cudaGetLastError();
}

template <bool kFast>
cudaError_t launch_cells(const BatchArgs& a, const void* ops, cudaStream_t s) {
  using C = CellCfg<Sys, N>;
  static bool attr = false;
  if (!attr) {
    cudaError_t e =
        cudaFuncSetAttribute(k_cells<Sys, N, kFast>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM_BYTES);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  const long long grid = (a.ncells - a.cell0 + C::CPB - 1) / C::CPB;
  if (grid <= 0) return cudaSuccess;
  k_cells<Sys, N, kFast><<<(unsigned)grid, C::THREADS, C::SMEM_BYTES, s>>>(a, *reinterpret_cast<const DevOps<N, double>*>(ops));
  return cudaGetLastError();
}

// fast = 1 (the FP32 modes): FP32 surface integral and DMP projections, the
// FP64 update as one fused multiply-add; fast = 0: FP64 in reference order
cudaError_t cells(const BatchArgs& a, const void* ops, int fast, cudaStream_t s) {
  return fast ? launch_cells<true>(a, ops, s) : launch_cells<false>(a, ops, s);
}

cudaError_t volume(const BatchArgs& a, const void* ops, cudaStream_t s) {
  const long long n = a.ncells * P2;
  if (n <= 0) return cudaSuccess;
  k_volume<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a, *reinterpret_cast<const DevOps<N, double>*>(ops));
  return cudaGetLastError();
}

#if ADERDG_SYS != 0
cudaError_t mark(const BatchArgs& a, cudaStream_t s) {
  if (a.ncells <= 0) return cudaSuccess;
  k_mark<Sys, N><<<(unsigned)((a.ncells + 255) / 256), 256, 0, s>>>(a);
  return cudaGetLastError();
}

template <class T>
int subcell_grid_t(int num_sms) {
  using C = SubCfg<Sys, N, T>;
  int per_sm = 0;
  cudaFuncSetAttribute(k_subcell<Sys, N, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM_BYTES);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_subcell<Sys, N, T>, C::THREADS, C::SMEM_BYTES) !=
      cudaSuccess)
    per_sm = 1;
  if (per_sm < 1) per_sm = 1;
  return per_sm * num_sms;
}

int subcell_grid(int num_sms, int fp32) { return fp32 ? subcell_grid_t<float>(num_sms) : subcell_grid_t<double>(num_sms); }

template <class T>
cudaError_t subcell_t(const BatchArgs& a, const void* ops, const FaceConst& fc, int grid, cudaStream_t s) {
  using C = SubCfg<Sys, N, T>;
  static bool attr = false;
  if (!attr) {
    cudaError_t e = cudaFuncSetAttribute(k_subcell<Sys, N, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, C::SMEM_BYTES);
    if (e != cudaSuccess) return e;
    attr = true;
  }
  k_subcell<Sys, N, T><<<grid, C::THREADS, C::SMEM_BYTES, s>>>(a, *reinterpret_cast<const DevOps<N, double>*>(ops), fc);
  return cudaGetLastError();
}

cudaError_t subcell(const BatchArgs& a, const void* ops, const FaceConst& fc, int grid, int fp32, cudaStream_t s) {
  return fp32 ? subcell_t<float>(a, ops, fc, grid, s) : subcell_t<double>(a, ops, fc, grid, s);
}

cudaError_t settle(const BatchArgs& a, const void* ops, int grid, cudaStream_t s) {
  k_settle<Sys, N><<<grid, 128, 0, s>>>(a, *reinterpret_cast<const DevOps<N, double>*>(ops));
  return cudaGetLastError();
}
#endif

}  // namespace

#define ADERDG_CAT2(a, b, c) a##b##_##c
#define ADERDG_CAT(a, b, c) ADERDG_CAT2(a, b, c)
void ADERDG_CAT(register_exact_, ADERDG_SYS, ADERDG_N)(KernelTable& t) {
  t.faces = &faces;
  t.cells = &cells;
  t.volume = &volume;
#if ADERDG_SYS != 0
  t.mark = &mark;
  t.subcell = &subcell;
  t.subcell_grid = &subcell_grid;
  t.settle = &settle;
#endif
}

}  // namespace aderdg
