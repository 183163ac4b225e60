// tables.h -- host-side launch table for one (system, N) kernel family.
//
// The kernels are templates on the PDE system and the degree N; each
// (system, N) pair is compiled in two translation units (predictor_tu.cu with
// fused multiply-adds, exact_tu.cu with --fmad=false) that fill one table.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <string>

#include "../../include/aderdg_gpu.h"
#include "common.cuh"
#include "setup.h"

namespace aderdg {

// candidates of the tuner (predictor.cuh PredVariant, cells.cuh CellCfg VAR)
constexpr int kPredVariantsMax = 7;
constexpr int kCellVariantsMax = 3;

struct KernelTable {
  int sys = -1, N = 0;
  // predictor translation unit
  size_t ops64_size = 0, ops32_size = 0;
  void (*make_ops64)(const HostOps&, void* out) = nullptr;
  void (*make_ops32)(const HostOps&, void* out) = nullptr;
  cudaError_t (*predictor)(const BatchArgs&, const void* ops, int fp32, bool phase, cudaStream_t) = nullptr;
  int pred_cells_per_cta[2] = {0, 0};
  int pred_threads[2] = {0, 0};
  // FP32 predictor candidates 1.. (predictor_var_tu.cu); [0] unused (the default)
  cudaError_t (*predictor_var[kPredVariantsMax])(const BatchArgs&, const void* ops, cudaStream_t) = {};
  int pred_var_cpb[kPredVariantsMax] = {}, pred_var_threads[kPredVariantsMax] = {};
  // FP32-mode cell-kernel candidates 1.. (cells_var_tu.cu); [0] unused (the default)
  cudaError_t (*cells_var[kCellVariantsMax])(const BatchArgs&, const void* ops64, cudaStream_t) = {};
  int cells_var_threads[kCellVariantsMax] = {};
  // FP32-mixed faces where they differ from the FP32 faces (Baer-Nunziato:
  // FP64 arithmetic on FP32 storage); null: use faces(..., fp32 = 1, ...)
  cudaError_t (*faces_mixed)(const BatchArgs&, const FaceConst&, cudaStream_t) = nullptr;
  // FP32-mixed subcell re-solve (FP64, reciprocal-sharing physics, fused
  // multiply-adds) and its persistent grid; null for advection-diffusion
  cudaError_t (*subcell_mixed)(const BatchArgs&, const void* ops64, const FaceConst&, int grid, cudaStream_t) = nullptr;
  int (*subcell_grid_mixed)(int num_sms) = nullptr;
  // exact translation unit
  cudaError_t (*faces)(const BatchArgs&, const FaceConst&, int fp32, cudaStream_t) = nullptr;
  cudaError_t (*cells)(const BatchArgs&, const void* ops64, int fast, cudaStream_t) = nullptr;
  cudaError_t (*volume)(const BatchArgs&, const void* ops64, cudaStream_t) = nullptr;
  cudaError_t (*mark)(const BatchArgs&, cudaStream_t) = nullptr;
  cudaError_t (*subcell)(const BatchArgs&, const void* ops64, const FaceConst&, int grid, int fp32, cudaStream_t) = nullptr;
  int (*subcell_grid)(int num_sms, int fp32) = nullptr;
  // FP32-mixed: DMP decisions k_cells left open, from FP64 values (k_settle);
  // grid CTAs persistent over the list
  cudaError_t (*settle)(const BatchArgs&, const void* ops64, int grid, cudaStream_t) = nullptr;
};

// On-device initial field of one simulation (initial.cu): uh at the
// Gauss-Legendre nodes and, when lh is non-null, the values at the subcell
// barycentres.  cudaErrorInvalidValue with *why set for an unknown field.
cudaError_t launch_initial_field(const aderdg_config& cfg, int ic, const double* params, double* uh, double* lh,
                                 cudaStream_t s, std::string* why);
// The subcell barycentre values of the cells with status != 0 only, into lh0
// and lh1 (the initial limiter's candidates of the cells it limited).
cudaError_t launch_initial_lh(const aderdg_config& cfg, int ic, const double* params, const int* status, double* lh0,
                              double* lh1, cudaStream_t s, std::string* why);

// Cell averages (or their primitive variables) of uh, [cell][V] (output.cu).
cudaError_t launch_cell_averages(const aderdg_config& cfg, const double* uh, int primitive, double* out,
                                 cudaStream_t s, std::string* why);
// Error of the cell averages of variable var against an exact field at time
// `time`: sums_dev[0] += sum |e|, sums_dev[1] += sum e^2, *max_dev = max |e| bits.
cudaError_t launch_error_norms(const aderdg_config& cfg, const double* uh, int ic, const double* params, int var,
                               double time, double* sums_dev, unsigned long long* max_dev, cudaStream_t s,
                               std::string* why);

// Returns the table for (sys, N) or nullptr when that pair was not built.
const KernelTable* kernel_table(int sys, int N);

// The tuner's choice for (system, N, precision) (registry.cu; zeros: the defaults).
aderdg_tuning tuning_of(int sys, int N, int precision);

// The FP32 modes' predictor and cell kernel in the tuned variant; FP64 keeps
// the reference-order kernels of its own.
inline cudaError_t launch_predictor(const KernelTable* kt, const BatchArgs& a, const void* ops, int precision,
                                    cudaStream_t s) {
  const int fp32 = precision != ADERDG_FP64 ? 1 : 0;
  if (fp32) {
    const int v = tuning_of(kt->sys, kt->N, precision).predictor;
    if (v > 0 && v < kPredVariantsMax && kt->predictor_var[v]) return kt->predictor_var[v](a, ops, s);
  }
  return kt->predictor(a, ops, fp32, false, s);
}
inline cudaError_t launch_cells(const KernelTable* kt, const BatchArgs& a, const void* ops64, int precision,
                                cudaStream_t s) {
  const int fast = precision != ADERDG_FP64 ? 1 : 0;
  if (fast) {
    const int v = tuning_of(kt->sys, kt->N, precision).cells;
    if (v > 0 && v < kCellVariantsMax && kt->cells_var[v]) return kt->cells_var[v](a, ops64, s);
  }
  return kt->cells(a, ops64, fast, s);
}
// the subcell kernel's persistent grid: the tuned CTAs per SM, at most max_grid
inline int subcell_launch_grid(const KernelTable* kt, int max_grid, int num_sms, int precision) {
  const int per = tuning_of(kt->sys, kt->N, precision).subcell_per_sm;
  if (per > 0 && per * num_sms < max_grid) return per * num_sms;
  return max_grid;
}

// The face kernel of a precision mode (aderdg_precision).
inline cudaError_t launch_faces(const KernelTable* kt, const BatchArgs& a, const FaceConst& fc, int precision,
                                cudaStream_t s) {
  if (precision == ADERDG_FP32_MIXED && kt->faces_mixed) return kt->faces_mixed(a, fc, s);
  return kt->faces(a, fc, precision != ADERDG_FP64 ? 1 : 0, s);
}
// The subcell re-solve of a precision mode: FP32 in the FP32-wide mode, FP64
// with the reciprocal-sharing physics in the FP32-mixed mode, FP64 in the
// reference's order otherwise.
inline int subcell_fp32(int precision) { return precision == ADERDG_FP32_WIDE ? 1 : 0; }
// max_grid: the most CTAs that fit (subcell_grid_of); the tuned CTAs per SM
// apply within it
inline cudaError_t launch_subcell(const KernelTable* kt, const BatchArgs& a, const void* ops64, const FaceConst& fc,
                                  int max_grid, int num_sms, int precision, cudaStream_t s) {
  const int grid = subcell_launch_grid(kt, max_grid, num_sms, precision);
  if (precision == ADERDG_FP32_MIXED && kt->subcell_mixed) return kt->subcell_mixed(a, ops64, fc, grid, s);
  return kt->subcell(a, ops64, fc, grid, subcell_fp32(precision), s);
}
inline int subcell_grid_of(const KernelTable* kt, int num_sms, int precision) {
  if (precision == ADERDG_FP32_MIXED && kt->subcell_grid_mixed) return kt->subcell_grid_mixed(num_sms);
  return kt->subcell_grid(num_sms, subcell_fp32(precision));
}

}  // namespace aderdg
