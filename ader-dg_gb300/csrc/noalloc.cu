// noalloc.cu -- the time-step (CFL) reduction for callers that cannot
// allocate device memory.
//
// Some hosts cannot call cudaMalloc: a solver embedded in a framework that
// owns every device allocation through its own pool, code that must not
// trigger the implicit device synchronisation cudaMalloc/cudaFree may cause,
// or a driver whose device arrays come from another runtime (OpenACC / CUDA
// Fortran data regions).  aderdg_calc_time_step needs a context, and creating
// one allocates.  This file gives those callers one entry point that
// allocates nothing: the caller passes the state and the output as device
// pointers it owns, and the only scratch -- one partial maximum per CTA and a
// completion ticket -- lives in a file-scope device array that every GPU
// loading this library holds until the process exits.
//
// Set-up: the first call on each device (with that device current) asks the
// runtime for the array's device address with cudaGetSymbolAddress and caches
// it, keyed on the CUDA context current at that call; make that first call
// before any stream capture.  A call in another context of that device (after
// cudaDeviceReset, for instance) looks the address up again.  Every call shares the
// array and leaves its contents behind, so each call clears the ticket before
// its kernel runs, and calls whose kernels overlap on the GPU race on the
// array: serialise them (one stream, or events).
//
// The kernel computes the same quantity as calc_time_step.f90 (Euler :9-52,
// BN :9-52, AD :9-57), in the same FP64 operation order as the time-step path
// of the context API (this unit is compiled with --fmad=false as well).
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/aderdg_gpu.h"
#include "common.cuh"
#include "physics.cuh"
#include "setup.h"

namespace aderdg {
void set_last_error(const std::string& msg);
int validate_config(const aderdg_config* c, std::string* why);
InstDesc make_inst_desc(const aderdg_config* cfg);
}

namespace {

constexpr int kThreads = 256;            // one cell per thread
constexpr int kMaxBlocks = 8192;         // partial maxima held in the scratch array
constexpr long long kMaxCells = (long long)kMaxBlocks * kThreads;  // 2,097,152 cells
constexpr int kMaxDevices = 64;

// [0, kMaxBlocks): per-CTA maximum of the CFL denominator (positive double bits)
// [kMaxBlocks]:    completion ticket
static __device__ __align__(256) unsigned long long g_scratch[kMaxBlocks + 1];

std::mutex g_mu;
// per device: the context the address was looked up in, and the address
struct Cached {
  CUcontext ctx;
  unsigned long long* addr;
};
Cached g_addr[kMaxDevices] = {};
PFN_cuCtxGetCurrent_v4000 g_ctx_current = nullptr;  // the driver's cuCtxGetCurrent, from the runtime

template <int SYS>
__device__ double node_denom(const aderdg::InstDesc& in, int N, const double* Q) {
  double denom = 0.0;
  if constexpr (SYS == aderdg::kSysAD) {
    const double factor = (double)(2 * N + 1);
    const double smax_v = fabs(in.ph.a);
    denom = denom + (aderdg::ADSys::max_eig_c(in.ph, 0) + 2.0 * smax_v * factor / in.dx) / in.dx;
    denom = denom + (aderdg::ADSys::max_eig_c(in.ph, 1) + 2.0 * smax_v * factor / in.dy) / in.dy;
  } else if constexpr (SYS == aderdg::kSysEuler) {
    denom = denom + aderdg::EulerSys::max_eig(in.ph, Q, 0) / in.dx;
    denom = denom + aderdg::EulerSys::max_eig(in.ph, Q, 1) / in.dy;
  } else {
    denom = denom + aderdg::BNSys::max_eig(in.ph, Q, 0) / in.dx;
    denom = denom + aderdg::BNSys::max_eig(in.ph, Q, 1) / in.dy;
  }
  return denom;
}

__device__ __forceinline__ unsigned long long umax(unsigned long long a, unsigned long long b) { return a > b ? a : b; }

template <int SYS, int V>
__global__ void __launch_bounds__(kThreads) k_cfl_noalloc(const double* __restrict__ uh, long long ncells, int N,
                                                          aderdg::InstDesc in, double time, double tend,
                                                          unsigned long long* scratch, double* dt_out) {
  __shared__ unsigned long long warp_max[kThreads / 32];
  __shared__ bool last;
  const int P2 = (N + 1) * (N + 1);
  const long long cell = (long long)blockIdx.x * kThreads + threadIdx.x;
  unsigned long long m = 0ull;
  if (cell < ncells) {
    const double* u = uh + (size_t)cell * P2 * V;
    for (int k = 0; k < P2; ++k) m = umax(m, (unsigned long long)__double_as_longlong(node_denom<SYS>(in, N, u + k * V)));
  }
  for (int o = 16; o > 0; o >>= 1) m = umax(m, __shfl_down_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) warp_max[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long b = 0ull;
    for (int w = 0; w < kThreads / 32; ++w) b = umax(b, warp_max[w]);
    scratch[blockIdx.x] = b;
    __threadfence();
    const unsigned long long ticket = atomicAdd(&scratch[kMaxBlocks], 1ull);
    last = ticket == (unsigned long long)gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return;
  // the last CTA folds the partial maxima and forms dt
  __threadfence();
  unsigned long long b = 0ull;
  for (int k = threadIdx.x; k < (int)gridDim.x; k += kThreads) b = umax(b, __ldcg(&scratch[k]));
  for (int o = 16; o > 0; o >>= 1) b = umax(b, __shfl_down_sync(0xffffffffu, b, o));
  if ((threadIdx.x & 31) == 0) warp_max[threadIdx.x >> 5] = b;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long mx = 0ull;
    for (int w = 0; w < kThreads / 32; ++w) mx = umax(mx, warp_max[w]);
    double dt = 1.0e20;
    dt = fmin(dt, in.cfl_pnpm / __longlong_as_double((long long)mx));
    if (time + dt > tend) dt = tend - time;
    *dt_out = dt;
    scratch[kMaxBlocks] = 0ull;  // leave the ticket cleared for the next call
  }
}

// the current context (null when none is current yet); called under g_mu
int current_context(CUcontext* ctx) {
  if (!g_ctx_current) {
    cudaDriverEntryPointQueryResult q = cudaDriverEntryPointSymbolNotFound;
    const cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", reinterpret_cast<void**>(&g_ctx_current),
                                                           4000, cudaEnableDefault, &q);
    if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !g_ctx_current) {
      g_ctx_current = nullptr;
      aderdg::set_last_error("cudaGetDriverEntryPointByVersion(cuCtxGetCurrent) failed");
      return ADERDG_ECUDA;
    }
  }
  if (g_ctx_current(ctx) != CUDA_SUCCESS) {
    aderdg::set_last_error("cuCtxGetCurrent failed");
    return ADERDG_ECUDA;
  }
  return ADERDG_OK;
}

int scratch_address(unsigned long long** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) {
    aderdg::set_last_error(std::string("cudaGetDevice: ") + cudaGetErrorString(e));
    return ADERDG_ECUDA;
  }
  if (dev < 0 || dev >= kMaxDevices) {
    aderdg::set_last_error("device ordinal beyond the supported 64");
    return ADERDG_EUNSUPPORTED;
  }
  std::lock_guard<std::mutex> lock(g_mu);
  CUcontext ctx = nullptr;
  int r = current_context(&ctx);
  if (r) return r;
  if (!ctx || g_addr[dev].ctx != ctx || !g_addr[dev].addr) {
    // set-up in this context (the lookup makes the device's primary context
    // current when none was)
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess || !p) {
      aderdg::set_last_error(std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      return ADERDG_ECUDA;
    }
    r = current_context(&ctx);
    if (r) return r;
    g_addr[dev] = Cached{ctx, static_cast<unsigned long long*>(p)};
  }
  *out = g_addr[dev].addr;
  return ADERDG_OK;
}

}  // namespace

extern "C" int aderdg_calc_time_step_noalloc(const aderdg_config* cfg, const double* uh, double time, double tend,
                                             double* dt, void* stream) {
  if (!cfg || !uh || !dt) {
    aderdg::set_last_error("null argument");
    return ADERDG_EINVAL;
  }
  std::string why;
  const int v = aderdg::validate_config(cfg, &why);  // the checks of aderdg_create
  if (v) {
    aderdg::set_last_error("aderdg_calc_time_step_noalloc: " + why);
    return v;
  }
  const long long ncells = (long long)cfg->imax * cfg->jmax;
  if (ncells > kMaxCells) {
    aderdg::set_last_error("aderdg_calc_time_step_noalloc: " + std::to_string(ncells) + " cells exceed the maximum of " +
                           std::to_string(kMaxCells) + " (the fixed scratch holds " + std::to_string(kMaxBlocks) +
                           " partial maxima of 256 cells each); use aderdg_calc_time_step");
    return ADERDG_ENOSPACE;
  }
  unsigned long long* scratch = nullptr;
  int r = scratch_address(&scratch);
  if (r) return r;
  const aderdg::InstDesc in = aderdg::make_inst_desc(cfg);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e = cudaMemsetAsync(scratch + kMaxBlocks, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess) {
    aderdg::set_last_error(std::string("cudaMemsetAsync: ") + cudaGetErrorString(e));
    return ADERDG_ECUDA;
  }
  const unsigned grid = (unsigned)((ncells + kThreads - 1) / kThreads);
  switch (cfg->system) {
    case ADERDG_SYS_ADVDIFF:
      k_cfl_noalloc<aderdg::kSysAD, 1><<<grid, kThreads, 0, s>>>(uh, ncells, cfg->N, in, time, tend, scratch, dt);
      break;
    case ADERDG_SYS_EULER:
      k_cfl_noalloc<aderdg::kSysEuler, 4><<<grid, kThreads, 0, s>>>(uh, ncells, cfg->N, in, time, tend, scratch, dt);
      break;
    default:
      k_cfl_noalloc<aderdg::kSysBN, 9><<<grid, kThreads, 0, s>>>(uh, ncells, cfg->N, in, time, tend, scratch, dt);
      break;
  }
  e = cudaGetLastError();
  if (e != cudaSuccess) {
    aderdg::set_last_error(std::string("k_cfl_noalloc launch: ") + cudaGetErrorString(e));
    return ADERDG_ECUDA;
  }
  return ADERDG_OK;
}
