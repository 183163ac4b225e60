// probe.cu -- measures the device's FP64 and FP32 FMA throughput, the
// denominators of the FP-pipe roofline of the predictor (an FP64- or
// FP32-pipe-bound kernel: it moves ~16 B of state per DOF-update but performs
// several hundred flops on it).  Eight independent FMA chains per thread keep
// the pipes busy; the result is written so nothing is optimised away.
#include <cuda_runtime.h>

#include "../../include/aderdg_gpu.h"
#include "physics.cuh"

namespace {

// the FP32-mixed mode's refined reciprocal and square root beside the
// correctly rounded operations, for the accuracy check (aderdg_probe_math)
__global__ void k_math(int n, const double* x, double* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double v = x[i];
  out[4 * (size_t)i + 0] = aderdg::mrcp<double>(v);
  out[4 * (size_t)i + 1] = 1.0 / v;
  out[4 * (size_t)i + 2] = aderdg::msqrt<double>(v);
  out[4 * (size_t)i + 3] = sqrt(v);
}

template <class R>
__global__ void __launch_bounds__(256) k_fma_chain(R* out, int iters, R seed) {
  R a0 = seed + threadIdx.x, a1 = a0 + R(1), a2 = a0 + R(2), a3 = a0 + R(3);
  R a4 = a0 + R(4), a5 = a0 + R(5), a6 = a0 + R(6), a7 = a0 + R(7);
  const R m = R(0.999999), c = R(1e-7);
  for (int k = 0; k < iters; ++k) {
#pragma unroll
    for (int u = 0; u < 16; ++u) {
      a0 = fma(a0, m, c); a1 = fma(a1, m, c); a2 = fma(a2, m, c); a3 = fma(a3, m, c);
      a4 = fma(a4, m, c); a5 = fma(a5, m, c); a6 = fma(a6, m, c); a7 = fma(a7, m, c);
    }
  }
  R s = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
  if (s == R(-12345.0)) out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <class R>
int measure(double* gflops, int sms) {
  R* out = nullptr;
  const int blocks = sms * 8, threads = 256;
  if (cudaMalloc(&out, sizeof(R) * blocks * threads) != cudaSuccess) return ADERDG_ENOMEM;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int iters = sizeof(R) == 8 ? 64 : 2048;
  k_fma_chain<R><<<blocks, threads>>>(out, iters, R(1));  // warm-up
  float best = 1e30f;
  for (int rep = 0; rep < 5; ++rep) {
    cudaEventRecord(e0);
    k_fma_chain<R><<<blocks, threads>>>(out, iters, R(1));
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess) return ADERDG_ECUDA;
  const double flops = 2.0 * 8.0 * 16.0 * (double)iters * blocks * threads;
  *gflops = flops / (best * 1e-3) / 1e9;
  return ADERDG_OK;
}

}  // namespace

extern "C" int aderdg_probe_peaks(double* fp64_gflops, double* fp32_gflops) {
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return ADERDG_ECUDA;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return ADERDG_ECUDA;
  int r = ADERDG_OK;
  if (fp64_gflops) r = measure<double>(fp64_gflops, sms);
  if (!r && fp32_gflops) r = measure<float>(fp32_gflops, sms);
  return r;
}

extern "C" int aderdg_host_alloc(size_t bytes, void** ptr) {
  if (!ptr) return ADERDG_EINVAL;
  *ptr = nullptr;
  if (bytes == 0) return ADERDG_OK;
  return cudaMallocHost(ptr, bytes) == cudaSuccess ? ADERDG_OK : ADERDG_ENOMEM;
}

extern "C" int aderdg_host_free(void* ptr) {
  if (!ptr) return ADERDG_OK;
  return cudaFreeHost(ptr) == cudaSuccess ? ADERDG_OK : ADERDG_ECUDA;
}

extern "C" int aderdg_probe_math(int n, const double* x, double* out) {
  if (n < 0 || (n > 0 && (!x || !out))) return ADERDG_EINVAL;
  if (n == 0) return ADERDG_OK;
  double *dx = nullptr, *dout = nullptr;
  if (cudaMalloc(&dx, sizeof(double) * n) != cudaSuccess) return ADERDG_ENOMEM;
  if (cudaMalloc(&dout, sizeof(double) * 4 * (size_t)n) != cudaSuccess) {
    cudaFree(dx);
    return ADERDG_ENOMEM;
  }
  int r = ADERDG_OK;
  if (cudaMemcpy(dx, x, sizeof(double) * n, cudaMemcpyHostToDevice) != cudaSuccess) r = ADERDG_ECUDA;
  if (!r) {
    k_math<<<(n + 255) / 256, 256>>>(n, dx, dout);
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemcpy(out, dout, sizeof(double) * 4 * (size_t)n, cudaMemcpyDeviceToHost) != cudaSuccess)
      r = ADERDG_ECUDA;
  }
  cudaFree(dx);
  cudaFree(dout);
  return r;
}
