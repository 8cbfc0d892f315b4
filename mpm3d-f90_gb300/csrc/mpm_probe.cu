// mpm_probe.cu -- the FP64 arithmetic ceiling of the device (the roofline of
// the FP64 forms of the step, which are bound by the FP64 pipe, not by HBM).
//
// Two kernels fill every SM with independent work: one runs kChains
// independent FP64 fused multiply-add chains per thread, one runs chains of
// FP64 divisions. The chains' results are folded into one value written by
// one thread, so nothing can be removed by the compiler. Each kernel is
// timed with CUDA events on a private stream; the best of `repeats`
// launches after a warm-up launch counts.
#include <cuda_runtime.h>

#include <algorithm>

#include "mpm3d_gpu.h"

namespace {

constexpr int kThreads = 256;
constexpr int kChains = 8;
constexpr int kFmaIters = 4096;
constexpr int kDivIters = 512;

__global__ void __launch_bounds__(kThreads) k_dfma(double a, double b, double* sink) {
  double x[kChains];
#pragma unroll
  for (int k = 0; k < kChains; ++k) x[k] = 1.0 + 1e-3 * (threadIdx.x + k);
  for (int i = 0; i < kFmaIters; ++i) {
#pragma unroll
    for (int k = 0; k < kChains; ++k) x[k] = fma(x[k], a, b);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < kChains; ++k) s += x[k];
  if (s == 12345.678) *sink = s;  // never true for the arguments used; keeps the chains live
}

__global__ void __launch_bounds__(kThreads) k_ddiv(double a, double* sink) {
  double x[kChains];
#pragma unroll
  for (int k = 0; k < kChains; ++k) x[k] = 1.5 + 1e-3 * (threadIdx.x + k);
  for (int i = 0; i < kDivIters; ++i) {
#pragma unroll
    for (int k = 0; k < kChains; ++k) x[k] = a / x[k];
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < kChains; ++k) s += x[k];
  if (s == 12345.678) *sink = s;
}

}  // namespace

extern "C" int mpm_fp64_ceiling(int device, int repeats, double* dfma_per_s, double* ddiv_per_s) {
  if (repeats < 1) repeats = 1;
  int prev = 0;
  if (cudaGetDevice(&prev) != cudaSuccess) return MPM_ERR_CUDA;
  if (device >= 0 && cudaSetDevice(device) != cudaSuccess) return MPM_ERR_CUDA;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device >= 0 ? device : prev);
  const int blocks = std::max(1, sms) * 8;  // eight 256-thread blocks per SM
  double* sink = nullptr;
  cudaStream_t st = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int r = MPM_OK;
  float best_fma = 1e30f, best_div = 1e30f;
  if (cudaMalloc(&sink, sizeof(double)) != cudaSuccess || cudaStreamCreate(&st) != cudaSuccess ||
      cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) {
    r = MPM_ERR_CUDA;
  } else {
    // a = 1 - 2^-20, b = 2^-30: the chains stay finite and away from 12345.678
    const double a = 1.0 - 9.5367431640625e-07, b = 9.313225746154785e-10;
    for (int it = 0; it <= repeats && !r; ++it) {
      float ms = 0.f;
      cudaEventRecord(e0, st);
      k_dfma<<<blocks, kThreads, 0, st>>>(a, b, sink);
      cudaEventRecord(e1, st);
      if (cudaEventSynchronize(e1) != cudaSuccess || cudaGetLastError() != cudaSuccess) r = MPM_ERR_CUDA;
      cudaEventElapsedTime(&ms, e0, e1);
      if (it > 0) best_fma = std::min(best_fma, ms);
      cudaEventRecord(e0, st);
      k_ddiv<<<blocks, kThreads, 0, st>>>(1.25, sink);
      cudaEventRecord(e1, st);
      if (cudaEventSynchronize(e1) != cudaSuccess || cudaGetLastError() != cudaSuccess) r = MPM_ERR_CUDA;
      cudaEventElapsedTime(&ms, e0, e1);
      if (it > 0) best_div = std::min(best_div, ms);
    }
  }
  const double threads = (double)blocks * kThreads * kChains;
  if (!r && dfma_per_s) *dfma_per_s = threads * kFmaIters / (best_fma * 1e-3);
  if (!r && ddiv_per_s) *ddiv_per_s = threads * kDivIters / (best_div * 1e-3);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (st) cudaStreamDestroy(st);
  if (sink) cudaFree(sink);
  cudaSetDevice(prev);
  return r;
}
