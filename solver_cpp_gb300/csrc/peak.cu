// peak.cu -- FP64 FMA throughput probe used as the FP64 roofline denominator.
//
// Each thread runs 8 independent FMA chains (enough instruction-level
// parallelism to keep the FP64 pipe busy); the grid covers every SM many times.
// Reported as TFLOP/s with one FMA = 2 flops.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/dgx.h"

namespace {
__global__ void k_dfma(double* out, int iters, double a, double b) {
  double x0 = threadIdx.x * 1e-9, x1 = x0 + 1e-9, x2 = x0 + 2e-9, x3 = x0 + 3e-9;
  double x4 = x0 + 4e-9, x5 = x0 + 5e-9, x6 = x0 + 6e-9, x7 = x0 + 7e-9;
  for (int i = 0; i < iters; ++i) {
    x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
    x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
  }
  double s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
  if (s == 12345.678) out[blockIdx.x] = s;   // keeps the chains live
}
}  // namespace

extern "C" dgx_status dgx_measure_fp64_peak(double* tflops, double* ms_out) {
  if (!tflops) return DGX_ERR_ARG;
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  double* d = nullptr;
  if (cudaMalloc(&d, sizeof(double) * 65536) != cudaSuccess) return DGX_ERR_NOMEM;
  const int threads = 256, blocks = sms * 8, iters = 16384;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0); cudaEventCreate(&e1);
  k_dfma<<<blocks, threads>>>(d, 64, 0.999999, 1e-7);          // warm-up
  float best = 1e30f;
  for (int rep = 0; rep < 5; ++rep) {
    cudaEventRecord(e0);
    k_dfma<<<blocks, threads>>>(d, iters, 0.999999, 1e-7);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0); cudaEventDestroy(e1);
  cudaFree(d);
  if (err != cudaSuccess) return DGX_ERR_CUDA;
  double flops = 2.0 * 8.0 * (double)iters * threads * blocks;
  *tflops = flops / (best * 1e-3) / 1e12;
  if (ms_out) *ms_out = best;
  return DGX_OK;
}
