// Measured FP64 rates of this GPU (the denominators of the plain form's
// roofline; the measured peaks cover HBM and bf16 only).
//   DMMA: mma.sync m8n8k4 f64 chains, 8 independent accumulators per thread
//   DFMA: fma chains, 8 independent accumulators per thread
#include <cuda_runtime.h>

#include "internal.h"

namespace tagpu {
namespace {

__global__ void dmma_rate_kernel(double* out, int iters) {
  const double a = threadIdx.x * 1e-3, b = 1.0 + blockIdx.x * 1e-6;
  double c[8][2] = {};
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int x = 0; x < 8; ++x)
      asm volatile(
          "mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
          : "+d"(c[x][0]), "+d"(c[x][1])
          : "d"(a), "d"(b));
  }
  double s = 0;
  for (int x = 0; x < 8; ++x) s += c[x][0] + c[x][1];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void dfma_rate_kernel(double* out, int iters) {
  const double a = threadIdx.x * 1e-3, b = 1.0 + blockIdx.x * 1e-9;
  double c[8];
  for (int x = 0; x < 8; ++x) c[x] = x;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int x = 0; x < 8; ++x) c[x] = fma(a, c[x], b);
  }
  double s = 0;
  for (int x = 0; x < 8; ++x) s += c[x];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

tagpu_status measure_fp64_rates(cudaStream_t s, int sm_count, double* dmma_tflops,
                                double* dfma_tflops) {
  const int blocks = sm_count * 4, threads = 256, iters = 4096;
  double* out = nullptr;
  if (cudaMallocAsync(&out, (size_t)blocks * threads * sizeof(double), s) != cudaSuccess)
    return TAGPU_ERR_NOMEM;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best_mma = 1e30f, best_fma = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    float ms = 0;
    cudaEventRecord(e0, s);
    dmma_rate_kernel<<<blocks, threads, 0, s>>>(out, iters);
    count_launch();
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best_mma) best_mma = ms;
    cudaEventRecord(e0, s);
    dfma_rate_kernel<<<blocks, threads, 0, s>>>(out, iters);
    count_launch();
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best_fma) best_fma = ms;
  }
  const double warps = (double)blocks * threads / 32;
  *dmma_tflops = 512.0 * 8 * iters * warps / best_mma / 1e9;            // 512 flops per mma
  *dfma_tflops = 16.0 * iters * (double)blocks * threads / best_fma / 1e9;  // 8 fma per iter
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFreeAsync(out, s);
  const cudaError_t e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? TAGPU_OK : TAGPU_ERR_CUDA;
}

}  // namespace tagpu
