// Measured rates of this GPU's warp-level (mma.sync) tensor paths and FP64
// FMA (the plain form's roofline denominators, and the evidence for which
// tensor path the emulated form runs on; the measured peaks cover HBM
// and tcgen05 bf16 only).
//   DMMA: mma.sync m8n8k4 f64 chains, 8 independent accumulators per thread
//   DFMA: fma chains, 8 independent accumulators per thread
//   IMMA: mma.sync m16n8k32 s8 x s8 -> s32 chains, 8 accumulators per thread
//   HMMA: mma.sync m16n8k16 bf16 x bf16 -> f32 chains, 8 accumulators
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

__global__ void imma_rate_kernel(int* out, int iters) {
  const uint32_t a = 0x01010101u * (threadIdx.x & 7), b = 0x01020304u + blockIdx.x;
  int c[8][4] = {};
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int x = 0; x < 8; ++x)
      asm volatile(
          "mma.sync.aligned.m16n8k32.row.col.s32.s8.s8.s32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
          "{%8,%9}, {%0,%1,%2,%3};"
          : "+r"(c[x][0]), "+r"(c[x][1]), "+r"(c[x][2]), "+r"(c[x][3])
          : "r"(a), "r"(a), "r"(a), "r"(a), "r"(b), "r"(b));
  }
  int s = 0;
  for (int x = 0; x < 8; ++x) s += c[x][0] + c[x][1] + c[x][2] + c[x][3];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void hmma_rate_kernel(float* out, int iters) {
  const uint32_t a = 0x3f803f80u, b = 0x3c003c00u + blockIdx.x;   // bf16 pairs
  float c[8][4] = {};
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int x = 0; x < 8; ++x)
      asm volatile(
          "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
          "{%8,%9}, {%0,%1,%2,%3};"
          : "+f"(c[x][0]), "+f"(c[x][1]), "+f"(c[x][2]), "+f"(c[x][3])
          : "r"(a), "r"(a), "r"(a), "r"(a), "r"(b), "r"(b));
  }
  float s = 0;
  for (int x = 0; x < 8; ++x) s += c[x][0] + c[x][1] + c[x][2] + c[x][3];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace

// Rates of the legacy warp-level tensor paths: INT8 (TOP/s) and bf16
// (TFLOP/s) mma.sync, best of three ~0.1 s runs.
tagpu_status measure_mma_sync_rates(cudaStream_t s, int sm_count, double* imma_tops,
                                    double* hmma_tflops) {
  const int blocks = sm_count * 4, threads = 256, iters = 8192;
  void* out = nullptr;
  if (cudaMallocAsync(&out, (size_t)blocks * threads * 4, s) != cudaSuccess)
    return TAGPU_ERR_NOMEM;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best_i = 1e30f, best_h = 1e30f;
  for (int rep = 0; rep < 3; ++rep) {
    float ms = 0;
    cudaEventRecord(e0, s);
    imma_rate_kernel<<<blocks, threads, 0, s>>>(static_cast<int*>(out), iters);
    count_launch();
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best_i) best_i = ms;
    cudaEventRecord(e0, s);
    hmma_rate_kernel<<<blocks, threads, 0, s>>>(static_cast<float*>(out), iters);
    count_launch();
    cudaEventRecord(e1, s);
    cudaEventSynchronize(e1);
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best_h) best_h = ms;
  }
  const double warps = (double)blocks * threads / 32;
  *imma_tops = 2.0 * 16 * 8 * 32 * 8 * iters * warps / best_i / 1e9;     // per mma: 8192 ops
  *hmma_tflops = 2.0 * 16 * 8 * 16 * 8 * iters * warps / best_h / 1e9;   // per mma: 4096 flops
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFreeAsync(out, s);
  const cudaError_t e = cudaStreamSynchronize(s);
  return e == cudaSuccess ? TAGPU_OK : TAGPU_ERR_CUDA;
}

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
