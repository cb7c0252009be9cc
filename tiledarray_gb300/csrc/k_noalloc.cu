// Allocation-free variant of kernel (b), the tile-pair list.
//
// For callers that cannot allocate device memory — for example code that runs
// while another framework owns every byte of the device through its own pool,
// or a latency-critical loop where an allocation (and the implicit
// synchronisation it may cause) is not acceptable.  The caller passes device
// pointers for every input and output; the only scratch the kernel needs (one
// pair count per result tile, between the counting and the scan pass) lives in
// a file-scope __device__ array of fixed size, so this entry point calls no
// cudaMalloc/cudaFree and no allocating library routine.
//
// Limits and sharing: M*N (result tiles) may not exceed kNoAllocMaxTiles
// (1,048,576; 8 MB of counts).  The array exists once per device that loads
// the library and lives until the process exits.  Every call shares it and it
// keeps the last call's contents; each call overwrites every count it uses
// before reading it, so nothing needs clearing, but calls whose kernels overlap
// on the GPU (for example on two streams) race on it.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "internal.h"

namespace tagpu {
namespace {

constexpr int64_t kNoAllocMaxTiles = int64_t(1) << 20;

static __device__ __align__(256) int64_t g_pair_counts[kNoAllocMaxTiles];

// Per-result-tile pair count (same predicate as pair_count_kernel, without the
// flop accounting).  One warp per result tile.
__global__ void noalloc_count_kernel(int64_t M, int64_t N, int64_t K,
                                     const float* __restrict__ C, float cthr,
                                     const float* __restrict__ L, float lthr,
                                     const float* __restrict__ R, float rthr,
                                     int64_t* __restrict__ counts) {
  const int lane = threadIdx.x & 31;
  const int64_t t = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (t >= M * N) return;
  const int64_t i = t / N, j = t - (t / N) * N;
  int64_t cnt = 0;
  if (!(C[t] < cthr)) {
    for (int64_t k0 = 0; k0 < K; k0 += 32) {
      const int64_t k = k0 + lane;
      const bool p = k < K && !(L[i * K + k] < lthr) && !(R[k * N + j] < rthr);
      cnt += __popc(__ballot_sync(0xffffffffu, p));
    }
  }
  if (lane == 0) counts[t] = cnt;
}

// Device address of g_pair_counts per device, looked up once.
std::mutex g_mu;
int64_t* g_addr[128] = {nullptr};

}  // namespace
}  // namespace tagpu

using namespace tagpu;

extern "C" tagpu_status tagpu_pair_list_noalloc(tagpu_ctx* ctx, int64_t M, int64_t N, int64_t K,
                                                const float* cnorm, float c_thr,
                                                const float* lnorm, float l_thr,
                                                const float* rnorm, float r_thr,
                                                int64_t* offsets, int32_t* kidx,
                                                int64_t kidx_cap, int64_t* npairs,
                                                void* stream) {
  if (!ctx) return TAGPU_ERR_INVALID;
  if (M < 0 || N < 0 || K < 0 || !offsets)
    return set_last_error(ctx, TAGPU_ERR_INVALID, "pair_list_noalloc: bad arguments");
  // M and N are bounded one at a time before their product is formed, so a
  // huge pair cannot overflow int64 and slip past the limit.
  if ((N > 0 && M > kNoAllocMaxTiles / N) || (M > 0 && N > kNoAllocMaxTiles / M))
    return set_last_error(ctx, TAGPU_ERR_INVALID,
                          "pair_list_noalloc: M*N result tiles above the fixed scratch of "
                          "1048576 tiles");
  if (M * N > 0 && (!cnorm || (K > 0 && (!lnorm || !rnorm))))
    return set_last_error(ctx, TAGPU_ERR_INVALID, "pair_list_noalloc: null input");
  const int dev = context_device(ctx);
  int prev_dev = -1;
  if (cudaGetDevice(&prev_dev) != cudaSuccess) {
    cudaGetLastError();
    prev_dev = -1;
  }
  if (dev < 0 || dev >= 128 || cudaSetDevice(dev) != cudaSuccess) {
    cudaGetLastError();
    return set_last_error(ctx, TAGPU_ERR_CUDA, "pair_list_noalloc: cannot select the device");
  }
  // the caller's current device is put back on every return below
  struct RestoreDevice {
    int d;
    ~RestoreDevice() {
      if (d >= 0) cudaSetDevice(d);
    }
  } restore{prev_dev};
  int64_t* counts = nullptr;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[dev]) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_pair_counts) != cudaSuccess || !p) {
        cudaGetLastError();
        return set_last_error(ctx, TAGPU_ERR_CUDA,
                              "pair_list_noalloc: scratch symbol address lookup failed");
      }
      g_addr[dev] = static_cast<int64_t*>(p);
    }
    counts = g_addr[dev];
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int64_t MN = M * N;
  if (MN > 0) {
    const int threads = 256;
    noalloc_count_kernel<<<(unsigned)((MN * 32 + threads - 1) / threads), threads, 0, s>>>(
        M, N, K, cnorm, c_thr, lnorm, l_thr, rnorm, r_thr, counts);
    count_launch();
  }
  launch_exclusive_scan(s, counts, MN, offsets);
  int64_t np = 0;
  if (cudaMemcpyAsync(&np, offsets + MN, sizeof(np), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess) {
    const cudaError_t ce = cudaGetLastError();
    return set_last_error(ctx, TAGPU_ERR_CUDA,
                          (std::string("pair_list_noalloc: pair count: ") + cudaGetErrorString(ce)).c_str());
  }
  if (npairs) *npairs = np;
  if (kidx) {
    if (kidx_cap < np)
      return set_last_error(ctx, TAGPU_ERR_INVALID, "pair_list_noalloc: kidx capacity too small");
    launch_pair_emit(s, M, N, K, cnorm, c_thr, lnorm, l_thr, rnorm, r_thr, offsets, kidx);
    if (cudaStreamSynchronize(s) != cudaSuccess) {
      const cudaError_t ce = cudaGetLastError();
      return set_last_error(ctx, TAGPU_ERR_CUDA,
                            (std::string("pair_list_noalloc: pair emission: ") +
                             cudaGetErrorString(ce)).c_str());
    }
  }
  const cudaError_t ce = cudaGetLastError();
  if (ce != cudaSuccess)
    return set_last_error(ctx, TAGPU_ERR_CUDA,
                          (std::string("pair_list_noalloc: ") + cudaGetErrorString(ce)).c_str());
  return TAGPU_OK;
}
