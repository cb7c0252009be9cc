// Kernels (a) and (b): SparseShape::gemm screening and the Summa tile-pair
// list, for sm_103a.
//
// (a) follows sparse_shape.h:1589-1684: L'[i,k] = L[i,k] * ksz[k],
//     R'[k,j] = R[k,j] * ksz[k], C[i,j] = |factor| * sum_k L'[i,k] * R'[k,j]
//     in float, then C < threshold -> 0 and counted.  The reference leaves the
//     summation order to sgemm; here it is k ascending with every product and
//     sum rounded separately (__fmul_rn / __fadd_rn, no FMA), the order the
//     CPU oracle uses, so the screened pattern is bit-exact.
// (b) follows dist_eval/contraction_eval.h:630-650, 1093-1161, 1348-1384: the
//     pair (i,k,j) exists iff result tile (i,j) is nonzero and both argument
//     tiles are nonzero; zero-ness is `norm < threshold` (sparse_shape.h:
//     495-523).  Pairs are emitted grouped by result tile (row-major) with k
//     ascending, so the reduction order per result tile is fixed.
#include <cuda_runtime.h>

#include "internal.h"

namespace tagpu {
namespace {

__global__ void shape_gemm_kernel(int64_t M, int64_t N, int64_t K,
                                  const float* __restrict__ L,
                                  const float* __restrict__ R,
                                  const float* __restrict__ ksz, float af,
                                  float thr, float* __restrict__ C,
                                  unsigned long long* zero_count) {
  const int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t total = M * N;
  unsigned zeros = 0;
  if (t < total) {
    const int64_t i = t / N, j = t - (t / N) * N;
    float v;
    if (K == 0) {
      v = __fmul_rn(__fmul_rn(L[i], R[j]), af);
    } else {
      float acc = 0.0f;
      const float* l = L + i * K;
      for (int64_t k = 0; k < K; ++k) {
        const float ks = ksz[k];
        const float a = __fmul_rn(l[k], ks);
        const float b = __fmul_rn(R[k * N + j], ks);
        acc = __fadd_rn(acc, __fmul_rn(a, b));
      }
      v = __fmul_rn(af, acc);
    }
    if (v < thr) {
      v = 0.0f;
      zeros = 1;
    }
    C[t] = v;
  }
  // one atomic per warp
  const unsigned b = __ballot_sync(0xffffffffu, zeros);
  if ((threadIdx.x & 31) == 0 && b) atomicAdd(zero_count, (unsigned long long)__popc(b));
}

// One warp per result tile: count the surviving k and accumulate
// 2*m*n*sum(k sizes) for the nonzero-block flop count.
__global__ void pair_count_kernel(int64_t M, int64_t N, int64_t K,
                                  const float* __restrict__ C, float cthr,
                                  const float* __restrict__ L, float lthr,
                                  const float* __restrict__ R, float rthr,
                                  const int32_t* __restrict__ msz,
                                  const int32_t* __restrict__ nsz,
                                  const int32_t* __restrict__ ksz,
                                  int64_t* __restrict__ counts, double* flops) {
  const int lane = threadIdx.x & 31;
  const int64_t t = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (t >= M * N) return;
  const int64_t i = t / N, j = t - (t / N) * N;
  int64_t cnt = 0;
  int64_t ksum = 0;
  if (!(C[t] < cthr)) {
    for (int64_t k0 = 0; k0 < K; k0 += 32) {
      const int64_t k = k0 + lane;
      bool p = false;
      if (k < K) p = !(L[i * K + k] < lthr) && !(R[k * N + j] < rthr);
      const unsigned b = __ballot_sync(0xffffffffu, p);
      cnt += __popc(b);
      if (p) ksum += ksz[k];
    }
  }
  for (int o = 16; o > 0; o >>= 1) ksum += __shfl_xor_sync(0xffffffffu, ksum, o);
  if (lane == 0) {
    counts[t] = cnt;
    if (ksum) atomicAdd(flops, 2.0 * (double)msz[i] * (double)nsz[j] * (double)ksum);
  }
}

__global__ void pair_emit_kernel(int64_t M, int64_t N, int64_t K,
                                 const float* __restrict__ C, float cthr,
                                 const float* __restrict__ L, float lthr,
                                 const float* __restrict__ R, float rthr,
                                 const int64_t* __restrict__ offsets,
                                 int32_t* __restrict__ kidx) {
  const int lane = threadIdx.x & 31;
  const int64_t t = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (t >= M * N) return;
  if (C[t] < cthr) return;
  const int64_t i = t / N, j = t - (t / N) * N;
  int64_t pos = offsets[t];
  for (int64_t k0 = 0; k0 < K; k0 += 32) {
    const int64_t k = k0 + lane;
    bool p = false;
    if (k < K) p = !(L[i * K + k] < lthr) && !(R[k * N + j] < rthr);
    const unsigned b = __ballot_sync(0xffffffffu, p);
    if (p) kidx[pos + __popc(b & ((1u << lane) - 1u))] = (int32_t)k;
    pos += __popc(b);
  }
}

// Single-CTA exclusive scan (1024 threads), chunked with a running carry.
// The lists scanned here have at most a few million entries.
__global__ void __launch_bounds__(1024) exclusive_scan_kernel(
    const int64_t* __restrict__ in, int64_t n, int64_t* __restrict__ out) {
  __shared__ int64_t warp_sums[32];
  __shared__ int64_t carry_s;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (tid == 0) carry_s = 0;
  __syncthreads();
  for (int64_t base = 0; base < n; base += 1024) {
    const int64_t idx = base + tid;
    const int64_t v = idx < n ? in[idx] : 0;
    int64_t x = v;
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
      int64_t w = warp_sums[lane];
      for (int o = 1; o < 32; o <<= 1) {
        const int64_t y = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += y;
      }
      warp_sums[lane] = w;
    }
    __syncthreads();
    const int64_t carry = carry_s;
    const int64_t incl = x + (warp ? warp_sums[warp - 1] : 0) + carry;
    if (idx < n) out[idx] = incl - v;
    __syncthreads();
    if (tid == 1023) carry_s = incl;
    __syncthreads();
  }
  if (tid == 0) out[n] = carry_s;
}

}  // namespace

void launch_shape_gemm(cudaStream_t s, int64_t M, int64_t N, int64_t K,
                       const float* L, const float* R, const float* ksz,
                       float abs_factor, float thr, float* C,
                       unsigned long long* zero_count) {
  const int64_t total = M * N;
  if (total == 0) return;
  const int threads = 256;
  const int64_t blocks = (total + threads - 1) / threads;
  shape_gemm_kernel<<<(unsigned)blocks, threads, 0, s>>>(M, N, K, L, R, ksz, abs_factor,
                                                         thr, C, zero_count);
  count_launch();
}

void launch_pair_count(cudaStream_t s, int64_t M, int64_t N, int64_t K,
                       const float* C, float cthr, const float* L, float lthr,
                       const float* R, float rthr, const int32_t* msz,
                       const int32_t* nsz, const int32_t* ksz, int64_t* counts,
                       double* flops) {
  const int64_t total = M * N;
  if (total == 0) return;
  const int threads = 256;
  const int64_t blocks = (total * 32 + threads - 1) / threads;
  pair_count_kernel<<<(unsigned)blocks, threads, 0, s>>>(M, N, K, C, cthr, L, lthr, R, rthr,
                                                         msz, nsz, ksz, counts, flops);
  count_launch();
}

void launch_exclusive_scan(cudaStream_t s, const int64_t* in, int64_t n, int64_t* out) {
  exclusive_scan_kernel<<<1, 1024, 0, s>>>(in, n, out);
  count_launch();
}

void launch_pair_emit(cudaStream_t s, int64_t M, int64_t N, int64_t K,
                      const float* C, float cthr, const float* L, float lthr,
                      const float* R, float rthr, const int64_t* offsets,
                      int32_t* kidx) {
  const int64_t total = M * N;
  if (total == 0) return;
  const int threads = 256;
  const int64_t blocks = (total * 32 + threads - 1) / threads;
  pair_emit_kernel<<<(unsigned)blocks, threads, 0, s>>>(M, N, K, C, cthr, L, lthr, R, rthr,
                                                        offsets, kidx);
  count_launch();
}

}  // namespace tagpu
