// Device-side synthetic operands and tile norms, for sm_103a.
//
// Values: element with global ordinal g (row-major over the array's element
// range) of tile t is value(seed, stream, g) * scale[t], where value is a
// counter-based hash (splitmix64) mapped to uniform[-1,1) or to the integers
// 0..100 (the `rand() % 101` data of the reference's tests).  The same
// definition is used on the host, so operands are identical everywhere.
//
// Norms: Tensor::norm (tensor/tensor.h:3768-3787) is sqrt of a sequential
// double sum of x*x in storage order (math/vector_op.h:561-577), stored as
// float.  A warp per tile estimates the sum and proves from an error bound
// which float the sequential sum rounds to, walking the tile in that order
// itself only when the bound cannot decide (tile_norms_kernel), so the norms
// (and the SparseShape built from them) match the host bit for bit.
#include <cuda_runtime.h>

#include "internal.h"

namespace tagpu {
namespace {

__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

__global__ void generate_kernel(GenDesc g, int64_t ntiles,
                                const int64_t* __restrict__ tile_lo,
                                const int32_t* __restrict__ tile_ext,
                                const int64_t* __restrict__ tile_off,
                                const double* __restrict__ tile_scale,
                                double* __restrict__ data) {
  const int64_t total = tile_off[ntiles];
  const uint64_t key = splitmix64(g.seed * 0x9E3779B97F4A7C15ull + g.stream);
  int64_t gstride[8];
  int64_t s = 1;
  for (int d = g.rank - 1; d >= 0; --d) {
    gstride[d] = s;
    s *= g.gext[d];
  }
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += (int64_t)gridDim.x * blockDim.x) {
    int64_t lo = 0, hi = ntiles;
    while (hi - lo > 1) {
      const int64_t mid = (lo + hi) >> 1;
      if (tile_off[mid] <= e) lo = mid; else hi = mid;
    }
    const int64_t t = lo;
    int64_t local = e - tile_off[t];
    int64_t gord = 0;
    for (int d = g.rank - 1; d >= 0; --d) {
      const int64_t ext = tile_ext[t * g.rank + d];
      const int64_t ix = local % ext;
      local /= ext;
      gord += (tile_lo[t * g.rank + d] + ix) * gstride[d];
    }
    const uint64_t h = splitmix64(key ^ (uint64_t)gord);
    double v = g.kind == 1 ? (double)(h % 101ull)
                           : __dsub_rn(__dmul_rn(__dmul_rn((double)(h >> 11), 0x1.0p-53), 2.0), 1.0);
    data[e] = __dmul_rn(v, tile_scale ? tile_scale[t] : 1.0);
  }
}

// Tile norms, bit-exact with the sequential order of the reference's serial
// reduction (math/vector_op.h:561-577 reduce_op_serial, used by Tensor::norm):
// s = fl(s + fl(x_i * x_i)) for i = 0..n-1, then float(sqrt(s)).
//
// One warp per tile.  The lanes sum fma(x, x, .) over a strided share of the
// tile (coalesced), giving an estimate S of the exact sum of squares with
// relative error at most gamma(n/32 + 5), gamma(m) = m u / (1 - m u),
// u = 2^-53.  The sequential sum differs from the exact one by at most
// gamma(n) of it (recursive summation of n rounded products, Higham,
// "Accuracy and Stability of Numerical Algorithms", 4.2), plus n * 2^-1074
// absolute where products fall below the normal range.  If both ends of
// that interval around S give the same float after the correctly rounded
// square root and the rounding to float (both monotonic), the sequential
// result gives it too; otherwise lane 0 runs the sequential loop itself.
// The fallback is rare: the interval is about n * 2^-52 wide relative to S
// against float spacing 2^-23, so a tile of n elements takes it with
// probability about n * 2^-29.
__global__ void tile_norms_kernel(int64_t ntiles, const int64_t* __restrict__ tile_off,
                                  const double* __restrict__ data, float* __restrict__ norms) {
  const int64_t t = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (t >= ntiles) return;
  const double* x = data + tile_off[t];
  const int64_t n = tile_off[t + 1] - tile_off[t];
  double a0 = 0.0, a1 = 0.0;
  int64_t i = lane;
  for (; i + 32 < n; i += 64) {
    const double u0 = x[i], u1 = x[i + 32];
    a0 = fma(u0, u0, a0);
    a1 = fma(u1, u1, a1);
  }
  if (i < n) a0 = fma(x[i], x[i], a0);
  double est = a0 + a1;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) est += __shfl_xor_sync(0xffffffffu, est, o);
  float out = 0.0f;
  bool exact = false;
  if (lane == 0) {
    const double u = 0x1.0p-53;
    const double m_est = (double)(n / 64 + 8), m_seq = (double)n + 2.0;
    // plus 4u for the roundings of the two ends themselves
    const double g = (m_seq + m_est) * u / (1.0 - (m_seq + m_est) * u) + 4.0 * u;
    const double tiny = ((double)n + 2.0) * 0x1.0p-1074 * 4.0;
    const double lo = est * (1.0 - g) - tiny, hi = est * (1.0 + g) + tiny;
    const float flo = __double2float_rn(__dsqrt_rn(lo > 0.0 ? lo : 0.0));
    const float fhi = __double2float_rn(__dsqrt_rn(hi));
    exact = flo == fhi && est == est && est < 1.0e300;
    out = flo;
  }
  exact = __shfl_sync(0xffffffffu, exact ? 1 : 0, 0) != 0;
  if (lane != 0) return;
  if (!exact) {
    double s = 0.0;
    for (int64_t k = 0; k < n; ++k) s = __dadd_rn(s, __dmul_rn(x[k], x[k]));
    out = __double2float_rn(__dsqrt_rn(s));
  }
  norms[t] = out;
}

}  // namespace

void launch_generate(cudaStream_t s, const GenDesc& g, int64_t ntiles,
                     const int64_t* tile_lo, const int32_t* tile_ext,
                     const int64_t* tile_off, const double* tile_scale, double* data) {
  if (ntiles <= 0) return;
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  generate_kernel<<<sms * 8, 256, 0, s>>>(g, ntiles, tile_lo, tile_ext, tile_off, tile_scale,
                                          data);
  count_launch();
}

void launch_tile_norms(cudaStream_t s, int64_t ntiles, const int64_t* tile_off,
                       const double* data, float* norms) {
  if (ntiles <= 0) return;
  const int threads = 256;   // eight tiles per block, a warp each
  tile_norms_kernel<<<(unsigned)((ntiles * 32 + threads - 1) / threads), threads, 0, s>>>(
      ntiles, tile_off, data, norms);
  count_launch();
}

}  // namespace tagpu
