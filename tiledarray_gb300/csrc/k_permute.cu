// Kernel (c): tile permutation into GEMM order, for sm_103a.
//
// Semantics follow tensor/permute.h:124-210 and permutation.h:60-78: result
// dimension perm[d] is argument dimension d, both row-major.  The reference
// fuses dimensions and runs blocked 2-D transposes (math/transpose.h:178);
// here every tile is decomposed into work items:
//   * the argument's fastest dimension stays fastest: items are groups of
//     contiguous rows, copied with coalesced loads and stores;
//   * otherwise the plane (b, a) of the argument's fastest dimension a and the
//     dimension b that becomes the result's fastest is cut into 32x32 blocks,
//     staged through shared memory so that both the load (along a) and the
//     store (along b) are coalesced; all other dimensions form the batch.
// All tiles of one array share the permutation; extents differ per tile.
// Index arithmetic is paid per item, not per element: a row-copy item is
// kRowsPerItem rows whose offsets are computed once into shared memory and
// then copied as one flat, coalesced element range; a transpose item is a
// strip of 32 x 32 blocks along the result's fastest dimension.
#include <cuda_runtime.h>

#include "internal.h"

namespace tagpu {
namespace {

constexpr int kRowsPerItem = 128;

struct TileGeom {
  int64_t e[8];       // argument extents
  int64_t is[8];      // argument strides
  int64_t os[8];      // result stride of argument dim d
  int64_t vol;
  int a, b;           // argument fastest dim, argument dim that becomes fastest
};

__host__ __device__ inline void make_geom(const PermuteDesc& d, const int32_t* ext,
                                          TileGeom& g) {
  const int r = d.rank;
  int64_t f[8];
  g.vol = 1;
  for (int x = 0; x < r; ++x) {
    g.e[x] = ext[x];
    g.vol *= ext[x];
    f[d.perm[x]] = ext[x];
  }
  int64_t s = 1;
  for (int x = r - 1; x >= 0; --x) {
    g.is[x] = s;
    s *= g.e[x];
  }
  int64_t fs[8];
  s = 1;
  for (int q = r - 1; q >= 0; --q) {
    fs[q] = s;
    s *= f[q];
  }
  for (int x = 0; x < r; ++x) g.os[x] = fs[d.perm[x]];
  g.a = r - 1;
  g.b = r - 1;
  for (int x = 0; x < r; ++x)
    if (d.perm[x] == r - 1) g.b = x;
}

__host__ __device__ inline int64_t items_of(const TileGeom& g) {
  if (g.vol == 0) return 0;
  if (g.a == g.b) {
    const int64_t rows = g.vol / g.e[g.a];
    return (rows + kRowsPerItem - 1) / kRowsPerItem;
  }
  const int64_t batch = g.vol / (g.e[g.a] * g.e[g.b]);
  return batch * ((g.e[g.a] + 31) / 32);
}

// offsets of the batch index `bi` over all dims except `skip0`/`skip1`
__device__ inline void batch_offsets(const TileGeom& g, int rank, int skip0, int skip1,
                                     int64_t bi, int64_t& in_off, int64_t& out_off) {
  in_off = 0;
  out_off = 0;
  for (int x = rank - 1; x >= 0; --x) {
    if (x == skip0 || x == skip1) continue;
    const int64_t ix = bi % g.e[x];
    bi /= g.e[x];
    in_off += ix * g.is[x];
    out_off += ix * g.os[x];
  }
}

__global__ void __launch_bounds__(256) permute_kernel(
    PermuteDesc d, int64_t ntiles, const int32_t* __restrict__ ext,
    const int64_t* __restrict__ in_off, const int64_t* __restrict__ out_off,
    const int64_t* __restrict__ item_start, int64_t nitems,
    const double* __restrict__ in, double* __restrict__ out) {
  __shared__ double buf[32][33];
  __shared__ int64_t s_io[kRowsPerItem], s_oo[kRowsPerItem];
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;  // 32 x 8
  for (int64_t item = blockIdx.x; item < nitems; item += gridDim.x) {
    // tile owning this item
    int64_t lo = 0, hi = ntiles;
    while (hi - lo > 1) {
      const int64_t mid = (lo + hi) >> 1;
      if (item_start[mid] <= item) lo = mid; else hi = mid;
    }
    const int64_t t = lo;
    TileGeom g;
    make_geom(d, ext + t * d.rank, g);
    const int64_t local = item - item_start[t];
    const double* src = in + in_off[t];
    double* dst = out + out_off[t];
    if (g.a == g.b) {
      const int64_t rowlen = g.e[g.a];
      const int64_t rows = g.vol / rowlen;
      const int64_t r0 = local * kRowsPerItem;
      const int nr = (int)(rows - r0 < kRowsPerItem ? rows - r0 : kRowsPerItem);
      for (int i = threadIdx.x; i < nr; i += blockDim.x) {
        int64_t io, oo;
        batch_offsets(g, d.rank, g.a, -1, r0 + i, io, oo);
        s_io[i] = io;
        s_oo[i] = oo;
      }
      __syncthreads();
      // one warp per row; 16-byte accesses when both ends are aligned
      for (int row = ty; row < nr; row += 8) {
        const double* sp = src + s_io[row];
        double* dp = dst + s_oo[row];
        if (((((uintptr_t)sp) | ((uintptr_t)dp)) & 15) == 0) {
          const int64_t half = rowlen >> 1;
          const double2* s2 = reinterpret_cast<const double2*>(sp);
          double2* d2 = reinterpret_cast<double2*>(dp);
#pragma unroll 2
          for (int64_t c = tx; c < half; c += 32) d2[c] = s2[c];
          if ((rowlen & 1) && tx == 0) dp[rowlen - 1] = sp[rowlen - 1];
        } else {
#pragma unroll 2
          for (int64_t c = tx; c < rowlen; c += 32) dp[c] = sp[c];
        }
      }
      __syncthreads();
    } else {
      // strip: batch index bi, block ab along a; all blocks along b
      const int64_t ea = g.e[g.a], eb = g.e[g.b];
      const int64_t na = (ea + 31) / 32;
      const int64_t bi = local / na, ab = local - bi * na;
      int64_t io, oo;
      batch_offsets(g, d.rank, g.a, g.b, bi, io, oo);
      const int64_t a0 = ab * 32;
      const int64_t isb = g.is[g.b], osa = g.os[g.a];
      for (int64_t b0 = 0; b0 < eb; b0 += 32) {
        // load: along a (stride 1 in the argument)
#pragma unroll
        for (int yy = ty; yy < 32; yy += 8) {
          const int64_t ib = b0 + yy, ia = a0 + tx;
          if (ib < eb && ia < ea) buf[yy][tx] = src[io + ib * isb + ia];
        }
        __syncthreads();
        // store: along b (stride 1 in the result)
#pragma unroll
        for (int yy = ty; yy < 32; yy += 8) {
          const int64_t ia = a0 + yy, ib = b0 + tx;
          if (ib < eb && ia < ea) dst[oo + ia * osa + ib] = buf[tx][yy];
        }
        __syncthreads();
      }
    }
  }
}

}  // namespace

int64_t permute_items(const PermuteDesc& d, const int64_t* ext) {
  int32_t e32[8];
  for (int x = 0; x < d.rank; ++x) e32[x] = (int32_t)ext[x];
  TileGeom g;
  make_geom(d, e32, g);
  return items_of(g);
}

void launch_permute(cudaStream_t s, const PermuteDesc& d, int64_t ntiles,
                    const int32_t* ext, const int64_t* in_off,
                    const int64_t* out_off, const int64_t* item_start,
                    int64_t nitems, const double* in, double* out) {
  if (nitems <= 0) return;
  int dev = 0, sms = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int64_t grid = nitems < (int64_t)sms * 16 ? nitems : (int64_t)sms * 16;
  permute_kernel<<<(unsigned)grid, 256, 0, s>>>(d, ntiles, ext, in_off, out_off, item_start,
                                                nitems, in, out);
  count_launch();
}

}  // namespace tagpu
