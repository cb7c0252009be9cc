// Kernel (d), plain form: grouped FP64 GEMM on the DMMA tensor cores
// (mma.sync m8n8k4 f64) over the compacted tile-pair list, for sm_103a.
//
// Reference semantics (tile_op/contract_reduce.h:367-452, tensor/tensor.h:
// 3132-3210, math/blas.h:171-177): result tile (i,j) is
// sum over its pairs k of alpha * op(A(i,k)) * op(B(k,j)), the first pair
// writing (beta = 0).  Here one CTA owns a 64x64 block of one result tile and
// walks the pair list of that tile in ascending k, accumulating in registers,
// so the reduction order is fixed and no atomics are needed.  alpha is applied
// once in the epilogue.  Uneven tile sizes are handled by zero-filled
// cp.async loads; transposed storage (Op::Trans) is folded into the loader.
#include <cuda_runtime.h>

#include "internal.h"

namespace tagpu {
namespace {

constexpr int BM = 64, BN = 64, BK = 16;
constexpr int SA = BK + 4;   // A row stride (doubles): conflict-free fragments
constexpr int SB = BN + 4;   // B row stride

__device__ __forceinline__ void cp_async8(void* smem, const void* gmem, bool pred) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  const int n = pred ? 8 : 0;
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;\n" ::"r"(s), "l"(gmem), "r"(n));
}
__device__ __forceinline__ void cp_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N)); }

__device__ __forceinline__ void dmma(double (&c)[2], double a, double b) {
  asm volatile(
      "mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
      : "+d"(c[0]), "+d"(c[1])
      : "d"(a), "d"(b));
}

struct Stage {
  double a[BM][SA];
  double b[BK][SB];
};

__global__ void __launch_bounds__(128) dmma_gemm_kernel(const GemmView* __restrict__ views,
                                                        const WorkItem* __restrict__ items,
                                                        int64_t nitems) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Stage* st = reinterpret_cast<Stage*>(smem_raw);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  const int g = lane >> 2, q = lane & 3;

  for (int64_t it = blockIdx.x; it < nitems; it += gridDim.x) {
    const WorkItem w = items[it];
    const GemmView& v = views[w.view];
    const int64_t t = w.tile;
    const int rb = w.rb, cb = w.cb;
    const int64_t i = t / v.Nt, j = t - (t / v.Nt) * v.Nt;
    const int m = v.msz[i], n = v.nsz[j];
    const int r0 = rb * BM, c0 = cb * BN;
    double acc[4][4][2];
#pragma unroll
    for (int x = 0; x < 4; ++x)
#pragma unroll
      for (int y = 0; y < 4; ++y) acc[x][y][0] = acc[x][y][1] = 0.0;

    const int64_t p0 = v.poff[t], p1 = v.poff[t + 1];
    // flattened (pair, k-chunk) iteration
    int64_t p = p0;
    int kk = 0, kcur = 0;
    const double* Ap = nullptr;
    const double* Bp = nullptr;
    auto advance_pair = [&]() {
      while (p < p1) {
        const int k = v.kidx[p];
        const int64_t ao = v.aoff[i * v.Kt + k], bo = v.boff[(int64_t)k * v.Nt + j];
        if (ao >= 0 && bo >= 0) {
          kk = v.ksz[k];
          Ap = v.A + ao + v.hel * (int64_t)m * kk;
          Bp = v.B + bo + v.hel * (int64_t)kk * n;
          kcur = 0;
          return true;
        }
        ++p;
      }
      return false;
    };
    auto load = [&](int buf) {
      Stage& s = st[buf];
      // A block: BM rows x BK k
#pragma unroll
      for (int e = tid; e < BM * BK; e += 128) {
        int r, c;
        if (v.a_trans) { r = e % BM; c = e / BM; } else { r = e / BK; c = e % BK; }
        const int gr = r0 + r, gc = kcur + c;
        const bool ok = gr < m && gc < kk;
        const double* src = v.a_trans ? Ap + (int64_t)(ok ? gc : 0) * m + (ok ? gr : 0)
                                      : Ap + (int64_t)(ok ? gr : 0) * kk + (ok ? gc : 0);
        cp_async8(&s.a[r][c], src, ok);
      }
#pragma unroll
      for (int e = tid; e < BK * BN; e += 128) {
        int r, c;
        if (v.b_trans) { c = e / BK; r = e % BK; } else { r = e / BN; c = e % BN; }
        const int gr = kcur + r, gc = c0 + c;
        const bool ok = gr < kk && gc < n;
        const double* src = v.b_trans ? Bp + (int64_t)(ok ? gc : 0) * kk + (ok ? gr : 0)
                                      : Bp + (int64_t)(ok ? gr : 0) * n + (ok ? gc : 0);
        cp_async8(&s.b[r][c], src, ok);
      }
      cp_commit();
    };
    auto next_chunk = [&]() -> bool {
      kcur += BK;
      if (kcur < kk) return true;
      ++p;
      return advance_pair();
    };

    // 8-row / 8-column groups of this warp's 32 x 32 sub-block inside the
    // tile: DMMAs on groups wholly past the tile edge (zero-filled, never
    // stored) are skipped, as are 4-k steps past the pair's k extent.
    const int xr = max(0, min(4, (m - r0 - wm + 7) / 8));
    const int yc = max(0, min(4, (n - c0 - wn + 7) / 8));
    bool have = advance_pair();
    int buf = 0;
    if (have) load(0);
    while (have) {
      const int kv = min(BK, kk - kcur);   // valid k of the chunk in `buf`
      const bool more = next_chunk();
      if (more) load(buf ^ 1);
      if (more) cp_wait<1>(); else cp_wait<0>();
      __syncthreads();
      const Stage& s = st[buf];
#pragma unroll
      for (int k4 = 0; k4 < BK; k4 += 4) {
        if (k4 >= kv) break;
        double af[4], bf[4];
#pragma unroll
        for (int x = 0; x < 4; ++x) af[x] = s.a[wm + x * 8 + g][k4 + q];
#pragma unroll
        for (int y = 0; y < 4; ++y) bf[y] = s.b[k4 + q][wn + y * 8 + g];
#pragma unroll
        for (int x = 0; x < 4; ++x)
#pragma unroll
          for (int y = 0; y < 4; ++y)
            if (x < xr && y < yc) dmma(acc[x][y], af[x], bf[y]);
      }
      __syncthreads();
      buf ^= 1;
      have = more;
    }

    // epilogue: C block rows r0.., cols c0..
    double* C = v.C + v.coff[t] + v.hel * (int64_t)m * n;
#pragma unroll
    for (int x = 0; x < 4; ++x) {
      const int gr = r0 + wm + x * 8 + g;
      if (gr >= m) continue;
#pragma unroll
      for (int y = 0; y < 4; ++y) {
        const int gc = c0 + wn + y * 8 + q * 2;
        if (gc < n) C[(int64_t)gr * n + gc] = v.alpha * acc[x][y][0];
        if (gc + 1 < n) C[(int64_t)gr * n + gc + 1] = v.alpha * acc[x][y][1];
      }
    }
  }
}

}  // namespace

void launch_dmma_gemm(cudaStream_t s, const GemmView* views, const WorkItem* items,
                      int64_t nitems, int sm_count) {
  if (nitems <= 0) return;
  const size_t smem = 2 * sizeof(Stage);
  static int per_sm = 0;
  if (per_sm == 0) {
    cudaFuncSetAttribute(dmma_gemm_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, dmma_gemm_kernel, 128, smem);
    if (per_sm < 1) per_sm = 1;
  }
  const int64_t grid = nitems < (int64_t)sm_count * per_sm ? nitems : (int64_t)sm_count * per_sm;
  dmma_gemm_kernel<<<(unsigned)grid, 128, smem, s>>>(views, items, nitems);
  count_launch();
}

}  // namespace tagpu
