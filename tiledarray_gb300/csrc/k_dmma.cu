// Kernel (d), plain form: grouped FP64 GEMM on the DMMA tensor cores
// (mma.sync m8n8k4 f64) over the compacted tile-pair list, for sm_103a.
//
// Reference semantics (tile_op/contract_reduce.h:367-452, tensor/tensor.h:
// 3132-3210, math/blas.h:171-177): result tile (i,j) is
// sum over its pairs k of alpha * op(A(i,k)) * op(B(k,j)), the first pair
// writing (beta = 0).  Here one CTA owns a 64x64 block of one result tile and
// walks the pair list of that tile in ascending k, accumulating in registers,
// so the reduction order is fixed and no atomics are needed.  alpha is applied
// once in the epilogue.  Operand blocks are staged by the TMA unit
// (cp.async.bulk, one copy per block row, completion on an mbarrier, two
// stages, every wait bounded by the context's limit); uneven tile sizes need
// no padding: k past a pair's extent reads as zero in the fragments, rows and
// columns past the tile are never stored.  Transposed storage (Op::Trans) is
// folded into the loader.
#include <cuda_runtime.h>

#include "internal.h"

namespace tagpu {
namespace {

constexpr int BM = 64, BN = 64, BK = 16;
// Shared-memory rows: a window of 16 (or 64) doubles lands 16-byte aligned
// at its row start with the data 0 or 1 double in (the row's offset), so a
// row holds 18 (66) doubles, padded to 20 (68) for conflict-free fragments.
constexpr int P16 = 20, P64 = 68;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ bool mbar_try(uint32_t a, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(a), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ uint64_t globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void dmma(double (&c)[2], double a, double b) {
  asm volatile(
      "mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
      : "+d"(c[0]), "+d"(c[1])
      : "d"(a), "d"(b));
}

// A stage: the A block (64 rows x 16 k, or 16 k rows x 64 for a transposed
// tile) and the B block (16 k rows x 64 columns, or 64 columns x 16 k),
// each as rows of bulk-copied windows, with the data offset of every row.
struct Stage {
  double a[BM * P16];   // >= BK * P64
  double b[BM * P16];
  uint8_t oa[BM], ob[BM];
};
static_assert(BM * P16 >= BK * P64, "stage rows");

// One row of a block: len doubles from global address src into the shared
// row dst (16-byte aligned).  The bulk copy (TMA, cp.async.bulk) moves the
// 16-byte aligned span that holds the row from its first element on: it
// starts up to 8 bytes before the row (inside the same allocation, whose
// base is 16-byte aligned) and stops at the last 16-byte boundary inside
// it; a last element beyond that boundary is copied with a plain load.
// Returns the bytes the bulk copy brings; *off = the row's data offset.
__device__ __forceinline__ uint32_t copy_row(double* dst, const double* src, int len,
                                             uint32_t bar, uint8_t* off) {
  const uintptr_t a = (uintptr_t)src;
  const uintptr_t ws = a & ~(uintptr_t)15, we = (a + (uintptr_t)len * 8) & ~(uintptr_t)15;
  const int o = (int)((a - ws) >> 3);
  *off = (uint8_t)o;
  uint32_t bytes = 0;
  if (we > ws) {
    bytes = (uint32_t)(we - ws);
    asm volatile("mbarrier.expect_tx.relaxed.cta.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(bytes)
                 : "memory");
    asm volatile(
        "cp.async.bulk.shared::cta.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        ::"r"(smem_u32(dst)), "l"((const void*)ws), "r"(bytes), "r"(bar)
        : "memory");
  }
  if ((a + (uintptr_t)len * 8) > we) dst[o + len - 1] = src[len - 1];   // the tail element
  return bytes;
}

__global__ void __launch_bounds__(128, 4) dmma_gemm_kernel(const GemmView* __restrict__ views,
                                                        const WorkItem* __restrict__ items,
                                                        int64_t nitems, int* __restrict__ err,
                                                        unsigned long long wait_ns) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Stage* st = reinterpret_cast<Stage*>(smem_raw);
  __shared__ __align__(8) uint64_t full[2];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  const int g = lane >> 2, q = lane & 3;
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&full[0])), "r"(128));
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&full[1])), "r"(128));
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // rows never copied keep offset 0, so every fragment index stays in its array
  if (tid < BM) st[0].oa[tid] = st[0].ob[tid] = st[1].oa[tid] = st[1].ob[tid] = 0;
  __syncthreads();
  uint32_t phase = 0;   // bit b: parity of stage b's next completion
  uint32_t pend = 0;    // bit b: stage b has a load in flight
  bool ok = true;

  for (int64_t it = blockIdx.x; it < nitems && ok; it += gridDim.x) {
    const WorkItem w = items[it];
    const GemmView& v = views[w.view];
    const int64_t t = w.tile;
    const int rb = w.rb, cb = w.cb;
    const int64_t i = t / v.Nt, j = t - (t / v.Nt) * v.Nt;
    const int m = v.msz[i], n = v.nsz[j];
    const int r0 = rb * BM, c0 = cb * BN;
    const int mv = min(BM, m - r0), nv = min(BN, n - c0);   // valid rows / columns
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
    // The rows of the chunk at kcur into stage buf: thread tid < 64 copies
    // row tid of a 64-row block, tid 64..79 row tid-64 of a 16-row block
    // (A's rows, then B's, as the layouts ask); every thread arrives.
    auto load = [&](int buf) {
      Stage& s = st[buf];
      const uint32_t bar = smem_u32(&full[buf]);
      const int kv = min(BK, kk - kcur);
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      if (tid < 64) {
        if (!v.a_trans) {   // A rows r0+tid, k kcur..: 64 rows of kv
          if (tid < mv) copy_row(&s.a[tid * P16], Ap + (int64_t)(r0 + tid) * kk + kcur, kv, bar, &s.oa[tid]);
        } else if (tid < BK) {   // A stored k x m: k row kcur+tid, columns r0..
          if (tid < kv) copy_row(&s.a[tid * P64], Ap + (int64_t)(kcur + tid) * m + r0, mv, bar, &s.oa[tid]);
        }
      } else if (tid < 64 + BM) {
        const int r = tid - 64;
        if (!v.b_trans) {   // B k rows kcur+r, columns c0..
          if (r < kv) copy_row(&s.b[r * P64], Bp + (int64_t)(kcur + r) * n + c0, nv, bar, &s.ob[r]);
        } else {            // B stored n x k: column c0+r, k kcur..
          if (r < nv) copy_row(&s.b[r * P16], Bp + (int64_t)(c0 + r) * kk + kcur, kv, bar, &s.ob[r]);
        }
      }
      asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
      pend |= 1u << buf;
    };
    auto next_chunk = [&]() -> bool {
      kcur += BK;
      if (kcur < kk) return true;
      ++p;
      return advance_pair();
    };

    // 8-row / 8-column groups of this warp's 32 x 32 sub-block inside the
    // tile: DMMAs on groups wholly past the tile edge (never stored) are
    // skipped, as are 4-k steps past the pair's k extent; k past it inside
    // a step read as zero.
    const int xr = max(0, min(4, (m - r0 - wm + 7) / 8));
    const int yc = max(0, min(4, (n - c0 - wn + 7) / 8));
    bool have = advance_pair();
    int buf = 0;
    if (have) load(0);
    while (have) {
      const int kv = min(BK, kk - kcur);   // valid k of the chunk in `buf`
      const bool more = next_chunk();
      if (more) load(buf ^ 1);
      // bounded wait for the chunk in `buf`
      {
        const uint32_t bar = smem_u32(&full[buf]), par = (phase >> buf) & 1u;
        if (!mbar_try(bar, par)) {
          const uint64_t t0 = globaltimer();
          while (!mbar_try(bar, par)) {
            if (globaltimer() - t0 > wait_ns) {
              atomicCAS(err, 0, 1);
              ok = false;
              break;
            }
          }
        }
        if (ok) {
          phase ^= 1u << buf;
          pend &= ~(1u << buf);
        }
      }
      if (__syncthreads_or(!ok)) {
        ok = false;
        break;
      }
      const Stage& s = st[buf];
      // fragment rows of the untransposed layouts: offsets read once per stage
      int abase[4], bbase[4];
#pragma unroll
      for (int x = 0; x < 4; ++x) {
        const int r = wm + x * 8 + g, c = wn + x * 8 + g;
        abase[x] = v.a_trans ? r : r * P16 + s.oa[r];
        bbase[x] = v.b_trans ? c * P16 + s.ob[c] : c;
      }
#pragma unroll
      for (int k4 = 0; k4 < BK; k4 += 4) {
        if (k4 >= kv) break;
        const int kq = k4 + q;
        const bool kin = kq < kv;
        const int ka = v.a_trans ? kq * P64 + s.oa[kq] : kq;
        const int kb = v.b_trans ? kq : kq * P64 + s.ob[kq];
        double af[4], bf[4];
#pragma unroll
        for (int x = 0; x < 4; ++x) af[x] = kin ? s.a[abase[x] + ka] : 0.0;
#pragma unroll
        for (int y = 0; y < 4; ++y) bf[y] = kin ? s.b[bbase[y] + kb] : 0.0;
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
    if (!ok) break;

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
  // copies of an aborted block land before the CTA exits (bounded)
  if (!ok) {
    const uint64_t t0 = globaltimer();
    for (int b = 0; b < 2; ++b)
      if ((pend >> b) & 1u)
        while (!mbar_try(smem_u32(&full[b]), (phase >> b) & 1u) &&
               globaltimer() - t0 < 4000000000ull) {
        }
  }
}

}  // namespace

void launch_dmma_gemm(cudaStream_t s, const GemmView* views, const WorkItem* items,
                      int64_t nitems, int* err, unsigned long long wait_ns, int sm_count) {
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
  dmma_gemm_kernel<<<(unsigned)grid, 128, smem, s>>>(views, items, nitems, err, wait_ns);
  count_launch();
}

}  // namespace tagpu
