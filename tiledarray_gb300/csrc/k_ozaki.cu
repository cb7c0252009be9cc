// Kernel (d), emulated-FP64 form: Ozaki-style split-integer slices on the
// tcgen05 tensor cores of sm_103a.
//
// What is computed: the same per-result-tile reduction as the plain DMMA
// kernel, C(i,j) = alpha * sum_k A(i,k) B(k,j) over the tile-pair list, with
// an error against FP64 of order 2^-(8S-1) relative per product (S = 7 by
// default: every result tile within about 2e-14 of the FP64 oracle).
//
// How:
//  * frames: every fused row r of A gets E_A[r] with |A[r,:]| < 2^E_A[r], every
//    fused column c of B gets E_B[c] (one pass over the operands, integer ops
//    on the IEEE bit fields);
//  * splitting (integer only): operands are cut into "bricks" (128 rows x 32 k
//    of A, 64 columns x 32 k of B, in global fused coordinates).  A brick's
//    deficit e is the smallest number of bits by which a nonzero element sits
//    below its row (column) frame; with m = floor(e / 8) whole digits, every
//    element a = x * 2^-(E-8m) rounded to 8S-1 fractional bits is cut into S
//    balanced base-256 digits d_1..d_S, |d_p| <= 128 (exact in bf16), a =
//    sum_p d_p 2^(1-8p), written as the K-major no-swizzle UMMA operand image
//    so that one bulk copy moves a brick into shared memory;
//  * products: slice pair (p, q) of a stage whose bricks have shifts mA, mB
//    lands on level t = p + q + mA + mB - M (M the output block's base), with
//    tcgen05.mma.kind::f16 (bf16 x bf16 -> fp32, M = 128, K = 16) into the
//    tensor-memory columns of level t (levels 2..TOP adjacent, 64 columns
//    each, TOP = min(S + 3, 9)); compile-time stage programs group the
//    products of one A slice into MMAs of several levels' width.  Levels
//    2..5 restart every 32, 16, 8, 8 stages and stay exact in fp32; levels
//    6..TOP sum over the whole block (the level comment below says why);
//  * draining: when a level's period ends the epilogue warps read it,
//    release it to the MMA warp at once through a per-level mbarrier (the
//    MMAs of the slices that do not touch it never wait), and fold it into
//    two int64 accumulators per element: hi (units of level 5) takes the
//    exact levels L_t * 2^(8(5-t)), lo (units of level TOP) the whole-block
//    levels L_t * 2^(8(TOP-t));
//  * recombination: at the end of an output block
//    C = alpha * 2^(E_A + E_B - 8M) * (hi * 2^(8(TOP-5)) + lo) * 2^(2-8 TOP),
//    the exact integer rounded once to double (exact_to_double), written
//    into the result tiles the block overlaps while the MMA warp already
//    runs the next block.
// Work is in global fused coordinates (output blocks 128 x 64, k blocks of
// 32), so uneven tiles cost no padding except at block-sparsity boundaries;
// a brick is stored only if some nonzero tile overlaps it, a k block is run
// for an output block only if both bricks exist.  Contributions of absent
// pairs are exact zeros, and output elements of zero result tiles are never
// written, so the result equals the tile-pair-list reduction.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <string>
#include <type_traits>
#include <vector>

#include "internal.h"

namespace tagpu {
namespace {

constexpr int BM = 128;            // output block rows (MMA M)
constexpr int BN = 64;             // output block columns (MMA N)
constexpr int BK = 32;             // k per stage (two MMA K = 16 steps)
// Level t collects t-1 digit products |d e| <= 2^14 per k.  Levels up to
// kExactTop are kept exact: level t restarts from zero every drain_period(t)
// stages (32 k each), the largest power of two <= 32 / (t-1) (32, 16, 8, 8
// for t = 2..5), so it never exceeds (t-1) * 32 * drain_period(t) * 2^14
// <= 2^24, where every fp32 sum of integers is exact.  Powers of two make
// the restarts of different levels fall on the same stages (every 8th), so
// the MMA warp waits for the epilogue at one stage in 8.  Levels above
// kExactTop (weight 2^-32 and below against level 2) accumulate over the
// whole output block in fp32 and are read once; their rounding stays below
// 2^-41 of sum_k |a_ik b_kj| per element, under FP64 GEMM's own worst-case
// bound.  The schedule is a fixed function of the stage index, so results do
// not depend on block order or row chunking.
constexpr int kExactTop = 5;
__host__ __device__ constexpr int drain_period(int t) {
  return t <= 2 ? 32 : t == 3 ? 16 : t <= 5 ? 8 : t <= 9 ? 4 : t <= 17 ? 2 : 1;
}
// Bit t set: level t (2..TOP) starts from zero at stage x of an output block.
template <int TOP>
__device__ __forceinline__ uint32_t restart_mask(int64_t x) {
  if (x == 0) return ((1u << (TOP + 1)) - 1u) & ~3u;
  uint32_t m = 0;
#pragma unroll
  for (int t = 2; t <= (TOP < kExactTop ? TOP : kExactTop); ++t)
    if (x % drain_period(t) == 0) m |= 1u << t;
  return m;
}
// Levels read by the epilogue after stage x of an n-stage block.
template <int TOP>
__device__ __forceinline__ uint32_t drain_mask(int64_t x, int64_t n) {
  return x + 1 == n ? restart_mask<TOP>(0) : restart_mask<TOP>(x + 1);
}
constexpr int A_SLICE_BYTES = BM * BK * 2;   // 8 KB
constexpr int B_SLICE_BYTES = BN * BK * 2;   // 4 KB
// Epilogue warps: EW of them, four per 32-lane quarter of tensor memory,
// each owning kCols of the block's 64 columns, and results staged kPass
// columns at a time (row stride kPass + 1 doubles: the row-per-lane writes
// hit distinct bank pairs per half warp).  Eight warps of 32 columns keep
// 168 registers a thread for the MMA issue of long-k blocks; sixteen warps
// of 16 columns (96 registers: five warps share a scheduler's register file)
// hold half the accumulators per thread and hide twice the conversion
// latency, which pays where blocks are short and the epilogue bounds the
// kernel.
template <int EW>
struct Epi {
  static_assert(EW == 8 || EW == 16, "eight or sixteen epilogue warps");
  static constexpr int kCols = BN * 4 / EW;            // 32 or 16
  static constexpr int kThreads = 64 + EW * 32;        // producer, MMA, epilogue warps
  static constexpr int kPass = EW == 8 ? 16 : 8;
  static constexpr int kLd = kPass + 1;
  static constexpr int kBytes = EW * 32 * kLd * 8;     // 34,816 or 36,864
};
// Launches whose units average at most this many 32-k stages take sixteen
// epilogue warps.
constexpr int64_t kShortStages = 128;
// Bound of the waits that let in-flight copies and MMAs finish before a CTA
// exits (they end within microseconds; the bound only keeps a broken launch
// from spinning forever).  The pipeline waits take their bound from the
// launch (wait_ns, host-settable, 4 s by default).
constexpr unsigned long long WAIT_NS = 4000000000ull;
// Brick shift of a brick with no nonzero element, and sum of shifts of a
// stage without products (a column block past its last B brick).
constexpr int32_t kNoShift = 1 << 20;

// ---------------------------------------------------------------------------
// PTX wrappers
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ uint64_t globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint32_t a, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(a), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t a, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(a), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t a) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(a) : "memory");
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
// Bounded wait: false after wait_ns or when another role has aborted.  The
// timer is read after the first failed try and then every 64 tries.
__device__ __forceinline__ bool mbar_wait(uint32_t a, uint32_t parity, volatile int* abort_s,
                                          unsigned long long wait_ns) {
  if (mbar_try(a, parity)) return true;
  const uint64_t t0 = globaltimer();
  for (uint32_t i = 0;; ++i) {
    if (mbar_try(a, parity)) return true;
    if ((i & 63) == 0) {
      if (*abort_s) return false;
      if (globaltimer() - t0 > wait_ns) return false;
    }
  }
}
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes,
                                         uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
      ::"r"(dst), "l"(src), "r"(bytes), "r"(mbar)
      : "memory");
}
// The same copy into the same shared-memory offset of every CTA of the
// cluster in `mask`; each destination's mbarrier (same offset) gets the bytes.
__device__ __forceinline__ void bulk_g2s_mc(uint32_t dst, const void* src, uint32_t bytes,
                                            uint32_t mbar, uint16_t mask) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.multicast::cluster"
      " [%0], [%1], %2, [%3], %4;"
      ::"r"(dst), "l"(src), "r"(bytes), "r"(mbar), "h"(mask)
      : "memory");
}
__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}
__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release.aligned;\n"
               "barrier.cluster.wait.acquire.aligned;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// Arrive on the mbarrier at this offset in every CTA of `mask` once the
// MMAs issued so far have completed.
__device__ __forceinline__ void tc_commit_mc(uint32_t mbar, uint16_t mask) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64"
      " [%0], %1;" ::"r"(mbar), "h"(mask)
      : "memory");
}
__device__ __forceinline__ void tc_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
               ::"r"(mbar)
               : "memory");
}
__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc,
                                       uint32_t idesc, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n"
      ::"r"(d_tmem), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void tmem_wait_ld() {
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// K-major, no-swizzle operand image: core matrices of 8 rows x 16 bytes,
// LBO = 128 B between the K-adjacent core matrices, SBO = 512 B between
// 8-row groups (a 32-k brick row group holds 4 core matrices).
__host__ __device__ inline uint32_t brick_offset(int row, int k) {
  return (uint32_t)((row >> 3) * 512 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}
__device__ __forceinline__ uint64_t make_desc(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)(128 >> 4) << 16;   // leading byte offset (K direction)
  d |= (uint64_t)(512 >> 4) << 32;   // stride byte offset (M/N direction)
  d |= (uint64_t)1 << 46;            // descriptor version for tcgen05
  return d;                          // base offset 0, layout SWIZZLE_NONE
}
// kind::f16 instruction descriptor: D f32, A/B bf16, K-major, M=128, N=n
// (n a multiple of 16, at most 256).
__host__ __device__ constexpr uint32_t idesc_n(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(BM >> 4) << 24);
}

// f * 2^sh as an exact int64, for an integer-valued float f with
// |f| * 2^sh < 2^62, from the float's bits (mantissa shifted by its
// exponent; zero shifts by at least 118 places down, clamped to 31).  The
// 16-warp epilogue uses it instead of a conversion instruction, which runs
// on this GPU's narrow FP64 pipe with a long latency; the 8-warp epilogue,
// short of issue slots rather than latency, keeps the instruction.
__device__ __forceinline__ int64_t float_to_ll_exact(float f, int sh) {
  const uint32_t b = __float_as_uint(f);
  const int e = (int)((b >> 23) & 0xff) - 150 + sh;
  const uint32_t m = (b & 0x7fffffu) | 0x800000u;
  const int64_t v = e >= 0 ? (int64_t)((uint64_t)m << e) : (int64_t)(m >> min(-e, 31));
  return (int)b < 0 ? -v : v;
}

// Correctly rounded double of (hi * 2^SH + lo) * 2^e2 from exact integers
// (|hi| < 2^61, |lo| < 2^62, 0 <= SH <= 32).  The value is first cut to a
// signed 64-bit window with the bits cut off ORed into its lowest bit
// (rounding to odd, which a later rounding to 53 bits turns into the correct
// rounding of the exact value, as the window keeps at least 55 bits); one
// conversion instruction then rounds the window to nearest even and an
// integer add on the exponent field scales it.  Rounding to odd needs no
// separate magnitude: in two's complement, truncating toward minus infinity
// and setting the lowest bit when anything was cut picks the odd neighbour
// for either sign.  The rare results outside the normal range take the FP64
// library route.
template <int SH>
__device__ __forceinline__ double exact_to_double(int64_t hi, int64_t lo, int e2) {
  static_assert(SH >= 0 && SH <= 32, "shift between the accumulators");
  int64_t y;
  int scale = e2;
  if constexpr (SH == 0) {
    y = hi + lo;
  } else {
    // W = H * 2^SH + r with 0 <= r < 2^SH
    const int64_t H = hi + (lo >> SH);
    const uint32_t r = SH == 32 ? (uint32_t)lo : ((uint32_t)lo & ((1u << (SH & 31)) - 1u));
    const int s = __clzll((long long)(H ^ (H >> 63))) - 1;   // redundant sign bits of H
    if (s >= SH) {   // W fits in 64 bits
      y = (int64_t)(((uint64_t)H << SH) | r);
    } else {
      const int d = SH - s;   // bits of r below the window, 1..SH
      y = (int64_t)(((uint64_t)H << s) | ((uint64_t)r >> d) | ((uint32_t)(r << (32 - d)) != 0u ? 1u : 0u));
      scale += d;
    }
  }
  if (y == 0) return 0.0;
  const double w = __ll2double_rn((long long)y);
  const long long bits = __double_as_longlong(w);
  const int ex = (int)((bits >> 52) & 0x7ff) + scale;
  if (ex < 1 || ex > 2046) return ldexp(w, scale);
  return __longlong_as_double(bits + ((long long)scale << 52));
}


struct OzParams {
  const uint8_t* Apack;      // A bricks, S * 8 KB each
  int64_t a_slot_base;       // first A brick slot held in Apack (row chunking)
  const uint8_t* Bpack;      // B bricks, S * 4 KB each
  const int32_t* brickA;     // RB x KBn -> slot or -1
  const int32_t* brickB;     // KBn x CB -> slot or -1
  const int32_t* blk;        // nblk x 2 (rb, cb), in scheduling order
  const int64_t* blk_rng;    // nblk x 2: [begin, end) of the block's k blocks in blk_kb
  int4* blk_ab;              // per k block of a unit: A slot, B slots of its two column
                             // blocks (the zero brick where absent), and the stage's
                             // digit shifts (shift_kernel, every run): bits 0-7 the
                             // shift of column block 0, 8-15 of column block 1, bit 16
                             // set when neither CTA has a product (stage not loaded)
  const int32_t* shiftA;     // per A brick slot: its deficit in bits, the least by which
                             // its elements sit below their row frames (kNoShift: all zero)
  const int32_t* shiftB;     // per B brick slot, likewise (slot of the zero brick: kNoShift)
  int32_t* unitM;            // per unit and column block: level base M | extra levels << 28
                             // (shift_kernel)
  unsigned long long* products;  // digit-slice products issued (128 x 64 x 32 each)
  int64_t nblk;
  int KBn, CB;
  const int32_t* EA;         // M_total frames (biased exponent; E = EA - 1022)
  const int32_t* EB;         // N_total frames
  const int32_t* row_tile;   // M_total
  const int32_t* row_local;
  const int32_t* col_tile;   // N_total
  const int32_t* col_local;
  const int32_t* msz;
  const int32_t* nsz;
  int64_t Nt;
  const int64_t* coff;       // Mt*Nt result tile offsets
  int64_t hel;               // fused element: its m x n matrix starts hel * m * n into a tile
  double alpha;
  double* C;
  int64_t M_total, N_total;
  int* err;                  // error flag (0 = ok)
};

template <int S, int EW>
struct Smem {
  static constexpr int kStages = (S * (A_SLICE_BYTES + B_SLICE_BYTES) * 3 <= 200 * 1024) ? 3 : 2;
  static constexpr int kStageBytes = S * (A_SLICE_BYTES + B_SLICE_BYTES);
  static constexpr int kBytes = kStages * kStageBytes + Epi<EW>::kBytes + 1024;
};

// ---------------------------------------------------------------------------
// Served mode: a persistent GEMM that takes units from a work queue
// ---------------------------------------------------------------------------
// The host publishes jobs (one contraction plan each, already split into
// digit bricks) into two lanes, 0 for short jobs and 1 for long ones.  The
// lane's units are numbered in publication order; a cluster's leader (rank
// 0 producer) claims the next unit of lane 0 if there is one, else of lane
// 1, so a short job published while a long one runs starts on the next
// cluster that finishes a unit.  Control words the host writes live in mapped
// host memory; claim counters and per-job unit counts in device memory.
constexpr int kQueueJobs = 1 << 16;   // jobs per lane between two resets
struct QueueJob {
  const void* view;          // the job's OzParams on the device
  int64_t first;             // number of its first unit in its lane
  int64_t units;             // units (pairs of output blocks)
  int32_t id;                // completion slot
  int32_t pad;
};
struct QueueArgs {
  const QueueJob* jobs[2];           // per lane, publication order (mapped)
  const volatile long long* published;   // [2] units published per lane (mapped)
  const volatile int* njobs;         // [2] jobs published per lane (mapped)
  const volatile int* stop;          // exit once nothing is left to claim (mapped)
  volatile int* job_done;            // [2 * kQueueJobs] 1 once a job finished (mapped)
  unsigned long long* claimed;       // [2] units claimed per lane (device)
  int* done_units;                   // [2 * kQueueJobs] CTA-units finished per job (device)
  unsigned long long idle_ns;        // exit after this long with nothing to claim
};
// A unit as the roles of a CTA see it; b < 0 ends the kernel.
struct QUnit {
  const OzParams* P;
  long long b;
  long long tag;             // job id | units << 20 (units < 2^43)
};

__device__ __forceinline__ long long ld_acquire_sys(const volatile long long* p) {
  long long v;
  asm volatile("ld.acquire.sys.global.s64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ int ld_acquire_sys(const volatile int* p) {
  int v;
  asm volatile("ld.acquire.sys.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
// Address of the same shared-memory location in CTA `rank` of the cluster.
__device__ __forceinline__ uint32_t mapa(uint32_t addr, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(addr), "r"(rank));
  return r;
}
__device__ __forceinline__ void st_cluster_u64(uint32_t addr, unsigned long long v) {
  asm volatile("st.shared::cluster.u64 [%0], %1;" ::"r"(addr), "l"(v) : "memory");
}
__device__ __forceinline__ void mbar_arrive_cluster(uint32_t addr) {
  asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(addr)
               : "memory");
}
// Bounded wait with cluster-scope acquire (the slot may have been written by
// the partner CTA).
__device__ __forceinline__ bool mbar_wait_cluster(uint32_t a, uint32_t parity,
                                                  volatile int* abort_s,
                                                  unsigned long long wait_ns) {
  auto try1 = [&]() {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    return ok != 0;
  };
  if (try1()) return true;
  const uint64_t t0 = globaltimer();
  for (uint32_t i = 0;; ++i) {
    if (try1()) return true;
    if ((i & 63) == 0) {
      if (*abort_s) return false;
      if (globaltimer() - t0 > wait_ns) return false;
    }
  }
}
// Claims the next unit (lane 0 before lane 1); false when there is none and
// the host asked to stop, the kernel has been idle for idle_ns, or a role
// aborted.  cache[l]: index of the lane's job the last claim fell into.
__device__ bool queue_claim(const QueueArgs& q, QUnit& u, int* cache, volatile int* abort_s) {
  const uint64_t t0 = globaltimer();
  for (;;) {
#pragma unroll
    for (int l = 0; l < 2; ++l) {
      const long long pub = ld_acquire_sys(&q.published[l]);
      unsigned long long c = *(volatile unsigned long long*)&q.claimed[l];
      while ((long long)c < pub) {
        const unsigned long long prev = atomicCAS(&q.claimed[l], c, c + 1);
        if (prev == c) {
          // the job holding unit c: jobs are published before their units
          const int nj = ld_acquire_sys(&q.njobs[l]);
          int j = cache[l] < nj ? cache[l] : nj - 1;
          while (j + 1 < nj && q.jobs[l][j + 1].first <= (long long)c) ++j;
          while (j > 0 && q.jobs[l][j].first > (long long)c) --j;
          cache[l] = j;
          const QueueJob& J = q.jobs[l][j];
          u.P = static_cast<const OzParams*>(J.view);
          u.b = (long long)c - J.first;
          u.tag = (long long)J.id | (J.units << 20);
          return true;
        }
        c = prev;
      }
    }
    if (*abort_s || ld_acquire_sys(q.stop)) return false;
    if (globaltimer() - t0 > q.idle_ns) return false;
    __nanosleep(500);
  }
}

// Output blocks of several contractions form one list: block gb belongs to
// view v with vstart[v] <= gb < vstart[v+1].
__device__ __forceinline__ int find_view(const int64_t* __restrict__ vstart, int nviews,
                                         int64_t gb) {
  int lo = 0, hi = nviews;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (vstart[mid] <= gb) lo = mid; else hi = mid;
  }
  return lo;
}

// MMAs of one stage with shift SH and last level L known at compile time:
// slice p feeds levels p+1+SH .. p+SH+min(L-p-SH, S) with B slices 1..,
// one MMA (two above N = 256) per slice and k step, every descriptor a
// constant offset from the stage's (descriptor address fields count 16-byte
// units).  Slices p0..p1 of k step ks, all with accumulate on.
template <int S, int SH, int L>
__device__ __forceinline__ void slices_full(uint32_t tmem, uint64_t ad0, uint64_t bd0, int ks,
                                            int p0, int p1) {
#pragma unroll
  for (int p = 1; p <= S; ++p) {
    const int nl = L - p - SH < S ? L - p - SH : S;
    if (nl > 0 && p >= p0 && p <= p1) {
      const uint64_t ad = ad0 + (uint64_t)((((p - 1) * A_SLICE_BYTES) >> 4) + ks * 16);
      const uint64_t bd = bd0 + (uint64_t)(ks * 16);
      const uint32_t d = tmem + (p - 1 + SH) * BN;
      const int nn = nl * BN;
      if (nn <= 256) {
        tc_mma(d, ad, bd, idesc_n(nn), 1u);
      } else {
        const int h = nn / 2;
        tc_mma(d, ad, bd, idesc_n(h), 1u);
        tc_mma(d + h, ad, bd + (uint64_t)(((h / 8) * 512) >> 4), idesc_n(h), 1u);
      }
    }
  }
}
// Levels lo..hi of slice p, k step ks (B slices from lo - p - SH).
template <int S, int SH>
__device__ __forceinline__ void slice_run(uint32_t tmem, uint64_t ad0, uint64_t bd0, int p, int ks,
                                          int lo, int hi, uint32_t acc) {
  if (hi < lo) return;
  const uint64_t ad = ad0 + (uint64_t)((((p - 1) * A_SLICE_BYTES) >> 4) + ks * 16);
  const uint64_t bd = bd0 + (uint64_t)((((lo - 1 - p - SH) * B_SLICE_BYTES) >> 4) + ks * 16);
  const uint32_t d = tmem + (lo - 2) * BN;
  const int nn = (hi - lo + 1) * BN;
  if (nn <= 256) {
    tc_mma(d, ad, bd, idesc_n(nn), acc);
  } else {
    const int h = nn / 2;
    tc_mma(d, ad, bd, idesc_n(h), acc);
    tc_mma(d + h, ad, bd + (uint64_t)(((h / 8) * 512) >> 4), idesc_n(h), acc);
  }
}
// The three stage programs, for a stage with no fresh level among its own:
//   kStageAll:     every slice (k step 0, then 1);
//   kStageRestartA: at a stage restarting levels zlo..5, every product on a
//                  level above 5 (each slice's run from level 6 up), issued
//                  before the wait: about two thirds of the stage's work
//                  covers the epilogue's reads of the restarting levels;
//   kStageRestartC: the rest once levels zlo..5 are free and marked fresh:
//                  slice 1's k step 0 in two runs, the restarting run
//                  [max(zlo, 2+SH), 5] with accumulate off, then the other
//                  slices' runs up to level 5.
enum { kStageAll = 0, kStageRestartA = 1, kStageRestartC = 2 };
template <int S, int SH, int L, int KIND>
__device__ __forceinline__ void stage_program(uint32_t tmem, uint64_t ad0, uint64_t bd0, int zlo) {
  if constexpr (KIND == kStageAll) {
    slices_full<S, SH, L>(tmem, ad0, bd0, 0, 1, S);
    slices_full<S, SH, L>(tmem, ad0, bd0, 1, 1, S);
  } else if constexpr (KIND == kStageRestartA) {
#pragma unroll
    for (int ks = 0; ks < 2; ++ks)
#pragma unroll
      for (int p = 1; p <= S; ++p) {
        const int top = p + SH + (L - p - SH < S ? L - p - SH : S);
        const int lo = p + 1 + SH > 6 ? p + 1 + SH : 6;
        slice_run<S, SH>(tmem, ad0, bd0, p, ks, lo, top, 1u);
      }
  } else {
    if constexpr (SH <= 3) {   // slice 1 starts at level 2 + SH <= 5
      const int lo = 2 + SH, top1 = (L < 1 + SH + S) ? L : 1 + SH + S;
      const int hi = top1 < 5 ? top1 : 5;
      const int f0 = zlo > lo ? zlo : lo;
      slice_run<S, SH>(tmem, ad0, bd0, 1, 0, lo, f0 - 1, 1u);
      slice_run<S, SH>(tmem, ad0, bd0, 1, 0, f0, hi, 0u);
#pragma unroll
      for (int ks = 0; ks < 2; ++ks)
#pragma unroll
        for (int p = 1 + (1 - ks); p <= 4 - SH; ++p) {
          const int top = p + SH + (L - p - SH < S ? L - p - SH : S);
          slice_run<S, SH>(tmem, ad0, bd0, p, ks, p + 1 + SH, top < 5 ? top : 5, 1u);
        }
    }
  }
}
// Selects the instance for a stage's shift s (0..S+1) and extra levels e.
template <int S, int SH, int KIND>
__device__ __forceinline__ void stage_dispatch(int s, int e, uint32_t tmem, uint64_t ad0,
                                               uint64_t bd0, int zlo) {
  if constexpr (SH <= S + 1) {
    if (s == SH) {
      if (e == 0) {
        stage_program<S, SH, S + 1, KIND>(tmem, ad0, bd0, zlo);
      } else if (e == 1) {
        if constexpr (S + 2 <= 9) stage_program<S, SH, S + 2, KIND>(tmem, ad0, bd0, zlo);
      } else {
        if constexpr (S + 3 <= 9) stage_program<S, SH, S + 3, KIND>(tmem, ad0, bd0, zlo);
      }
    } else {
      stage_dispatch<S, SH + 1, KIND>(s, e, tmem, ad0, bd0, zlo);
    }
  }
}

// Digit shifts.  A brick's digits are cut relative to its rows' frames lowered
// by 8 m bits: e, the brick's deficit, is the smallest number of bits by
// which an element sits below its row frame, and m = floor(e / 8) whole
// digits (split_kernel).  Operands that decay along k so keep all 8S-1 bits
// in every brick instead of losing the bits between the brick and its row
// maximum.  Product (p, q) of a stage whose bricks have mA and mB then has
// weight 2^(2 - 8(p + q + mA + mB)) against the row and column frames.
// An output block counts its levels from its base M = the smallest mA + mB
// over its stages: product (p, q) of a stage with s = mA + mB - M lands on
// level p + q + s.  Since mA + mB floors each deficit separately, the
// block's largest contributions (deficit min(eA + eB) bits) may lie up to
// u = min(eA + eB) - 8M < 15 bits below the base, so the block keeps
// E = (u + 3) / 8 extra levels: pairs with p + q + s <= S + 1 + E are kept,
// which puts the truncation at least 8S + 4 bits below the block's own
// magnitude, as without shifts.  A stage with s >= S + E has no product
// left; a stage that neither CTA of the cluster needs is not loaded at all.
//
// Lazy zeroing: a level restarts by being marked fresh; the first MMA that
// writes a fresh level does so with accumulate off.  A level still fresh at a
// drain got no product in its period, and the epilogue skips it.
template <int S, bool Q, int EW>
__global__ void __cluster_dims__(2, 1, 1) __launch_bounds__(Epi<EW>::kThreads, 1) ozaki_gemm_kernel(
    const OzParams* __restrict__ views, const int64_t* __restrict__ vstart, int nviews,
    int64_t nblk_total, int* __restrict__ err, unsigned long long wait_ns,
    const QueueArgs* __restrict__ qa) {
  constexpr int STAGES = Smem<S, EW>::kStages;
  constexpr int STAGE_BYTES = Smem<S, EW>::kStageBytes;
  constexpr int EPI_WARPS = EW;
  constexpr int EPI_COLS = Epi<EW>::kCols;
  constexpr int EPI_PASS = Epi<EW>::kPass;
  constexpr int EPI_LD = Epi<EW>::kLd;
  // levels 2..TOP are MMA targets: S + 1 of them and up to two extra, as
  // many as the 512 tensor-memory columns hold (one extra for S = 7)
  constexpr int TOP = S + 3 < 9 ? S + 3 : 9;
  static_assert((TOP - 1) * BN <= 512, "levels exceed tensor memory");
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ __align__(8) uint64_t bar_full[STAGES], bar_empty[STAGES];
  __shared__ __align__(8) uint64_t bar_acc_full, bar_level[TOP + 1], bar_done;
  __shared__ uint32_t tmem_base_s;
  __shared__ uint32_t fresh_ring[4];   // per drain: levels that got no product
  __shared__ volatile int abort_s;
  // served mode: units handed from the cluster leader to the roles of both CTAs
  __shared__ __align__(8) QUnit q_ring[4];
  __shared__ __align__(8) uint64_t q_full[4], q_empty[4], epi_done;

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint8_t* stage_base = (uint8_t*)(((uintptr_t)smem + 1023) & ~(uintptr_t)1023);
  // The two CTAs of a cluster run the two output blocks of a unit: rank r
  // owns column block 2c + r; each loads half of the shared A brick into both.
  const uint32_t rank = cluster_rank();
  const int64_t unit0 = blockIdx.x >> 1, unit_step = gridDim.x >> 1;

  if (threadIdx.x == 0) {
    for (int s = 0; s < STAGES; ++s) {
      mbar_init(smem_u32(&bar_full[s]), 1);
      mbar_init(smem_u32(&bar_empty[s]), 2);   // both CTAs' MMAs have read the stage
    }
    // a drain is ready once the MMAs before it completed (commit) and the MMA
    // warp has published the drain's fresh levels (arrive)
    mbar_init(smem_u32(&bar_acc_full), 2);
    for (int t = 0; t <= TOP; ++t) mbar_init(smem_u32(&bar_level[t]), EPI_WARPS);  // per warp
    mbar_init(smem_u32(&bar_done), 1);
    for (int i = 0; i < 4; ++i) {
      mbar_init(smem_u32(&q_full[i]), 1);
      // consumers of a slot: MMA + epilogue warps of rank 0, producer, MMA
      // and epilogue warps of rank 1 (only rank 0's barrier is used)
      mbar_init(smem_u32(&q_empty[i]), 3 + 2 * EPI_WARPS);
    }
    mbar_init(smem_u32(&epi_done), EPI_WARPS);
    abort_s = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;"
                 ::"r"(smem_u32(&tmem_base_s)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  tc_fence_before();
  __syncthreads();
  cluster_sync();   // the partner's barriers exist before any multicast or remote arrive
  tc_fence_after();
  const uint32_t tmem = tmem_base_s;
  // level t (2..TOP) accumulates in tensor-memory columns [(t-2)*BN, (t-1)*BN)

  auto fail = [&](int code) {
    abort_s = 1;
    atomicCAS(err, 0, code);
  };
  // Served mode, a consumer warp: the next unit from the ring; lane 0 then
  // releases the slot to the cluster leader.  false ends the warp's loop.
  int qslot = 0;
  uint32_t qph = 0;
  auto ring_read = [&](int slot) {
    const volatile long long* w = reinterpret_cast<const volatile long long*>(&q_ring[slot]);
    QUnit u;
    u.P = reinterpret_cast<const OzParams*>(w[0]);
    u.b = w[1];
    u.tag = w[2];
    return u;
  };
  auto ring_take = [&](QUnit& u) -> bool {
    if (!mbar_wait_cluster(smem_u32(&q_full[qslot]), qph, &abort_s, wait_ns)) {
      fail(6);
      return false;
    }
    u = ring_read(qslot);
    __syncwarp();
    if (lane == 0) {
      const uint32_t e = smem_u32(&q_empty[qslot]);
      if (rank == 0) mbar_arrive(e); else mbar_arrive_cluster(mapa(e, 0));
    }
    if (++qslot == 4) {
      qslot = 0;
      qph ^= 1;
    }
    return u.b >= 0;
  };

  if (warp == 0) {
    // ------------------------------------------------------------ producer
    // The whole warp loads 32 (A slot, B slot, shifts) entries at a time;
    // lane 0 waits for free stages and issues the two bulk copies of each
    // stage either CTA has products for.
    int stage = 0;
    uint32_t phase = 0;
    uint32_t issued_parity[STAGES];
    bool issued[STAGES];
    for (int s = 0; s < STAGES; ++s) issued[s] = false;
    bool ok = true;
    // loads of one unit's stages
    // A stage loads the slices its products use: slice p and B slice q meet
    // on level p + q + s <= L, so a column block needs the first
    // min(S, L - 1 - s) slices of both bricks.  The A prefix is the larger of
    // the two column blocks' (both CTAs receive the multicast halves).
    int64_t gb = unit0;
    int cache[2] = {0, 0};
    for (;;) {
      // the next unit: the static stride, or (served) the cluster leader
      // claims one and hands it to both CTAs through the ring
      const OzParams* Pp = nullptr;
      int64_t b = 0;
      if constexpr (!Q) {
        if (gb >= nblk_total || !ok) break;
        const int vi = find_view(vstart, nviews, gb);
        Pp = &views[vi];
        b = gb - vstart[vi];
        gb += unit_step;
      } else if (rank == 0) {
        QUnit u;
        if (lane == 0) {
          bool got = mbar_wait(smem_u32(&q_empty[qslot]), qph ^ 1, &abort_s, wait_ns);
          if (!got) fail(7);
          got = got && queue_claim(*qa, u, cache, &abort_s);
          if (!got) {
            u.P = nullptr;
            u.b = -1;
            u.tag = 0;
          }
          const uint32_t slot = smem_u32(&q_ring[qslot]);
          const uint32_t rslot = mapa(slot, 1);
          q_ring[qslot] = u;
          st_cluster_u64(rslot, (unsigned long long)(uintptr_t)u.P);
          st_cluster_u64(rslot + 8, (unsigned long long)u.b);
          st_cluster_u64(rslot + 16, (unsigned long long)u.tag);
          mbar_arrive(smem_u32(&q_full[qslot]));
          mbar_arrive_cluster(mapa(smem_u32(&q_full[qslot]), 1));
        }
        __syncwarp();
        u = ring_read(qslot);
        if (++qslot == 4) {
          qslot = 0;
          qph ^= 1;
        }
        if (u.b < 0 || !ok) break;
        Pp = u.P;
        b = u.b;
      } else {
        QUnit u;
        if (!ok || !ring_take(u)) break;
        Pp = u.P;
        b = u.b;
      }
      const OzParams& P = *Pp;
      const int64_t x0 = P.blk_rng[2 * b], x1 = P.blk_rng[2 * b + 1];
      const int L0 = S + 1 + (int)((uint32_t)P.unitM[2 * b] >> 28);
      const int L1 = S + 1 + (int)((uint32_t)P.unitM[2 * b + 1] >> 28);
      for (int64_t xb = x0; xb < x1 && ok; xb += 32) {
        int4 mine = make_int4(0, 0, 0, 0);
        if (xb + lane < x1) mine = P.blk_ab[xb + lane];
        const int cnt = (int)(x1 - xb < 32 ? x1 - xb : 32);
        for (int j = 0; j < cnt; ++j) {
          const int sa = __shfl_sync(0xffffffffu, mine.x, j);
          const int sb = __shfl_sync(0xffffffffu, rank ? mine.z : mine.y, j);
          const int w = __shfl_sync(0xffffffffu, mine.w, j);
          if ((w >> 16) & 1) continue;   // neither CTA has a product at this stage
          if (lane == 0) {
            if (!mbar_wait(smem_u32(&bar_empty[stage]), phase ^ 1, &abort_s, wait_ns)) {
              fail(1);
              ok = false;
            } else {
              uint8_t* dst = stage_base + stage * STAGE_BYTES;
              const uint32_t full = smem_u32(&bar_full[stage]);
              const int need0 = max(0, min(S, L0 - 1 - (w & 0xff)));
              const int need1 = max(0, min(S, L1 - 1 - ((w >> 8) & 0xff)));
              const int na = max(need0, need1), nb = rank ? need1 : need0;
              // this CTA's half of the A prefix into both CTAs, then its own B
              // prefix; the stage (both A halves + B) completes here
              const uint32_t half_a = (uint32_t)na * (A_SLICE_BYTES / 2);   // multiple of 16
              mbar_expect_tx(full, (uint32_t)(na * A_SLICE_BYTES + nb * B_SLICE_BYTES));
              bulk_g2s_mc(smem_u32(dst) + rank * half_a,
                          P.Apack + (size_t)(sa - P.a_slot_base) * (S * A_SLICE_BYTES) +
                              rank * half_a,
                          half_a, full, (uint16_t)3);
              if (nb > 0)
                bulk_g2s(smem_u32(dst + S * A_SLICE_BYTES),
                         P.Bpack + (size_t)sb * (S * B_SLICE_BYTES), (uint32_t)nb * B_SLICE_BYTES,
                         full);
              issued[stage] = true;
              issued_parity[stage] = phase;
            }
          }
          ok = __shfl_sync(0xffffffffu, ok ? 1 : 0, 0) != 0;
          if (!ok) break;
          if (++stage == STAGES) {
            stage = 0;
            phase ^= 1;
          }
        }
      }
    }
    // copies still in flight land before the CTA may exit
    if (lane == 0)
      for (int s = 0; s < STAGES; ++s)
        if (issued[s] &&
            !mbar_wait(smem_u32(&bar_full[s]), issued_parity[s], &abort_s, WAIT_NS)) {
          const uint64_t t0 = globaltimer();
          while (!mbar_try(smem_u32(&bar_full[s]), issued_parity[s]) &&
                 globaltimer() - t0 < WAIT_NS) {
          }
        }
  } else if (warp == 1) {
    // ------------------------------------------------------------ MMA issuer
    // Level t lives in tensor-memory columns [(t-2)*BN, (t-1)*BN) and the S
    // B slices of a stage are contiguous in the K-major image, so the
    // products of A slice p with B slices q = q0..q1 (levels p+q+s) form ONE
    // MMA of N = (q1-q0+1)*BN (two of half that width above 256).  At shift
    // s, with L = S+1+E the block's last level, slice p feeds levels
    // p+1+s .. p+s+min(L-p-s, S): for s = 0, E = 0, 8 MMAs of N >= 160 and
    // one of 64 per k step for S = 6.  Lane 0 issues; the other lanes join
    // the waits.
    //
    // At a stage where levels restart (restart_mask), the MMAs whose lowest
    // level lies above every restarting level go first; then the warp waits
    // until the epilogue has read the restarting levels, marks them fresh and
    // issues the rest, slice 1 first (its range starts lowest).  An MMA over
    // levels of which some are fresh is split into runs, fresh runs with
    // accumulate off.
    auto mma_run = [&](uint32_t sb, int p, int ks, int q0, int t0, int nlev, uint32_t acc) {
      const uint32_t a = sb + (p - 1) * A_SLICE_BYTES + ks * 256;
      const uint32_t b0 = sb + S * A_SLICE_BYTES + (q0 - 1) * B_SLICE_BYTES + ks * 256;
      const int n = nlev * BN;
      const uint32_t d0 = tmem + (t0 - 2) * BN;
      if (n <= 256) {
        tc_mma(d0, make_desc(a), make_desc(b0), idesc_n(n), acc);
      } else {
        const int h = n / 2;   // a multiple of 32: B rows start on 8-row groups
        tc_mma(d0, make_desc(a), make_desc(b0), idesc_n(h), acc);
        tc_mma(d0 + h, make_desc(a), make_desc(b0 + (h / 8) * 512), idesc_n(h), acc);
      }
    };
    uint32_t fresh = 0;          // bit t: level t restarted and not written since (lane 0)
    // Slice p at shift s up to level L, split by fresh runs (lane 0).
    auto issue = [&](uint32_t sb, int p, int ks, int s, int L) {
      const int lo = p + 1 + s, hi = p + s + min(L - p - s, S);
      if (hi < lo) return;   // no level of this slice is kept (callers exclude it)
      const uint32_t span = ((2u << hi) - 1u) & ~((1u << lo) - 1u);
      if (!(fresh & span)) {
        mma_run(sb, p, ks, 1, lo, hi - lo + 1, 1u);
        return;
      }
      int t = lo;
      while (t <= hi) {
        const uint32_t f = (fresh >> t) & 1u;
        int u = t;
        while (u + 1 <= hi && ((fresh >> (u + 1)) & 1u) == f) ++u;
        mma_run(sb, p, ks, t - p - s, t, u - t + 1, f ? 0u : 1u);
        t = u + 1;
      }
      fresh &= ~span;
    };
    int stage = 0;
    uint32_t phase = 0;
    uint32_t level_parity = 0;   // bit t: parity of the next read of level t to wait for
    uint32_t level_used = 0;     // bit t: level t has been drained before
    int64_t events = 0;          // drains published
    bool ok = true;
    auto wait_level = [&](int t) -> bool {
      if (level_used & (1u << t)) {
        if (!mbar_wait(smem_u32(&bar_level[t]), (level_parity >> t) & 1u, &abort_s, wait_ns)) {
          fail(3);
          return false;
        }
        level_parity ^= 1u << t;
        tc_fence_after();
      }
      level_used |= 1u << t;
      return true;
    };
    int64_t gb = unit0;
    for (;;) {
      const OzParams* Pp = nullptr;
      int64_t b = 0;
      if constexpr (!Q) {
        if (gb >= nblk_total || !ok) break;
        const int vi = find_view(vstart, nviews, gb);
        Pp = &views[vi];
        b = gb - vstart[vi];
        gb += unit_step;
      } else {
        QUnit u;
        if (!ok || !ring_take(u)) break;
        Pp = u.P;
        b = u.b;
      }
      const OzParams& P = *Pp;
      const int64_t x0 = P.blk_rng[2 * b];
      const int64_t n = P.blk_rng[2 * b + 1] - x0;
      const int L = S + 1 + (int)((uint32_t)P.unitM[2 * b + rank] >> 28);
      const uint32_t* wsrc = reinterpret_cast<const uint32_t*>(P.blk_ab + x0) + 3;
      uint32_t wnext = lane < n ? wsrc[4 * lane] : 0u;
      for (int64_t xb = 0; xb < n && ok; xb += 32) {
        const uint32_t wcur = wnext;   // the next 32 entries' shifts load meanwhile
        if (xb + 32 + lane < n) wnext = wsrc[4 * (xb + 32 + lane)];
        const int cnt = (int)(n - xb < 32 ? n - xb : 32);
        for (int j = 0; j < cnt && ok; ++j) {
          const int64_t x = xb + j;
          const uint32_t w = __shfl_sync(0xffffffffu, wcur, j);
          const int s = (int)((w >> (8 * rank)) & 0xffu);
          const bool loaded = !((w >> 16) & 1u);
          const bool has = loaded && s + 2 <= L;   // this CTA multiplies at this stage
          const uint32_t z = restart_mask<TOP>(x);
          uint32_t sbase = 0;
          if (loaded) {
            if (!mbar_wait(smem_u32(&bar_full[stage]), phase, &abort_s, wait_ns)) {
              fail(2);
              ok = false;
              break;
            }
            tc_fence_after();
            sbase = smem_u32(stage_base + stage * STAGE_BYTES);
          }
          if (!z) {
            if (lane == 0 && has) {
              const uint32_t span = ((2u << L) - 1u) & ~((1u << (2 + s)) - 1u);
              if (!(fresh & span)) {
                // common case: every level of the stage is written already
                stage_dispatch<S, 0, kStageAll>(s, L - S - 1, tmem, make_desc(sbase),
                                                make_desc(sbase + S * A_SLICE_BYTES), 0);
              } else {
#pragma unroll
                for (int ks = 0; ks < 2; ++ks)
#pragma unroll
                  for (int p = 1; p <= S; ++p)
                    if (p + 1 + s <= L) issue(sbase, p, ks, s, L);
              }
            }
          } else if (x == 0) {
            // a block's first stage: every level restarts.  Levels are read
            // by the epilogue from the top down, so each slice goes out as
            // soon as its lowest level is free.
#pragma unroll
            for (int t = TOP; t >= 2; --t) {
              if (!wait_level(t)) {
                ok = false;
                break;
              }
              fresh |= 1u << t;
              const int p = t - 1 - s;
              if (lane == 0 && has && p >= 1 && p <= S && p + 1 + s <= L) {
                issue(sbase, p, 0, s, L);
                issue(sbase, p, 1, s, L);
              }
              __syncwarp();
            }
            if (!ok) break;
          } else {
            // a restart of levels zlo..5 (periods end together at multiples
            // of 8 stages, so z is always such a run)
            const int tmax = 31 - __clz(z);
            const int zlo = __ffs(z) - 1;
            const uint32_t span = ((2u << L) - 1u) & ~((1u << (2 + s)) - 1u);
            const bool quick = S >= 4 && !(fresh & span) && tmax == 5;
            const uint64_t ad0 = make_desc(sbase), bd0 = make_desc(sbase + S * A_SLICE_BYTES);
            if (lane == 0 && has) {
              if (quick) {
                stage_dispatch<S, 0, kStageRestartA>(s, L - S - 1, tmem, ad0, bd0, zlo);
              } else {
#pragma unroll
                for (int ks = 0; ks < 2; ++ks)
#pragma unroll
                  for (int p = 1; p <= S; ++p)
                    if (p + 1 + s > tmax && p + 1 + s <= L) issue(sbase, p, ks, s, L);
              }
            }
            __syncwarp();
#pragma unroll
            for (int t = TOP; t >= 2; --t)
              if ((z >> t) & 1u)
                if (!wait_level(t)) {
                  ok = false;
                  break;
                }
            if (!ok) break;
            fresh |= z;
            if (lane == 0 && has) {
              if (quick) {
                stage_dispatch<S, 0, kStageRestartC>(s, L - S - 1, tmem, ad0, bd0, zlo);
                fresh &= ~span;
              } else {
#pragma unroll
                for (int ks = 0; ks < 2; ++ks)
#pragma unroll
                  for (int p = 1; p <= S; ++p)
                    if (p + 1 + s <= tmax && p + 1 + s <= L) issue(sbase, p, ks, s, L);
              }
            }
          }
          __syncwarp();
          if (loaded) {
            // both CTAs write into this stage (the A halves): release it in both
            if (lane == 0) tc_commit_mc(smem_u32(&bar_empty[stage]), (uint16_t)3);
            __syncwarp();
            if (++stage == STAGES) {
              stage = 0;
              phase ^= 1;
            }
          }
          const uint32_t dm = drain_mask<TOP>(x, n);
          if (dm) {
            if (lane == 0) {
              fresh_ring[events & 3] = fresh & dm;
              tc_commit(smem_u32(&bar_acc_full));
              mbar_arrive(smem_u32(&bar_acc_full));
            }
            __syncwarp();
            ++events;
          }
        }
      }
        }
    // nothing may be in flight when tensor memory is released
    if (lane == 0) tc_commit(smem_u32(&bar_done));
    __syncwarp();
    {
      const uint64_t t0 = globaltimer();
      while (!mbar_try(smem_u32(&bar_done), 0) && globaltimer() - t0 < WAIT_NS) {
      }
    }
  } else {
    // ------------------------------------------------------------ epilogue
    // warp % 4 selects the 32 tensor-memory lanes (rows) a warp may access,
    // (warp - 2) / 4 the EPI_COLS of the 64 columns it owns.  After
    // each stage that ends a level's period (drain_mask), that level is read
    // (unless it got no product in the period), released to the MMA warp at
    // once, and folded into two int64 accumulators per element: hi in units
    // of level 5 takes the exact levels (L_t * 2^(8(5-t)), t <= 5; level 2's
    // periods sum below 2^32 for K <= 2^18, so hi stays below 2^57) and lo in
    // units of level TOP takes the whole-block levels (L_t * 2^(8(TOP-t)),
    // t >= 6, each read once per block, below 2^59 together).
    const int quarter = warp & 3;
    const int cq = (warp - 2) >> 2;
    const int rloc = quarter * 32 + lane;
    const uint32_t lane_addr = tmem + ((uint32_t)(quarter * 32) << 16) + cq * EPI_COLS;
    int64_t events = 0;
    bool ok = true;
    int64_t hi[EPI_COLS], lo[EPI_COLS];
#pragma unroll
    for (int j = 0; j < EPI_COLS; ++j) hi[j] = lo[j] = 0;
    int64_t gb = unit0;
    uint32_t nunits = 0;
    for (;;) {
      const OzParams* Pp = nullptr;
      int64_t b = 0;
      long long tag = 0;
      if constexpr (!Q) {
        if (gb >= nblk_total || !ok) break;
        const int vi = find_view(vstart, nviews, gb);
        Pp = &views[vi];
        b = gb - vstart[vi];
        gb += unit_step;
      } else {
        QUnit u;
        if (!ok || !ring_take(u)) break;
        Pp = u.P;
        b = u.b;
        tag = u.tag;
      }
      const OzParams& P = *Pp;
      const int rb = P.blk[2 * b], cb = 2 * P.blk[2 * b + 1] + (int)rank;
      const int64_t n = P.blk_rng[2 * b + 1] - P.blk_rng[2 * b];
      for (int64_t x = 0; x < n; ++x) {
        const uint32_t dm = drain_mask<TOP>(x, n);
        if (!dm) continue;
        if (!mbar_wait(smem_u32(&bar_acc_full), (uint32_t)(events & 1), &abort_s, wait_ns)) {
          fail(4);
          ok = false;
          break;
        }
        const uint32_t fm = fresh_ring[events & 3];
        ++events;
        tc_fence_after();
#pragma unroll
        for (int t = TOP; t >= 2; --t) {
          if (!((dm >> t) & 1u)) continue;
          if ((fm >> t) & 1u) {   // no product since the restart: the level is zero
            __syncwarp();
            if (lane == 0) mbar_arrive(smem_u32(&bar_level[t]));
            continue;
          }
          float v0[16], v1[16];
          tmem_ld16(lane_addr + (t - 2) * BN, v0);
          if constexpr (EPI_COLS == 32) tmem_ld16(lane_addr + (t - 2) * BN + 16, v1);
          tmem_wait_ld();
          tc_fence_before();
          __syncwarp();   // every lane's reads are done: one arrival per warp
          if (lane == 0) mbar_arrive(smem_u32(&bar_level[t]));
          if (t > kExactTop) {
            // whole-block fp32 sum: integer valued, possibly beyond 2^31
            const int sh = 8 * (TOP - t);
#pragma unroll
            for (int j = 0; j < 16; ++j) {
              if constexpr (EPI_COLS == 32) {
                lo[j] += (int64_t)__float2ll_rn(v0[j]) << sh;
                lo[16 + j] += (int64_t)__float2ll_rn(v1[j]) << sh;
              } else {
                lo[j] += float_to_ll_exact(v0[j], sh);
              }
            }
          } else {
            const int sh = 8 * (kExactTop - t);
#pragma unroll
            for (int j = 0; j < 16; ++j) {
              hi[j] += (int64_t)__float2int_rn(v0[j]) << sh;
              if constexpr (EPI_COLS == 32) hi[16 + j] += (int64_t)__float2int_rn(v1[j]) << sh;
            }
          }
        }
      }
      if (!ok) break;
      // recombination: C = alpha * 2^(E_A + E_B - 8 M) * (hi * 2^(8(TOP-5)) + lo) * u_TOP,
      // exact integer to correctly rounded double, then one multiply by alpha.
      // The column data of the warp's EPI_COLS columns is loaded one column
      // per lane and broadcast by shuffles, the row's per thread, and the
      // tile offset once per result tile crossed: every load is issued before
      // the first store, so the stores do not serialise reloads behind them.
      {
        const uint32_t full = 0xffffffffu;
        const int64_t gcl = (int64_t)cb * BN + cq * EPI_COLS + lane;
        const bool cok = lane < EPI_COLS && gcl < P.N_total;
        const int tj_l = cok ? P.col_tile[gcl] : -1;
        const int cl_l = cok ? P.col_local[gcl] : 0;
        const int eb_l = cok ? P.EB[gcl] - 1022 : 0;
        const int nn_l = cok ? P.nsz[tj_l] : 0;
        const int64_t gr = (int64_t)rb * BM + rloc;
        const bool rok = gr < P.M_total;
        const int ti_l = rok ? P.row_tile[gr] : -1;
        const int64_t mrow_l = rok ? P.hel * P.msz[ti_l] + P.row_local[gr] : 0;
        const int e2 = (2 - 8 * TOP) + (rok ? P.EA[gr] - 1022 : 0) -
                       8 * (int)((uint32_t)P.unitM[2 * b + rank] & 0x0FFFFFFFu);
        const int64_t* __restrict__ coff = P.coff;
        const int64_t Nt = P.Nt;
        double* __restrict__ const Cout = P.C;
        const double alpha = P.alpha;
        const bool unit_alpha = alpha == 1.0;
        double* sb = reinterpret_cast<double*>(stage_base + STAGES * STAGE_BYTES) +
                     (warp - 2) * 32 * EPI_LD;
        // Passes of EPI_PASS columns: each lane converts its row's values
        // into the warp's staging rows, then the warp writes them out with
        // lane = column (32 / EPI_PASS rows at a time), so every store
        // instruction writes whole 8 * EPI_PASS-byte row segments.
#pragma unroll
        for (int hc = 0; hc < EPI_COLS / EPI_PASS; ++hc) {
#pragma unroll
          for (int c = 0; c < EPI_PASS; ++c) {
            const int j = EPI_PASS * hc + c;
            const int eb = __shfl_sync(full, eb_l, j);
            const double v = exact_to_double<8 * (TOP - kExactTop)>(hi[j], lo[j], e2 + eb);
            sb[lane * EPI_LD + c] = unit_alpha ? v : alpha * v;
          }
          __syncwarp();
          const int c = lane % EPI_PASS;
          const int tj = __shfl_sync(full, tj_l, EPI_PASS * hc + c);
          const int cl = __shfl_sync(full, cl_l, EPI_PASS * hc + c);
          const int64_t nn = __shfl_sync(full, nn_l, EPI_PASS * hc + c);
          int ti_prev = -1;
          int64_t off = -1;
          constexpr int RPS = 32 / EPI_PASS;   // rows per store instruction
#pragma unroll 4
          for (int i = 0; i < 32 / RPS; ++i) {
            const int r = RPS * i + lane / EPI_PASS;
            const int ti = __shfl_sync(full, ti_l, r);
            const int64_t mrow = __shfl_sync(full, mrow_l, r);
            if (ti >= 0 && tj >= 0) {
              if (ti != ti_prev) {
                off = coff[(int64_t)ti * Nt + tj];
                ti_prev = ti;
              }
              if (off >= 0) Cout[off + mrow * nn + cl] = sb[r * EPI_LD + c];
            }
          }
          __syncwarp();
        }
      }
#pragma unroll
      for (int j = 0; j < EPI_COLS; ++j) hi[j] = lo[j] = 0;
      if constexpr (Q) {
        // Each finished unit is counted per job once all epilogue warps have
        // stored their results; the count reaching both CTAs of every unit
        // marks the job done for the host.
        __syncwarp();
        if (lane == 0) mbar_arrive(smem_u32(&epi_done));
        if (warp == 2) {
          if (!mbar_wait(smem_u32(&epi_done), nunits & 1u, &abort_s, wait_ns)) {
            fail(8);
            break;
          }
          if (lane == 0) {
            const int job = (int)(tag & 0xFFFFF);
            const long long units = tag >> 20;
            __threadfence_system();
            const int prev = atomicAdd(&qa->done_units[job], 1);
            if ((long long)prev + 1 == 2 * units) {
              __threadfence_system();
              asm volatile("st.release.sys.global.s32 [%0], %1;" ::"l"(&qa->job_done[job]), "r"(1)
                           : "memory");
            }
          }
          __syncwarp();
        }
        ++nunits;
      }
    }
  }
  tc_fence_before();
  __syncthreads();
  // the partner no longer copies into this CTA's shared memory nor arrives on
  // its barriers once it has passed this point
  cluster_sync();
  tc_fence_after();
  if (warp == 1) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem));
  }
}

// Stage shifts of every unit (one warp per unit, all views of a launch).
// From the bricks' deficits eA, eB (bits) and whole-digit shifts
// mA = eA / 8, mB = eB / 8: each column block's base M = min(mA + mB) and
// extra levels E = (min(eA + eB) - 8M + 3) / 8 (at most 2, and at most 1
// for S = 7, whose levels 2..9 fill the tensor memory), packed as
// unitM = M | E << 28; per stage s = mA + mB - M for each column block
// (clipped to 255), bit 16 set when neither column block has a product
// (s >= S + E).  Also counts the digit-slice products the GEMM will issue.
__global__ void shift_kernel(const OzParams* __restrict__ views, const int64_t* __restrict__ vstart,
                             int nviews, int64_t nblk_total, int S) {
  const int lane = threadIdx.x & 31;
  const int64_t gb = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (gb >= nblk_total) return;
  const int vi = find_view(vstart, nviews, gb);
  const OzParams& P = views[vi];
  const int64_t b = gb - vstart[vi];
  const int64_t x0 = P.blk_rng[2 * b], x1 = P.blk_rng[2 * b + 1];
  // deficits of the stage's A brick and its two B bricks (kNoShift: absent)
  auto deficits = [&](int64_t x, int& a, int& b0, int& b1) {
    const int4 e = P.blk_ab[x];
    a = P.shiftA[e.x];
    b0 = P.shiftB[e.y];
    b1 = P.shiftB[e.z];
  };
  int M[2] = {kNoShift, kNoShift}, T[2] = {kNoShift, kNoShift};
  for (int64_t x = x0 + lane; x < x1; x += 32) {
    int a, bb[2];
    deficits(x, a, bb[0], bb[1]);
#pragma unroll
    for (int c = 0; c < 2; ++c)
      if (a < kNoShift && bb[c] < kNoShift) {
        M[c] = min(M[c], (a >> 3) + (bb[c] >> 3));
        T[c] = min(T[c], a + bb[c]);
      }
  }
#pragma unroll
  for (int c = 0; c < 2; ++c)
    for (int o = 16; o > 0; o >>= 1) {
      M[c] = min(M[c], __shfl_xor_sync(0xffffffffu, M[c], o));
      T[c] = min(T[c], __shfl_xor_sync(0xffffffffu, T[c], o));
    }
  int E[2];
  const int emax = min(2, 9 - (S + 1));   // levels 2..9 fill the tensor memory
#pragma unroll
  for (int c = 0; c < 2; ++c) E[c] = M[c] >= kNoShift ? 0 : min(emax, (T[c] - 8 * M[c] + 3) >> 3);
  unsigned long long prod = 0;
  for (int64_t x = x0 + lane; x < x1; x += 32) {
    int a, bb[2];
    deficits(x, a, bb[0], bb[1]);
    int sh[2];
    bool none = true;
#pragma unroll
    for (int c = 0; c < 2; ++c) {
      const int L = S + 1 + E[c];
      sh[c] = 255;
      if (a < kNoShift && bb[c] < kNoShift) sh[c] = min(255, (a >> 3) + (bb[c] >> 3) - M[c]);
      if (sh[c] + 2 <= L) {
        none = false;
        for (int p = 1; p <= S; ++p) prod += (unsigned long long)max(0, min(L - p - sh[c], S));
      }
    }
    reinterpret_cast<int32_t*>(P.blk_ab + x)[3] = sh[0] | (sh[1] << 8) | ((none ? 1 : 0) << 16);
  }
  for (int o = 16; o > 0; o >>= 1) prod += __shfl_xor_sync(0xffffffffu, prod, o);
  if (lane == 0) {
    P.unitM[2 * b] = M[0] | (E[0] << 28);
    P.unitM[2 * b + 1] = M[1] | (E[1] << 28);
    if (prod) atomicAdd(P.products, prod);
  }
}

// ---------------------------------------------------------------------------
// frames, bricks and splitting
// ---------------------------------------------------------------------------

// Element (row, k) of an operand in GEMM order.  A: rows = M, tile (i,k) is
// m x kk (trans: kk x m).  B is seen as its transpose: rows = N, tile (k,j)
// is kk x n (trans: n x kk).
struct OperandView {
  const double* data;
  const int64_t* off;        // tile offsets
  int64_t rowt, kt;          // tile grid (rows, k) in this view
  int64_t off_stride_row, off_stride_k;  // off index = rt*sr + kt*sk
  const int32_t* rsz;        // tile sizes along rows
  const int32_t* ksz;        // tile sizes along k
  int row_contig;            // 1: element (r, k) at r * 1 + k * rows_in_tile
  int64_t hel;               // fused element: its matrix starts hel * rows * k into a tile
};

__device__ __forceinline__ int exp_field(double x) {
  return (int)((__double_as_longlong(x) >> 52) & 0x7ff);
}

// A frame job: one operand of one contraction.  Its work items are
// (row tile, chunk of kFrameRows rows, k tile), row-chunk major: row tile rt
// owns chunks [chunk0[rt], chunk0[rt+1]).  Items of all jobs of a launch are
// numbered consecutively from each job's item0.
constexpr int kFrameRows = 64;
struct FrameJob {
  OperandView v;
  const int32_t* row_start;   // first fused row of every row tile
  const int32_t* chunk0;      // rowt + 1 entries
  int32_t* E;                 // frames of the operand's fused rows
  int64_t item0;
};

// Frames: max biased exponent of every operand row over its k, folded into
// the row's frame with atomicMax.  One CTA per work item (64 rows of one
// operand tile), so long fused rows and tall tiles both spread over many
// CTAs and no CTA is idle.  Both storage orders are read coalesced: rows of a
// row-major tile by warps along k, columns of a transposed tile by threads
// along the rows.
__global__ void __launch_bounds__(256) frame_kernel(const FrameJob* __restrict__ jobs,
                                                    int njobs) {
  const int64_t g = blockIdx.x;
  int lo = 0, hi = njobs;
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (jobs[mid].item0 <= g) lo = mid; else hi = mid;
  }
  const FrameJob& J = jobs[lo];
  const OperandView& v = J.v;
  const int64_t i = g - J.item0;
  const int64_t q = i / v.kt, ktile = i - q * v.kt;   // q: global row chunk of the job
  int a = 0, b = (int)v.rowt;                          // row tile owning chunk q
  while (b - a > 1) {
    const int mid = (a + b) >> 1;
    if (J.chunk0[mid] <= q) a = mid; else b = mid;
  }
  const int64_t rt = a;
  const int64_t o = v.off[rt * v.off_stride_row + ktile * v.off_stride_k];
  if (o < 0) return;
  const int m = v.rsz[rt], kk = v.ksz[ktile];
  const int r0 = (int)(q - J.chunk0[rt]) * kFrameRows, r1 = min(m, r0 + kFrameRows);
  const double* base = v.data + o + v.hel * m * kk;
  int32_t* Er = J.E + J.row_start[rt];
  if (v.row_contig) {              // element (r, k) at k * m + r
    const int r = r0 + (threadIdx.x % kFrameRows);
    const int kq = threadIdx.x / kFrameRows, nq = blockDim.x / kFrameRows;
    int e = 0;
    if (r < r1)
#pragma unroll 4   // several loads in flight per thread
      for (int k = kq; k < kk; k += nq) e = max(e, exp_field(base[(int64_t)k * m + r]));
    if (e > 0) atomicMax(&Er[r], e);
  } else {                         // element (r, k) at r * kk + k
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int r = r0 + warp; r < r1; r += blockDim.x >> 5) {
      int e = 0;
#pragma unroll 4
      for (int k = lane; k < kk; k += 32) e = max(e, exp_field(base[(int64_t)r * kk + k]));
      for (int s = 16; s > 0; s >>= 1) e = max(e, __shfl_xor_sync(0xffffffffu, e, s));
      if (lane == 0 && e > 0) atomicMax(&Er[r], e);
    }
  }
}

// Zeroing of int32 ranges (frames, error flags) of many plans in one launch.
struct ZeroJob {
  int32_t* p;
  int64_t n;
};
__global__ void zero_kernel(const ZeroJob* __restrict__ jobs) {
  const ZeroJob J = jobs[blockIdx.x];
  for (int64_t i = threadIdx.x; i < J.n; i += blockDim.x) J.p[i] = 0;
}

// Digits of one element: fixed point round(x * 2^(8S-1-E)) (E = frame -
// 1022), cut into S balanced base-256 digits, f[0] the most significant,
// each returned as the bit pattern of the exact float (|d| <= 128), whose
// high half is the bf16 digit and whose low half is zero.
template <int S>
__device__ __forceinline__ void split_digits(double x, int frame, uint32_t (&f)[S]) {
  int64_t fx = 0;
  const uint64_t bits = (uint64_t)__double_as_longlong(x);
  const int be = (int)((bits >> 52) & 0x7ff);
  if (frame > 0 && (bits << 1) != 0) {
    uint64_t mant = bits & 0xFFFFFFFFFFFFFull;
    int bexp = be;
    if (be == 0) {
      bexp = 1;  // subnormal
    } else {
      mant |= 1ull << 52;
    }
    const int E = frame - 1022;
    const int sh = 1075 + E - (8 * S - 1) - bexp;   // >= 53 - (8S - 1): negative only for S = 7
    uint64_t q;
    if (sh <= 0) {
      q = mant << (-sh);
    } else if (sh >= 64) {
      q = 0;
    } else {
      q = (mant >> sh) + ((mant >> (sh - 1)) & 1ull);  // round half up in magnitude
    }
    fx = (bits >> 63) ? -(int64_t)q : (int64_t)q;
  }
  // The balanced digits of the recurrence d = ((v + 128) & 255) - 128,
  // v = (v - d) / 256 from the least significant digit: adding 128 at each of
  // the S - 1 lower digit positions makes digit q (counted from the least
  // significant) byte q of the sum minus 128, and leaves the top digit as the
  // sum shifted down by 8 (S - 1).  |fx| <= 2^(8S-1), so the sum does not
  // overflow.  A byte b becomes the float b - 128 exactly as
  // (2^23 + b) - (2^23 + 128): one byte permute and one float add.
  constexpr uint64_t kBias = 0x8080808080808080ull >> (8 * (9 - S));
  const uint64_t u = (uint64_t)fx + kBias;
  const uint32_t ul = (uint32_t)u, uh = (uint32_t)(u >> 32);
#pragma unroll
  for (int q = 0; q < S - 1; ++q)
    f[S - 1 - q] = __float_as_uint(
        __fadd_rn(__uint_as_float(__byte_perm(q < 4 ? ul : uh, 0x4B000000u, 0x7540u | (q & 3))),
                  -8388736.0f));
  f[0] = __float_as_uint((float)(int)((int64_t)u >> (8 * (S - 1))));
}

// A split job: the bricks of one operand (or of one row chunk of it) of one
// contraction.  Bricks of all jobs of a launch are numbered consecutively
// from each job's brick0.
struct SplitJob {
  OperandView v;
  const int32_t *row_tile, *row_local, *k_tile, *k_local;
  const int32_t *row_ext, *k_ext;   // extent of the tile holding each fused row / k
  const int32_t* E;           // frames of the operand's fused rows
  int64_t rows_total, k_total;
  const int32_t* bricks;      // nbricks x 2 (row block, k block)
  const int4* hdr;            // per brick: tile of its first / last row, of its first / last k
  int64_t nbricks;
  uint8_t* pack;              // brick i of the job at pack + i * S * ROWS * 64 bytes
  int32_t* shift;             // brick i's deficit e in bits (kNoShift: all zero)
  int64_t brick0;
};

// Split staging layout in shared memory: the 16 bytes of (row r, k group
// g = k / 8) sit at chunk g * (ROWS + 1) + r of a slice.  The four k groups
// of one row land in distinct bank groups (lanes along k store 2 bytes each
// without conflicts) and the rows of one group are consecutive chunks (lanes
// along rows store 16 bytes each without conflicts).  The copy-out reorders
// the chunks into the K-major core-matrix image (brick_offset).
template <int ROWS>
__device__ __forceinline__ uint32_t stage_chunk(int r, int g) {
  return (uint32_t)(g * (ROWS + 1) + r) * 16;
}

// One CTA per brick (grid-stride over the bricks of all jobs): gather
// ROWS x 32 elements, split them into S digit slices, write the brick image.
// The brick's row and k maps (tile, local index, frame, tile extent) and the
// offsets of the tiles it overlaps are staged in shared memory first, so an
// element costs one independent data load; a thread issues all its loads
// before it splits.  Row-major tiles are read by warps along rows with lanes
// along k, transposed tiles by threads that own eight k of one row with
// lanes along rows: both coalesced.  A brick over more than kTable tiles
// (tiles of a few elements) looks tile offsets up in global memory.
template <int S, int ROWS>
__global__ void __launch_bounds__(256, ROWS == BM ? 4 : 5) split_kernel(const SplitJob* __restrict__ jobs, int njobs,
                                                    int64_t total) {
  constexpr int SLICE = ROWS * BK * 2;        // image bytes per slice
  constexpr int SPAD = 4 * (ROWS + 1) * 16;   // staged bytes per slice
  constexpr int EPT = ROWS * BK / 256;        // elements per thread
  constexpr int kTable = 256;
  static_assert(EPT % 8 == 0, "a transposed-tile thread owns whole k groups");
  extern __shared__ __align__(16) uint8_t img[];
  __shared__ int s_rt[ROWS], s_lr[ROWS], s_fr[ROWS], s_m[ROWS];
  __shared__ int s_kt[BK], s_lk[BK], s_kk[BK];
  __shared__ int64_t s_off[kTable];
  __shared__ int s_shift;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  // A brick's header (its job, index, block coordinates and tile ranges) is
  // fetched one iteration ahead, so its loads overlap the previous brick.
  struct Hdr {
    int job;
    int64_t bi;
    int rb, kb;
    int4 h;
  };
  auto fetch = [&](int64_t g) {
    Hdr x;
    int lo = 0, hi = njobs;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (jobs[mid].brick0 <= g) lo = mid; else hi = mid;
    }
    x.job = lo;
    x.bi = g - jobs[lo].brick0;
    x.rb = jobs[lo].bricks[2 * x.bi];
    x.kb = jobs[lo].bricks[2 * x.bi + 1];
    x.h = jobs[lo].hdr[x.bi];
    return x;
  };
  Hdr cur{};
  if (blockIdx.x < total) cur = fetch(blockIdx.x);
  for (int64_t gbi = blockIdx.x; gbi < total; gbi += gridDim.x) {
    Hdr nxt = cur;
    if (gbi + gridDim.x < total) nxt = fetch(gbi + gridDim.x);
    const SplitJob& J = jobs[cur.job];
    const OperandView& v = J.v;
    const int64_t rows_total = J.rows_total, k_total = J.k_total;
    const int64_t bi = cur.bi;
    const int64_t r0 = (int64_t)cur.rb * ROWS, k0 = (int64_t)cur.kb * BK;
    const int rt0 = cur.h.x, kt0 = cur.h.z;
    const int nr = cur.h.y - rt0 + 1, nk = cur.h.w - kt0 + 1;
    const bool staged = nr * nk <= kTable;
    // every reader of the previous brick's shift passed the barrier after
    // its split before any thread gets here
    if (threadIdx.x == 0) s_shift = kNoShift;
    for (int i = threadIdx.x; i < ROWS; i += blockDim.x) {
      const int64_t gr = r0 + i;
      if (gr < rows_total) {
        s_rt[i] = J.row_tile[gr];
        s_lr[i] = J.row_local[gr];
        s_fr[i] = J.E[gr];
        s_m[i] = J.row_ext[gr];
      } else {
        s_rt[i] = -1;
        s_fr[i] = 0;
      }
    }
    if (threadIdx.x < BK) {
      const int64_t gk = k0 + threadIdx.x;
      if (gk < k_total) {
        s_kt[threadIdx.x] = J.k_tile[gk];
        s_lk[threadIdx.x] = J.k_local[gk];
        s_kk[threadIdx.x] = J.k_ext[gk];
      } else {
        s_kt[threadIdx.x] = -1;
      }
    }
    if (staged) {
      for (int t = threadIdx.x; t < nr * nk; t += blockDim.x) {
        const int a = t / nk, b = t - a * nk;
        const int64_t o =
            v.off[(int64_t)(rt0 + a) * v.off_stride_row + (int64_t)(kt0 + b) * v.off_stride_k];
        s_off[t] = o < 0 || v.hel == 0 ? o : o + v.hel * v.rsz[rt0 + a] * v.ksz[kt0 + b];
      }
    }
    __syncthreads();
    const double* __restrict__ data = v.data;
    double x[EPT];
    // All loads of the thread, with the tile offsets from shared memory
    // (ST) or looked up per element; two instantiations, so the staged path
    // carries no global offset loads.
    auto load_all = [&](auto st_c) {
      constexpr bool ST = decltype(st_c)::value;
      // start of the element's matrix in tile (rt, kt), -1 if absent
      auto tile_off = [&](int rt, int kt, int m, int kk) -> int64_t {
        if constexpr (ST) {
          return s_off[(rt - rt0) * nk + (kt - kt0)];
        } else {
          const int64_t o =
              v.off[(int64_t)rt * v.off_stride_row + (int64_t)kt * v.off_stride_k];
          return o < 0 ? o : o + v.hel * m * kk;
        }
      };
      if (!v.row_contig) {
        // element (r, k) at o + lr * kk + lk: lanes along k, rows warp + 8 i
        const int k = lane, kt = s_kt[k], lk = s_lk[k], kk = kt >= 0 ? s_kk[k] : 0;
#pragma unroll
        for (int i = 0; i < EPT; ++i) {
          const int r = warp + 8 * i, rt = s_rt[r];
          double val = 0.0;
          if (rt >= 0 && kt >= 0) {
            const int64_t o = tile_off(rt, kt, ST ? 0 : s_m[r], kk);
            if (o >= 0) val = data[o + (int64_t)s_lr[r] * kk + lk];
          }
          x[i] = val;
        }
      } else {
        // element (r, k) at o + lk * m + lr: a thread owns row r = 32 (item /
        // 4) + lane and the eight k of group item % 4
#pragma unroll
        for (int i = 0; i < EPT / 8; ++i) {
          const int item = warp + 8 * i, r = (item >> 2) * 32 + lane, g = item & 3;
          const int rt = s_rt[r], lr = s_lr[r], m = s_m[r];
#pragma unroll
          for (int j = 0; j < 8; ++j) {
            const int k = 8 * g + j, kt = s_kt[k];
            double val = 0.0;
            if (rt >= 0 && kt >= 0) {
              const int64_t o = tile_off(rt, kt, m, ST ? 0 : s_kk[k]);
              if (o >= 0) val = data[o + (int64_t)s_lk[k] * m + lr];
            }
            x[8 * i + j] = val;
          }
        }
      }
    };
    if (staged)
      load_all(std::true_type{});
    else
      load_all(std::false_type{});
    // Brick deficit e: the smallest number of bits by which a nonzero element
    // sits below its row frame (subnormals count as exponent 1); the digits
    // are cut against 2^(frame - 8m), m = floor(e / 8) whole digits.
    {
      int eloc = kNoShift;
      // nonzero tested on the bit pattern (±0 is zero): an FP64 compare
      // would run on this GPU's narrow FP64 pipe once per element
      auto see = [&](double val, int fr) {
        const uint64_t bits = (uint64_t)__double_as_longlong(val);
        if ((bits << 1) != 0 && fr > 0)
          eloc = min(eloc, fr - max((int)((bits >> 52) & 0x7ff), 1));
      };
      if (!v.row_contig) {
#pragma unroll
        for (int i = 0; i < EPT; ++i) see(x[i], s_fr[warp + 8 * i]);
      } else {
#pragma unroll
        for (int i = 0; i < EPT / 8; ++i) {
          const int item = warp + 8 * i, r = (item >> 2) * 32 + lane;
#pragma unroll
          for (int j = 0; j < 8; ++j) see(x[8 * i + j], s_fr[r]);
        }
      }
      for (int o = 16; o > 0; o >>= 1) eloc = min(eloc, __shfl_xor_sync(0xffffffffu, eloc, o));
      if (lane == 0 && eloc < kNoShift) atomicMin(&s_shift, eloc);
    }
    __syncthreads();
    const int m = s_shift;
    const int dfr = m < kNoShift ? 8 * (m >> 3) : 0;   // frame reduction of every row
    if (!v.row_contig) {
      const int k = lane;
      uint8_t* c0 = img + stage_chunk<ROWS>(0, k >> 3) + (k & 7) * 2;
#pragma unroll
      for (int i = 0; i < EPT; ++i) {
        const int r = warp + 8 * i;
        uint32_t h[S];
        split_digits<S>(x[i], s_fr[r] - dfr, h);
#pragma unroll
        for (int p = 0; p < S; ++p)
          *reinterpret_cast<uint16_t*>(c0 + r * 16 + p * SPAD) = (uint16_t)(h[p] >> 16);
      }
    } else {
#pragma unroll
      for (int i = 0; i < EPT / 8; ++i) {
        const int item = warp + 8 * i, r = (item >> 2) * 32 + lane, g = item & 3;
        const int fr = s_fr[r] - dfr;
        uint32_t w[S][4];
#pragma unroll
        for (int j = 0; j < 8; j += 2) {
          uint32_t h0[S], h1[S];
          split_digits<S>(x[8 * i + j], fr, h0);
          split_digits<S>(x[8 * i + j + 1], fr, h1);
          // the bf16 halves of k = j (low) and j + 1 (high)
#pragma unroll
          for (int p = 0; p < S; ++p) w[p][j >> 1] = __byte_perm(h0[p], h1[p], 0x7632u);
        }
        uint8_t* c = img + stage_chunk<ROWS>(r, g);
#pragma unroll
        for (int p = 0; p < S; ++p)
          *reinterpret_cast<uint4*>(c + p * SPAD) = make_uint4(w[p][0], w[p][1], w[p][2], w[p][3]);
      }
    }
    if (threadIdx.x == 0) J.shift[bi] = m;
    __syncthreads();
    // Copy-out in image order (chunk c of a slice: row 8 (c / 32) + c % 8,
    // k group (c / 8) % 4).  The maps and staged offsets are not read again,
    // so the next brick may restage them while slow threads still copy; its
    // first barrier orders its stores into img after this copy.
    constexpr int CH = SLICE / 16;
    uint8_t* dst = J.pack + (size_t)bi * S * SLICE;
    for (int i = threadIdx.x; i < S * CH; i += blockDim.x) {
      const int p = i / CH, c = i - p * CH;
      const int r = (c >> 5) * 8 + (c & 7), g = (c >> 3) & 3;   // brick_offset(r, 8 g) == 16 c
      *reinterpret_cast<uint4*>(dst + p * SLICE + brick_offset(r, 8 * g)) =
          *reinterpret_cast<const uint4*>(img + p * SPAD + stage_chunk<ROWS>(r, g));
    }
    cur = nxt;
  }
}

// Does any present tile overlap brick (row block, k block)?
__global__ void brick_flag_kernel(OperandView v, const int32_t* __restrict__ row_tile,
                                  const int32_t* __restrict__ k_tile, int64_t rows_total,
                                  int64_t k_total, int ROWS, int64_t RB, int64_t KB,
                                  int64_t* __restrict__ flag) {
  const int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= RB * KB) return;
  const int64_t rb = x / KB, kb = x - (x / KB) * KB;
  const int64_t r0 = rb * ROWS, r1 = min(rows_total, r0 + ROWS) - 1;
  const int64_t k0 = kb * BK, k1 = min(k_total, k0 + BK) - 1;
  int64_t f = 0;
  for (int rt = row_tile[r0]; rt <= row_tile[r1] && !f; ++rt)
    for (int kt = k_tile[k0]; kt <= k_tile[k1]; ++kt)
      if (v.off[(int64_t)rt * v.off_stride_row + (int64_t)kt * v.off_stride_k] >= 0) {
        f = 1;
        break;
      }
  flag[x] = f;
}

// Slot of every flagged (block, k block) x = block * KB + k block, and the
// list of flagged pairs.  With CBt > 0 the slot map is written transposed,
// at k block * CBt + block (the B bricks' (k block, column block) order).
__global__ void brick_slot_kernel(const int64_t* __restrict__ flag,
                                  const int64_t* __restrict__ scan, int64_t n, int64_t KB,
                                  int32_t* __restrict__ slot, int32_t* __restrict__ list,
                                  int64_t CBt) {
  const int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= n) return;
  const int64_t blk = x / KB, kb = x - blk * KB;
  const int64_t at = CBt > 0 ? kb * CBt + blk : x;
  if (flag[x]) {
    const int64_t s = scan[x];
    slot[at] = (int32_t)s;
    list[2 * s] = (int32_t)blk;
    list[2 * s + 1] = (int32_t)kb;
  } else {
    slot[at] = -1;
  }
}

// Tile ranges of every brick of a list: the tiles of its first and last
// row and of its first and last k (rows and k in fused GEMM order).
__global__ void brick_hdr_kernel(const int32_t* __restrict__ list, int64_t n,
                                 const int32_t* __restrict__ row_tile,
                                 const int32_t* __restrict__ k_tile, int64_t rows_total,
                                 int64_t k_total, int ROWS, int4* __restrict__ hdr) {
  const int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= n) return;
  const int64_t r0 = (int64_t)list[2 * x] * ROWS, k0 = (int64_t)list[2 * x + 1] * BK;
  hdr[x] = make_int4(row_tile[r0], row_tile[min(rows_total, r0 + ROWS) - 1], k_tile[k0],
                     k_tile[min(k_total, k0 + BK) - 1]);
}

// Units of work are pairs of output blocks (rb, 2c) and (rb, 2c+1), run by
// the two CTAs of a cluster, which share the A brick of every k block.
// One warp per unit: a column block is active if it overlaps a nonzero
// result tile; the unit's k list is every k block whose A brick exists and
// whose B brick exists for an active column block of the pair.
__device__ __forceinline__ bool block_active(const int32_t* __restrict__ row_tile,
                                             const int32_t* __restrict__ col_tile,
                                             const int64_t* __restrict__ coff, int64_t Nt,
                                             int64_t M_total, int64_t N_total, int64_t rb,
                                             int64_t cb) {
  const int64_t r0 = rb * BM, r1 = min(M_total, r0 + BM) - 1;
  const int64_t c0 = cb * BN;
  if (c0 >= N_total) return false;
  const int64_t c1 = min(N_total, c0 + BN) - 1;
  for (int it = row_tile[r0]; it <= row_tile[r1]; ++it)
    for (int jt = col_tile[c0]; jt <= col_tile[c1]; ++jt)
      if (coff[(int64_t)it * Nt + jt] >= 0) return true;
  return false;
}

__global__ void block_kernel(const int32_t* __restrict__ brickA, const int32_t* __restrict__ brickB,
                             const int32_t* __restrict__ row_tile,
                             const int32_t* __restrict__ col_tile, const int64_t* __restrict__ coff,
                             int64_t Nt, int64_t M_total, int64_t N_total, int64_t RB, int64_t CB,
                             int64_t KB, const int64_t* __restrict__ offs /* null: count */,
                             int64_t* __restrict__ counts, int32_t* __restrict__ kbs) {
  const int lane = threadIdx.x & 31;
  const int64_t CP = (CB + 1) / 2;
  const int64_t x = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (x >= RB * CP) return;
  const int64_t rb = x / CP, cp = x - (x / CP) * CP;
  const int64_t cb0 = 2 * cp, cb1 = 2 * cp + 1;
  const bool act0 = block_active(row_tile, col_tile, coff, Nt, M_total, N_total, rb, cb0);
  const bool act1 =
      cb1 < CB && block_active(row_tile, col_tile, coff, Nt, M_total, N_total, rb, cb1);
  int64_t cnt = 0;
  int64_t pos = offs ? offs[x] : 0;
  if (act0 || act1) {
    for (int64_t k0 = 0; k0 < KB; k0 += 32) {
      const int64_t kb = k0 + lane;
      bool p = kb < KB && brickA[rb * KB + kb] >= 0;
      if (p) p = (act0 && brickB[kb * CB + cb0] >= 0) || (act1 && brickB[kb * CB + cb1] >= 0);
      const unsigned bm = __ballot_sync(0xffffffffu, p);
      if (offs && p) kbs[pos + __popc(bm & ((1u << lane) - 1u))] = (int32_t)kb;
      pos += __popc(bm);
      cnt += __popc(bm);
    }
  }
  if (!offs && lane == 0) counts[x] = cnt;
}

__global__ void block_list_kernel(const int64_t* __restrict__ counts,
                                  const int64_t* __restrict__ scan_blocks, int64_t n, int64_t CP,
                                  int32_t* __restrict__ blk) {
  const int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= n || counts[x] == 0) return;
  const int64_t s = scan_blocks[x];
  blk[2 * s] = (int32_t)(x / CP);
  blk[2 * s + 1] = (int32_t)(x - (x / CP) * CP);
}

// Brick slots of every (unit, k block): one warp per unit.  A column block
// without a B brick at this k (or past the last column, or inactive) reads
// the zero brick `zero_b`.
__global__ void slot_pairs_kernel(const int32_t* __restrict__ blk, const int64_t* __restrict__ off,
                                  int64_t nblk, const int32_t* __restrict__ kbs,
                                  const int32_t* __restrict__ brickA,
                                  const int32_t* __restrict__ brickB, int64_t KB, int64_t CB,
                                  const int32_t* __restrict__ row_tile,
                                  const int32_t* __restrict__ col_tile,
                                  const int64_t* __restrict__ coff, int64_t Nt, int64_t M_total,
                                  int64_t N_total, int32_t zero_b, int4* __restrict__ out) {
  const int lane = threadIdx.x & 31;
  const int64_t b = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  if (b >= nblk) return;
  const int64_t rb = blk[2 * b], cb0 = 2 * (int64_t)blk[2 * b + 1], cb1 = cb0 + 1;
  const bool act0 = block_active(row_tile, col_tile, coff, Nt, M_total, N_total, rb, cb0);
  const bool act1 =
      cb1 < CB && block_active(row_tile, col_tile, coff, Nt, M_total, N_total, rb, cb1);
  for (int64_t x = off[b] + lane; x < off[b + 1]; x += 32) {
    const int64_t kb = kbs[x];
    int32_t b0 = act0 ? brickB[kb * CB + cb0] : -1;
    int32_t b1 = act1 ? brickB[kb * CB + cb1] : -1;
    out[x] = make_int4(brickA[rb * KB + kb], b0 >= 0 ? b0 : zero_b, b1 >= 0 ? b1 : zero_b, 0);
  }
}

__global__ void flag_nonzero_kernel(const int64_t* __restrict__ counts, int64_t n,
                                    int64_t* __restrict__ flag) {
  const int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (x < n) flag[x] = counts[x] > 0 ? 1 : 0;
}

__global__ void gather_offsets_kernel(const int64_t* __restrict__ counts,
                                      const int64_t* __restrict__ scan_counts,
                                      const int64_t* __restrict__ scan_blocks, int64_t n,
                                      int64_t* __restrict__ blk_off) {
  const int64_t x = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= n) return;
  if (counts[x] > 0) blk_off[scan_blocks[x]] = scan_counts[x];
  if (x == n - 1) blk_off[scan_blocks[n]] = scan_counts[n];
}

inline unsigned blocks_for(int64_t n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

struct DevVec {
  void* p = nullptr;
  size_t bytes = 0;
};

// All device state of one emulated contraction (scratch).
struct OzakiPlan {
  cudaStream_t s = nullptr;
  int S = 6;
  int64_t M_total = 0, N_total = 0, K_total = 0;
  int64_t RB = 0, KB = 0, CB = 0;
  int64_t nA = 0, nB = 0, nblk = 0, nkb = 0;
  OperandView va{}, vb{};
  std::vector<DevVec> bufs;
  int32_t *row_tile = nullptr, *row_local = nullptr, *k_tile = nullptr, *k_local = nullptr,
          *col_tile = nullptr, *col_local = nullptr, *rstart = nullptr, *cstart = nullptr;
  int32_t *row_ext = nullptr, *k_ext = nullptr, *col_ext = nullptr;   // tile extent per index
  int4 *hdrA = nullptr, *hdrB = nullptr;   // brick headers of listA / listB
  int4* blk_ab = nullptr;
  int32_t *EA = nullptr, *EB = nullptr, *brickA = nullptr, *brickB = nullptr, *listA = nullptr,
          *listB = nullptr, *blk = nullptr, *blk_kb = nullptr;
  int64_t *blk_off = nullptr, *blk_rng = nullptr;
  // frame work: per row tile the first 64-row chunk (prefix), per operand
  int32_t *chunk0_a = nullptr, *chunk0_b = nullptr;
  int64_t frame_items_a = 0, frame_items_b = 0;
  // work tables of the frame and split launches (host copies and device)
  FrameJob h_frames[2];                    // A, B
  SplitJob h_split_b;
  std::vector<SplitJob> h_split_a;         // one per row chunk
  FrameJob* d_frames = nullptr;
  SplitJob* d_split_b = nullptr;
  SplitJob* d_split_a = nullptr;
  uint8_t *Apack = nullptr, *Bpack = nullptr;
  int32_t *shiftA = nullptr, *shiftB = nullptr, *unitM = nullptr;   // digit shifts
  unsigned long long* products = nullptr;  // digit-slice products issued per run
  unsigned long long wait_ns = 4000000000ull;  // bound of the GEMM's pipeline waits
  int* err = nullptr;
  OzParams P{};
  OzParams* d_params = nullptr;   // P on the device (single-view launches)
  int64_t* d_vstart = nullptr;    // {0, nblk}
  // row chunking: A bricks are built and consumed one range of row blocks at
  // a time when all of them would not fit next to the operands
  int nchunk = 1;
  std::vector<int64_t> chunk_slot{0, 0};   // A slot boundaries
  std::vector<int64_t> chunk_blk{0, 0};    // block boundaries (scheduling order)
  OzParams* d_chunk_params = nullptr;
  int64_t* d_chunk_vstart = nullptr;
  std::vector<int64_t> chunk_rb{0, 0};     // row-block boundaries of the chunks
  // schedule (results do not depend on it): super-tile of the block order
  int tune_gr = 4, tune_gc = 19;
  int epi_warps = 0;   // epilogue width chosen by the autotuner, 0: by stage count
  std::vector<int32_t> h_blk;              // blocks (rb, cb) in discovery order
  std::vector<int64_t> h_off;              // their k-list offsets
  size_t bytes = 0;
  ~OzakiPlan() {
    for (auto& b : bufs)
      if (b.p) cudaFreeAsync(b.p, s);
  }
  template <typename T>
  tagpu_status alloc(T** p, size_t n, std::string* e) {
    void* q = nullptr;
    const size_t bytes_ = std::max<size_t>(1, n) * sizeof(T);
    cudaError_t ce = pool_alloc(&q, bytes_, s);
    if (ce != cudaSuccess) {
      *e = std::string("ozaki scratch allocation failed: ") + cudaGetErrorString(ce);
      return TAGPU_ERR_NOMEM;
    }
    bufs.push_back({q, bytes_});
    bytes += bytes_;
    *p = static_cast<T*>(q);
    return TAGPU_OK;
  }
  template <typename T>
  tagpu_status upload(T** p, const std::vector<T>& v, std::string* e) {
    tagpu_status st = alloc(p, v.size(), e);
    if (st) return st;
    if (!v.empty()) cudaMemcpyAsync(*p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s);
    return TAGPU_OK;
  }
  // Several int32 vectors in one allocation and one copy (each starts on a
  // 16-byte boundary): fewer host round trips than one upload per vector.
  tagpu_status upload_many(const std::vector<std::pair<int32_t**, const std::vector<int32_t>*>>& v,
                           std::string* e) {
    std::vector<size_t> at;
    size_t n = 0;
    for (const auto& x : v) {
      at.push_back(n);
      n += (std::max<size_t>(1, x.second->size()) + 3) & ~(size_t)3;
    }
    std::vector<int32_t> host(n, 0);
    for (size_t i = 0; i < v.size(); ++i)
      std::copy(v[i].second->begin(), v[i].second->end(), host.begin() + at[i]);
    int32_t* d = nullptr;
    tagpu_status st = alloc(&d, n, e);
    if (st) return st;
    cudaMemcpyAsync(d, host.data(), n * sizeof(int32_t), cudaMemcpyHostToDevice, s);
    for (size_t i = 0; i < v.size(); ++i) *v[i].first = d + at[i];
    return TAGPU_OK;
  }
};

namespace {

constexpr int kMaxDevices = 128;

// Co-resident clusters of the GEMM kernel on the current device (the
// shared-memory attribute is set on first use, per device).
template <int S, bool Q, int EW>
int gemm_clusters(int sm_count) {
  const size_t smem = Smem<S, EW>::kBytes;
  static bool set[kMaxDevices] = {};
  static int clusters[kMaxDevices] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= kMaxDevices) dev = 0;
  if (!set[dev]) {
    cudaFuncSetAttribute(ozaki_gemm_kernel<S, Q, EW>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
    // A persistent grid larger than what fits at once would leave the extra
    // clusters to start after others finish their whole share.
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(2 * (sm_count / 2)), 1, 1);
    cfg.blockDim = dim3(Epi<EW>::kThreads, 1, 1);
    cfg.dynamicSmemBytes = smem;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, ozaki_gemm_kernel<S, Q, EW>, &cfg) != cudaSuccess ||
        n <= 0) {
      cudaGetLastError();
      n = sm_count / 2;
    }
    clusters[dev] = std::min(n, sm_count / 2);
    set[dev] = true;
    if (const char* e = getenv("TAGPU_VERBOSE"))
      if (atoi(e) > 0)
        fprintf(stderr, "tagpu: emulated GEMM (S=%d%s, %d epilogue warps) on device %d: %d "
                "co-resident clusters of 2 (%d SMs)\n", S, Q ? ", served" : "", EW, dev, n,
                sm_count);
  }
  return clusters[dev];
}

template <int S, int EW>
void launch_gemm_ew(const OzParams* views, const int64_t* vstart, int nviews, int64_t nblk,
                    int* err, int sm_count, unsigned long long wait_ns, cudaStream_t st) {
  const int clusters = gemm_clusters<S, false, EW>(sm_count);
  // clusters of two CTAs, one unit (pair of output blocks) at a time each
  const int64_t grid = 2 * std::min<int64_t>(nblk, clusters);
  if (grid > 0) {
    // stage shifts from the digit bricks just split, then the GEMM
    shift_kernel<<<blocks_for(nblk * 32, 256), 256, 0, st>>>(views, vstart, nviews, nblk, S);
    count_launch();
    ozaki_gemm_kernel<S, false, EW><<<(unsigned)grid, Epi<EW>::kThreads, Smem<S, EW>::kBytes,
                                      st>>>(views, vstart, nviews, nblk, err, wait_ns, nullptr);
    count_launch();
  }
}

template <int S>
void launch_gemm_t(const OzParams* views, const int64_t* vstart, int nviews, int64_t nblk,
                   int64_t nstages, int epi_warps, int* err, int sm_count,
                   unsigned long long wait_ns, cudaStream_t st) {
  // the width from the autotuner (epi_warps 8 or 16), else by the units'
  // average stage count; TAGPU_EPILOGUE_WARPS=8 or 16 overrides both
  // (results are the same)
  bool wide = epi_warps ? epi_warps == 16 : nstages <= kShortStages * nblk;
  if (const char* e = getenv("TAGPU_EPILOGUE_WARPS")) {
    const int w = atoi(e);
    if (w == 8 || w == 16) wide = w == 16;
  }
  if (wide)
    launch_gemm_ew<S, 16>(views, vstart, nviews, nblk, err, sm_count, wait_ns, st);
  else
    launch_gemm_ew<S, 8>(views, vstart, nviews, nblk, err, sm_count, wait_ns, st);
}

// The persistent served GEMM: all co-resident clusters but `reserve`, which
// stay free for the kernels that prepare requests.
template <int S>
void launch_served_t(const QueueArgs* qa, int* err, int sm_count, int reserve,
                     unsigned long long wait_ns, cudaStream_t st) {
  const int clusters = std::max(1, gemm_clusters<S, true, 8>(sm_count) - reserve);
  ozaki_gemm_kernel<S, true, 8><<<(unsigned)(2 * clusters), Epi<8>::kThreads, Smem<S, 8>::kBytes,
                                  st>>>(nullptr, nullptr, 0, 0, err, wait_ns, qa);
  count_launch();
}

// Dynamic shared memory of a split CTA: S staged slices of ROWS x 32 digits.
constexpr int split_smem(int S, int rows) { return S * 4 * (rows + 1) * 16; }

template <int S>
void launch_split_t(const SplitJob* d_jobs, int njobs, int64_t total, bool a_side,
                    int sm_count, cudaStream_t st) {
  // the shared-memory attribute and the residency are per device
  static bool set[kMaxDevices] = {};
  static int resident[kMaxDevices][2] = {};
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev < 0 || dev >= kMaxDevices) dev = 0;
  if (!set[dev]) {
    cudaFuncSetAttribute(split_kernel<S, BM>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         split_smem(S, BM));
    cudaFuncSetAttribute(split_kernel<S, BN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         split_smem(S, BN));
    int ra = 0, rb = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ra, split_kernel<S, BM>, 256, split_smem(S, BM));
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&rb, split_kernel<S, BN>, 256, split_smem(S, BN));
    resident[dev][0] = std::max(ra, 1);
    resident[dev][1] = std::max(rb, 1);
    set[dev] = true;
  }
  if (total <= 0 || njobs <= 0) return;
  // one wave of resident CTAs, each striding over the bricks
  const int grid = (int)std::min<int64_t>(total, (int64_t)sm_count * resident[dev][a_side ? 0 : 1]);
  if (a_side)
    split_kernel<S, BM><<<grid, 256, split_smem(S, BM), st>>>(d_jobs, njobs, total);
  else
    split_kernel<S, BN><<<grid, 256, split_smem(S, BN), st>>>(d_jobs, njobs, total);
  count_launch();
}

// Splits of a table of jobs of one side (A: 128-row bricks, B: 64-column).
void launch_split(int S, const SplitJob* d_jobs, int njobs, int64_t total, bool a_side,
                  int sm_count, cudaStream_t st) {
  switch (S) {
    case 2: launch_split_t<2>(d_jobs, njobs, total, a_side, sm_count, st); break;
    case 3: launch_split_t<3>(d_jobs, njobs, total, a_side, sm_count, st); break;
    case 4: launch_split_t<4>(d_jobs, njobs, total, a_side, sm_count, st); break;
    case 5: launch_split_t<5>(d_jobs, njobs, total, a_side, sm_count, st); break;
    case 7: launch_split_t<7>(d_jobs, njobs, total, a_side, sm_count, st); break;
    default: launch_split_t<6>(d_jobs, njobs, total, a_side, sm_count, st); break;
  }
}

// Frames of a table of jobs with `items` work items in all.
void launch_frames(const FrameJob* d_jobs, int njobs, int64_t items, cudaStream_t s) {
  if (items <= 0 || njobs <= 0) return;
  frame_kernel<<<(unsigned)items, 256, 0, s>>>(d_jobs, njobs);
  count_launch();
}

void index_maps(const int32_t* sz, int64_t n, std::vector<int32_t>& tile,
                std::vector<int32_t>& local, std::vector<int32_t>& start) {
  tile.clear();
  local.clear();
  start.assign(n + 1, 0);
  for (int64_t t = 0; t < n; ++t) {
    start[t + 1] = start[t] + sz[t];
    for (int32_t x = 0; x < sz[t]; ++x) {
      tile.push_back((int32_t)t);
      local.push_back(x);
    }
  }
}

}  // namespace

// Scheduling order of the units (pairs of output blocks).
// Units are sorted by row chunk, then by super-tiles of gr row blocks x gc
// column-block pairs (with 76 clusters, 4 x 19 is one wave), so clusters
// running together share A bricks (gc ways, on top of the pair's multicast)
// and B bricks (gr ways) in L2.  Results do not depend on the schedule: the
// order of every block's sums is fixed by its own unit's k list.
tagpu_status ozaki_schedule(OzakiPlan* pl, int gr, int gc, std::string* err) {
  if (gr < 1 || gc < 1) {
    *err = "bad emulated-form schedule";
    return TAGPU_ERR_INVALID;
  }
  cudaStream_t s = pl->s;
  pl->tune_gr = gr;
  pl->tune_gc = gc;
  const auto& hb = pl->h_blk;
  const auto& ho = pl->h_off;
  const int64_t nsc = ((pl->CB + 1) / 2 + gc - 1) / gc;   // super-tile columns (pairs)
  const auto& crb = pl->chunk_rb;
  auto chunk_of = [&](int64_t rb) {
    return (int64_t)(std::upper_bound(crb.begin(), crb.end(), rb) - crb.begin()) - 1;
  };
  std::vector<std::pair<std::pair<int64_t, int64_t>, int64_t>> key(pl->nblk);
  for (int64_t b = 0; b < pl->nblk; ++b) {
    const int64_t rb = hb[2 * b], cb = hb[2 * b + 1];
    const int64_t tile = (rb / gr) * nsc + cb / gc;
    key[b] = {{chunk_of(rb), tile * gr * gc + (cb % gc) * gr + (rb % gr)}, b};
  }
  std::sort(key.begin(), key.end());
  std::vector<int32_t> nb(2 * pl->nblk);
  std::vector<int64_t> rng(2 * pl->nblk);
  pl->chunk_blk.assign(pl->nchunk + 1, pl->nblk);
  for (int64_t i = pl->nblk - 1; i >= 0; --i) pl->chunk_blk[key[i].first.first] = i;
  for (int c = pl->nchunk - 1; c >= 0; --c)
    pl->chunk_blk[c] = std::min(pl->chunk_blk[c], pl->chunk_blk[c + 1]);
  for (int64_t i = 0; i < pl->nblk; ++i) {
    const int64_t b = key[i].second;
    nb[2 * i] = hb[2 * b];
    nb[2 * i + 1] = hb[2 * b + 1];
    rng[2 * i] = ho[b];
    rng[2 * i + 1] = ho[b + 1];
  }
  if (pl->nblk) {
    cudaMemcpyAsync(pl->blk, nb.data(), nb.size() * 4, cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(pl->blk_rng, rng.data(), rng.size() * 8, cudaMemcpyHostToDevice, s);
  }
  // the slot pairs follow the k lists, which did not move
  if (pl->nchunk > 1) {
    std::vector<OzParams> cp(pl->nchunk, pl->P);
    std::vector<int64_t> cv(2 * pl->nchunk);
    for (int c = 0; c < pl->nchunk; ++c) {
      cp[c].blk = pl->P.blk + 2 * pl->chunk_blk[c];
      cp[c].blk_rng = pl->P.blk_rng + 2 * pl->chunk_blk[c];
      cp[c].nblk = pl->chunk_blk[c + 1] - pl->chunk_blk[c];
      cp[c].a_slot_base = pl->chunk_slot[c];
      cp[c].unitM = pl->P.unitM + 2 * pl->chunk_blk[c];
      cv[2 * c] = 0;
      cv[2 * c + 1] = cp[c].nblk;
    }
    cudaMemcpyAsync(pl->d_chunk_params, cp.data(), cp.size() * sizeof(OzParams),
                    cudaMemcpyHostToDevice, s);
    cudaMemcpyAsync(pl->d_chunk_vstart, cv.data(), cv.size() * 8, cudaMemcpyHostToDevice, s);
  }
  const int64_t vs[2] = {0, pl->nblk};
  cudaMemcpyAsync(pl->d_params, &pl->P, sizeof(OzParams), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(pl->d_vstart, vs, sizeof(vs), cudaMemcpyHostToDevice, s);
  const cudaError_t ce = cudaStreamSynchronize(s);
  if (ce != cudaSuccess) {
    *err = std::string("ozaki schedule: ") + cudaGetErrorString(ce);
    return TAGPU_ERR_CUDA;
  }
  return TAGPU_OK;
}

// Plan: index maps, brick maps, block lists, scratch.  Host reads back only
// the counts that size the allocations.
tagpu_status ozaki_plan(cudaStream_t s, const GemmView& v, const int32_t* h_msz,
                        const int32_t* h_nsz, const int32_t* h_ksz, int slices,
                        OzakiPlan** out, std::string* err) {
  if (slices < 2 || slices > 7) {
    *err = "emulated form supports 2..7 slices";
    return TAGPU_ERR_INVALID;
  }
  auto pl = std::make_unique<OzakiPlan>();
  pl->s = s;
  pl->S = slices;
  std::vector<int32_t> rt, rl, rs, kt_, kl, ks, ct, cl, cs;
  index_maps(h_msz, v.Mt, rt, rl, rs);
  std::vector<int32_t> c0a(1, 0), c0b(1, 0);
  for (int64_t i = 0; i < v.Mt; ++i)
    c0a.push_back(c0a.back() + (h_msz[i] + kFrameRows - 1) / kFrameRows);
  for (int64_t j = 0; j < v.Nt; ++j)
    c0b.push_back(c0b.back() + (h_nsz[j] + kFrameRows - 1) / kFrameRows);
  pl->frame_items_a = (int64_t)c0a.back() * v.Kt;
  pl->frame_items_b = (int64_t)c0b.back() * v.Kt;
  index_maps(h_ksz, v.Kt, kt_, kl, ks);
  index_maps(h_nsz, v.Nt, ct, cl, cs);
  pl->M_total = (int64_t)rt.size();
  pl->K_total = (int64_t)kt_.size();
  pl->N_total = (int64_t)ct.size();
  if (pl->M_total == 0 || pl->N_total == 0 || pl->K_total == 0) {
    *err = "empty GEMM";
    return TAGPU_ERR_INVALID;
  }
  if (pl->K_total > (1ll << 18)) {
    *err = "emulated form: contracted extent above 262144 (the top level would leave the "
           "exact fp32 range)";
    return TAGPU_ERR_UNSUPPORTED;
  }
  pl->RB = (pl->M_total + BM - 1) / BM;
  pl->CB = (pl->N_total + BN - 1) / BN;
  pl->KB = (pl->K_total + BK - 1) / BK;
  auto extents = [](const std::vector<int32_t>& tile, const int32_t* sz) {
    std::vector<int32_t> e(tile.size());
    for (size_t i = 0; i < tile.size(); ++i) e[i] = sz[tile[i]];
    return e;
  };
  tagpu_status st;
  const std::vector<int32_t> row_e = extents(rt, h_msz), k_e = extents(kt_, h_ksz),
                             col_e = extents(ct, h_nsz);
  if ((st = pl->upload_many({{&pl->row_ext, &row_e}, {&pl->k_ext, &k_e}, {&pl->col_ext, &col_e},
                             {&pl->row_tile, &rt}, {&pl->row_local, &rl}, {&pl->rstart, &rs},
                             {&pl->k_tile, &kt_}, {&pl->k_local, &kl}, {&pl->col_tile, &ct},
                             {&pl->col_local, &cl}, {&pl->cstart, &cs}},
                            err)) ||
      (st = pl->alloc(&pl->EA, pl->M_total, err)) || (st = pl->alloc(&pl->EB, pl->N_total, err)) ||
      (st = pl->alloc(&pl->err, 1, err)))
    return st;
  // operand views in (rows, k) form
  OperandView& a = pl->va;
  a.data = v.A;
  a.off = v.aoff;
  a.rowt = v.Mt;
  a.kt = v.Kt;
  a.off_stride_row = v.Kt;
  a.off_stride_k = 1;
  a.rsz = v.msz;
  a.ksz = v.ksz;
  a.row_contig = v.a_trans;  // trans: tile stored k x m, rows contiguous
  a.hel = v.hel;
  OperandView& b = pl->vb;
  b.data = v.B;
  b.off = v.boff;
  b.rowt = v.Nt;
  b.kt = v.Kt;
  b.off_stride_row = 1;       // boff index = k * Nt + n
  b.off_stride_k = v.Nt;
  b.rsz = v.nsz;
  b.ksz = v.ksz;
  b.row_contig = v.b_trans ? 0 : 1;  // k x n storage: rows (n) contiguous
  b.hel = v.hel;
  // brick maps: A and B flag passes, one host read of both counts
  int64_t *flag = nullptr, *scan = nullptr, *flag_b = nullptr, *scan_b0 = nullptr;
  const int64_t nfa = pl->RB * pl->KB, nfb = pl->CB * pl->KB;
  if ((st = pl->alloc(&flag, nfa, err)) || (st = pl->alloc(&scan, nfa + 1, err)) ||
      (st = pl->alloc(&flag_b, nfb, err)) || (st = pl->alloc(&scan_b0, nfb + 1, err)) ||
      (st = pl->alloc(&pl->brickA, nfa, err)) || (st = pl->alloc(&pl->listA, 2 * nfa, err)) ||
      (st = pl->alloc(&pl->brickB, nfb, err)) || (st = pl->alloc(&pl->listB, 2 * nfb, err)))
    return st;
  brick_flag_kernel<<<blocks_for(nfa, 256), 256, 0, s>>>(a, pl->row_tile, pl->k_tile, pl->M_total,
                                                         pl->K_total, BM, pl->RB, pl->KB, flag);
  count_launch();
  launch_exclusive_scan(s, flag, nfa, scan);
  brick_slot_kernel<<<blocks_for(nfa, 256), 256, 0, s>>>(flag, scan, nfa, pl->KB, pl->brickA,
                                                         pl->listA, 0);
  count_launch();
  // B bricks are indexed (k block, column block) in the GEMM; the flag pass
  // runs over (column block, k block) and the slots are written transposed
  brick_flag_kernel<<<blocks_for(nfb, 256), 256, 0, s>>>(b, pl->col_tile, pl->k_tile,
                                                         pl->N_total, pl->K_total, BN, pl->CB,
                                                         pl->KB, flag_b);
  count_launch();
  launch_exclusive_scan(s, flag_b, nfb, scan_b0);
  brick_slot_kernel<<<blocks_for(nfb, 256), 256, 0, s>>>(flag_b, scan_b0, nfb, pl->KB,
                                                         pl->brickB, pl->listB, pl->CB);
  count_launch();
  cudaMemcpyAsync(&pl->nA, scan + nfa, 8, cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(&pl->nB, scan_b0 + nfb, 8, cudaMemcpyDeviceToHost, s);
  cudaStreamSynchronize(s);
  if ((st = pl->alloc(&pl->hdrA, pl->nA, err)) || (st = pl->alloc(&pl->hdrB, pl->nB, err)))
    return st;
  if (pl->nA) {
    brick_hdr_kernel<<<blocks_for(pl->nA, 256), 256, 0, s>>>(
        pl->listA, pl->nA, pl->row_tile, pl->k_tile, pl->M_total, pl->K_total, BM, pl->hdrA);
    count_launch();
  }
  if (pl->nB) {
    brick_hdr_kernel<<<blocks_for(pl->nB, 256), 256, 0, s>>>(
        pl->listB, pl->nB, pl->col_tile, pl->k_tile, pl->N_total, pl->K_total, BN, pl->hdrB);
    count_launch();
  }
  // units (pairs of output blocks) and their k-block lists
  const int64_t CP = (pl->CB + 1) / 2;
  const int64_t nob = pl->RB * CP;
  int64_t *counts = nullptr, *scan_c = nullptr, *bflag = nullptr, *scan_b = nullptr;
  if ((st = pl->alloc(&counts, nob, err)) || (st = pl->alloc(&scan_c, nob + 1, err)) ||
      (st = pl->alloc(&bflag, nob, err)) || (st = pl->alloc(&scan_b, nob + 1, err)))
    return st;
  block_kernel<<<blocks_for(nob * 32, 256), 256, 0, s>>>(
      pl->brickA, pl->brickB, pl->row_tile, pl->col_tile, v.coff, v.Nt, pl->M_total, pl->N_total,
      pl->RB, pl->CB, pl->KB, nullptr, counts, nullptr);
  count_launch();
  launch_exclusive_scan(s, counts, nob, scan_c);
  flag_nonzero_kernel<<<blocks_for(nob, 256), 256, 0, s>>>(counts, nob, bflag);
  count_launch();
  launch_exclusive_scan(s, bflag, nob, scan_b);
  cudaMemcpyAsync(&pl->nkb, scan_c + nob, 8, cudaMemcpyDeviceToHost, s);
  cudaMemcpyAsync(&pl->nblk, scan_b + nob, 8, cudaMemcpyDeviceToHost, s);
  cudaStreamSynchronize(s);
  if ((st = pl->alloc(&pl->blk, 2 * pl->nblk, err)) ||
      (st = pl->alloc(&pl->blk_off, pl->nblk + 1, err)) ||
      (st = pl->alloc(&pl->blk_kb, pl->nkb, err)))
    return st;
  block_kernel<<<blocks_for(nob * 32, 256), 256, 0, s>>>(
      pl->brickA, pl->brickB, pl->row_tile, pl->col_tile, v.coff, v.Nt, pl->M_total, pl->N_total,
      pl->RB, pl->CB, pl->KB, scan_c, counts, pl->blk_kb);
  count_launch();
  block_list_kernel<<<blocks_for(nob, 256), 256, 0, s>>>(counts, scan_b, nob, CP, pl->blk);
  count_launch();
  gather_offsets_kernel<<<blocks_for(nob, 256), 256, 0, s>>>(counts, scan_c, scan_b, nob,
                                                             pl->blk_off);
  count_launch();
  if ((st = pl->alloc(&pl->blk_ab, pl->nkb, err))) return st;
  if (pl->nblk) {
    slot_pairs_kernel<<<blocks_for(pl->nblk * 32, 256), 256, 0, s>>>(
        pl->blk, pl->blk_off, pl->nblk, pl->blk_kb, pl->brickA, pl->brickB, pl->KB, pl->CB,
        pl->row_tile, pl->col_tile, v.coff, v.Nt, pl->M_total, pl->N_total, (int32_t)pl->nB,
        pl->blk_ab);
    count_launch();
  }
  // Row chunking: when the A bricks would not fit next to everything else,
  // they are built and consumed one range of row blocks at a time.
  const size_t a_brick = (size_t)slices * A_SLICE_BYTES, b_brick = (size_t)slices * B_SLICE_BYTES;
  std::vector<int64_t> chunk_rb{0, pl->RB};
  pl->chunk_slot = {0, pl->nA};
  {
    size_t free_b = 0, total_b = 0;
    cudaMemGetInfo(&free_b, &total_b);
    size_t budget = free_b / 2;
    if (const char* e = getenv("TAGPU_OZAKI_A_BYTES")) budget = (size_t)atof(e);
    budget = std::max<size_t>(budget, a_brick * (size_t)pl->KB);  // at least one row block
    if (a_brick * (size_t)pl->nA > budget && pl->nA > 0) {
      std::vector<int32_t> la(2 * pl->nA);
      cudaMemcpyAsync(la.data(), pl->listA, la.size() * 4, cudaMemcpyDeviceToHost, s);
      cudaStreamSynchronize(s);
      chunk_rb = {0};
      pl->chunk_slot = {0};
      const int64_t per = (int64_t)(budget / a_brick);
      for (int64_t x = 0; x < pl->nA; ++x) {
        if (x - pl->chunk_slot.back() >= per && (x == 0 || la[2 * x] != la[2 * (x - 1)])) {
          pl->chunk_slot.push_back(x);
          chunk_rb.push_back(la[2 * x]);
        }
      }
      pl->chunk_slot.push_back(pl->nA);
      chunk_rb.push_back(pl->RB);
    }
    pl->nchunk = (int)pl->chunk_slot.size() - 1;
  }
  pl->chunk_rb = chunk_rb;
  pl->h_blk.resize(2 * pl->nblk);
  pl->h_off.resize(pl->nblk + 1);
  if (pl->nblk) {
    cudaMemcpyAsync(pl->h_blk.data(), pl->blk, pl->h_blk.size() * 4, cudaMemcpyDeviceToHost, s);
    cudaMemcpyAsync(pl->h_off.data(), pl->blk_off, pl->h_off.size() * 8, cudaMemcpyDeviceToHost,
                    s);
    cudaStreamSynchronize(s);
  }
  if ((st = pl->alloc(&pl->blk_rng, 2 * pl->nblk, err))) return st;
  // operand slices (A: the largest chunk)
  int64_t max_slots = 0;
  for (int c = 0; c < pl->nchunk; ++c)
    max_slots = std::max(max_slots, pl->chunk_slot[c + 1] - pl->chunk_slot[c]);
  if ((st = pl->alloc(&pl->Apack, a_brick * max_slots, err)) ||
      (st = pl->alloc(&pl->Bpack, b_brick * (pl->nB + 1), err)))
    return st;
  if ((st = pl->alloc(&pl->shiftA, pl->nA, err)) ||
      (st = pl->alloc(&pl->shiftB, pl->nB + 1, err)) ||
      (st = pl->alloc(&pl->unitM, 2 * pl->nblk, err)) || (st = pl->alloc(&pl->products, 1, err)))
    return st;
  // brick nB: all digits zero, read by a unit's column block where it has no
  // B brick of its own; its shift marks it empty (0x3F3F3F3F >= kNoShift)
  cudaMemsetAsync(pl->Bpack + b_brick * pl->nB, 0, b_brick, s);
  cudaMemsetAsync(pl->shiftB + pl->nB, 0x3F, sizeof(int32_t), s);
  cudaError_t ce = cudaGetLastError();
  if (ce != cudaSuccess) {
    *err = std::string("ozaki planning: ") + cudaGetErrorString(ce);
    return TAGPU_ERR_CUDA;
  }
  OzParams& P = pl->P;
  P.Apack = pl->Apack;
  P.Bpack = pl->Bpack;
  P.brickA = pl->brickA;
  P.brickB = pl->brickB;
  P.blk = pl->blk;
  P.blk_rng = pl->blk_rng;
  P.blk_ab = pl->blk_ab;
  P.nblk = pl->nblk;
  P.KBn = (int)pl->KB;
  P.CB = (int)pl->CB;
  P.EA = pl->EA;
  P.EB = pl->EB;
  P.row_tile = pl->row_tile;
  P.row_local = pl->row_local;
  P.col_tile = pl->col_tile;
  P.col_local = pl->col_local;
  P.msz = v.msz;
  P.nsz = v.nsz;
  P.Nt = v.Nt;
  P.coff = v.coff;
  P.hel = v.hel;
  P.alpha = v.alpha;
  P.C = v.C;
  P.M_total = pl->M_total;
  P.N_total = pl->N_total;
  P.err = pl->err;
  P.a_slot_base = 0;
  P.shiftA = pl->shiftA;
  P.shiftB = pl->shiftB;
  P.unitM = pl->unitM;
  P.products = pl->products;
  if (pl->nchunk > 1 && ((st = pl->alloc(&pl->d_chunk_params, pl->nchunk, err)) ||
                         (st = pl->alloc(&pl->d_chunk_vstart, 2 * pl->nchunk, err))))
    return st;
  if ((st = pl->alloc(&pl->d_params, 1, err)) || (st = pl->alloc(&pl->d_vstart, 2, err)))
    return st;
  if ((st = ozaki_schedule(pl.get(), pl->tune_gr, pl->tune_gc, err))) return st;
  // work tables of the frame and split launches
  if ((st = pl->upload(&pl->chunk0_a, c0a, err)) || (st = pl->upload(&pl->chunk0_b, c0b, err)))
    return st;
  pl->h_frames[0] = FrameJob{pl->va, pl->rstart, pl->chunk0_a, pl->EA, 0};
  pl->h_frames[1] = FrameJob{pl->vb, pl->cstart, pl->chunk0_b, pl->EB, pl->frame_items_a};
  pl->h_split_b = SplitJob{pl->vb,      pl->col_tile, pl->col_local, pl->k_tile,
                           pl->k_local, pl->col_ext,  pl->k_ext,     pl->EB,
                           pl->N_total, pl->K_total,  pl->listB,     pl->hdrB,
                           pl->nB,      pl->Bpack,    pl->shiftB,    0};
  pl->h_split_a.clear();
  for (int c = 0; c < pl->nchunk; ++c)
    pl->h_split_a.push_back(SplitJob{pl->va, pl->row_tile, pl->row_local, pl->k_tile,
                                     pl->k_local, pl->row_ext, pl->k_ext, pl->EA, pl->M_total,
                                     pl->K_total, pl->listA + 2 * pl->chunk_slot[c],
                                     pl->hdrA + pl->chunk_slot[c],
                                     pl->chunk_slot[c + 1] - pl->chunk_slot[c], pl->Apack,
                                     pl->shiftA + pl->chunk_slot[c], 0});
  {
    const std::vector<FrameJob> fj(pl->h_frames, pl->h_frames + 2);
    const std::vector<SplitJob> sb(1, pl->h_split_b);
    if ((st = pl->upload(&pl->d_frames, fj, err)) || (st = pl->upload(&pl->d_split_b, sb, err)) ||
        (st = pl->upload(&pl->d_split_a, pl->h_split_a, err)))
      return st;
  }
  *out = pl.release();
  return TAGPU_OK;
}

// Frames, splitting and the GEMM; no host synchronisation.
void ozaki_enqueue(OzakiPlan* pl, int sm_count, cudaStream_t s) {
  cudaMemsetAsync(pl->EA, 0, pl->M_total * 4, s);
  cudaMemsetAsync(pl->EB, 0, pl->N_total * 4, s);
  cudaMemsetAsync(pl->err, 0, 4, s);
  cudaMemsetAsync(pl->products, 0, sizeof(unsigned long long), s);
  launch_frames(pl->d_frames, 2, pl->frame_items_a + pl->frame_items_b, s);
  launch_split(pl->S, pl->d_split_b, 1, pl->nB, false, sm_count, s);
  // chunked plans split A chunk by chunk inside ozaki_enqueue_gemm
  if (pl->nchunk == 1) launch_split(pl->S, pl->d_split_a, 1, pl->nA, true, sm_count, s);
}

void ozaki_enqueue_gemm_views(const void* d_params, const int64_t* d_vstart, int nviews,
                              int64_t nblk, int64_t nstages, int slices, int* d_err,
                              int sm_count, unsigned long long wait_ns, cudaStream_t s,
                              int epi_warps) {
  const OzParams* v = static_cast<const OzParams*>(d_params);
  const int64_t k = nstages;
  const int w = epi_warps;
  switch (slices) {
    case 2: launch_gemm_t<2>(v, d_vstart, nviews, nblk, k, w, d_err, sm_count, wait_ns, s); break;
    case 3: launch_gemm_t<3>(v, d_vstart, nviews, nblk, k, w, d_err, sm_count, wait_ns, s); break;
    case 4: launch_gemm_t<4>(v, d_vstart, nviews, nblk, k, w, d_err, sm_count, wait_ns, s); break;
    case 5: launch_gemm_t<5>(v, d_vstart, nviews, nblk, k, w, d_err, sm_count, wait_ns, s); break;
    case 7: launch_gemm_t<7>(v, d_vstart, nviews, nblk, k, w, d_err, sm_count, wait_ns, s); break;
    default: launch_gemm_t<6>(v, d_vstart, nviews, nblk, k, w, d_err, sm_count, wait_ns, s); break;
  }
}

void ozaki_enqueue_gemm(OzakiPlan* pl, int sm_count, cudaStream_t s) {
  if (pl->nchunk == 1) {
    ozaki_enqueue_gemm_views(pl->d_params, pl->d_vstart, 1, pl->nblk, pl->nkb, pl->S, pl->err,
                             sm_count, pl->wait_ns, s, pl->epi_warps);
    return;
  }
  for (int c = 0; c < pl->nchunk; ++c) {
    launch_split(pl->S, pl->d_split_a + c, 1, pl->h_split_a[c].nbricks, true, sm_count, s);
    // a chunk's units take the plan's average stage count
    const int64_t units = pl->chunk_blk[c + 1] - pl->chunk_blk[c];
    const int64_t stages = pl->nblk ? (int64_t)((double)pl->nkb * units / pl->nblk) : 0;
    ozaki_enqueue_gemm_views(pl->d_chunk_params + c, pl->d_chunk_vstart + 2 * c, 1, units,
                             stages, pl->S, pl->err, sm_count, pl->wait_ns, s, pl->epi_warps);
  }
}

int ozaki_chunks(const OzakiPlan* pl) { return pl->nchunk; }

int64_t ozaki_stages(const OzakiPlan* pl) { return pl->nkb; }

namespace {
template <typename T>
void append_bytes(std::vector<uint8_t>* out, const T& x) {
  const uint8_t* p = reinterpret_cast<const uint8_t*>(&x);
  out->insert(out->end(), p, p + sizeof(T));
}
}  // namespace

void ozaki_group_tables(OzakiPlan* const* pls, int n, std::vector<uint8_t>* zero_jobs,
                        std::vector<uint8_t>* frame_jobs, std::vector<uint8_t>* split_a,
                        std::vector<uint8_t>* split_b, OzGroupDims* d) {
  zero_jobs->clear();
  frame_jobs->clear();
  split_a->clear();
  split_b->clear();
  *d = OzGroupDims{};
  for (int i = 0; i < n; ++i) {
    OzakiPlan* pl = pls[i];
    append_bytes(zero_jobs, ZeroJob{pl->EA, pl->M_total});
    append_bytes(zero_jobs, ZeroJob{pl->EB, pl->N_total});
    append_bytes(zero_jobs, ZeroJob{pl->err, 1});
    append_bytes(zero_jobs, ZeroJob{reinterpret_cast<int32_t*>(pl->products), 2});
    d->nzero += 4;
    for (int x = 0; x < 2; ++x) {
      FrameJob f = pl->h_frames[x];
      f.item0 = d->frame_items;
      d->frame_items += x == 0 ? pl->frame_items_a : pl->frame_items_b;
      append_bytes(frame_jobs, f);
      ++d->nframe;
    }
    SplitJob a = pl->h_split_a[0];
    a.brick0 = d->split_a_bricks;
    d->split_a_bricks += a.nbricks;
    append_bytes(split_a, a);
    ++d->nsplit_a;
    SplitJob b = pl->h_split_b;
    b.brick0 = d->split_b_bricks;
    d->split_b_bricks += b.nbricks;
    append_bytes(split_b, b);
    ++d->nsplit_b;
  }
}

void ozaki_group_enqueue(const void* zero_jobs, const void* frame_jobs, const void* split_a,
                         const void* split_b, const OzGroupDims& d, int S, int sm_count,
                         cudaStream_t s) {
  if (d.nzero > 0) {
    zero_kernel<<<(unsigned)d.nzero, 256, 0, s>>>(static_cast<const ZeroJob*>(zero_jobs));
    count_launch();
  }
  launch_frames(static_cast<const FrameJob*>(frame_jobs), d.nframe, d.frame_items, s);
  launch_split(S, static_cast<const SplitJob*>(split_b), d.nsplit_b, d.split_b_bricks, false,
               sm_count, s);
  launch_split(S, static_cast<const SplitJob*>(split_a), d.nsplit_a, d.split_a_bricks, true,
               sm_count, s);
}

// Autotuner: times the schedules of the emulated GEMM on the contraction
// itself (frames and digit bricks built once), keeps the fastest, and caches
// the choice per shape bucket (slices, log2 of the fused extents, density
// decile) in a text file, one "bucket gr gc chunk ms" line per bucket.
namespace {
std::string tune_bucket(const OzakiPlan* pl) {
  auto l2 = [](int64_t x) {
    int b = 0;
    while ((int64_t(1) << (b + 1)) <= x) ++b;
    return b;
  };
  const double dens = pl->nblk ? (double)pl->nkb / ((double)pl->nblk * (double)pl->KB) : 0.0;
  char buf[128];
  snprintf(buf, sizeof(buf), "S%d_M%d_N%d_K%d_d%d", pl->S, l2(pl->M_total), l2(pl->N_total),
           l2(pl->K_total), (int)(dens * 10));
  return buf;
}
}  // namespace

tagpu_status ozaki_autotune(OzakiPlan* pl, int sm_count, cudaStream_t s, const char* cache,
                            std::string* log, std::string* err) {
  const std::string key = tune_bucket(pl);
  if (cache && *cache) {
    if (FILE* f = fopen(cache, "r")) {
      char line[256];
      while (fgets(line, sizeof(line), f)) {
        char k[128], extra[8];
        int gr, gc, ew = 0;
        double ms;
        // "bucket rows cols ms epilogue-warps" (lines without the width
        // leave it to the stage count)
        const int n = sscanf(line, "%127s %d %d %lf %d %7s", k, &gr, &gc, &ms, &ew, extra);
        if ((n == 4 || n == 5) && key == k) {
          fclose(f);
          if (log) *log = "cached " + key;
          pl->epi_warps = n == 5 && (ew == 8 || ew == 16) ? ew : 0;
          return ozaki_schedule(pl, gr, gc, err);
        }
      }
      fclose(f);
    }
  }
  ozaki_enqueue(pl, sm_count, s);  // frames and bricks for the timing runs
  pl->epi_warps = 0;               // the block orders are timed with the width by stage count
  const int shapes[][2] = {{4, 19}, {2, 38}, {8, 10}, {1, 76}, {19, 4}, {6, 13}, {3, 25}, {12, 6}};
  std::string all;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  int bgr = pl->tune_gr, bgc = pl->tune_gc;
  tagpu_status st = TAGPU_OK;
  for (const auto& sh : shapes) {
    if ((st = ozaki_schedule(pl, sh[0], sh[1], err))) break;
    float t = 1e30f;
    for (int rep = 0; rep < 2; ++rep) {
      cudaEventRecord(e0, s);
      ozaki_enqueue_gemm(pl, sm_count, s);
      cudaEventRecord(e1, s);
      cudaEventSynchronize(e1);
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      t = std::min(t, ms);
    }
    char one[64];
    snprintf(one, sizeof(one), " %dx%d:%.3f", sh[0], sh[1], t);
    all += one;
    if (t < best) {
      best = t;
      bgr = sh[0];
      bgc = sh[1];
    }
  }
  if (st) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return st;
  }
  if ((st = ozaki_schedule(pl, bgr, bgc, err))) {
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return st;
  }
  // the epilogue width: the best order above ran with the width the stage
  // count picks; time the other one on it and keep the faster
  const int auto_w = pl->nkb <= kShortStages * pl->nblk ? 16 : 8;
  int best_w = auto_w;
  {
    pl->epi_warps = auto_w == 16 ? 8 : 16;
    float t = 1e30f;
    for (int rep = 0; rep < 2; ++rep) {
      cudaEventRecord(e0, s);
      ozaki_enqueue_gemm(pl, sm_count, s);
      cudaEventRecord(e1, s);
      cudaEventSynchronize(e1);
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      t = std::min(t, ms);
    }
    char one[64];
    snprintf(one, sizeof(one), "; %d warps on %dx%d:%.3f", pl->epi_warps, bgr, bgc, t);
    all += one;
    if (t < best) {
      best = t;
      best_w = pl->epi_warps;
    }
    pl->epi_warps = best_w;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (cache && *cache) {
    if (FILE* f = fopen(cache, "a")) {
      fprintf(f, "%s %d %d %.4f %d\n", key.c_str(), bgr, bgc, best, best_w);
      fclose(f);
    }
  }
  if (log) {
    char buf[256];
    snprintf(buf, sizeof(buf), "tuned %s: super-tile %dx%d, %d epilogue warps, %.3f ms (ms per "
             "shape:", key.c_str(), bgr, bgc, best_w, best);
    *log = std::string(buf) + all + ")";
  }
  if (const char* e = getenv("TAGPU_VERBOSE"))
    if (atoi(e) > 0) fprintf(stderr, "tagpu: %s\n", log ? log->c_str() : all.c_str());
  return TAGPU_OK;
}

size_t ozaki_params_size() { return sizeof(OzParams); }
void ozaki_params(const OzakiPlan* pl, void* out) { *static_cast<OzParams*>(out) = pl->P; }
int ozaki_slices(const OzakiPlan* pl) { return pl->S; }
int* ozaki_error_flag(OzakiPlan* pl) { return pl->err; }

int ozaki_error(OzakiPlan* pl) {
  int e = 0;
  cudaMemcpyAsync(&e, pl->err, 4, cudaMemcpyDeviceToHost, pl->s);
  cudaStreamSynchronize(pl->s);
  return e;
}

size_t ozaki_scratch_bytes(const OzakiPlan* pl) { return pl->bytes; }
void ozaki_set_wait(OzakiPlan* pl, unsigned long long wait_ns) { pl->wait_ns = wait_ns; }

// bf16 flops of the digit-slice MMAs the last run issued (128 x 64 x 32
// multiply-adds per slice product); synchronises.
double ozaki_mma_flops(OzakiPlan* pl) {
  unsigned long long n = 0;
  cudaMemcpyAsync(&n, pl->products, sizeof(n), cudaMemcpyDeviceToHost, pl->s);
  cudaStreamSynchronize(pl->s);
  return (double)n * 2.0 * BM * BN * BK;
}
int64_t ozaki_units(const OzakiPlan* pl) { return pl->nblk; }
void ozaki_destroy(OzakiPlan* pl) { delete pl; }

// ---------------------------------------------------------------------------
// served mode (host side)
// ---------------------------------------------------------------------------
// Control block in mapped, page-locked host memory: the host publishes with
// release stores, the kernel reads with acquire loads (the GPU of this
// system is cache-coherent with host memory).
struct ServeMapped {
  long long published[2];
  int njobs[2];
  int stop;
  int pad;
  int job_done[2 * kQueueJobs];
  QueueJob jobs[2][kQueueJobs];
};

struct OzakiServe {
  int S = 6;
  int sm_count = 0, reserve = 0;
  unsigned long long wait_ns = 4000000000ull;
  cudaStream_t stream = nullptr;     // the persistent kernel's stream
  ServeMapped* h = nullptr;          // host view
  ServeMapped* d = nullptr;          // device view of the same memory
  unsigned long long* claimed = nullptr;
  int* done_units = nullptr;
  int* err = nullptr;
  QueueArgs* d_args = nullptr;
  cudaEvent_t ev = nullptr;          // recorded after each launch
  bool running = false;
  int next_id = 0;
  long long lane_units[2] = {0, 0};
  int lane_jobs[2] = {0, 0};
  ~OzakiServe() {
    if (running && h) {
      __atomic_store_n(&h->stop, 1, __ATOMIC_RELEASE);
      cudaStreamSynchronize(stream);
    }
    if (ev) cudaEventDestroy(ev);
    if (d_args) cudaFree(d_args);
    if (claimed) cudaFree(claimed);
    if (done_units) cudaFree(done_units);
    if (err) cudaFree(err);
    if (h) cudaFreeHost(h);
  }
};

tagpu_status ozaki_serve_create(int S, int sm_count, int reserve, unsigned long long wait_ns,
                                cudaStream_t stream, OzakiServe** out, std::string* err) {
  if (S < 2 || S > 7) {
    *err = "served emulated form supports 2..7 slices";
    return TAGPU_ERR_INVALID;
  }
  auto q = std::make_unique<OzakiServe>();
  q->S = S;
  q->sm_count = sm_count;
  q->reserve = reserve;
  q->wait_ns = wait_ns;
  q->stream = stream;
  void* hp = nullptr;
  if (cudaHostAlloc(&hp, sizeof(ServeMapped), cudaHostAllocMapped) != cudaSuccess) {
    cudaGetLastError();
    *err = "served mode: mapped host control block allocation failed";
    return TAGPU_ERR_NOMEM;
  }
  q->h = static_cast<ServeMapped*>(hp);
  memset(q->h, 0, sizeof(ServeMapped));
  void* dp = nullptr;
  if (cudaHostGetDevicePointer(&dp, hp, 0) != cudaSuccess) {
    cudaGetLastError();
    *err = "served mode: mapped control block has no device address";
    return TAGPU_ERR_CUDA;
  }
  q->d = static_cast<ServeMapped*>(dp);
  if (cudaMalloc(&q->claimed, 2 * sizeof(unsigned long long)) != cudaSuccess ||
      cudaMalloc(&q->done_units, 2 * kQueueJobs * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&q->err, sizeof(int)) != cudaSuccess ||
      cudaMalloc(&q->d_args, sizeof(QueueArgs)) != cudaSuccess) {
    cudaGetLastError();
    *err = "served mode: device allocation failed";
    return TAGPU_ERR_NOMEM;
  }
  QueueArgs a{};
  a.jobs[0] = q->d->jobs[0];
  a.jobs[1] = q->d->jobs[1];
  a.published = q->d->published;
  a.njobs = q->d->njobs;
  a.stop = &q->d->stop;
  a.job_done = q->d->job_done;
  a.claimed = q->claimed;
  a.done_units = q->done_units;
  a.idle_ns = 20000000ull;   // a kernel with nothing to claim for 20 ms exits
  cudaMemcpyAsync(q->d_args, &a, sizeof(a), cudaMemcpyHostToDevice, stream);
  cudaMemsetAsync(q->claimed, 0, 2 * sizeof(unsigned long long), stream);
  cudaMemsetAsync(q->done_units, 0, 2 * kQueueJobs * sizeof(int), stream);
  cudaMemsetAsync(q->err, 0, sizeof(int), stream);
  cudaEventCreateWithFlags(&q->ev, cudaEventDisableTiming);
  if (cudaStreamSynchronize(stream) != cudaSuccess) {
    const cudaError_t ce = cudaGetLastError();
    *err = std::string("served mode setup: ") + cudaGetErrorString(ce);
    return TAGPU_ERR_CUDA;
  }
  *out = q.release();
  return TAGPU_OK;
}

void ozaki_serve_destroy(OzakiServe* q) { delete q; }

// Frames, digit splits and stage shifts of a plan on stream s, for a served
// job (its GEMM runs in the served kernel).  Plans split in row chunks are
// not served.
void ozaki_prepare_served(OzakiPlan* pl, int sm_count, cudaStream_t s) {
  ozaki_enqueue(pl, sm_count, s);
  if (pl->nblk > 0) {
    shift_kernel<<<blocks_for(pl->nblk * 32, 256), 256, 0, s>>>(pl->d_params, pl->d_vstart, 1,
                                                                pl->nblk, pl->S);
    count_launch();
  }
}

int ozaki_serve_publish(OzakiServe* q, OzakiPlan* pl, int lane) {
  if (pl->nblk <= 0) return -2;   // nothing to run: done at once
  if (q->next_id >= 2 * kQueueJobs || q->lane_jobs[lane] >= kQueueJobs) return -1;
  const int id = q->next_id++;
  const int j = q->lane_jobs[lane]++;
  QueueJob& J = q->h->jobs[lane][j];
  J.view = pl->d_params;
  J.first = q->lane_units[lane];
  J.units = pl->nblk;
  J.id = id;
  J.pad = 0;
  q->lane_units[lane] += pl->nblk;
  __atomic_store_n(&q->h->njobs[lane], j + 1, __ATOMIC_RELEASE);
  __atomic_store_n(&q->h->published[lane], q->lane_units[lane], __ATOMIC_RELEASE);
  return id;
}

bool ozaki_serve_done(const OzakiServe* q, int job) {
  return job < 0 || __atomic_load_n(&q->h->job_done[job], __ATOMIC_ACQUIRE) != 0;
}

// Launches the served kernel unless it is running; a kernel that has exited
// reports its error flag (0: it ran out of work, else a bounded wait ran out
// and the jobs it held are lost).
tagpu_status ozaki_serve_kick(OzakiServe* q, int* exited_error, std::string* err) {
  *exited_error = 0;
  if (q->running) {
    const cudaError_t ce = cudaEventQuery(q->ev);
    if (ce == cudaErrorNotReady) return TAGPU_OK;
    q->running = false;
    if (ce != cudaSuccess) {
      cudaGetLastError();
      *err = std::string("served GEMM: ") + cudaGetErrorString(ce);
      return TAGPU_ERR_CUDA;
    }
    int e = 0;
    cudaMemcpyAsync(&e, q->err, sizeof(int), cudaMemcpyDeviceToHost, q->stream);
    cudaMemsetAsync(q->err, 0, sizeof(int), q->stream);
    cudaStreamSynchronize(q->stream);
    *exited_error = e;
  }
  if (*exited_error) return TAGPU_OK;   // the caller fails the lost jobs, then kicks again
  __atomic_store_n(&q->h->stop, 0, __ATOMIC_RELEASE);
  switch (q->S) {
    case 2: launch_served_t<2>(q->d_args, q->err, q->sm_count, q->reserve, q->wait_ns, q->stream); break;
    case 3: launch_served_t<3>(q->d_args, q->err, q->sm_count, q->reserve, q->wait_ns, q->stream); break;
    case 4: launch_served_t<4>(q->d_args, q->err, q->sm_count, q->reserve, q->wait_ns, q->stream); break;
    case 5: launch_served_t<5>(q->d_args, q->err, q->sm_count, q->reserve, q->wait_ns, q->stream); break;
    case 7: launch_served_t<7>(q->d_args, q->err, q->sm_count, q->reserve, q->wait_ns, q->stream); break;
    default: launch_served_t<6>(q->d_args, q->err, q->sm_count, q->reserve, q->wait_ns, q->stream); break;
  }
  const cudaError_t le = cudaGetLastError();
  if (le != cudaSuccess) {
    *err = std::string("served GEMM launch: ") + cudaGetErrorString(le);
    return TAGPU_ERR_CUDA;
  }
  cudaEventRecord(q->ev, q->stream);
  q->running = true;
  return TAGPU_OK;
}

// With no job in flight: the kernel is stopped (it exits at once, nothing is
// left to claim) and the counters go back to zero so the job tables start
// over.
tagpu_status ozaki_serve_reset(OzakiServe* q, std::string* err) {
  if (!q->running && q->next_id == 0) return TAGPU_OK;
  if (q->running) {
    __atomic_store_n(&q->h->stop, 1, __ATOMIC_RELEASE);
    cudaStreamSynchronize(q->stream);
    q->running = false;
  }
  const int used = q->next_id;
  __atomic_store_n(&q->h->published[0], 0ll, __ATOMIC_RELEASE);
  __atomic_store_n(&q->h->published[1], 0ll, __ATOMIC_RELEASE);
  __atomic_store_n(&q->h->njobs[0], 0, __ATOMIC_RELEASE);
  __atomic_store_n(&q->h->njobs[1], 0, __ATOMIC_RELEASE);
  memset(q->h->job_done, 0, sizeof(int) * (size_t)std::max(used, 0));
  cudaMemsetAsync(q->claimed, 0, 2 * sizeof(unsigned long long), q->stream);
  if (used > 0) cudaMemsetAsync(q->done_units, 0, sizeof(int) * (size_t)used, q->stream);
  cudaMemsetAsync(q->err, 0, sizeof(int), q->stream);
  const cudaError_t ce = cudaStreamSynchronize(q->stream);
  q->next_id = 0;
  q->lane_units[0] = q->lane_units[1] = 0;
  q->lane_jobs[0] = q->lane_jobs[1] = 0;
  if (ce != cudaSuccess) {
    *err = std::string("served mode reset: ") + cudaGetErrorString(ce);
    return TAGPU_ERR_CUDA;
  }
  return TAGPU_OK;
}

int ozaki_serve_slices(const OzakiServe* q) { return q->S; }
int ozaki_stage_count(const OzakiPlan* pl) { return (int)std::min<int64_t>(pl->nkb, 1 << 30); }

}  // namespace tagpu
