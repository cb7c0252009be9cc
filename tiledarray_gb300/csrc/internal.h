// Internal declarations shared by the host library (tagpu.cpp) and the
// kernel translation units (*.cu).  Not part of the C ABI.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/tagpu.h"

namespace tagpu {

// cudaMallocAsync from the device's default pool.  The pool keeps freed
// blocks (release threshold: never), and under a mix of very large and small
// requests its free memory can be too fragmented for a large block; on
// failure the stream's pending frees are waited for, the pool's unused memory
// is returned to the device and the allocation is tried once more.
inline cudaError_t pool_alloc(void** p, size_t bytes, cudaStream_t s) {
  cudaError_t e = cudaMallocAsync(p, bytes, s);
  if (e == cudaSuccess) return e;
  cudaGetLastError();
  int dev = 0;
  cudaMemPool_t pool;
  if (cudaStreamSynchronize(s) != cudaSuccess || cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetDefaultMemPool(&pool, dev) != cudaSuccess) {
    cudaGetLastError();
    return e;
  }
  cudaMemPoolTrimTo(pool, 0);
  e = cudaMallocAsync(p, bytes, s);
  if (e != cudaSuccess) cudaGetLastError();
  return e;
}

// Kernel launches made by this library (every launch site counts itself).
void count_launch();
int64_t launch_count();

// Record a message as the context's last error and return `st`.
tagpu_status set_last_error(tagpu_ctx* ctx, tagpu_status st, const char* msg);
// Device ordinal of a context.
int context_device(const tagpu_ctx* ctx);

// ---------------------------------------------------------------------------
// kernel launchers (defined in the .cu files); all asynchronous on `s`
// ---------------------------------------------------------------------------

// (a) SparseShape::gemm screening: float, k ascending, no FMA.
void launch_shape_gemm(cudaStream_t s, int64_t M, int64_t N, int64_t K,
                       const float* L, const float* R, const float* ksz,
                       float abs_factor, float thr, float* C,
                       unsigned long long* zero_count);

// (b) pair list: per-result-tile counts and flops, exclusive scan, emission.
void launch_pair_count(cudaStream_t s, int64_t M, int64_t N, int64_t K,
                       const float* C, float cthr, const float* L, float lthr,
                       const float* R, float rthr, const int32_t* msz,
                       const int32_t* nsz, const int32_t* ksz, int64_t* counts,
                       double* flops);
void launch_exclusive_scan(cudaStream_t s, const int64_t* in, int64_t n,
                           int64_t* out /* n+1 */);
void launch_pair_emit(cudaStream_t s, int64_t M, int64_t N, int64_t K,
                      const float* C, float cthr, const float* L, float lthr,
                      const float* R, float rthr, const int64_t* offsets,
                      int32_t* kidx);

// (c) tile permutation.  Tiles of one array share `perm`; each tile has its
// own extents.  ext: ntiles x rank argument extents; in_off / out_off:
// element offsets; item_start: ntiles+1 prefix sums of per-tile work items.
struct PermuteDesc {
  int rank;
  int perm[8];
};
// Tile-wise sum R = C + P over one run of elements of a result tile
// (c or p < 0: that argument tile is absent and the other is copied).
struct AddChunk {
  int64_t r, c, p, len;
};
// Host <-> device copy of array storage by a kernel over a coherent host
// link; usable when `host` is registered host memory whose address the
// device can dereference on a platform that shares the host page tables.
bool link_copy_usable(const void* host);
void launch_link_copy(cudaStream_t s, void* dst, const void* src, size_t bytes);
void launch_add_tiles(cudaStream_t s, const AddChunk* chunks, int64_t nchunks, const double* C,
                      const double* P, double* R);

void launch_permute(cudaStream_t s, const PermuteDesc& d, int64_t ntiles,
                    const int32_t* ext, const int64_t* in_off,
                    const int64_t* out_off, const int64_t* item_start,
                    int64_t nitems, const double* in, double* out);
// Work items a tile of the given extents needs (host-side helper shared with
// the kernel's decomposition).
int64_t permute_items(const PermuteDesc& d, const int64_t* ext);

// FP64 tensor (DMMA) and FMA rates measured with dependent-chain loops.
tagpu_status measure_fp64_rates(cudaStream_t s, int sm_count, double* dmma_tflops,
                                double* dfma_tflops);
// INT8 (TOP/s) and bf16 (TFLOP/s) rates of the warp-level mma.sync path.
tagpu_status measure_mma_sync_rates(cudaStream_t s, int sm_count, double* imma_tops,
                                    double* hmma_tflops);

// Generation of synthetic operands and sequential tile norms.
struct GenDesc {
  int rank;
  int64_t gext[8];    // global element extents
  uint64_t seed, stream;
  int kind;
};
void launch_generate(cudaStream_t s, const GenDesc& g, int64_t ntiles,
                     const int64_t* tile_lo /* ntiles x rank */,
                     const int32_t* tile_ext /* ntiles x rank */,
                     const int64_t* tile_off /* ntiles+1 prefix */,
                     const double* tile_scale, double* data);
void launch_tile_norms(cudaStream_t s, int64_t ntiles, const int64_t* tile_off,
                       const double* data, float* norms);

// (d) plain FP64 DMMA GEMM over the pair list.
struct GemmView {
  int64_t Mt, Nt, Kt;
  const int32_t* msz;     // Mt fused row sizes
  const int32_t* nsz;     // Nt
  const int32_t* ksz;     // Kt
  const double* A;        // left tile data
  const int64_t* aoff;    // Mt*Kt offsets, -1 absent
  int a_trans;            // tile stored k x m
  const double* B;
  const int64_t* boff;    // Kt*Nt
  int b_trans;            // tile stored n x k
  const int64_t* poff;    // Mt*Nt+1 pair offsets
  const int32_t* kidx;    // pair k
  double alpha;
  double* C;
  const int64_t* coff;    // Mt*Nt result offsets, -1 zero tile
  // general products: this view is element `hel` of a fused-mode slab; the
  // element's matrix inside a tile of extent (fused..., rows, cols) starts
  // hel * rows * cols elements into the tile (0 for ordinary contractions)
  int64_t hel;
};
// One 64x64 output block of one result tile of one contraction.
struct WorkItem {
  int64_t tile;       // result tile ordinal (row-major over Mt x Nt)
  int32_t view;       // index into the GemmView array
  int16_t rb, cb;     // 64-row / 64-column block within the tile
};
void launch_dmma_gemm(cudaStream_t s, const GemmView* views, const WorkItem* items,
                      int64_t nitems, int* err, unsigned long long wait_ns, int sm_count);

// (d) emulated FP64 (Ozaki scheme, bf16 digit slices on tcgen05).
// ozaki_plan sizes and fills the scratch (index maps, brick maps, block
// lists; host synchronises to read counts); ozaki_enqueue runs the frames and
// the digit splitting, ozaki_enqueue_gemm the tensor-core GEMM; neither
// synchronises, so both can be captured in a CUDA graph.
struct OzakiPlan;
tagpu_status ozaki_plan(cudaStream_t s, const GemmView& v, const int32_t* h_msz,
                        const int32_t* h_nsz, const int32_t* h_ksz, int slices,
                        OzakiPlan** out, std::string* err);
void ozaki_enqueue(OzakiPlan* pl, int sm_count, cudaStream_t s);
void ozaki_enqueue_gemm(OzakiPlan* pl, int sm_count, cudaStream_t s);
// One launch over the output blocks of several plans with the same slice
// count: d_params holds their parameter blocks (ozaki_params), d_vstart the
// prefix sums of their block counts; nstages their units' 32-k stages in
// total (it picks the epilogue width unless epi_warps, 8 or 16, fixes it);
// d_err receives a wait timeout (each
// pipeline wait gives up after wait_ns).  Runs the stage-shift pass first.
void ozaki_enqueue_gemm_views(const void* d_params, const int64_t* d_vstart, int nviews,
                              int64_t nblk, int64_t nstages, int slices, int* d_err,
                              int sm_count, unsigned long long wait_ns, cudaStream_t s,
                              int epi_warps = 0);
// 32-k stages over all units of a plan.
int64_t ozaki_stages(const OzakiPlan* pl);
// Number of row chunks (1 unless the A digit bricks would not fit at once;
// chunked plans are launched on their own, not grouped with others).
int ozaki_chunks(const OzakiPlan* pl);
// Times the block-order schedules on this contraction and applies
// the fastest; cache: file of tuned buckets (NULL or "" = no cache).
tagpu_status ozaki_autotune(OzakiPlan* pl, int sm_count, cudaStream_t s, const char* cache,
                            std::string* log, std::string* err);
size_t ozaki_params_size();
void ozaki_params(const OzakiPlan* pl, void* out);
int ozaki_slices(const OzakiPlan* pl);
int* ozaki_error_flag(OzakiPlan* pl);
int ozaki_error(OzakiPlan* pl);   // synchronises; 0 = ok
size_t ozaki_scratch_bytes(const OzakiPlan* pl);
// Bound of the GEMM's pipeline waits for later runs of this plan.
void ozaki_set_wait(OzakiPlan* pl, unsigned long long wait_ns);
// bf16 flops of the digit-slice MMAs the last run issued; synchronises.
double ozaki_mma_flops(OzakiPlan* pl);
// Frames and digit splits of several plans of one digit count (none split in
// row chunks) in one launch per step: the host builds the job tables (bytes
// to upload as they are), the enqueue runs zeroing, frames, B and A splits.
struct OzGroupDims {
  int nzero = 0, nframe = 0, nsplit_a = 0, nsplit_b = 0;
  int64_t frame_items = 0, split_a_bricks = 0, split_b_bricks = 0;
};
void ozaki_group_tables(OzakiPlan* const* pls, int n, std::vector<uint8_t>* zero_jobs,
                        std::vector<uint8_t>* frame_jobs, std::vector<uint8_t>* split_a,
                        std::vector<uint8_t>* split_b, OzGroupDims* d);
void ozaki_group_enqueue(const void* zero_jobs, const void* frame_jobs, const void* split_a,
                         const void* split_b, const OzGroupDims& d, int S, int sm_count,
                         cudaStream_t s);
// Units of the GEMM schedule (a unit is a pair of output blocks run by the
// two CTAs of a cluster); multi-view launches offset their views by these.
int64_t ozaki_units(const OzakiPlan* pl);
void ozaki_destroy(OzakiPlan* pl);
// (unit, k block) stages of a plan: its GEMM work in stages of 32 k.
int ozaki_stage_count(const OzakiPlan* pl);

// Served mode: one persistent emulated GEMM (slice count S) that takes units
// from a work queue.  Jobs (prepared plans) are published into lane 0 (short)
// or lane 1 (long); lane 0 is claimed first.  Every call below is made by one
// host thread.
struct OzakiServe;
// `reserve` co-resident clusters stay free for the kernels preparing requests.
tagpu_status ozaki_serve_create(int S, int sm_count, int reserve, unsigned long long wait_ns,
                                cudaStream_t stream, OzakiServe** out, std::string* err);
void ozaki_serve_destroy(OzakiServe* q);   // stops the kernel, frees the queue
int ozaki_serve_slices(const OzakiServe* q);
// Frames, digit splits and stage shifts of a plan on stream s (no GEMM);
// plans split in row chunks (ozaki_chunks > 1) are not served.
void ozaki_prepare_served(OzakiPlan* pl, int sm_count, cudaStream_t s);
// Publishes a prepared plan; returns its job id, -2 for a plan without units
// (done at once), -1 when the job tables are full (reset first).
int ozaki_serve_publish(OzakiServe* q, OzakiPlan* pl, int lane);
bool ozaki_serve_done(const OzakiServe* q, int job);
// Launches the kernel unless it runs.  *exited_error: the kernel had exited
// with a bounded wait run out (its claimed jobs are lost; reset, then kick).
tagpu_status ozaki_serve_kick(OzakiServe* q, int* exited_error, std::string* err);
// With no job in flight: stops the kernel and restarts the job tables.
tagpu_status ozaki_serve_reset(OzakiServe* q, std::string* err);

}  // namespace tagpu
