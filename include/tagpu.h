/*
 * tagpu — C ABI of the GB300-native block-sparse contraction engine.
 *
 * The engine replaces TiledArray's block-sparse contraction path
 *   C("i,j") = A("i,k") * B("k,j"),  R("a,b,i,j") = V("a,b,c,d") * T("c,d,i,j")
 * on one GPU.  Every entry point is extern "C", takes plain pointers and
 * sizes, and returns a tagpu_status; nothing throws across this boundary.
 * The message of the last failure on a context is tagpu_last_error().
 *
 * Reference interfaces replaced (paths relative to the TiledArray source):
 *   tagpu_init / tagpu_shutdown       TiledArray::initialize / finalize
 *                                     (tiledarray.cpp:84-185)
 *   tagpu_threshold_get / _set        SparseShape<float>::threshold()
 *                                     (sparse_shape.h:548-557, 1941-1942)
 *   tagpu_array_create                DistArray(world, TiledRange[, shape])
 *                                     (dist_array.h:63; tiled_range.h:33;
 *                                      tiled_range1.h:47)
 *   tagpu_array_set_shape             SparseShape(norms, trange[, do_not_scale])
 *                                     (sparse_shape.h:335-348, 407-422)
 *   tagpu_array_upload / _download    DistArray::set / find of Tensor tiles
 *   tagpu_array_generate              make_array with a per-tile norm op
 *                                     (conversions/make_array.h:151-199) over
 *                                     device-generated tiles
 *   tagpu_contract                    TsrExpr::operator= of a contraction
 *                                     (expressions/tsr_expr.h:132-138 ->
 *                                      expr.h:377-430 -> cont_engine.h:354-677
 *                                      -> dist_eval/contraction_eval.h)
 *   tagpu_shape_gemm                  SparseShape::gemm (sparse_shape.h:1589-1684)
 *   tagpu_pair_list                   Summa tile-pair set
 *                                     (dist_eval/contraction_eval.h:630-650,
 *                                      1093-1161, 1348-1384)
 *   tagpu_permute                     Tensor permute (tensor/permute.h:124-210)
 *   tagpu_batch_*                     many independent TsrExpr assignments
 *                                     evaluated together (one persistent launch)
 *   tagpu_server_*                    no counterpart: request loop for served
 *                                     contractions
 *
 * Ownership: arrays are owned by the caller and freed with
 * tagpu_array_destroy; device storage belongs to the context.  Host buffers
 * passed in are copied before the call returns.
 * Threading: a context serialises its own work; tagpu_server_submit may be
 * called from many host threads.
 */
#ifndef TAGPU_H
#define TAGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum tagpu_status {
  TAGPU_OK = 0,
  TAGPU_ERR_INVALID = 1,      /* malformed argument (TA_EXCEPTION analogue) */
  TAGPU_ERR_UNSUPPORTED = 2,  /* expression form not on this path */
  TAGPU_ERR_NOMEM = 3,        /* device allocation failed or over budget */
  TAGPU_ERR_CUDA = 4,         /* CUDA runtime error */
  TAGPU_ERR_TIMEOUT = 5,      /* a bounded device or host wait ran out */
  TAGPU_ERR_REJECTED = 6,     /* server admission rejected the request */
  TAGPU_ERR_NOT_READY = 7,    /* server request still in flight */
  TAGPU_ERR_STATE = 8         /* object used in the wrong state */
} tagpu_status;

typedef enum tagpu_precision {
  TAGPU_PRECISION_FP64 = 0,   /* plain FP64: DMMA (mma.sync f64) */
  TAGPU_PRECISION_OZAKI = 1   /* emulated FP64: exact integer slices on the
                                 tcgen05 tensor cores, FP64 recombination */
} tagpu_precision;

typedef struct tagpu_config {
  int device;                 /* CUDA device ordinal */
  size_t hbm_budget_bytes;    /* 0 = no budget */
} tagpu_config;

typedef struct tagpu_ctx tagpu_ctx;
typedef struct tagpu_array tagpu_array;

tagpu_status tagpu_init(const tagpu_config* cfg, tagpu_ctx** out);
tagpu_status tagpu_shutdown(tagpu_ctx* ctx);
const char* tagpu_last_error(const tagpu_ctx* ctx);
const char* tagpu_status_string(tagpu_status s);
/* Blocks until all work queued on the context has finished. */
tagpu_status tagpu_sync(tagpu_ctx* ctx);

/* CUDA-event timing on the context's stream: start records an event, stop
 * records a second one, waits for it and returns the elapsed milliseconds. */
tagpu_status tagpu_timer_start(tagpu_ctx* ctx);
tagpu_status tagpu_timer_stop(tagpu_ctx* ctx, double* ms);

/* Measured FP64 rates of the context's GPU (TFLOP/s): DMMA (mma.sync f64)
 * and FMA, from short dependent-chain loops (~0.1 s).  No counterpart in the
 * reference; used as the plain form's roofline denominator. */
tagpu_status tagpu_device_fp64_rates(tagpu_ctx* ctx, double* dmma_tflops, double* dfma_tflops);
/* Measured rates of the warp-level tensor path (mma.sync) of the context's
 * GPU: INT8 m16n8k32 (TOP/s) and bf16 m16n8k16 (TFLOP/s), ~0.3 s.  No
 * counterpart in the reference; the evidence for the emulated form's choice
 * of the tcgen05 bf16 path over INT8 (tcgen05 kind::i8 does not exist on
 * sm_103a, leaving INT8 only on mma.sync). */
tagpu_status tagpu_device_mma_sync_rates(tagpu_ctx* ctx, double* imma_tops, double* hmma_tflops);

/* Bound of every pipeline wait inside the emulated GEMM (seconds, default
 * 4).  A wait that runs out makes the kernel abort cleanly (in-flight copies
 * and MMAs finish, tensor memory is released) and the call return
 * TAGPU_ERR_TIMEOUT; the context stays usable.  Applies to contractions
 * planned after the call (a batch keeps the bound it was captured with).
 * No counterpart in the reference. */
tagpu_status tagpu_set_wait_limit(tagpu_ctx* ctx, double seconds);

/* Default screening threshold used for new result shapes; initial value is
 * FLT_EPSILON as in SparseShape<float>. */
float tagpu_threshold_get(const tagpu_ctx* ctx);
void tagpu_threshold_set(tagpu_ctx* ctx, float threshold);

/* ---- arrays --------------------------------------------------------------
 * hashmarks[d] holds ntiles[d]+1 increasing boundaries of dimension d
 * (TiledRange1).  rank <= 8.  A new array is dense (DensePolicy) until a
 * shape is set.  It holds no device memory until it is first written
 * (upload, generate, a shape) or read; an array read before it was written
 * holds zero tiles. */
tagpu_status tagpu_array_create(tagpu_ctx* ctx, int rank, const int64_t* ntiles,
                                const int64_t* const* hashmarks,
                                tagpu_array** out);
tagpu_status tagpu_array_destroy(tagpu_array* a);

/* SparseShape semantics: norms holds one Frobenius norm per tile (tile grid,
 * row-major).  Unless do_not_scale, they are divided by the tile volume;
 * values below `threshold` (negative: the context default) are zeroed.
 * Passing norms == NULL makes the array dense. */
tagpu_status tagpu_array_set_shape(tagpu_array* a, const float* norms,
                                   int do_not_scale, float threshold);

/* Host tiles: the nonzero tiles in tile-ordinal order, each row-major over
 * its own range, concatenated; n = total element count
 * (tagpu_array_info().elements).  Registered host memory (tagpu_host_alloc
 * buffers, or memory the caller registered with CUDA) moves with a copy
 * kernel over a coherent host link; other memory with cudaMemcpyAsync.
 * Both calls return when the copy is complete. */
tagpu_status tagpu_array_upload(tagpu_array* a, const double* tiles, int64_t n);
tagpu_status tagpu_array_download(const tagpu_array* a, double* tiles, int64_t n);

/* Device-side synthetic operand: element with global ordinal g in tile t
 * gets value(seed, stream, g) * tile_scale[t]; kind 0 = uniform[-1,1),
 * kind 1 = integers hash % 101.  Tiles with tile_scale[t] == 0 are absent.
 * tile_scale == NULL means 1 for every tile.  If compute_shape, the shape is
 * set from the device tile norms (make_array semantics) with `threshold`
 * (negative: context default) and tiles below it are dropped. */
tagpu_status tagpu_array_generate(tagpu_array* a, uint64_t seed, uint64_t stream,
                                  int kind, const double* tile_scale,
                                  int compute_shape, float threshold);

/* Pinned host buffers for staging operands and results (no counterpart in
 * the reference, whose tiles live in host memory): anonymous mappings on
 * base pages registered with CUDA (cudaHostAlloc memory where registration
 * fails).  Free with tagpu_host_free. */
tagpu_status tagpu_host_alloc(tagpu_ctx* ctx, size_t bytes, void** p);
tagpu_status tagpu_host_free(tagpu_ctx* ctx, void* p);

/* Archive I/O: DistArray::serialize (dist_array.h:1583-1592, store) and its
 * input form (:1603-1645, load) for a single-rank world, in that order: type
 * tag, world size and rank, TiledRange, shape, stored-tile count, then each
 * stored tile's range and row-major data.  Fixed-width little-endian fields
 * (the layout is written out in tiledarray_gb300/csrc/tagpu.cpp); tiles stream
 * through a pinned staging buffer.  A file that is not such an archive, or
 * whose tiles do not match its shape, is TAGPU_ERR_INVALID. */
tagpu_status tagpu_array_save(const tagpu_array* a, const char* path);
tagpu_status tagpu_array_load(tagpu_ctx* ctx, const char* path, tagpu_array** a);

/* The byte stream DistArray::serialize (dist_array.h:1583-1590) hands a
 * MADNESS binary archive on one rank, for exchange with TiledArray programs:
 * typeid hash of the array type, world size 1, rank 0, the TiledRange
 * (tiled_range.h:392; tiled_range1.h:405; range.h:1143-1157), the shape
 * (SparseShape: norm tensor, tile-extent vectors, zero count,
 * sparse_shape.h:1918-1923; DenseShape: nothing), typeid hash of the pmap
 * type, the tile count and every stored tile as a Tensor<double>
 * (tensor/tensor.h:1389-1416).  The two hash codes belong to the C++
 * implementation of the TiledArray build that reads or wrote the stream:
 * serialize writes the values given, deserialize returns the values read.
 * `sparse` says whether the stream holds a SparseShape (TSpArrayD) or a
 * DenseShape (TArrayD); the stream does not record it.  Multi-rank streams
 * are rejected (one rank's stream holds only that rank's tiles). */
tagpu_status tagpu_array_serialize(const tagpu_array* a, const char* path,
                                   uint64_t array_type_hash, uint64_t pmap_type_hash);
tagpu_status tagpu_array_deserialize(tagpu_ctx* ctx, const char* path, int sparse,
                                     tagpu_array** a, uint64_t* array_type_hash,
                                     uint64_t* pmap_type_hash);

/* TiledArray::truncate (conversions/truncate.h:52-80): the shape is rebuilt
 * from the Frobenius norms of the stored tiles (computed on the device in
 * storage order, as Tensor::norm), scaled by tile volume, with `threshold`
 * (negative: the context default); tiles below it are dropped and the rest
 * compacted in place.  Zero tiles stay zero.  A dense array is left as is. */
tagpu_status tagpu_array_truncate(tagpu_array* a, float threshold);

typedef struct tagpu_array_info {
  int rank;
  int dense;                  /* 1: DensePolicy */
  int64_t ntiles_total;       /* tile-grid volume */
  int64_t nonzero_tiles;
  int64_t zero_tiles;         /* SparseShape zero_tile_count */
  int64_t elements;           /* stored elements (sum of nonzero tile volumes) */
  float threshold;            /* the shape's own threshold */
  size_t device_bytes;
  int64_t ntiles[8];          /* tiles per dimension (first `rank` entries) */
} tagpu_array_info;
tagpu_status tagpu_array_get_info(const tagpu_array* a, tagpu_array_info* info);
/* Scaled tile norms (tile grid, row-major). */
tagpu_status tagpu_array_get_norms(const tagpu_array* a, float* norms);
/* Element offset of every tile in the upload/download buffer, -1 if zero. */
tagpu_status tagpu_array_get_tile_offsets(const tagpu_array* a, int64_t* offsets);
/* One tile to the host: `DistArray::find(i).get()` (dist_array.h:717-733)
 * for tile ordinal `ordinal` (row-major over the tile grid); n must equal the
 * tile's volume.  A zero tile is TAGPU_ERR_INVALID. */
tagpu_status tagpu_array_get_tile(const tagpu_array* a, int64_t ordinal, double* tile,
                                  int64_t n);
/* Tiling of the array: hashmarks of dimension d (ntiles[d]+1 values). */
tagpu_status tagpu_array_get_hashmarks(const tagpu_array* a, int d,
                                       int64_t* hashmarks);

/* ---- contraction -------------------------------------------------------- */
typedef struct tagpu_contract_opts {
  int precision;              /* tagpu_precision */
  int slices;                 /* Ozaki slices per operand, 2..7, 0 = default (7:
                                 55-bit digits; 6 is faster, 47-bit) */
  float threshold;            /* result screening threshold, <0 = default */
  int autotune;               /* emulated form: time the GEMM schedules (block
                                 order, epilogue width) on first use of a
                                 shape bucket and cache the fastest in the file
                                 named by TAGPU_TUNE_CACHE (results do not
                                 depend on the schedule); also enabled by the
                                 environment variable TAGPU_AUTOTUNE=1 */
} tagpu_contract_opts;

typedef struct tagpu_contract_stats {
  int64_t result_tiles;       /* M_t * N_t */
  int64_t nonzero_result_tiles;
  int64_t zero_tiles;         /* result SparseShape zero count */
  int64_t pairs;              /* |tile-pair list| */
  double flops;               /* 2 * sum over pairs of m*k*n */
  double ms_shape;            /* kernel (a) */
  double ms_pairs;            /* kernel (b) */
  double ms_permute;          /* kernel (c), arguments and result */
  double ms_split;            /* Ozaki slicing */
  double ms_gemm;             /* kernel (d) */
  double ms_total;            /* whole call, host wall clock */
  int left_permtype, right_permtype; /* 1 identity, 2 transpose, 3 general */
  int precision;
  int slices;
  int64_t gemm_blocks;        /* output blocks the GEMM ran */
  int64_t gemm_launches;      /* GEMM-phase kernel launches */
  int64_t kernel_launches;    /* every kernel the call launched */
  double mma_flops;           /* emulated form: bf16 flops of the digit-slice
                                 MMAs issued (stages and slice pairs whose
                                 products fall below the kept levels are
                                 not issued) */
} tagpu_contract_stats;

/* c = alpha * A(a_idx) * B(b_idx) with index strings like "i,k".  *c is a new
 * array (the target); the result shape is SparseShape::gemm of the argument
 * shapes with the result threshold.  General (fused-index) products, where an
 * index appears in both arguments and the target (c("b,i,k") =
 * a("b,i,j") * b("b,j,k"), batched outer and Hadamard products included),
 * follow ContEngine's general path: SparseShape::gemm_batched
 * (sparse_shape.h:1707-1885) per fused tile slab, a matrix product per fused
 * element (in the emulated form, one digit-slice GEMM plan per fused
 * element, all of them in grouped launches); they need congruent fused and
 * contracted tilings. */
tagpu_status tagpu_contract(tagpu_ctx* ctx, const char* c_idx, double alpha,
                            tagpu_array* A, const char* a_idx, tagpu_array* B,
                            const char* b_idx, const tagpu_contract_opts* opts,
                            tagpu_array** c);
tagpu_status tagpu_last_stats(const tagpu_ctx* ctx, tagpu_contract_stats* st);

/* c += alpha * A(a_idx) * B(b_idx): `C("i,j") += A("i,k") * B("k,j")`
 * (expressions/tsr_expr.h:146-152, an AddExpr of the target and the
 * product).  The product is formed as by tagpu_contract in the target's index
 * order and must have the target's tiling; the new shape is SparseShape::add
 * (sparse_shape.h:1309-1328): float sum of the two scaled norms, zero below
 * the context threshold.  Tiles present in both are summed with one rounding,
 * a tile present in one is copied.  Dense and sparse policies do not mix.
 * Statistics of the product are in tagpu_last_stats. */
tagpu_status tagpu_contract_accumulate(tagpu_ctx* ctx, const char* c_idx, double alpha,
                                       tagpu_array* A, const char* a_idx, tagpu_array* B,
                                       const char* b_idx, const tagpu_contract_opts* opts,
                                       tagpu_array* C);

/* ---- single steps, host buffers (for parity tests) ----------------------- */
/* Kernel (a): result[M x N] = |factor| * (left[M x K] * k_sizes) x
 * (right[K x N] * k_sizes) in float, k ascending, screened by threshold.
 * K == 0 (k_sizes NULL) is the outer-product branch. */
tagpu_status tagpu_shape_gemm(tagpu_ctx* ctx, int64_t M, int64_t N, int64_t K,
                              const float* left, const float* right,
                              const float* k_sizes, double factor,
                              float threshold, float* result,
                              int64_t* zero_count);
/* Kernel (b): CSR tile-pair list.  offsets: M*N+1; kidx capacity kidx_cap
 * (pass kidx NULL to count only). */
tagpu_status tagpu_pair_list(tagpu_ctx* ctx, int64_t M, int64_t N, int64_t K,
                             const float* cnorm, float c_thr,
                             const float* lnorm, float l_thr,
                             const float* rnorm, float r_thr, int64_t* offsets,
                             int32_t* kidx, int64_t kidx_cap, int64_t* npairs);
/* Kernel (b) without any device allocation.  No counterpart in the
 * reference: it serves callers that cannot allocate device memory (a host
 * application whose device memory is owned by another framework's pool, or a
 * latency-critical loop that must not allocate).  Every pointer is a device
 * pointer supplied by the caller (offsets: M*N+1 entries; kidx: kidx_cap
 * entries or NULL to count only); *npairs is written on the host.  The only
 * scratch is a fixed per-device array of 2^20 result-tile counts inside the
 * library, so M*N above 1,048,576 is rejected (TAGPU_ERR_INVALID).  The first
 * call on a device looks the array up (make it before any stream capture);
 * calls whose work overlaps on the GPU share the array and race.  stream:
 * a cudaStream_t, NULL for the legacy default stream. */
tagpu_status tagpu_pair_list_noalloc(tagpu_ctx* ctx, int64_t M, int64_t N, int64_t K,
                                     const float* cnorm, float c_thr,
                                     const float* lnorm, float l_thr,
                                     const float* rnorm, float r_thr,
                                     int64_t* offsets, int32_t* kidx, int64_t kidx_cap,
                                     int64_t* npairs, void* stream);
/* Kernel (c): out = permute(in, perm), result dim perm[d] = arg dim d. */
tagpu_status tagpu_permute(tagpu_ctx* ctx, int rank, const int64_t* extents,
                           const int32_t* perm, const double* in, double* out);

/* ---- batched evaluation --------------------------------------------------- */
typedef struct tagpu_batch tagpu_batch;
tagpu_status tagpu_batch_create(tagpu_ctx* ctx, tagpu_batch** out);
/* Adds c = alpha * A(a_idx) * B(b_idx); *c is created now and filled by run. */
tagpu_status tagpu_batch_add(tagpu_batch* b, const char* c_idx, double alpha,
                             tagpu_array* A, const char* a_idx, tagpu_array* B,
                             const char* b_idx, const tagpu_contract_opts* opts,
                             tagpu_array** c);
/* First call plans every contraction and captures the launch sequence in a
 * CUDA graph; later calls replay the graph (operands may change values, not
 * shapes). */
tagpu_status tagpu_batch_run(tagpu_batch* b);
tagpu_status tagpu_batch_stats(const tagpu_batch* b, tagpu_contract_stats* st);
tagpu_status tagpu_batch_destroy(tagpu_batch* b);

/* ---- serving: continuous batching of contraction requests --------------- */
typedef struct tagpu_server tagpu_server;
typedef struct tagpu_server_config {
  size_t hbm_budget_bytes;    /* admission budget for results and scratch;
                                 0 = no budget */
  int max_batch;              /* contractions per launch, 0 = 64 */
  int precision;              /* default precision of requests */
  int slices;                 /* default Ozaki slices, 0 = 7 */
} tagpu_server_config;
typedef struct tagpu_request {
  const char* c_idx;
  double alpha;
  tagpu_array* A;
  const char* a_idx;
  tagpu_array* B;
  const char* b_idx;
  int precision;              /* < 0: server default */
  int slices;                 /* <= 0: server default */
} tagpu_request;
typedef struct tagpu_request_result {
  tagpu_status status;        /* status of the contraction itself */
  double latency_ms;          /* submit -> result ready */
  double queue_ms;            /* submit -> admitted */
  double flops;               /* nonzero-block flops */
  int64_t pairs;
  int batch_size;             /* contractions in its launch */
  uint64_t batch_id;
} tagpu_request_result;
typedef struct tagpu_server_stats {
  int64_t submitted, completed, rejected, failed, batches;
  double p50_ms, p99_ms, mean_ms; /* latency of completed requests */
  double flops;               /* total nonzero-block flops completed */
  double wall_ms;             /* first submit -> last completion */
  size_t bytes_in_use, peak_bytes;
} tagpu_server_stats;

/* Starts the request loop on its own host thread.  Requests reference arrays
 * that stay resident on the device; a request whose footprint bound exceeds
 * the budget is rejected at submit (TAGPU_ERR_REJECTED); others wait until
 * enough of the budget is free and are batched with whatever else is
 * admitted.  While one batch runs on the GPU the next one is planned. */
tagpu_status tagpu_server_start(tagpu_ctx* ctx, const tagpu_server_config* cfg,
                                tagpu_server** out);
/* Thread-safe. */
tagpu_status tagpu_server_submit(tagpu_server* s, const tagpu_request* req, uint64_t* id);
/* TAGPU_ERR_NOT_READY while in flight; on TAGPU_OK *c (may be NULL to drop
 * it) receives the result array, owned by the caller from then on. */
tagpu_status tagpu_server_poll(tagpu_server* s, uint64_t id, tagpu_array** c,
                               tagpu_request_result* res);
/* Blocks up to timeout_ms (< 0: no limit) then behaves like poll. */
tagpu_status tagpu_server_wait(tagpu_server* s, uint64_t id, double timeout_ms,
                               tagpu_array** c, tagpu_request_result* res);
tagpu_status tagpu_server_get_stats(tagpu_server* s, tagpu_server_stats* st);
/* Finishes queued work, then stops the loop and frees the server. */
tagpu_status tagpu_server_stop(tagpu_server* s);

#ifdef __cplusplus
}
#endif

#endif /* TAGPU_H */
