/*
 * CPU oracle for the block-sparse contraction path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library restates, in plain C++, the
 * algorithm TiledArray uses for C("i,j") = A("i,k") * B("k,j") on block-sparse
 * arrays.  It is used by tests/ as the checker, by __graft_entry__.smoke() to
 * check one small GPU invocation, and by bench.py's CPU-baseline leg.  The
 * product library (libtagpu) never links, loads or calls it.
 *
 * Parity pins (the reference cannot be compiled here: it needs MADNESS,
 * Boost, BTAS, BLAS++ and MPI):
 *   - integer-valued data, for which every FP64 sum is exact, compared with an
 *     independent dense numpy evaluation (the stand-in for the Eigen
 *     expectation the reference's own tests build);
 *   - the SparseShape::gemm expectation formula of the reference's own test
 *     (tests/sparse_shape.cpp:1478-1541);
 *   - fixtures under tests/golden/ restating the reference's test scenarios.
 *
 * Floating-point order is fixed here and compiled with -ffp-contract=off:
 *   - tile norms: sequential double sum of x*x in storage order
 *     (tensor/tensor.h:3768-3787, math/vector_op.h:561-577);
 *   - shape scaling: float, recursive outer product of inverse tile sizes
 *     (sparse_shape.h:106-131, 150-215);
 *   - shape gemm: float, k ascending, no fused multiply-add
 *     (sparse_shape.h:1589-1684; the reference defers the order to sgemm).
 */
#ifndef TAGPU_ORACLE_H
#define TAGPU_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Counter-based generator shared by the oracle and the device generator. */
uint64_t orc_hash(uint64_t seed, uint64_t stream, uint64_t ordinal);
double orc_uniform(uint64_t seed, uint64_t stream, uint64_t ordinal);

/* Fill one tile: element e of the tile (row-major over the tile's range) gets
 * the value for global element ordinal ord(e), times `scale`.
 * kind 0: uniform[-1,1); kind 1: integer hash % 101 (the reference tests'
 * rand() % 101 data).  rank <= 8. */
void orc_fill_tile(int rank, const int64_t* lo, const int64_t* hi,
                   const int64_t* global_extent, uint64_t seed, uint64_t stream,
                   int kind, double scale, double* out);

/* Tensor::norm of a tile: float(sqrt(sum_{i} x_i*x_i)), sequential. */
float orc_tile_norm(int64_t n, const double* x);

/* SparseShape(norms, trange) scaling: norms (row-major over the tile grid)
 * are scaled in place by the inverse tile volume and screened.
 * sizes: concatenated per-dim tile sizes (float), ntiles[d] entries each.
 * Returns the zero-tile count. */
int64_t orc_scale_norms(int rank, const int64_t* ntiles, const float* sizes,
                        float threshold, float* norms);

/* SparseShape::gemm on norms already in GEMM order.
 * left: M x K, right: K x N, k_sizes: K (outer product of contracted tile
 * sizes; pass NULL and K = 0 for an outer product).  Writes M x N result norms
 * and returns the zero count. */
int64_t orc_shape_gemm(int64_t M, int64_t N, int64_t K, const float* left,
                       const float* right, const float* k_sizes, double factor,
                       float threshold, float* result);

/* recursive_outer_product of size vectors (sparse_shape.h:106-131), with an
 * optional reciprocal (InverseVolume).  out must hold prod(ntiles) floats. */
void orc_outer_sizes(int rank, const int64_t* ntiles, const float* sizes,
                     int inverse, float* out);

/* Summa pair set: (i,k,j) with C(i,j) >= c_thr, L(i,k) >= l_thr,
 * R(k,j) >= r_thr.  offsets: M*N+1 entries (CSR over result tiles in
 * row-major order), kidx: the k of every pair, ascending per result tile.
 * Pass kidx == NULL to count only.  Returns the pair count. */
int64_t orc_pairs(int64_t M, int64_t N, int64_t K, const float* cnorm,
                  float c_thr, const float* lnorm, float l_thr,
                  const float* rnorm, float r_thr, int64_t* offsets,
                  int32_t* kidx);

/* Tensor permute: result dim perm[d] = argument dim d (permutation.h:60-78,
 * tensor/permute.h:124-210).  extents: argument extents. */
void orc_permute_f64(int rank, const int64_t* extents, const int32_t* perm,
                     const double* in, double* out);
void orc_permute_f32(int rank, const int64_t* extents, const int32_t* perm,
                     const float* in, float* out);

/* Per-result-tile reduction over the pair list, GEMM order.
 * Left tile (i,k) is m_i x k_k row-major (left_trans = 0) or k_k x m_i
 * (left_trans = 1); right tile (k,j) is k_k x n_j (right_trans = 0) or
 * n_j x k_k (right_trans = 1).  Offsets are element offsets into the tile
 * data, -1 for an absent tile.  Result tiles: m_i x n_j at res_off[i*N+j]
 * (-1: zero tile, skipped).  First pair writes C = alpha*A*B, later pairs
 * C += alpha*A*B (tensor/tensor.h:3132-3210, tile_op/contract_reduce.h:367-452).
 * nthreads: worker threads over result tiles (0 = hardware concurrency).
 * dgemm: optional cblas_dgemm-compatible ILP64 function pointer; NULL uses
 * the oracle's own k-ascending loop. */
typedef void (*orc_cblas_dgemm_fn)(int layout, int transa, int transb,
                                   int64_t m, int64_t n, int64_t k,
                                   double alpha, const double* a, int64_t lda,
                                   const double* b, int64_t ldb, double beta,
                                   double* c, int64_t ldc);
void orc_contract(int64_t M, int64_t N, int64_t K, const int64_t* msz,
                  const int64_t* nsz, const int64_t* ksz, const double* left,
                  const int64_t* left_off, int left_trans, const double* right,
                  const int64_t* right_off, int right_trans,
                  const int64_t* offsets, const int32_t* kidx, double alpha,
                  double* result, const int64_t* res_off, int nthreads,
                  orc_cblas_dgemm_fn dgemm);

/* Same as orc_contract restricted to the result tiles listed in `tiles`
 * (row-major result tile ordinals); used for a bounded CPU-baseline sample. */
void orc_contract_subset(int64_t M, int64_t N, int64_t K, const int64_t* msz,
                         const int64_t* nsz, const int64_t* ksz,
                         const double* left, const int64_t* left_off,
                         int left_trans, const double* right,
                         const int64_t* right_off, int right_trans,
                         const int64_t* offsets, const int32_t* kidx,
                         double alpha, double* result, const int64_t* res_off,
                         const int64_t* tiles, int64_t ntiles_sel,
                         int nthreads, orc_cblas_dgemm_fn dgemm);

#ifdef __cplusplus
}
#endif

#endif
