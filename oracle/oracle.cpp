// CPU oracle for the block-sparse contraction path.  TEST INFRASTRUCTURE ONLY:
// see oracle.h for what it restates and how it is pinned.  Compiled with
// -ffp-contract=off so that every multiply and add rounds separately.
#include "oracle.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

namespace {

inline uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// recursive_outer_product (sparse_shape.h:106-131): split the modes at
// middle = ceil(dim/2), recurse, and take the row-major outer product with
// float multiplication.
std::vector<float> outer_sizes(int rank, const int64_t* ntiles,
                               const float* const* sv, bool inverse) {
  if (rank == 1) {
    std::vector<float> r(ntiles[0]);
    for (int64_t i = 0; i < ntiles[0]; ++i)
      r[i] = inverse ? 1.0f / sv[0][i] : sv[0][i];
    return r;
  }
  const int middle = (rank >> 1) + (rank & 1);
  std::vector<float> left = outer_sizes(middle, ntiles, sv, inverse);
  std::vector<float> right =
      outer_sizes(rank - middle, ntiles + middle, sv + middle, inverse);
  std::vector<float> r(left.size() * right.size());
  for (size_t i = 0; i < left.size(); ++i)
    for (size_t j = 0; j < right.size(); ++j)
      r[i * right.size() + j] = left[i] * right[j];
  return r;
}

std::vector<const float*> split_sizes(int rank, const int64_t* ntiles,
                                      const float* sizes) {
  std::vector<const float*> sv(rank);
  const float* p = sizes;
  for (int d = 0; d < rank; ++d) {
    sv[d] = p;
    p += ntiles[d];
  }
  return sv;
}

template <typename T>
void permute_impl(int rank, const int64_t* extents, const int32_t* perm,
                  const T* in, T* out) {
  // result extent[perm[d]] = arg extent[d]; walk the argument in storage
  // order and scatter each element to its permuted ordinal.
  int64_t rext[8], rstride[8], amap[8];
  for (int d = 0; d < rank; ++d) rext[perm[d]] = extents[d];
  int64_t s = 1;
  for (int d = rank - 1; d >= 0; --d) {
    rstride[d] = s;
    s *= rext[d];
  }
  const int64_t vol = s;
  for (int d = 0; d < rank; ++d) amap[d] = rstride[perm[d]];
  int64_t idx[8] = {0};
  int64_t rord = 0;
  for (int64_t ord = 0; ord < vol; ++ord) {
    out[rord] = in[ord];
    for (int d = rank - 1; d >= 0; --d) {
      ++idx[d];
      rord += amap[d];
      if (idx[d] < extents[d]) break;
      rord -= amap[d] * idx[d];
      idx[d] = 0;
    }
  }
}

struct ContractArgs {
  int64_t M, N, K;
  const int64_t *msz, *nsz, *ksz;
  const double* left;
  const int64_t* left_off;
  int left_trans;
  const double* right;
  const int64_t* right_off;
  int right_trans;
  const int64_t* offsets;
  const int32_t* kidx;
  double alpha;
  double* result;
  const int64_t* res_off;
  orc_cblas_dgemm_fn dgemm;
};

void contract_tile(const ContractArgs& a, int64_t t) {
  if (a.res_off[t] < 0) return;
  const int64_t i = t / a.N, j = t % a.N;
  const int64_t m = a.msz[i], n = a.nsz[j];
  double* c = a.result + a.res_off[t];
  bool first = true;
  for (int64_t p = a.offsets[t]; p < a.offsets[t + 1]; ++p) {
    const int64_t k = a.kidx[p];
    const int64_t kk = a.ksz[k];
    const int64_t lo = a.left_off[i * a.K + k];
    const int64_t ro = a.right_off[k * a.N + j];
    if (lo < 0 || ro < 0) continue;  // pair list built from shapes; data absent
    const double* A = a.left + lo;
    const double* B = a.right + ro;
    if (a.dgemm) {
      a.dgemm(101, a.left_trans ? 112 : 111, a.right_trans ? 112 : 111, m, n,
              kk, a.alpha, A, a.left_trans ? m : kk, B, a.right_trans ? kk : n,
              first ? 0.0 : 1.0, c, n);
    } else {
      for (int64_t r = 0; r < m; ++r) {
        for (int64_t q = 0; q < n; ++q) {
          double s = 0.0;
          for (int64_t x = 0; x < kk; ++x) {
            const double av = a.left_trans ? A[x * m + r] : A[r * kk + x];
            const double bv = a.right_trans ? B[q * kk + x] : B[x * n + q];
            s = s + av * bv;
          }
          const double v = a.alpha * s;
          c[r * n + q] = first ? v : c[r * n + q] + v;
        }
      }
    }
    first = false;
  }
  if (first) std::memset(c, 0, sizeof(double) * m * n);
}

void run_tiles(const ContractArgs& a, const int64_t* tiles, int64_t ntiles,
               int nthreads) {
  if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
  std::atomic<int64_t> next{0};
  auto worker = [&]() {
    for (;;) {
      const int64_t x = next.fetch_add(1);
      if (x >= ntiles) break;
      contract_tile(a, tiles ? tiles[x] : x);
    }
  };
  if (nthreads == 1) {
    worker();
    return;
  }
  std::vector<std::thread> pool;
  for (int t = 0; t < nthreads; ++t) pool.emplace_back(worker);
  for (auto& th : pool) th.join();
}

}  // namespace

extern "C" {

uint64_t orc_hash(uint64_t seed, uint64_t stream, uint64_t ordinal) {
  return splitmix64(splitmix64(seed * 0x9E3779B97F4A7C15ull + stream) ^ ordinal);
}

double orc_uniform(uint64_t seed, uint64_t stream, uint64_t ordinal) {
  const uint64_t h = orc_hash(seed, stream, ordinal);
  return (double)(h >> 11) * 0x1.0p-53 * 2.0 - 1.0;
}

void orc_fill_tile(int rank, const int64_t* lo, const int64_t* hi,
                   const int64_t* global_extent, uint64_t seed, uint64_t stream,
                   int kind, double scale, double* out) {
  int64_t gstride[8];
  int64_t s = 1;
  for (int d = rank - 1; d >= 0; --d) {
    gstride[d] = s;
    s *= global_extent[d];
  }
  int64_t vol = 1;
  for (int d = 0; d < rank; ++d) vol *= hi[d] - lo[d];
  if (vol == 0) return;
  int64_t idx[8];
  for (int d = 0; d < rank; ++d) idx[d] = lo[d];
  for (int64_t e = 0; e < vol; ++e) {
    int64_t g = 0;
    for (int d = 0; d < rank; ++d) g += idx[d] * gstride[d];
    const uint64_t h = orc_hash(seed, stream, (uint64_t)g);
    double v = kind == 1 ? (double)(h % 101ull)
                         : (double)(h >> 11) * 0x1.0p-53 * 2.0 - 1.0;
    out[e] = v * scale;
    for (int d = rank - 1; d >= 0; --d) {
      if (++idx[d] < hi[d]) break;
      idx[d] = lo[d];
    }
  }
}

float orc_tile_norm(int64_t n, const double* x) {
  double s = 0.0;
  for (int64_t i = 0; i < n; ++i) s = s + x[i] * x[i];
  return (float)std::sqrt(s);
}

void orc_outer_sizes(int rank, const int64_t* ntiles, const float* sizes,
                     int inverse, float* out) {
  auto sv = split_sizes(rank, ntiles, sizes);
  auto r = outer_sizes(rank, ntiles, sv.data(), inverse != 0);
  std::copy(r.begin(), r.end(), out);
}

int64_t orc_scale_norms(int rank, const int64_t* ntiles, const float* sizes,
                        float threshold, float* norms) {
  auto sv = split_sizes(rank, ntiles, sizes);
  int64_t zeros = 0;
  if (rank == 1) {
    for (int64_t i = 0; i < ntiles[0]; ++i) {
      norms[i] /= sv[0][i];
      if (norms[i] < threshold) {
        norms[i] = 0.0f;
        ++zeros;
      }
    }
    return zeros;
  }
  const int middle = (rank >> 1) + (rank & 1);
  auto left = outer_sizes(middle, ntiles, sv.data(), true);
  auto right = outer_sizes(rank - middle, ntiles + middle, sv.data() + middle, true);
  for (size_t i = 0; i < left.size(); ++i) {
    for (size_t j = 0; j < right.size(); ++j) {
      float& v = norms[i * right.size() + j];
      const float xy = left[i] * right[j];
      v = v * xy;
      if (v < threshold) {
        v = 0.0f;
        ++zeros;
      }
    }
  }
  return zeros;
}

int64_t orc_shape_gemm(int64_t M, int64_t N, int64_t K, const float* left,
                       const float* right, const float* k_sizes, double factor,
                       float threshold, float* result) {
  const float abs_factor = (float)std::fabs(factor);
  int64_t zeros = 0;
  if (K == 0) {
    for (int64_t i = 0; i < M; ++i)
      for (int64_t j = 0; j < N; ++j) {
        float v = left[i] * right[j];
        v = v * abs_factor;
        if (v < threshold) {
          v = 0.0f;
          ++zeros;
        }
        result[i * N + j] = v;
      }
    return zeros;
  }
  std::vector<float> l(M * K), r(K * N);
  for (int64_t i = 0; i < M; ++i)
    for (int64_t k = 0; k < K; ++k) l[i * K + k] = left[i * K + k] * k_sizes[k];
  for (int64_t k = 0; k < K; ++k)
    for (int64_t j = 0; j < N; ++j) r[k * N + j] = right[k * N + j] * k_sizes[k];
  for (int64_t i = 0; i < M; ++i) {
    for (int64_t j = 0; j < N; ++j) {
      float s = 0.0f;
      for (int64_t k = 0; k < K; ++k) s = s + l[i * K + k] * r[k * N + j];
      float v = abs_factor * s;
      if (v < threshold) {
        v = 0.0f;
        ++zeros;
      }
      result[i * N + j] = v;
    }
  }
  return zeros;
}

int64_t orc_pairs(int64_t M, int64_t N, int64_t K, const float* cnorm,
                  float c_thr, const float* lnorm, float l_thr,
                  const float* rnorm, float r_thr, int64_t* offsets,
                  int32_t* kidx) {
  int64_t n = 0;
  for (int64_t i = 0; i < M; ++i) {
    for (int64_t j = 0; j < N; ++j) {
      if (offsets) offsets[i * N + j] = n;
      if (cnorm[i * N + j] < c_thr) continue;
      for (int64_t k = 0; k < K; ++k) {
        if (lnorm[i * K + k] < l_thr || rnorm[k * N + j] < r_thr) continue;
        if (kidx) kidx[n] = (int32_t)k;
        ++n;
      }
    }
  }
  if (offsets) offsets[M * N] = n;
  return n;
}

void orc_permute_f64(int rank, const int64_t* extents, const int32_t* perm,
                     const double* in, double* out) {
  permute_impl(rank, extents, perm, in, out);
}

void orc_permute_f32(int rank, const int64_t* extents, const int32_t* perm,
                     const float* in, float* out) {
  permute_impl(rank, extents, perm, in, out);
}

void orc_contract(int64_t M, int64_t N, int64_t K, const int64_t* msz,
                  const int64_t* nsz, const int64_t* ksz, const double* left,
                  const int64_t* left_off, int left_trans, const double* right,
                  const int64_t* right_off, int right_trans,
                  const int64_t* offsets, const int32_t* kidx, double alpha,
                  double* result, const int64_t* res_off, int nthreads,
                  orc_cblas_dgemm_fn dgemm) {
  ContractArgs a{M,         N,     K,        msz,    nsz,     ksz,
                 left,      left_off,        left_trans,     right,
                 right_off, right_trans,     offsets, kidx,  alpha,
                 result,    res_off,         dgemm};
  run_tiles(a, nullptr, M * N, nthreads);
}

void orc_contract_subset(int64_t M, int64_t N, int64_t K, const int64_t* msz,
                         const int64_t* nsz, const int64_t* ksz,
                         const double* left, const int64_t* left_off,
                         int left_trans, const double* right,
                         const int64_t* right_off, int right_trans,
                         const int64_t* offsets, const int32_t* kidx,
                         double alpha, double* result, const int64_t* res_off,
                         const int64_t* tiles, int64_t ntiles_sel,
                         int nthreads, orc_cblas_dgemm_fn dgemm) {
  ContractArgs a{M,         N,     K,        msz,    nsz,     ksz,
                 left,      left_off,        left_trans,     right,
                 right_off, right_trans,     offsets, kidx,  alpha,
                 result,    res_off,         dgemm};
  run_tiles(a, tiles, ntiles_sel, nthreads);
}

}  // extern "C"
