// tagpu host library: the C ABI of include/tagpu.h.
//
// The expression semantics are TiledArray's (paths relative to its source):
//   index parsing / product classification  expressions/mult_engine.h:300-360
//   layout choice (permtypes)               expressions/permopt.h:258-396,
//                                           expressions/binary_engine.h:101-176
//   fused GEMM dimensions                   math/gemm_helper.h:57-90, 252-273
//   result tiling and shape                 expressions/cont_engine.h:354-535,
//                                           642-677
//   shape construction and scaling          sparse_shape.h:150-237, 335-422
// Host code only plans; every step that touches tile data or norms runs in a
// kernel (k_*.cu).  Compiled with -ffp-contract=off: the float shape algebra
// done here (size vectors, scaling) rounds each operation separately, as the
// CPU reference does.
#include <cuda_runtime.h>
#include <sys/mman.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <thread>
#include <unordered_map>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <limits>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "internal.h"

using namespace tagpu;

// ---------------------------------------------------------------------------
// context and arrays
// ---------------------------------------------------------------------------

struct tagpu_ctx {
  int device = 0;
  int sm_count = 0;
  cudaStream_t stream = nullptr;
  float threshold = std::numeric_limits<float>::epsilon();
  size_t budget = 0;
  std::atomic<size_t> used{0};
  std::string err;
  tagpu_contract_stats last{};
  std::recursive_mutex mu;
  cudaEvent_t t0 = nullptr, t1 = nullptr;
  // bound of every pipeline wait in the emulated GEMM (tagpu_set_wait_limit)
  unsigned long long wait_ns = 4000000000ull;
};

struct tagpu_array {
  tagpu_ctx* ctx = nullptr;
  int rank = 0;
  std::vector<std::vector<int64_t>> hm;  // hashmarks per dim
  std::vector<int64_t> nt;               // tiles per dim
  bool dense = true;
  std::vector<float> norms;              // scaled norms (sparse only)
  float threshold = 0.0f;                // the shape's own threshold
  int64_t zero_count = 0;
  std::vector<int64_t> off;              // element offset per tile, -1 zero
  int64_t elements = 0;
  double* data = nullptr;                // device
  size_t bytes = 0;

  int64_t ntiles() const {
    int64_t n = 1;
    for (auto x : nt) n *= x;
    return n;
  }
  void tile_index(int64_t ord, int64_t* idx) const {
    for (int d = rank - 1; d >= 0; --d) {
      idx[d] = nt[d] ? ord % nt[d] : 0;
      ord = nt[d] ? ord / nt[d] : 0;
    }
  }
  int64_t tile_volume(int64_t ord) const {
    int64_t idx[8];
    tile_index(ord, idx);
    int64_t v = 1;
    for (int d = 0; d < rank; ++d) v *= hm[d][idx[d] + 1] - hm[d][idx[d]];
    return v;
  }
  bool tile_is_zero(int64_t ord) const {
    if (dense) return false;
    return norms[ord] < threshold;
  }
  ~tagpu_array();  // releases the device storage
};

namespace {

tagpu_status fail(tagpu_ctx* ctx, tagpu_status st, const char* fmt, ...) {
  if (ctx) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    ctx->err = buf;
  }
  return st;
}

#define CUDA_TRY(ctx, call)                                                          \
  do {                                                                               \
    cudaError_t e_ = (call);                                                         \
    if (e_ != cudaSuccess)                                                           \
      return fail((ctx), TAGPU_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

tagpu_status dev_alloc(tagpu_ctx* ctx, void** p, size_t bytes) {
  *p = nullptr;
  if (bytes == 0) return TAGPU_OK;
  if (ctx->budget && ctx->used.load() + bytes > ctx->budget)
    return fail(ctx, TAGPU_ERR_NOMEM, "device budget exceeded: %zu + %zu > %zu bytes",
                ctx->used.load(), bytes, ctx->budget);
  cudaError_t e = pool_alloc(p, bytes, ctx->stream);
  if (e != cudaSuccess) {
    return fail(ctx, TAGPU_ERR_NOMEM, "cudaMallocAsync(%zu) failed: %s", bytes,
                cudaGetErrorString(e));
  }
  ctx->used += bytes;
  return TAGPU_OK;
}

void dev_free(tagpu_ctx* ctx, void* p, size_t bytes) {
  if (!p) return;
  cudaFreeAsync(p, ctx->stream);
  ctx->used -= bytes;
}

}  // namespace

tagpu_array::~tagpu_array() {
  if (data) dev_free(ctx, data, bytes);
}

namespace tagpu {
static std::atomic<int64_t> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
int64_t launch_count() { return g_launches.load(std::memory_order_relaxed); }

tagpu_status set_last_error(tagpu_ctx* ctx, tagpu_status st, const char* msg) {
  if (ctx) ctx->err = msg;
  return st;
}
int context_device(const tagpu_ctx* ctx) { return ctx ? ctx->device : -1; }
}  // namespace tagpu

namespace {

// Scoped device buffer on the context stream.
struct DBuf {
  tagpu_ctx* ctx = nullptr;
  void* p = nullptr;
  size_t n = 0;
  DBuf() = default;
  explicit DBuf(tagpu_ctx* c) : ctx(c) {}
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  ~DBuf() { release(); }
  void release() {
    if (p) dev_free(ctx, p, n);
    p = nullptr;
    n = 0;
  }
  tagpu_status alloc(size_t bytes) {
    release();
    tagpu_status st = dev_alloc(ctx, &p, bytes);
    if (st == TAGPU_OK) n = bytes;
    return st;
  }
  template <typename T>
  T* as() const { return static_cast<T*>(p); }
};

template <typename T>
tagpu_status upload_vec(tagpu_ctx* ctx, DBuf& b, const std::vector<T>& v) {
  tagpu_status st = b.alloc(std::max<size_t>(1, v.size()) * sizeof(T));
  if (st) return st;
  if (!v.empty())
    CUDA_TRY(ctx, cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice,
                                  ctx->stream));
  return TAGPU_OK;
}

// recursive_outer_product (sparse_shape.h:106-131): split at ceil(d/2),
// recurse, row-major outer product in float.
std::vector<float> outer_sizes(const std::vector<std::vector<float>>& sv, size_t b, size_t e,
                               bool inverse) {
  if (e - b == 1) {
    std::vector<float> r(sv[b].size());
    for (size_t i = 0; i < r.size(); ++i) r[i] = inverse ? 1.0f / sv[b][i] : sv[b][i];
    return r;
  }
  const size_t dim = e - b;
  const size_t middle = (dim >> 1) + (dim & 1);
  auto l = outer_sizes(sv, b, b + middle, inverse);
  auto r = outer_sizes(sv, b + middle, e, inverse);
  std::vector<float> out(l.size() * r.size());
  for (size_t i = 0; i < l.size(); ++i)
    for (size_t j = 0; j < r.size(); ++j) out[i * r.size() + j] = l[i] * r[j];
  return out;
}

std::vector<std::vector<float>> size_vectors(const tagpu_array* a) {
  std::vector<std::vector<float>> sv(a->rank);
  for (int d = 0; d < a->rank; ++d) {
    sv[d].resize(a->nt[d]);
    for (int64_t i = 0; i < a->nt[d]; ++i) sv[d][i] = (float)(a->hm[d][i + 1] - a->hm[d][i]);
  }
  return sv;
}

// scale_tile_norms<InverseVolume, Screen> (sparse_shape.h:150-215)
int64_t scale_norms(const tagpu_array* a, std::vector<float>& norms, float thr) {
  auto sv = size_vectors(a);
  int64_t zeros = 0;
  if (a->rank == 1) {
    for (size_t i = 0; i < norms.size(); ++i) {
      norms[i] /= sv[0][i];
      if (norms[i] < thr) {
        norms[i] = 0.0f;
        ++zeros;
      }
    }
    return zeros;
  }
  if (a->rank == 0) return 0;
  const size_t middle = (a->rank >> 1) + (a->rank & 1);
  auto l = outer_sizes(sv, 0, middle, true);
  auto r = outer_sizes(sv, middle, a->rank, true);
  for (size_t i = 0; i < l.size(); ++i)
    for (size_t j = 0; j < r.size(); ++j) {
      float& v = norms[i * r.size() + j];
      const float xy = l[i] * r[j];
      v = v * xy;
      if (v < thr) {
        v = 0.0f;
        ++zeros;
      }
    }
  return zeros;
}

// Recompute offsets for a packed layout of the currently nonzero tiles.
void pack_offsets(tagpu_array* a) {
  const int64_t n = a->ntiles();
  a->off.assign(n, -1);
  int64_t pos = 0;
  for (int64_t t = 0; t < n; ++t) {
    if (a->tile_is_zero(t)) continue;
    a->off[t] = pos;
    pos += a->tile_volume(t);
  }
  a->elements = pos;
}

tagpu_status ensure_storage(tagpu_array* a) {
  tagpu_ctx* ctx = a->ctx;
  const size_t need = (size_t)a->elements * sizeof(double);
  if (a->data && a->bytes == need) return TAGPU_OK;
  if (a->data) dev_free(ctx, a->data, a->bytes);
  a->data = nullptr;
  a->bytes = 0;
  if (need == 0) return TAGPU_OK;
  void* p = nullptr;
  tagpu_status st = dev_alloc(ctx, &p, need);
  if (st) return st;
  a->data = static_cast<double*>(p);
  a->bytes = need;
  return TAGPU_OK;
}

// An array made by tagpu_array_create holds no device memory until it is
// written (upload, generate, a shape, a contraction result) or read; a read of
// an array never written sees zero tiles, like a TiledArray DistArray whose
// tiles were initialised to zero.  So an operand too large for the device can
// still be described (and a request naming it refused by admission).
tagpu_status materialize(const tagpu_array* ca) {
  tagpu_array* a = const_cast<tagpu_array*>(ca);
  if (a->data || a->elements == 0) return TAGPU_OK;
  tagpu_status st = ensure_storage(a);
  if (st) return st;
  CUDA_TRY(a->ctx, cudaMemsetAsync(a->data, 0, a->bytes, a->ctx->stream));
  return TAGPU_OK;
}

tagpu_array* new_array(tagpu_ctx* ctx, const std::vector<std::vector<int64_t>>& hm) {
  auto* a = new tagpu_array;
  a->ctx = ctx;
  a->rank = (int)hm.size();
  a->hm = hm;
  a->nt.resize(a->rank);
  for (int d = 0; d < a->rank; ++d) a->nt[d] = (int64_t)hm[d].size() - 1;
  a->threshold = ctx->threshold;
  pack_offsets(a);
  return a;
}

// ---------------------------------------------------------------------------
// index lists and the permutation optimizer
// ---------------------------------------------------------------------------

bool parse_indices(const char* s, std::vector<std::string>& out) {
  out.clear();
  if (!s) return false;
  std::string cur;
  auto flush = [&]() -> bool {
    size_t b = cur.find_first_not_of(" \t"), e = cur.find_last_not_of(" \t");
    if (b == std::string::npos) return false;
    out.push_back(cur.substr(b, e - b + 1));
    cur.clear();
    return true;
  };
  bool any = false;
  for (const char* p = s; *p; ++p) {
    if (*p == ',') {
      if (!flush()) return false;
      any = true;
    } else {
      cur.push_back(*p);
    }
  }
  if (cur.find_first_not_of(" \t") != std::string::npos) {
    flush();
  } else if (any) {
    return false;  // trailing comma
  }
  for (size_t i = 0; i < out.size(); ++i)
    for (size_t j = i + 1; j < out.size(); ++j)
      if (out[i] == out[j]) return false;
  return true;
}

int find_idx(const std::vector<std::string>& v, const std::string& x) {
  for (size_t i = 0; i < v.size(); ++i)
    if (v[i] == x) return (int)i;
  return -1;
}

enum { IDENTITY = 1, MATRIX_TRANSPOSE = 2, GENERAL = 3 };

// GEMMPermutationOptimizer::compute_index_list_contraction (permopt.h:258-376)
struct PermOpt {
  std::vector<std::string> left, right, result;
  int lop = GENERAL, rop = GENERAL;
};

PermOpt permopt(const std::vector<std::string>& L, const std::vector<std::string>& R,
                bool prefer_left) {
  PermOpt o;
  const size_t lr = L.size(), rr = R.size();
  for (auto& v : L) {
    if (find_idx(R, v) < 0) {
      o.left.push_back(v);
      o.result.push_back(v);
    } else {
      o.right.push_back(v);
    }
  }
  const size_t inner = o.right.size(), lo = o.left.size(), ro = rr - inner;
  if (inner == 0) {
    for (auto& v : R) {
      o.right.push_back(v);
      o.result.push_back(v);
    }
    return o;
  }
  bool ordered = true, lnt = true, lt = true, rnt = true, rt = true;
  const bool perm_left = lr < rr || (lr == rr && prefer_left);
  for (size_t i = 0; i < rr; ++i) {
    const std::string& idx = R[i];
    const int jj = find_idx(L, idx);
    if (jj < 0) {
      o.right.push_back(idx);
      o.result.push_back(idx);
      continue;
    }
    const size_t j = (size_t)jj;
    const size_t x = o.left.size() - lo;
    ordered = ordered && o.right[x] == idx;
    lnt = lnt && j >= lo;
    lt = lt && j < inner;
    rnt = rnt && i < inner;
    rt = rt && i >= ro;
    if (ordered) {
      o.left.push_back(idx);
    } else if (perm_left) {
      o.left.push_back(idx);
      o.right[x] = idx;
      lnt = lt = false;
    } else {
      o.left.push_back(o.right[x]);
      rnt = rt = false;
    }
  }
  o.lop = lnt ? IDENTITY : (lt ? MATRIX_TRANSPOSE : GENERAL);
  o.rop = rnt ? IDENTITY : (rt ? MATRIX_TRANSPOSE : GENERAL);
  return o;
}

// perm with result dim perm[d] = argument dim d, mapping src order to dst
std::vector<int> perm_between(const std::vector<std::string>& src,
                              const std::vector<std::string>& dst) {
  std::vector<int> p(src.size());
  for (size_t d = 0; d < src.size(); ++d) p[d] = find_idx(dst, src[d]);
  return p;
}

bool is_identity(const std::vector<int>& p) {
  for (size_t d = 0; d < p.size(); ++d)
    if (p[d] != (int)d) return false;
  return true;
}

template <typename T>
std::vector<T> permute_grid(const std::vector<T>& in, const std::vector<int64_t>& ext,
                            const std::vector<int>& perm) {
  const int r = (int)ext.size();
  std::vector<T> out(in.size());
  if (in.empty()) return out;
  std::vector<int64_t> rext(r), rs(r), amap(r), idx(r, 0);
  for (int d = 0; d < r; ++d) rext[perm[d]] = ext[d];
  int64_t s = 1;
  for (int d = r - 1; d >= 0; --d) {
    rs[d] = s;
    s *= rext[d];
  }
  for (int d = 0; d < r; ++d) amap[d] = rs[perm[d]];
  int64_t ro = 0;
  for (size_t o = 0; o < in.size(); ++o) {
    out[ro] = in[o];
    for (int d = r - 1; d >= 0; --d) {
      ++idx[d];
      ro += amap[d];
      if (idx[d] < ext[d]) break;
      ro -= amap[d] * idx[d];
      idx[d] = 0;
    }
  }
  return out;
}

struct EventTimer {
  cudaEvent_t a, b;
  cudaStream_t s;
  explicit EventTimer(cudaStream_t st) : s(st) {
    cudaEventCreate(&a);
    cudaEventCreate(&b);
    cudaEventRecord(a, s);
  }
  void stop() { cudaEventRecord(b, s); }
  double ms() {
    cudaEventSynchronize(b);
    float f = 0;
    cudaEventElapsedTime(&f, a, b);
    return f;
  }
  ~EventTimer() {
    cudaEventDestroy(a);
    cudaEventDestroy(b);
  }
};

}  // namespace

// ---------------------------------------------------------------------------
// C ABI: context
// ---------------------------------------------------------------------------

extern "C" {

const char* tagpu_status_string(tagpu_status s) {
  switch (s) {
    case TAGPU_OK: return "ok";
    case TAGPU_ERR_INVALID: return "invalid argument";
    case TAGPU_ERR_UNSUPPORTED: return "unsupported";
    case TAGPU_ERR_NOMEM: return "out of device memory";
    case TAGPU_ERR_CUDA: return "CUDA error";
    case TAGPU_ERR_TIMEOUT: return "timeout";
    case TAGPU_ERR_REJECTED: return "rejected";
    case TAGPU_ERR_NOT_READY: return "not ready";
    case TAGPU_ERR_STATE: return "bad state";
  }
  return "unknown";
}

tagpu_status tagpu_init(const tagpu_config* cfg, tagpu_ctx** out) {
  if (!out) return TAGPU_ERR_INVALID;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return TAGPU_ERR_CUDA;
  }
  auto* ctx = new tagpu_ctx;
  ctx->device = cfg ? cfg->device : 0;
  ctx->budget = cfg ? cfg->hbm_budget_bytes : 0;
  if (ctx->device < 0 || ctx->device >= ndev) {
    delete ctx;
    return TAGPU_ERR_INVALID;
  }
  if (cudaSetDevice(ctx->device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete ctx;
    return TAGPU_ERR_CUDA;
  }
  cudaDeviceGetAttribute(&ctx->sm_count, cudaDevAttrMultiProcessorCount, ctx->device);
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, ctx->device) == cudaSuccess) {
    uint64_t thr = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  *out = ctx;
  return TAGPU_OK;
}

tagpu_status tagpu_shutdown(tagpu_ctx* ctx) {
  if (!ctx) return TAGPU_ERR_INVALID;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  if (ctx->t0) cudaEventDestroy(ctx->t0);
  if (ctx->t1) cudaEventDestroy(ctx->t1);
  cudaStreamDestroy(ctx->stream);
  delete ctx;
  return TAGPU_OK;
}

const char* tagpu_last_error(const tagpu_ctx* ctx) { return ctx ? ctx->err.c_str() : ""; }

tagpu_status tagpu_sync(tagpu_ctx* ctx) {
  if (!ctx) return TAGPU_ERR_INVALID;
  CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return TAGPU_OK;
}

tagpu_status tagpu_timer_start(tagpu_ctx* ctx) {
  if (!ctx) return TAGPU_ERR_INVALID;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  if (!ctx->t0) {
    CUDA_TRY(ctx, cudaEventCreate(&ctx->t0));
    CUDA_TRY(ctx, cudaEventCreate(&ctx->t1));
  }
  CUDA_TRY(ctx, cudaEventRecord(ctx->t0, ctx->stream));
  return TAGPU_OK;
}

tagpu_status tagpu_timer_stop(tagpu_ctx* ctx, double* ms) {
  if (!ctx || !ms || !ctx->t0) return TAGPU_ERR_INVALID;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  CUDA_TRY(ctx, cudaEventRecord(ctx->t1, ctx->stream));
  CUDA_TRY(ctx, cudaEventSynchronize(ctx->t1));
  float f = 0;
  CUDA_TRY(ctx, cudaEventElapsedTime(&f, ctx->t0, ctx->t1));
  *ms = f;
  return TAGPU_OK;
}

tagpu_status tagpu_device_fp64_rates(tagpu_ctx* ctx, double* dmma_tflops, double* dfma_tflops) {
  if (!ctx || !dmma_tflops || !dfma_tflops) return TAGPU_ERR_INVALID;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  tagpu_status st = measure_fp64_rates(ctx->stream, ctx->sm_count, dmma_tflops, dfma_tflops);
  if (st) return fail(ctx, st, "FP64 rate measurement failed");
  return TAGPU_OK;
}

tagpu_status tagpu_device_mma_sync_rates(tagpu_ctx* ctx, double* imma_tops, double* hmma_tflops) {
  if (!ctx || !imma_tops || !hmma_tflops) return TAGPU_ERR_INVALID;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  tagpu_status st = measure_mma_sync_rates(ctx->stream, ctx->sm_count, imma_tops, hmma_tflops);
  if (st) return fail(ctx, st, "mma.sync rate measurement failed");
  return TAGPU_OK;
}

float tagpu_threshold_get(const tagpu_ctx* ctx) { return ctx ? ctx->threshold : 0.0f; }
void tagpu_threshold_set(tagpu_ctx* ctx, float t) {
  if (ctx) ctx->threshold = t;
}

tagpu_status tagpu_set_wait_limit(tagpu_ctx* ctx, double seconds) {
  if (!ctx) return TAGPU_ERR_INVALID;
  if (!(seconds > 0.0) || seconds > 3600.0)
    return fail(ctx, TAGPU_ERR_INVALID, "wait limit must lie in (0, 3600] seconds");
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  const double ns = seconds * 1e9;
  ctx->wait_ns = ns < 1.0 ? 1ull : (unsigned long long)ns;
  return TAGPU_OK;
}

// ---------------------------------------------------------------------------
// C ABI: arrays
// ---------------------------------------------------------------------------

tagpu_status tagpu_array_create(tagpu_ctx* ctx, int rank, const int64_t* ntiles,
                                const int64_t* const* hashmarks, tagpu_array** out) {
  if (!ctx || !out) return TAGPU_ERR_INVALID;
  *out = nullptr;
  if (rank < 0 || rank > 8 || (rank > 0 && (!ntiles || !hashmarks)))
    return fail(ctx, TAGPU_ERR_INVALID, "array rank must be 0..8");
  std::vector<std::vector<int64_t>> hm(rank);
  for (int d = 0; d < rank; ++d) {
    if (ntiles[d] < 0 || !hashmarks[d])
      return fail(ctx, TAGPU_ERR_INVALID, "dimension %d: bad tiling", d);
    hm[d].assign(hashmarks[d], hashmarks[d] + ntiles[d] + 1);
    for (int64_t i = 0; i < ntiles[d]; ++i)
      if (hm[d][i + 1] < hm[d][i])
        return fail(ctx, TAGPU_ERR_INVALID, "dimension %d: hashmarks must not decrease", d);
  }
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  *out = new_array(ctx, hm);   // storage on first write or read
  return TAGPU_OK;
}

tagpu_status tagpu_array_destroy(tagpu_array* a) {
  if (!a) return TAGPU_ERR_INVALID;
  std::lock_guard<std::recursive_mutex> lk(a->ctx->mu);
  cudaSetDevice(a->ctx->device);
  delete a;
  return TAGPU_OK;
}

tagpu_status tagpu_array_set_shape(tagpu_array* a, const float* norms, int do_not_scale,
                                   float threshold) {
  if (!a) return TAGPU_ERR_INVALID;
  tagpu_ctx* ctx = a->ctx;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  if (!norms) {
    a->dense = true;
    a->norms.clear();
    a->zero_count = 0;
  } else {
    const float thr = threshold < 0 ? ctx->threshold : threshold;
    a->dense = false;
    a->norms.assign(norms, norms + a->ntiles());
    a->threshold = thr;
    if (!do_not_scale) {
      a->zero_count = scale_norms(a, a->norms, thr);
    } else {
      a->zero_count = 0;
      for (auto& v : a->norms)
        if (v < thr) {
          v = 0.0f;
          ++a->zero_count;
        }
    }
  }
  pack_offsets(a);
  return ensure_storage(a);
}

tagpu_status tagpu_array_upload(tagpu_array* a, const double* tiles, int64_t n) {
  if (!a) return TAGPU_ERR_INVALID;
  tagpu_ctx* ctx = a->ctx;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  if (n != a->elements)
    return fail(ctx, TAGPU_ERR_INVALID, "upload: %lld elements given, array stores %lld",
                (long long)n, (long long)a->elements);
  if (n && !tiles) return fail(ctx, TAGPU_ERR_INVALID, "upload: null buffer");
  // the packed host layout equals the device layout iff offsets are packed
  pack_offsets(a);
  tagpu_status st = ensure_storage(a);
  if (st) return st;
  if (n) {
    if (link_copy_usable(tiles))
      launch_link_copy(ctx->stream, a->data, tiles, n * sizeof(double));
    else
      CUDA_TRY(ctx, cudaMemcpyAsync(a->data, tiles, n * sizeof(double), cudaMemcpyHostToDevice,
                                    ctx->stream));
  }
  CUDA_TRY(ctx, cudaGetLastError());
  CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return TAGPU_OK;
}

tagpu_status tagpu_array_download(const tagpu_array* a, double* tiles, int64_t n) {
  if (!a) return TAGPU_ERR_INVALID;
  tagpu_ctx* ctx = a->ctx;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  if (n != a->elements)
    return fail(ctx, TAGPU_ERR_INVALID, "download: buffer holds %lld elements, array %lld",
                (long long)n, (long long)a->elements);
  if (n && !tiles) return fail(ctx, TAGPU_ERR_INVALID, "download: null buffer");
  if (tagpu_status st = materialize(a)) return st;
  if (n) {
    if (link_copy_usable(tiles))
      launch_link_copy(ctx->stream, tiles, a->data, n * sizeof(double));
    else
      CUDA_TRY(ctx, cudaMemcpyAsync(tiles, a->data, n * sizeof(double), cudaMemcpyDeviceToHost,
                                    ctx->stream));
  }
  CUDA_TRY(ctx, cudaGetLastError());
  CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return TAGPU_OK;
}

// After a shape change: the stored tiles `present` (ordinal order, at element
// offsets `offs` of a->data) move to the offsets of the tiles the new shape
// keeps.  Compaction is in place: surviving tiles move to lower addresses in
// ordinal order; a tile whose source and destination overlap goes through a
// bounce buffer of one tile, disjoint runs are single copies.
static tagpu_status compact_tiles(tagpu_ctx* ctx, tagpu_array* a,
                                  const std::vector<int64_t>& present,
                                  const std::vector<int64_t>& offs) {
  tagpu_status st;
  const int64_t np = (int64_t)present.size();
  pack_offsets(a);  // offsets of the tiles that survived the shape
  DBuf bounce(ctx);
  int64_t x = 0;
  while (x < np) {
    const int64_t t = present[x];
    const int64_t dst = a->off[t];
    if (dst < 0 || dst == offs[x]) {
      ++x;
      continue;
    }
    const int64_t len = offs[x + 1] - offs[x];
    if (dst + len <= offs[x]) {
      CUDA_TRY(ctx, cudaMemcpyAsync(a->data + dst, a->data + offs[x], len * sizeof(double),
                                    cudaMemcpyDeviceToDevice, ctx->stream));
    } else {
      if (bounce.n < (size_t)len * sizeof(double) && (st = bounce.alloc(len * sizeof(double))))
        return st;
      CUDA_TRY(ctx, cudaMemcpyAsync(bounce.p, a->data + offs[x], len * sizeof(double),
                                    cudaMemcpyDeviceToDevice, ctx->stream));
      CUDA_TRY(ctx, cudaMemcpyAsync(a->data + dst, bounce.p, len * sizeof(double),
                                    cudaMemcpyDeviceToDevice, ctx->stream));
    }
    ++x;
  }
  CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  // release the tail the dropped tiles occupied (kept if no room to move)
  const size_t keep = (size_t)a->elements * sizeof(double);
  if (keep < a->bytes) {
    void* p = nullptr;
    if (keep && (st = dev_alloc(ctx, &p, keep)) == TAGPU_OK) {
      CUDA_TRY(ctx, cudaMemcpyAsync(p, a->data, keep, cudaMemcpyDeviceToDevice, ctx->stream));
      dev_free(ctx, a->data, a->bytes);
      a->data = static_cast<double*>(p);
      a->bytes = keep;
    } else if (!keep) {
      dev_free(ctx, a->data, a->bytes);
      a->data = nullptr;
      a->bytes = 0;
    }
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  }
  return TAGPU_OK;
}

tagpu_status tagpu_array_generate(tagpu_array* a, uint64_t seed, uint64_t stream, int kind,
                                  const double* tile_scale, int compute_shape,
                                  float threshold) {
  if (!a) return TAGPU_ERR_INVALID;
  tagpu_ctx* ctx = a->ctx;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  if (kind != 0 && kind != 1) return fail(ctx, TAGPU_ERR_INVALID, "generate: kind must be 0 or 1");
  const int64_t n = a->ntiles();
  // tiles generated: with compute_shape those with a nonzero scale (the shape
  // follows from their norms); without it, every tile the current shape keeps
  // (a zero scale then gives a zero tile)
  std::vector<int64_t> lo, offs(1, 0), present;
  std::vector<int32_t> ext;
  std::vector<double> scale;
  int64_t idx[8];
  for (int64_t t = 0; t < n; ++t) {
    const double sc = tile_scale ? tile_scale[t] : 1.0;
    if (compute_shape ? sc == 0.0 : a->tile_is_zero(t)) continue;
    a->tile_index(t, idx);
    for (int d = 0; d < a->rank; ++d) {
      lo.push_back(a->hm[d][idx[d]] - a->hm[d][0]);
      ext.push_back((int32_t)(a->hm[d][idx[d] + 1] - a->hm[d][idx[d]]));
    }
    scale.push_back(sc);
    present.push_back(t);
    offs.push_back(offs.back() + a->tile_volume(t));
  }
  const int64_t np = (int64_t)present.size();
  // Generate straight into the array's storage laid out over the present
  // tiles (tile ordinal order), so peak memory is the array itself.
  DBuf dlo(ctx), dext(ctx), doff(ctx), dsc(ctx);
  tagpu_status st;
  if ((st = upload_vec(ctx, dlo, lo)) || (st = upload_vec(ctx, dext, ext)) ||
      (st = upload_vec(ctx, doff, offs)) || (st = upload_vec(ctx, dsc, scale)))
    return st;
  const size_t need = (size_t)offs.back() * sizeof(double);
  if (a->bytes != need) {
    if (a->data) dev_free(ctx, a->data, a->bytes);
    a->data = nullptr;
    a->bytes = 0;
    if (need) {
      void* p = nullptr;
      if ((st = dev_alloc(ctx, &p, need))) return st;
      a->data = static_cast<double*>(p);
      a->bytes = need;
    }
  }
  GenDesc g{};
  g.rank = a->rank;
  for (int d = 0; d < a->rank; ++d) g.gext[d] = a->hm[d].back() - a->hm[d][0];
  g.seed = seed;
  g.stream = stream;
  g.kind = kind;
  launch_generate(ctx->stream, g, np, dlo.as<int64_t>(), dext.as<int32_t>(), doff.as<int64_t>(),
                  dsc.as<double>(), a->data);
  CUDA_TRY(ctx, cudaGetLastError());
  if (compute_shape) {
    DBuf dn(ctx);
    if ((st = dn.alloc(std::max<int64_t>(1, np) * sizeof(float)))) return st;
    launch_tile_norms(ctx->stream, np, doff.as<int64_t>(), a->data, dn.as<float>());
    CUDA_TRY(ctx, cudaGetLastError());
    std::vector<float> pn(np);
    if (np)
      CUDA_TRY(ctx, cudaMemcpyAsync(pn.data(), dn.p, np * sizeof(float), cudaMemcpyDeviceToHost,
                                    ctx->stream));
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    std::vector<float> norms(n, 0.0f);
    for (int64_t x = 0; x < np; ++x) norms[present[x]] = pn[x];
    const float thr = threshold < 0 ? ctx->threshold : threshold;
    a->dense = false;
    a->threshold = thr;
    a->norms = norms;
    a->zero_count = scale_norms(a, a->norms, thr);
  }
  return compact_tiles(ctx, a, present, offs);
}

tagpu_status tagpu_array_truncate(tagpu_array* a, float threshold) {
  if (!a) return TAGPU_ERR_INVALID;
  tagpu_ctx* ctx = a->ctx;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  if (a->dense) return TAGPU_OK;   // DensePolicy: no-op
  cudaSetDevice(ctx->device);
  if (tagpu_status st = materialize(a)) return st;
  const float thr = threshold < 0 ? ctx->threshold : threshold;
  const int64_t n = a->ntiles();
  std::vector<int64_t> present, offs(1, 0);
  for (int64_t t = 0; t < n; ++t) {
    if (a->off[t] < 0) continue;
    present.push_back(t);
    offs.push_back(offs.back() + a->tile_volume(t));
  }
  const int64_t np = (int64_t)present.size();
  tagpu_status st;
  DBuf doff(ctx), dn(ctx);
  if ((st = upload_vec(ctx, doff, offs)) ||
      (st = dn.alloc(std::max<int64_t>(1, np) * sizeof(float))))
    return st;
  launch_tile_norms(ctx->stream, np, doff.as<int64_t>(), a->data, dn.as<float>());
  CUDA_TRY(ctx, cudaGetLastError());
  std::vector<float> pn(np);
  if (np)
    CUDA_TRY(ctx, cudaMemcpyAsync(pn.data(), dn.p, np * sizeof(float), cudaMemcpyDeviceToHost,
                                  ctx->stream));
  CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  std::vector<float> norms(n, 0.0f);
  for (int64_t x = 0; x < np; ++x) norms[present[x]] = pn[x];
  a->threshold = thr;
  a->norms = norms;
  a->zero_count = scale_norms(a, a->norms, thr);
  return compact_tiles(ctx, a, present, offs);
}

tagpu_status tagpu_array_get_info(const tagpu_array* a, tagpu_array_info* info) {
  if (!a || !info) return TAGPU_ERR_INVALID;
  info->rank = a->rank;
  info->dense = a->dense ? 1 : 0;
  info->ntiles_total = a->ntiles();
  int64_t nz = 0;
  for (auto o : a->off) nz += o >= 0;
  info->nonzero_tiles = nz;
  info->zero_tiles = a->dense ? 0 : a->zero_count;
  info->elements = a->elements;
  info->threshold = a->threshold;
  info->device_bytes = a->bytes;
  for (int d = 0; d < 8; ++d) info->ntiles[d] = d < a->rank ? a->nt[d] : 0;
  return TAGPU_OK;
}

tagpu_status tagpu_array_get_norms(const tagpu_array* a, float* norms) {
  if (!a || !norms) return TAGPU_ERR_INVALID;
  const int64_t n = a->ntiles();
  if (a->dense) {
    for (int64_t t = 0; t < n; ++t) norms[t] = std::numeric_limits<float>::infinity();
  } else {
    std::copy(a->norms.begin(), a->norms.end(), norms);
  }
  return TAGPU_OK;
}

tagpu_status tagpu_array_get_tile_offsets(const tagpu_array* a, int64_t* offsets) {
  if (!a || !offsets) return TAGPU_ERR_INVALID;
  std::copy(a->off.begin(), a->off.end(), offsets);
  return TAGPU_OK;
}

tagpu_status tagpu_array_get_tile(const tagpu_array* a, int64_t ordinal, double* tile,
                                  int64_t n) {
  if (!a) return TAGPU_ERR_INVALID;
  tagpu_ctx* ctx = a->ctx;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  if (ordinal < 0 || ordinal >= (int64_t)a->off.size())
    return fail(ctx, TAGPU_ERR_INVALID, "get_tile: ordinal %lld outside the tile grid",
                (long long)ordinal);
  if (a->off[ordinal] < 0)
    return fail(ctx, TAGPU_ERR_INVALID, "get_tile: tile %lld is zero", (long long)ordinal);
  const int64_t vol = a->tile_volume(ordinal);
  if (n != vol)
    return fail(ctx, TAGPU_ERR_INVALID, "get_tile: buffer holds %lld elements, tile %lld",
                (long long)n, (long long)vol);
  if (n && !tile) return fail(ctx, TAGPU_ERR_INVALID, "get_tile: null buffer");
  cudaSetDevice(ctx->device);
  if (tagpu_status st = materialize(a)) return st;
  if (n)
    CUDA_TRY(ctx, cudaMemcpyAsync(tile, a->data + a->off[ordinal], n * sizeof(double),
                                  cudaMemcpyDeviceToHost, ctx->stream));
  CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return TAGPU_OK;
}

// ---- archive I/O ------------------------------------------------------------
// The order of DistArray::serialize (dist_array.h:1583-1592) with a
// single-rank world: a type tag, world size and rank, the TiledRange, the
// shape, the number of stored tiles, then each stored tile (its range and its
// row-major data) in ordinal order.  Little endian, fixed-width fields:
//   "TAGPUARR" u32 version=1 | u32 type tag (1 = Tensor<double>)
//   i64 world size (1) | i64 world rank (0)
//   u32 rank | per dimension: i64 ntiles, i64 hashmarks[ntiles + 1]
//   u8 dense | f32 threshold | i64 zero tiles | f32 scaled norms[tiles] (sparse)
//   i64 stored tiles | per tile: i64 ordinal, i64 lo[rank], i64 hi[rank],
//                                f64 data[volume]
// Tiles move through a pinned staging buffer, so arrays larger than host
// memory stream through.
}  // extern "C"

namespace {
struct HostMap {
  void* base;
  size_t len;
  bool mapped;   // mmap + cudaHostRegister (else cudaHostAlloc)
};
std::mutex& host_maps_mu() {
  static std::mutex m;
  return m;
}
std::unordered_map<void*, HostMap>& host_maps() {
  static std::unordered_map<void*, HostMap> m;
  return m;
}
constexpr char kArchiveMagic[8] = {'T', 'A', 'G', 'P', 'U', 'A', 'R', 'R'};
constexpr size_t kStage = size_t(64) << 20;

struct PinnedStage {
  void* p = nullptr;
  PinnedStage() {
    if (cudaMallocHost(&p, kStage) != cudaSuccess) p = nullptr;
  }
  ~PinnedStage() {
    if (p) cudaFreeHost(p);
  }
};

struct File {
  FILE* f = nullptr;
  File(const char* path, const char* mode) : f(fopen(path, mode)) {}
  ~File() {
    if (f) fclose(f);
  }
  template <typename T>
  bool put(const T& x) { return fwrite(&x, sizeof(T), 1, f) == 1; }
  template <typename T>
  bool get(T& x) { return fread(&x, sizeof(T), 1, f) == 1; }
};
}  // namespace

extern "C" {

// Host buffers: an anonymous mapping on base pages (huge pages gave the host
// link no measurable gain), touched and registered with CUDA; cudaHostAlloc
// where that fails.  The mapping of each buffer is remembered for the free.
tagpu_status tagpu_host_alloc(tagpu_ctx* ctx, size_t bytes, void** p) {
  if (!ctx || !p) return TAGPU_ERR_INVALID;
  *p = nullptr;
  cudaSetDevice(ctx->device);
  if (bytes == 0) return TAGPU_OK;
  {
    void* m = mmap(nullptr, bytes, PROT_READ | PROT_WRITE, MAP_PRIVATE | MAP_ANONYMOUS, -1, 0);
    if (m != MAP_FAILED) {
      madvise(m, bytes, MADV_NOHUGEPAGE);
      memset(m, 0, bytes);
      if (cudaHostRegister(m, bytes, cudaHostRegisterDefault) == cudaSuccess) {
        std::lock_guard<std::mutex> lk(host_maps_mu());
        host_maps()[m] = HostMap{m, bytes, true};
        *p = m;
        return TAGPU_OK;
      }
      cudaGetLastError();
      munmap(m, bytes);
    }
  }
  const cudaError_t e = cudaHostAlloc(p, bytes, cudaHostAllocDefault);
  if (e != cudaSuccess) {
    *p = nullptr;
    return fail(ctx, TAGPU_ERR_NOMEM, "cudaHostAlloc(%zu) failed: %s", bytes,
                cudaGetErrorString(e));
  }
  std::lock_guard<std::mutex> lk(host_maps_mu());
  host_maps()[*p] = HostMap{*p, bytes, false};
  return TAGPU_OK;
}

tagpu_status tagpu_host_free(tagpu_ctx* ctx, void* p) {
  if (!ctx) return TAGPU_ERR_INVALID;
  if (!p) return TAGPU_OK;
  HostMap hm{};
  {
    std::lock_guard<std::mutex> lk(host_maps_mu());
    auto it = host_maps().find(p);
    if (it == host_maps().end())
      return fail(ctx, TAGPU_ERR_INVALID, "host_free: not a tagpu host buffer");
    hm = it->second;
    host_maps().erase(it);
  }
  if (hm.mapped) {
    cudaHostUnregister(p);
    munmap(hm.base, hm.len);
  } else {
    cudaFreeHost(p);
  }
  return TAGPU_OK;
}

tagpu_status tagpu_array_save(const tagpu_array* a, const char* path) {
  if (!a || !path) return TAGPU_ERR_INVALID;
  tagpu_ctx* ctx = a->ctx;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  if (tagpu_status st = materialize(a)) return st;
  File out(path, "wb");
  if (!out.f) return fail(ctx, TAGPU_ERR_INVALID, "save: cannot open %s", path);
  PinnedStage stage;
  if (!stage.p) return fail(ctx, TAGPU_ERR_NOMEM, "save: no pinned staging buffer");
  bool ok = fwrite(kArchiveMagic, 1, 8, out.f) == 8;
  ok = ok && out.put<uint32_t>(1) && out.put<uint32_t>(1) && out.put<int64_t>(1) &&
       out.put<int64_t>(0) && out.put<uint32_t>((uint32_t)a->rank);
  for (int d = 0; d < a->rank && ok; ++d) {
    ok = out.put<int64_t>(a->nt[d]) &&
         fwrite(a->hm[d].data(), 8, a->hm[d].size(), out.f) == a->hm[d].size();
  }
  const int64_t n = a->ntiles();
  ok = ok && out.put<uint8_t>(a->dense ? 1 : 0) && out.put<float>(a->threshold) &&
       out.put<int64_t>(a->zero_count);
  if (ok && !a->dense) ok = fwrite(a->norms.data(), 4, (size_t)n, out.f) == (size_t)n;
  int64_t count = 0;
  for (int64_t t = 0; t < n; ++t) count += a->off[t] >= 0;
  ok = ok && out.put<int64_t>(count);
  int64_t idx[8];
  for (int64_t t = 0; t < n && ok; ++t) {
    if (a->off[t] < 0) continue;
    a->tile_index(t, idx);
    ok = out.put<int64_t>(t);
    for (int d = 0; d < a->rank && ok; ++d) ok = out.put<int64_t>(a->hm[d][idx[d]]);
    for (int d = 0; d < a->rank && ok; ++d) ok = out.put<int64_t>(a->hm[d][idx[d] + 1]);
    const size_t bytes = (size_t)a->tile_volume(t) * sizeof(double);
    for (size_t x = 0; x < bytes && ok; x += kStage) {
      const size_t m = std::min(kStage, bytes - x);
      CUDA_TRY(ctx, cudaMemcpyAsync(stage.p, (const uint8_t*)(a->data + a->off[t]) + x, m,
                                    cudaMemcpyDeviceToHost, ctx->stream));
      CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
      ok = fwrite(stage.p, 1, m, out.f) == m;
    }
  }
  if (!ok) return fail(ctx, TAGPU_ERR_INVALID, "save: write to %s failed", path);
  return TAGPU_OK;
}

tagpu_status tagpu_array_load(tagpu_ctx* ctx, const char* path, tagpu_array** out_a) {
  if (!ctx || !path || !out_a) return TAGPU_ERR_INVALID;
  *out_a = nullptr;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  File in(path, "rb");
  if (!in.f) return fail(ctx, TAGPU_ERR_INVALID, "load: cannot open %s", path);
  auto bad = [&](const char* what) {
    return fail(ctx, TAGPU_ERR_INVALID, "load: %s: %s", path, what);
  };
  char magic[8];
  uint32_t version = 0, tag = 0, rank = 0;
  int64_t wsize = 0, wrank = 0;
  if (fread(magic, 1, 8, in.f) != 8 || memcmp(magic, kArchiveMagic, 8) != 0)
    return bad("not an array archive");
  if (!in.get(version) || version != 1) return bad("unknown archive version");
  if (!in.get(tag) || tag != 1) return bad("tile type is not Tensor<double>");
  if (!in.get(wsize) || !in.get(wrank) || wsize != 1 || wrank != 0)
    return bad("archive of another world");
  if (!in.get(rank) || rank > 8) return bad("bad rank");
  std::vector<std::vector<int64_t>> hm(rank);
  for (uint32_t d = 0; d < rank; ++d) {
    int64_t nt = -1;
    if (!in.get(nt) || nt < 0 || nt > (int64_t(1) << 32)) return bad("bad tile count");
    hm[d].resize((size_t)nt + 1);
    if (fread(hm[d].data(), 8, hm[d].size(), in.f) != hm[d].size()) return bad("truncated");
    for (int64_t i = 0; i < nt; ++i)
      if (hm[d][i + 1] < hm[d][i]) return bad("hashmarks decrease");
  }
  std::unique_ptr<tagpu_array> a(new_array(ctx, hm));
  uint8_t dense = 1;
  float thr = 0.0f;
  int64_t zeros = 0;
  if (!in.get(dense) || !in.get(thr) || !in.get(zeros)) return bad("truncated");
  const int64_t n = a->ntiles();
  a->dense = dense != 0;
  if (!a->dense) {
    a->norms.resize((size_t)n);
    if (fread(a->norms.data(), 4, (size_t)n, in.f) != (size_t)n) return bad("truncated");
    a->threshold = thr;
    a->zero_count = zeros;
  }
  pack_offsets(a.get());
  tagpu_status st = ensure_storage(a.get());
  if (st) return st;
  int64_t count = -1, expect = 0;
  for (int64_t t = 0; t < n; ++t) expect += a->off[t] >= 0;
  if (!in.get(count) || count != expect) return bad("stored tiles do not match the shape");
  PinnedStage stage;
  if (!stage.p) return fail(ctx, TAGPU_ERR_NOMEM, "load: no pinned staging buffer");
  int64_t idx[8];
  for (int64_t c = 0; c < count; ++c) {
    int64_t t = -1;
    if (!in.get(t) || t < 0 || t >= n || a->off[t] < 0) return bad("bad tile ordinal");
    a->tile_index(t, idx);
    for (uint32_t d = 0; d < rank; ++d) {
      int64_t lo = 0;
      if (!in.get(lo) || lo != a->hm[d][idx[d]]) return bad("tile range mismatch");
    }
    for (uint32_t d = 0; d < rank; ++d) {
      int64_t hi = 0;
      if (!in.get(hi) || hi != a->hm[d][idx[d] + 1]) return bad("tile range mismatch");
    }
    const size_t bytes = (size_t)a->tile_volume(t) * sizeof(double);
    for (size_t x = 0; x < bytes; x += kStage) {
      const size_t m = std::min(kStage, bytes - x);
      if (fread(stage.p, 1, m, in.f) != m) return bad("truncated tile data");
      CUDA_TRY(ctx, cudaMemcpyAsync((uint8_t*)(a->data + a->off[t]) + x, stage.p, m,
                                    cudaMemcpyHostToDevice, ctx->stream));
      CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    }
  }
  *out_a = a.release();
  return TAGPU_OK;
}

// ---------------------------------------------------------------------------
// Archives in DistArray::serialize field order (one rank)
// ---------------------------------------------------------------------------
// The stream a MADNESS binary archive receives from DistArray::serialize
// (dist_array.h:1583-1590) for one rank: every scalar is its raw
// little-endian bytes, arrays written through archive::wrap carry no length,
// vectors carry a size_t count first.
//   u64 typeid(DistArray).hash_code, i32 world size, i32 world rank,
//   TiledRange  (tiled_range.h:392):  Range tiles, Range elements,
//               u64 modes, per mode TiledRange1 (tiled_range1.h:405):
//               Range1 tiles, Range1 elements, u64 ntiles, Range1 per tile
//   shape       SparseShape (sparse_shape.h:1918-1923): Tensor<float> of the
//               scaled norms, per mode ValArray<float> of tile extents
//               (u64 size + floats, val_array.h:454-457), u64 zero count;
//               DenseShape writes nothing (dense_shape.h:390)
//   u64 typeid(pmap).hash_code, i64 tile count,
//   per stored tile Tensor<double> (tensor/tensor.h:1389-1416):
//               u8 empty, Range, u64 nbatch, f64 data[volume * nbatch]
// Range (range.h:1143-1157): u32 rank, i64 lobound[r], upbound[r],
// extent[r], stride[r] (row-major), i64 offset = sum lobound * stride,
// u64 volume.  Range1 (range1.h:195-204): i64 first, i64 second.
// The two hash codes are values of the writer's C++ implementation; they are
// passed through, never interpreted.
namespace {
struct SerialRange {
  std::vector<int64_t> lo, up;
};
bool put_range(File& f, const std::vector<int64_t>& lo, const std::vector<int64_t>& up) {
  const uint32_t r = (uint32_t)lo.size();
  bool ok = f.put<uint32_t>(r);
  std::vector<int64_t> ext(r), stride(r);
  int64_t vol = 1, off = 0;
  for (int d = (int)r - 1; d >= 0; --d) {
    ext[d] = up[d] - lo[d];
    stride[d] = vol;
    off += lo[d] * stride[d];
    vol *= ext[d];
  }
  for (auto* v : {&lo, &up, (const std::vector<int64_t>*)&ext,
                  (const std::vector<int64_t>*)&stride})
    for (int64_t x : *v) ok = ok && f.put<int64_t>(x);
  return ok && f.put<int64_t>(off) && f.put<uint64_t>((uint64_t)vol);
}
// Reads a Range and checks that its derived fields agree with its bounds.
bool get_range(File& f, SerialRange* r, uint32_t max_rank = 8) {
  uint32_t rank = 0;
  if (!f.get(rank) || rank > max_rank) return false;
  std::vector<int64_t> v(4 * (size_t)rank);
  for (auto& x : v)
    if (!f.get(x)) return false;
  int64_t off = 0;
  uint64_t vol = 0;
  if (!f.get(off) || !f.get(vol)) return false;
  r->lo.assign(v.begin(), v.begin() + rank);
  r->up.assign(v.begin() + rank, v.begin() + 2 * rank);
  int64_t evol = 1, eoff = 0;
  for (int d = (int)rank - 1; d >= 0; --d) {
    const int64_t ext = r->up[d] - r->lo[d];
    if (ext < 0 || v[2 * rank + d] != ext || v[3 * rank + d] != evol) return false;
    eoff += r->lo[d] * evol;
    evol *= ext;
  }
  return eoff == off && (uint64_t)evol == vol;
}
}  // namespace

tagpu_status tagpu_array_serialize(const tagpu_array* a, const char* path,
                                   uint64_t array_type_hash, uint64_t pmap_type_hash) {
  if (!a || !path) return TAGPU_ERR_INVALID;
  tagpu_ctx* ctx = a->ctx;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  if (tagpu_status st = materialize(a)) return st;
  File out(path, "wb");
  if (!out.f) return fail(ctx, TAGPU_ERR_INVALID, "serialize: cannot open %s", path);
  PinnedStage stage;
  if (!stage.p) return fail(ctx, TAGPU_ERR_NOMEM, "serialize: no pinned staging buffer");
  const int r = a->rank;
  bool ok = out.put<uint64_t>(array_type_hash) && out.put<int32_t>(1) && out.put<int32_t>(0);
  // TiledRange: tile range, element range, the modes' TiledRange1
  std::vector<int64_t> z(r, 0), nt(r), elo(r), eup(r);
  for (int d = 0; d < r; ++d) {
    nt[d] = a->nt[d];
    elo[d] = a->hm[d].front();
    eup[d] = a->hm[d].back();
  }
  ok = ok && put_range(out, z, nt) && put_range(out, elo, eup) && out.put<uint64_t>((uint64_t)r);
  for (int d = 0; d < r && ok; ++d) {
    ok = out.put<int64_t>(0) && out.put<int64_t>(a->nt[d]) && out.put<int64_t>(elo[d]) &&
         out.put<int64_t>(eup[d]) && out.put<uint64_t>((uint64_t)a->nt[d]);
    for (int64_t i = 0; i < a->nt[d] && ok; ++i)
      ok = out.put<int64_t>(a->hm[d][i]) && out.put<int64_t>(a->hm[d][i + 1]);
  }
  const int64_t n = a->ntiles();
  if (!a->dense) {
    // SparseShape: the norm tensor over the tile range (nbatch 1), the tile
    // extents of every mode as floats, the zero-tile count
    ok = ok && out.put<uint8_t>(n == 0 ? 1 : 0);
    if (n > 0) {
      ok = ok && put_range(out, z, nt) && out.put<uint64_t>(1) &&
           fwrite(a->norms.data(), 4, (size_t)n, out.f) == (size_t)n;
    }
    for (int d = 0; d < r && ok; ++d) {
      ok = out.put<uint64_t>((uint64_t)a->nt[d]);
      for (int64_t i = 0; i < a->nt[d] && ok; ++i)
        ok = out.put<float>((float)(a->hm[d][i + 1] - a->hm[d][i]));
    }
    ok = ok && out.put<uint64_t>((uint64_t)a->zero_count);
  }
  int64_t count = 0;
  for (int64_t t = 0; t < n; ++t) count += a->off[t] >= 0;
  ok = ok && out.put<uint64_t>(pmap_type_hash) && out.put<int64_t>(count);
  int64_t idx[8];
  std::vector<int64_t> lo(r), up(r);
  for (int64_t t = 0; t < n && ok; ++t) {
    if (a->off[t] < 0) continue;
    a->tile_index(t, idx);
    for (int d = 0; d < r; ++d) {
      lo[d] = a->hm[d][idx[d]];
      up[d] = a->hm[d][idx[d] + 1];
    }
    ok = out.put<uint8_t>(0) && put_range(out, lo, up) && out.put<uint64_t>(1);
    const size_t bytes = (size_t)a->tile_volume(t) * sizeof(double);
    for (size_t x = 0; x < bytes && ok; x += kStage) {
      const size_t m = std::min(kStage, bytes - x);
      CUDA_TRY(ctx, cudaMemcpyAsync(stage.p, (const uint8_t*)(a->data + a->off[t]) + x, m,
                                    cudaMemcpyDeviceToHost, ctx->stream));
      CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
      ok = fwrite(stage.p, 1, m, out.f) == m;
    }
  }
  if (!ok) return fail(ctx, TAGPU_ERR_INVALID, "serialize: write to %s failed", path);
  return TAGPU_OK;
}

tagpu_status tagpu_array_deserialize(tagpu_ctx* ctx, const char* path, int sparse,
                                     tagpu_array** out_a, uint64_t* array_type_hash,
                                     uint64_t* pmap_type_hash) {
  if (!ctx || !path || !out_a) return TAGPU_ERR_INVALID;
  *out_a = nullptr;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  File in(path, "rb");
  if (!in.f) return fail(ctx, TAGPU_ERR_INVALID, "deserialize: cannot open %s", path);
  auto bad = [&](const char* what) {
    return fail(ctx, TAGPU_ERR_INVALID, "deserialize: %s: %s", path, what);
  };
  uint64_t th = 0, ph = 0;
  int32_t wsize = 0, wrank = 0;
  if (!in.get(th) || !in.get(wsize) || !in.get(wrank)) return bad("truncated header");
  if (wsize != 1 || wrank != 0)
    return bad("archive of a multi-rank world (one rank's tiles only); this engine is one rank");
  SerialRange tr, er;
  uint64_t modes = 0;
  if (!get_range(in, &tr) || !get_range(in, &er) || !in.get(modes) || modes != tr.lo.size())
    return bad("bad TiledRange");
  const int r = (int)modes;
  std::vector<std::vector<int64_t>> hm(r);
  for (int d = 0; d < r; ++d) {
    int64_t t0, t1, e0, e1;
    uint64_t cnt = 0;
    if (!in.get(t0) || !in.get(t1) || !in.get(e0) || !in.get(e1) || !in.get(cnt))
      return bad("bad TiledRange1");
    if (t0 != tr.lo[d] || t1 != tr.up[d] || e0 != er.lo[d] || e1 != er.up[d] ||
        (int64_t)cnt != t1 - t0 || cnt > (uint64_t(1) << 32))
      return bad("TiledRange1 disagrees with the TiledRange");
    hm[d].reserve(cnt + 1);
    for (uint64_t i = 0; i < cnt; ++i) {
      int64_t f = 0, s = 0;
      if (!in.get(f) || !in.get(s) || s < f) return bad("bad tile range");
      if (i == 0) {
        if (f != e0) return bad("first tile does not start the element range");
        hm[d].push_back(f);
      } else if (f != hm[d].back()) {
        return bad("tiles of a mode leave gaps");
      }
      hm[d].push_back(s);
    }
    if (cnt == 0) hm[d].push_back(e0);
    if (hm[d].back() != e1) return bad("tiles do not end the element range");
  }
  std::unique_ptr<tagpu_array> a(new_array(ctx, hm));
  const int64_t n = a->ntiles();
  if (sparse) {
    uint8_t empty = 1;
    if (!in.get(empty)) return bad("truncated shape");
    a->dense = false;
    a->norms.assign((size_t)n, 0.0f);
    if (!empty) {
      SerialRange nr;
      uint64_t nb = 0;
      if (!get_range(in, &nr) || !in.get(nb) || nb != 1 || nr.lo != std::vector<int64_t>(r, 0) ||
          nr.up != tr.up)
        return bad("norm tensor does not span the tile range");
      if (fread(a->norms.data(), 4, (size_t)n, in.f) != (size_t)n) return bad("truncated norms");
    }
    for (int d = 0; d < r; ++d) {
      uint64_t sz = 0;
      if (!in.get(sz) || (int64_t)sz != a->nt[d]) return bad("bad size vector");
      for (uint64_t i = 0; i < sz; ++i) {
        float x = 0;
        if (!in.get(x) || x != (float)(hm[d][i + 1] - hm[d][i]))
          return bad("size vector disagrees with the tiling");
      }
    }
    uint64_t zc = 0;
    if (!in.get(zc)) return bad("truncated shape");
    int64_t zeros = 0;
    for (float x : a->norms) zeros += x == 0.0f;
    if ((int64_t)zc != zeros) return bad("zero-tile count disagrees with the norms");
    a->zero_count = zeros;
    // The writer's threshold is process-wide and not stored; every tile with
    // a nonzero norm was kept by it, so the array's threshold is the context
    // default lowered, if need be, to the smallest nonzero norm.
    float thr = ctx->threshold;
    for (float x : a->norms)
      if (x > 0.0f && x < thr) thr = x;
    a->threshold = thr;
  }
  int64_t count = -1;
  if (!in.get(ph) || !in.get(count)) return bad("truncated");
  pack_offsets(a.get());
  tagpu_status st = ensure_storage(a.get());
  if (st) return st;
  int64_t expect = 0;
  for (int64_t t = 0; t < n; ++t) expect += a->off[t] >= 0;
  if (count != expect) return bad("stored tiles do not match the shape");
  PinnedStage stage;
  if (!stage.p) return fail(ctx, TAGPU_ERR_NOMEM, "deserialize: no pinned staging buffer");
  std::vector<char> seen((size_t)n, 0);
  for (int64_t c = 0; c < count; ++c) {
    uint8_t empty = 1;
    SerialRange tr1;
    uint64_t nb = 0;
    if (!in.get(empty) || empty || !get_range(in, &tr1) || !in.get(nb) || nb != 1 ||
        (int)tr1.lo.size() != r)
      return bad("bad tile header");
    // the tile's ordinal from its lower bounds
    int64_t t = 0;
    for (int d = 0; d < r; ++d) {
      const auto it = std::lower_bound(hm[d].begin(), hm[d].end() - 1, tr1.lo[d]);
      if (it == hm[d].end() - 1 || *it != tr1.lo[d] || *(it + 1) != tr1.up[d])
        return bad("tile range is not a tile of the TiledRange");
      t = t * a->nt[d] + (it - hm[d].begin());
    }
    if (a->off[t] < 0 || seen[t]) return bad("tile absent from the shape or repeated");
    seen[t] = 1;
    const size_t bytes = (size_t)a->tile_volume(t) * sizeof(double);
    for (size_t x = 0; x < bytes; x += kStage) {
      const size_t m = std::min(kStage, bytes - x);
      if (fread(stage.p, 1, m, in.f) != m) return bad("truncated tile data");
      CUDA_TRY(ctx, cudaMemcpyAsync((uint8_t*)(a->data + a->off[t]) + x, stage.p, m,
                                    cudaMemcpyHostToDevice, ctx->stream));
      CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    }
  }
  if (array_type_hash) *array_type_hash = th;
  if (pmap_type_hash) *pmap_type_hash = ph;
  *out_a = a.release();
  return TAGPU_OK;
}

tagpu_status tagpu_array_get_hashmarks(const tagpu_array* a, int d, int64_t* hashmarks) {
  if (!a || !hashmarks || d < 0 || d >= a->rank) return TAGPU_ERR_INVALID;
  std::copy(a->hm[d].begin(), a->hm[d].end(), hashmarks);
  return TAGPU_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// contraction: plan (host + kernels a/b, allocations) then enqueue (kernel d
// and the result permutation, no host synchronisation, capturable)
// ---------------------------------------------------------------------------

namespace tagpu {

// Tile permutation of a whole array, planned once and enqueued any number of
// times (the descriptors live on the device).
struct PermutePlan {
  PermuteDesc pd{};
  int64_t ntl = 0, nitems = 0;
  DBuf ext, in_off, out_off, item_start;
  explicit PermutePlan(tagpu_ctx* c) : ext(c), in_off(c), out_off(c), item_start(c) {}

  // dst must already have the permuted tiling and packed offsets
  tagpu_status build(const tagpu_array* a, const std::vector<int>& perm,
                     const tagpu_array* dst) {
    tagpu_ctx* ctx = a->ctx;
    pd.rank = a->rank;
    for (int d = 0; d < a->rank; ++d) pd.perm[d] = perm[d];
    std::vector<int32_t> e32;
    std::vector<int64_t> io, oo, is(1, 0);
    int64_t idx[8], nidx[8], e[8];
    for (int64_t t = 0; t < a->ntiles(); ++t) {
      if (a->off[t] < 0) continue;
      a->tile_index(t, idx);
      for (int d = 0; d < a->rank; ++d) {
        e[d] = a->hm[d][idx[d] + 1] - a->hm[d][idx[d]];
        e32.push_back((int32_t)e[d]);
        nidx[perm[d]] = idx[d];
      }
      int64_t no = 0;
      for (int d = 0; d < a->rank; ++d) no = no * dst->nt[d] + nidx[d];
      io.push_back(a->off[t]);
      oo.push_back(dst->off[no]);
      is.push_back(is.back() + (a->rank ? permute_items(pd, e) : 0));
    }
    ntl = (int64_t)io.size();
    nitems = is.back();
    tagpu_status st;
    if ((st = upload_vec(ctx, ext, e32)) || (st = upload_vec(ctx, in_off, io)) ||
        (st = upload_vec(ctx, out_off, oo)) || (st = upload_vec(ctx, item_start, is)))
      return st;
    return TAGPU_OK;
  }
  void enqueue(cudaStream_t s, const double* in, double* out) const {
    if (ntl == 0) return;
    if (pd.rank == 0) {
      cudaMemcpyAsync(out, in, sizeof(double), cudaMemcpyDeviceToDevice, s);
      return;
    }
    launch_permute(s, pd, ntl, ext.as<int32_t>(), in_off.as<int64_t>(), out_off.as<int64_t>(),
                   item_start.as<int64_t>(), nitems, in, out);
  }
};

// New array with the permuted tiling, norms and packed storage (no data).
tagpu_array* permuted_layout(const tagpu_array* a, const std::vector<int>& perm) {
  std::vector<std::vector<int64_t>> nhm(a->rank);
  for (int d = 0; d < a->rank; ++d) nhm[perm[d]] = a->hm[d];
  tagpu_array* r = new_array(a->ctx, nhm);
  r->dense = a->dense;
  r->threshold = a->threshold;
  r->zero_count = a->zero_count;
  if (!a->dense) r->norms = permute_grid(a->norms, a->nt, perm);
  pack_offsets(r);
  return r;
}

// Everything one contraction needs after planning.
struct Contraction {
  tagpu_ctx* ctx;
  std::vector<std::string> ai, bi, ci;
  PermOpt po;
  int inner = 0, lorank = 0;
  std::vector<int> lperm, rperm, cperm;
  int64_t Mt = 1, Nt = 1, Kt = 1;
  // general products: nfused leading fused (Hadamard) modes in the canonical
  // layouts (fused, left free, contracted) x (fused, contracted, right free)
  // -> (fused, left free, right free); Ht fused tiles ("slabs") of hsz
  // elements each; every per-slab array (norms, offsets, pairs) is stored
  // slab after slab.  Ordinary contractions: nfused 0, Ht 1.
  int nfused = 0;
  int64_t Ht = 1;
  std::vector<int32_t> hsz{1};
  std::vector<GemmView> gviews;         // general products: one view per fused element
  std::vector<int32_t> msz, nsz, ksz;
  std::vector<float> kfl;               // k_sizes (float) for the shape gemm
  std::vector<float> ln, rn;            // GEMM-order norms
  float lthr = 0, rthr = 0, cthr = 0;
  bool dense = false;
  double alpha = 1.0;
  int precision = TAGPU_PRECISION_FP64;
  int slices = 7;
  // operands in GEMM order
  tagpu_array* Aop = nullptr;
  tagpu_array* Bop = nullptr;
  std::unique_ptr<tagpu_array> Aown, Bown;
  int a_trans = 0, b_trans = 0;
  std::vector<int64_t> aoff, boff;
  // result in GEMM order (left outer, right outer) and in the target order
  std::unique_ptr<tagpu_array> C, Cfinal;
  std::unique_ptr<PermutePlan> post;
  std::vector<float> cn;
  int64_t zero_count = 0;
  int64_t npairs = 0;
  double flops = 0;
  // device state
  DBuf d_msz, d_nsz, d_ksz, d_aoff, d_boff, d_poff, d_kidx, d_coff;
  std::vector<WorkItem> items;
  GemmView view{};                      // fixed at plan time (device pointers)
  double* post_in = nullptr;            // GEMM-order result
  double* post_out = nullptr;           // target-order result
  tagpu_contract_stats st{};
  // emulated form scratch: one plan per GEMM view (one for an ordinary
  // contraction, one per fused element for a general product)
  std::vector<OzakiPlan*> ozs;
  size_t oz_bytes = 0;
  std::string tune_log;
  explicit Contraction(tagpu_ctx* c)
      : ctx(c), d_msz(c), d_nsz(c), d_ksz(c), d_aoff(c), d_boff(c), d_poff(c), d_kidx(c),
        d_coff(c) {}
  ~Contraction();
  tagpu_array* result() { return Cfinal ? Cfinal.get() : C.get(); }
  bool emulated() const { return precision == TAGPU_PRECISION_OZAKI && !ozs.empty(); }
};

Contraction::~Contraction() {
  for (OzakiPlan* pl : ozs) ozaki_destroy(pl);
  ctx->used -= oz_bytes;
}

}  // namespace tagpu

namespace {

std::vector<int32_t> fused_sizes(const tagpu_array* a, const std::vector<int>& dims) {
  std::vector<int32_t> out(1, 1);
  for (int d : dims) {
    std::vector<int32_t> nxt;
    nxt.reserve(out.size() * a->nt[d]);
    for (auto x : out)
      for (int64_t t = 0; t < a->nt[d]; ++t)
        nxt.push_back(x * (int32_t)(a->hm[d][t + 1] - a->hm[d][t]));
    out.swap(nxt);
  }
  return out;
}

// General (fused-index) product, ContEngine::init_struct_general and
// SparseShape::gemm_batched (sparse_shape.h:1707-1885): indices in both
// arguments and the target are fused, in both arguments only contracted, in
// one argument and the target free.  Arguments go to the canonical layouts
// (fused, left free, contracted) and (fused, contracted, right free), the
// result is (fused, left free, right free), permuted to the target after.
tagpu_status plan_general(Contraction& c, tagpu_array* A, tagpu_array* B) {
  tagpu_ctx* ctx = c.ctx;
  std::vector<std::string> F, L, K, R;
  for (auto& x : c.ai) {
    const bool inB = find_idx(c.bi, x) >= 0, inC = find_idx(c.ci, x) >= 0;
    if (inB && inC) F.push_back(x);
    else if (inB) K.push_back(x);
    else if (inC) L.push_back(x);
    else return fail(ctx, TAGPU_ERR_UNSUPPORTED, "index '%s' is summed over one argument only",
                     x.c_str());
  }
  for (auto& x : c.bi) {
    const bool inA = find_idx(c.ai, x) >= 0, inC = find_idx(c.ci, x) >= 0;
    if (!inA && inC) R.push_back(x);
    else if (!inA) return fail(ctx, TAGPU_ERR_UNSUPPORTED,
                               "index '%s' is summed over one argument only", x.c_str());
  }
  for (auto& x : c.ci)
    if (find_idx(c.ai, x) < 0 && find_idx(c.bi, x) < 0)
      return fail(ctx, TAGPU_ERR_INVALID, "target index '%s' is in neither argument", x.c_str());
  if (c.ci.size() != F.size() + L.size() + R.size())
    return fail(ctx, TAGPU_ERR_INVALID, "target indices repeat");
  c.po = PermOpt{};
  c.po.left = F;
  c.po.left.insert(c.po.left.end(), L.begin(), L.end());
  c.po.left.insert(c.po.left.end(), K.begin(), K.end());
  c.po.right = F;
  c.po.right.insert(c.po.right.end(), K.begin(), K.end());
  c.po.right.insert(c.po.right.end(), R.begin(), R.end());
  c.po.result = F;
  c.po.result.insert(c.po.result.end(), L.begin(), L.end());
  c.po.result.insert(c.po.result.end(), R.begin(), R.end());
  c.po.lop = c.po.rop = GENERAL;
  c.nfused = (int)F.size();
  c.inner = (int)K.size();
  c.lorank = (int)L.size();
  c.lperm = perm_between(c.ai, c.po.left);
  c.rperm = perm_between(c.bi, c.po.right);
  c.cperm = perm_between(c.po.result, c.ci);
  std::vector<int> f_dims, lo_dims, li_dims, ro_dims;
  for (auto& x : F) f_dims.push_back(find_idx(c.ai, x));
  for (auto& x : L) lo_dims.push_back(find_idx(c.ai, x));
  for (auto& x : K) li_dims.push_back(find_idx(c.ai, x));
  for (auto& x : R) ro_dims.push_back(find_idx(c.bi, x));
  for (auto* v : {&F, &K})
    for (auto& x : *v)
      if (A->hm[find_idx(c.ai, x)] != B->hm[find_idx(c.bi, x)])
        return fail(ctx, TAGPU_ERR_INVALID,
                    "the %s dimensions '%s' of the arguments are not congruent",
                    v == &F ? "fused" : "contracted", x.c_str());
  c.hsz = fused_sizes(A, f_dims);
  c.Ht = (int64_t)c.hsz.size();
  c.msz = fused_sizes(A, lo_dims);
  c.ksz = fused_sizes(A, li_dims);
  c.nsz = fused_sizes(B, ro_dims);
  c.Mt = (int64_t)c.msz.size();
  c.Kt = (int64_t)c.ksz.size();
  c.Nt = (int64_t)c.nsz.size();
  if (c.inner > 0) {
    auto sv = size_vectors(A);
    std::vector<std::vector<float>> ksv;
    for (int d : li_dims) ksv.push_back(sv[d]);
    c.kfl = outer_sizes(ksv, 0, ksv.size(), false);
  }
  return TAGPU_OK;
}

// Parse, classify, choose layouts, GEMM-order sizes and norms.
tagpu_status plan_contraction(Contraction& c, const char* c_idx, double alpha, tagpu_array* A,
                              const char* a_idx, tagpu_array* B, const char* b_idx,
                              float cthr) {
  tagpu_ctx* ctx = c.ctx;
  if (!parse_indices(a_idx, c.ai) || !parse_indices(b_idx, c.bi) || !parse_indices(c_idx, c.ci))
    return fail(ctx, TAGPU_ERR_INVALID, "malformed index list");
  if ((int)c.ai.size() != A->rank || (int)c.bi.size() != B->rank)
    return fail(ctx, TAGPU_ERR_INVALID, "index list rank does not match the array rank");
  if (A->dense != B->dense)
    return fail(ctx, TAGPU_ERR_UNSUPPORTED, "dense and sparse arguments cannot be mixed");
  bool general = false;
  for (auto& x : c.ci)
    general = general || (find_idx(c.ai, x) >= 0 && find_idx(c.bi, x) >= 0);
  if (general) {
    tagpu_status e = plan_general(c, A, B);
    if (e) return e;
    c.dense = A->dense;
    c.alpha = alpha;
    c.cthr = cthr;
    if (c.dense) {
      c.ln.assign(c.Ht * c.Mt * c.Kt, 1.0f);
      c.rn.assign(c.Ht * c.Kt * c.Nt, 1.0f);
      c.lthr = c.rthr = 0.0f;
    } else {
      c.ln = permute_grid(A->norms, A->nt, c.lperm);
      c.rn = permute_grid(B->norms, B->nt, c.rperm);
      c.lthr = A->threshold;
      c.rthr = B->threshold;
    }
    return TAGPU_OK;
  }
  // TensorProduct::Contraction: every target index is free in exactly one
  // argument, every other index is shared by both arguments
  for (auto& x : c.ci) {
    const bool inA = find_idx(c.ai, x) >= 0, inB = find_idx(c.bi, x) >= 0;
    if (inA == inB)
      return fail(ctx, TAGPU_ERR_UNSUPPORTED,
                  "index '%s' is not a free index of exactly one argument "
                  "(Hadamard and general products are not on this path)", x.c_str());
  }
  for (auto& x : c.ai)
    if (find_idx(c.bi, x) < 0 && find_idx(c.ci, x) < 0)
      return fail(ctx, TAGPU_ERR_UNSUPPORTED, "index '%s' is summed over one argument only",
                  x.c_str());
  for (auto& x : c.bi)
    if (find_idx(c.ai, x) < 0 && find_idx(c.ci, x) < 0)
      return fail(ctx, TAGPU_ERR_UNSUPPORTED, "index '%s' is summed over one argument only",
                  x.c_str());
  c.po = permopt(c.ai, c.bi, true);
  c.inner = (int)(c.ai.size() + c.bi.size() - c.po.result.size()) / 2;
  c.lorank = (int)c.ai.size() - c.inner;
  c.lperm = perm_between(c.ai, c.po.left);
  c.rperm = perm_between(c.bi, c.po.right);
  c.cperm = perm_between(c.po.result, c.ci);
  for (int x = 0; x < c.inner; ++x) {
    const std::string& v = c.po.left[c.lorank + x];
    const int da = find_idx(c.ai, v), db = find_idx(c.bi, v);
    if (A->hm[da] != B->hm[db])
      return fail(ctx, TAGPU_ERR_INVALID,
                  "the contracted dimensions '%s' of the arguments are not congruent",
                  v.c_str());
  }
  std::vector<int> lo_dims, li_dims, ro_dims;
  for (int x = 0; x < c.lorank; ++x) lo_dims.push_back(find_idx(c.ai, c.po.left[x]));
  for (int x = 0; x < c.inner; ++x) li_dims.push_back(find_idx(c.ai, c.po.left[c.lorank + x]));
  for (size_t x = c.inner; x < c.po.right.size(); ++x)
    ro_dims.push_back(find_idx(c.bi, c.po.right[x]));
  c.msz = fused_sizes(A, lo_dims);
  c.ksz = fused_sizes(A, li_dims);
  c.nsz = fused_sizes(B, ro_dims);
  c.Mt = (int64_t)c.msz.size();
  c.Kt = (int64_t)c.ksz.size();
  c.Nt = (int64_t)c.nsz.size();
  if (c.inner > 0) {
    auto sv = size_vectors(A);
    std::vector<std::vector<float>> ksv;
    for (int d : li_dims) ksv.push_back(sv[d]);
    c.kfl = outer_sizes(ksv, 0, ksv.size(), false);
  }
  c.dense = A->dense;
  c.alpha = alpha;
  c.cthr = cthr;
  if (c.dense) {
    c.ln.assign(c.Mt * c.Kt, 1.0f);
    c.rn.assign(c.Kt * c.Nt, 1.0f);
    c.lthr = c.rthr = 0.0f;
  } else {
    c.ln = permute_grid(A->norms, A->nt, c.lperm);
    c.rn = permute_grid(B->norms, B->nt, c.rperm);
    c.lthr = A->threshold;
    c.rthr = B->threshold;
  }
  return TAGPU_OK;
}

// Steps (a) and (b) on the device, slab by slab for general products
// (SparseShape::gemm_batched contracts every fused-tile slab as gemm does).
tagpu_status run_shape_and_pairs(Contraction& c) {
  tagpu_ctx* ctx = c.ctx;
  cudaStream_t s = ctx->stream;
  const int64_t H = c.Ht, MN = c.Mt * c.Nt, TOT = H * MN;
  const int64_t lslab = c.Mt * c.Kt, rslab = c.Kt * c.Nt;   // per-slab norm counts
  DBuf dL(ctx), dR(ctx), dK(ctx), dC(ctx), dz(ctx), dcnt(ctx), dfl(ctx);
  tagpu_status e;
  if ((e = upload_vec(ctx, dL, c.ln)) || (e = upload_vec(ctx, dR, c.rn)) ||
      (e = upload_vec(ctx, dK, c.kfl)) || (e = upload_vec(ctx, c.d_msz, c.msz)) ||
      (e = upload_vec(ctx, c.d_nsz, c.nsz)) || (e = upload_vec(ctx, c.d_ksz, c.ksz)))
    return e;
  if ((e = dC.alloc(std::max<int64_t>(1, TOT) * sizeof(float))) ||
      (e = dz.alloc(sizeof(unsigned long long))) ||
      (e = dcnt.alloc(std::max<int64_t>(1, TOT) * sizeof(int64_t))) ||
      (e = dfl.alloc(std::max<int64_t>(1, H) * sizeof(double))) ||
      (e = c.d_poff.alloc((TOT + 1) * sizeof(int64_t))))
    return e;
  CUDA_TRY(ctx, cudaMemsetAsync(dz.p, 0, sizeof(unsigned long long), s));
  CUDA_TRY(ctx, cudaMemsetAsync(dfl.p, 0, std::max<int64_t>(1, H) * sizeof(double), s));
  const float af = (float)std::fabs(c.alpha);
  {
    EventTimer tm(s);
    if (c.dense) {
      // DenseShape::gemm (dense_shape.h:378-390): every result tile present
      std::vector<float> ones(std::max<int64_t>(1, TOT), 1.0f);
      CUDA_TRY(ctx, cudaMemcpyAsync(dC.p, ones.data(), ones.size() * sizeof(float),
                                    cudaMemcpyHostToDevice, s));
      CUDA_TRY(ctx, cudaStreamSynchronize(s));
    } else if (c.inner > 0 && c.kfl.empty()) {
      CUDA_TRY(ctx, cudaMemsetAsync(dC.p, 0, std::max<int64_t>(1, TOT) * sizeof(float), s));
      unsigned long long z = 0.0f < c.cthr ? (unsigned long long)TOT : 0ull;
      CUDA_TRY(ctx, cudaMemcpyAsync(dz.p, &z, sizeof(z), cudaMemcpyHostToDevice, s));
      CUDA_TRY(ctx, cudaStreamSynchronize(s));
    } else {
      for (int64_t h = 0; h < H; ++h)
        launch_shape_gemm(s, c.Mt, c.Nt, c.inner > 0 ? c.Kt : 0, dL.as<float>() + h * lslab,
                          dR.as<float>() + h * rslab, dK.as<float>(), af, c.cthr,
                          dC.as<float>() + h * MN, dz.as<unsigned long long>());
    }
    tm.stop();
    CUDA_TRY(ctx, cudaGetLastError());
    c.st.ms_shape = tm.ms();
  }
  c.cn.resize(TOT);
  unsigned long long zc = 0;
  if (TOT)
    CUDA_TRY(ctx, cudaMemcpyAsync(c.cn.data(), dC.p, TOT * sizeof(float), cudaMemcpyDeviceToHost,
                                  s));
  CUDA_TRY(ctx, cudaMemcpyAsync(&zc, dz.p, sizeof(zc), cudaMemcpyDeviceToHost, s));
  {
    EventTimer tm(s);
    const float cthr = c.dense ? 0.0f : c.cthr;
    for (int64_t h = 0; h < H; ++h)
      launch_pair_count(s, c.Mt, c.Nt, c.Kt, dC.as<float>() + h * MN, cthr,
                        dL.as<float>() + h * lslab, c.lthr, dR.as<float>() + h * rslab, c.rthr,
                        c.d_msz.as<int32_t>(), c.d_nsz.as<int32_t>(), c.d_ksz.as<int32_t>(),
                        dcnt.as<int64_t>() + h * MN, dfl.as<double>() + h);
    launch_exclusive_scan(s, dcnt.as<int64_t>(), TOT, c.d_poff.as<int64_t>());
    CUDA_TRY(ctx, cudaGetLastError());
    int64_t np = 0;
    std::vector<double> fl(std::max<int64_t>(1, H), 0.0);
    CUDA_TRY(ctx, cudaMemcpyAsync(&np, c.d_poff.as<int64_t>() + TOT, sizeof(int64_t),
                                  cudaMemcpyDeviceToHost, s));
    CUDA_TRY(ctx, cudaMemcpyAsync(fl.data(), dfl.p, fl.size() * sizeof(double),
                                  cudaMemcpyDeviceToHost, s));
    CUDA_TRY(ctx, cudaStreamSynchronize(s));
    c.npairs = np;
    // a slab's tile pairs run once per fused element of the slab
    c.flops = 0.0;
    for (int64_t h = 0; h < H; ++h) c.flops += fl[h] * (double)c.hsz[h];
    if ((e = c.d_kidx.alloc(std::max<int64_t>(1, np) * sizeof(int32_t)))) return e;
    for (int64_t h = 0; h < H; ++h)
      launch_pair_emit(s, c.Mt, c.Nt, c.Kt, dC.as<float>() + h * MN, cthr,
                       dL.as<float>() + h * lslab, c.lthr, dR.as<float>() + h * rslab, c.rthr,
                       c.d_poff.as<int64_t>() + h * MN, c.d_kidx.as<int32_t>());
    tm.stop();
    CUDA_TRY(ctx, cudaGetLastError());
    c.st.ms_pairs = tm.ms();
  }
  c.zero_count = c.dense ? 0 : (int64_t)zc;
  return TAGPU_OK;
}

// Operands in GEMM order: explicit permutation for `general`, transposition
// fused into the GEMM loaders otherwise (binary_engine.h:159-175).
tagpu_status prepare_operands(Contraction& c, tagpu_array* A, tagpu_array* B) {
  tagpu_ctx* ctx = c.ctx;
  tagpu_status e;
  if ((e = materialize(A)) || (e = materialize(B))) return e;
  auto explicit_permute = [&](tagpu_array* X, const std::vector<int>& perm,
                              std::unique_ptr<tagpu_array>& own) -> tagpu_status {
    own.reset(permuted_layout(X, perm));
    tagpu_status st = ensure_storage(own.get());
    if (st) return st;
    PermutePlan pp(ctx);
    if ((st = pp.build(X, perm, own.get()))) return st;
    EventTimer tm(ctx->stream);
    pp.enqueue(ctx->stream, X->data, own->data);
    tm.stop();
    CUDA_TRY(ctx, cudaGetLastError());
    c.st.ms_permute += tm.ms();
    return TAGPU_OK;
  };
  if (c.po.lop == GENERAL && !is_identity(c.lperm)) {
    if ((e = explicit_permute(A, c.lperm, c.Aown))) return e;
    c.Aop = c.Aown.get();
    c.a_trans = 0;
  } else {
    c.Aop = A;
    c.a_trans = (c.po.lop == MATRIX_TRANSPOSE && !is_identity(c.lperm)) ? 1 : 0;
  }
  if (c.po.rop == GENERAL && !is_identity(c.rperm)) {
    if ((e = explicit_permute(B, c.rperm, c.Bown))) return e;
    c.Bop = c.Bown.get();
    c.b_trans = 0;
  } else {
    c.Bop = B;
    c.b_trans = (c.po.rop == MATRIX_TRANSPOSE && !is_identity(c.rperm)) ? 1 : 0;
  }
  c.aoff.assign(c.Ht * c.Mt * c.Kt, -1);
  c.boff.assign(c.Ht * c.Kt * c.Nt, -1);
  if (c.nfused > 0) {
    // canonical layouts: the argument's own tile order, slab after slab
    for (int64_t t = 0; t < (int64_t)c.aoff.size(); ++t) c.aoff[t] = c.Aop->off[t];
    for (int64_t t = 0; t < (int64_t)c.boff.size(); ++t) c.boff[t] = c.Bop->off[t];
  } else if (c.inner == 0) {
    for (int64_t m = 0; m < c.Mt; ++m) c.aoff[m] = c.Aop->off[m];
    for (int64_t n = 0; n < c.Nt; ++n) c.boff[n] = c.Bop->off[n];
    c.a_trans = c.b_trans = 0;
  } else {
    for (int64_t m = 0; m < c.Mt; ++m)
      for (int64_t k = 0; k < c.Kt; ++k)
        c.aoff[m * c.Kt + k] = c.Aop->off[c.a_trans ? k * c.Mt + m : m * c.Kt + k];
    for (int64_t k = 0; k < c.Kt; ++k)
      for (int64_t n = 0; n < c.Nt; ++n)
        c.boff[k * c.Nt + n] = c.Bop->off[c.b_trans ? n * c.Kt + k : k * c.Nt + n];
  }
  if ((e = upload_vec(ctx, c.d_aoff, c.aoff)) || (e = upload_vec(ctx, c.d_boff, c.boff)))
    return e;
  return TAGPU_OK;
}

// Result arrays: GEMM order (written by kernel d) and, when the target order
// differs, the permuted target (contract_reduce.h:370-381).
tagpu_status make_result(Contraction& c, tagpu_array* A, tagpu_array* B) {
  tagpu_ctx* ctx = c.ctx;
  std::vector<std::vector<int64_t>> hm;
  // fused modes (general products), then the left outer, then the right outer
  for (int x = 0; x < c.nfused + c.lorank; ++x)
    hm.push_back(A->hm[find_idx(c.ai, c.po.left[x])]);
  for (size_t x = c.nfused + c.inner; x < c.po.right.size(); ++x)
    hm.push_back(B->hm[find_idx(c.bi, c.po.right[x])]);
  c.C.reset(new_array(ctx, hm));
  tagpu_array* C = c.C.get();
  C->dense = c.dense;
  C->threshold = c.cthr;
  if (!c.dense) {
    C->norms = c.cn;
    C->norms.resize(C->ntiles(), 0.0f);
  }
  C->zero_count = c.zero_count;
  pack_offsets(C);
  tagpu_status e = ensure_storage(C);
  if (e) return e;
  std::vector<int64_t> coff(c.Ht * c.Mt * c.Nt, -1);
  for (int64_t t = 0; t < (int64_t)coff.size() && t < C->ntiles(); ++t) coff[t] = C->off[t];
  if ((e = upload_vec(ctx, c.d_coff, coff))) return e;
  if (!is_identity(c.cperm)) {
    c.Cfinal.reset(permuted_layout(C, c.cperm));
    if ((e = ensure_storage(c.Cfinal.get()))) return e;
    c.post.reset(new PermutePlan(ctx));
    if ((e = c.post->build(C, c.cperm, c.Cfinal.get()))) return e;
  }
  return TAGPU_OK;
}

GemmView gemm_view(Contraction& c) {
  GemmView v{};
  v.Mt = c.Mt;
  v.Nt = c.Nt;
  v.Kt = c.Kt;
  v.msz = c.d_msz.as<int32_t>();
  v.nsz = c.d_nsz.as<int32_t>();
  v.ksz = c.d_ksz.as<int32_t>();
  v.A = c.Aop->data;
  v.aoff = c.d_aoff.as<int64_t>();
  v.a_trans = c.a_trans;
  v.B = c.Bop->data;
  v.boff = c.d_boff.as<int64_t>();
  v.b_trans = c.b_trans;
  v.poff = c.d_poff.as<int64_t>();
  v.kidx = c.d_kidx.as<int32_t>();
  v.alpha = c.alpha;
  v.C = c.C->data;
  v.coff = c.d_coff.as<int64_t>();
  return v;
}

tagpu_status build_dmma_items(Contraction& c, int32_t view) {
  c.items.clear();
  for (int64_t t = 0; t < c.Mt * c.Nt; ++t) {
    if (c.C->off[t] < 0) continue;
    const int64_t i = t / c.Nt, j = t % c.Nt;
    const int64_t rbs = (c.msz[i] + 63) / 64, cbs = (c.nsz[j] + 63) / 64;
    if (rbs > 32767 || cbs > 32767)
      return fail(c.ctx, TAGPU_ERR_UNSUPPORTED, "fused tile extent above 2097088");
    for (int64_t rb = 0; rb < rbs; ++rb)
      for (int64_t cb = 0; cb < cbs; ++cb)
        c.items.push_back(WorkItem{t, view, (int16_t)rb, (int16_t)cb});
  }
  return TAGPU_OK;
}

// Full planning of one contraction.
// General products: one view per fused element (the slab's tile, pair and
// result offsets; the element's matrices inside the slab's tiles) and the
// work items of its nonzero result tiles.
tagpu_status build_general_items(Contraction& c, bool with_items) {
  c.items.clear();
  c.gviews.clear();
  const GemmView base = gemm_view(c);
  const int64_t MN = c.Mt * c.Nt;
  for (int64_t h = 0; h < c.Ht; ++h) {
    for (int64_t el = 0; el < c.hsz[h]; ++el) {
      GemmView v = base;
      v.aoff = base.aoff + h * c.Mt * c.Kt;
      v.boff = base.boff + h * c.Kt * c.Nt;
      v.poff = base.poff + h * MN;
      v.coff = base.coff + h * MN;
      v.hel = el;
      const int32_t vid = (int32_t)c.gviews.size();
      c.gviews.push_back(v);
      if (!with_items) continue;
      for (int64_t t = 0; t < MN; ++t) {
        if (c.C->off[h * MN + t] < 0) continue;
        const int64_t i = t / c.Nt, j = t % c.Nt;
        const int64_t rbs = (c.msz[i] + 63) / 64, cbs = (c.nsz[j] + 63) / 64;
        if (rbs > 32767 || cbs > 32767)
          return fail(c.ctx, TAGPU_ERR_UNSUPPORTED, "fused tile extent above 2097088");
        for (int64_t rb = 0; rb < rbs; ++rb)
          for (int64_t cb = 0; cb < cbs; ++cb)
            c.items.push_back(WorkItem{t, vid, (int16_t)rb, (int16_t)cb});
      }
    }
  }
  return TAGPU_OK;
}

tagpu_status plan_all(Contraction& c, const char* c_idx, double alpha, tagpu_array* A,
                      const char* a_idx, tagpu_array* B, const char* b_idx,
                      const tagpu_contract_opts* opts) {
  tagpu_ctx* ctx = c.ctx;
  c.precision = opts ? opts->precision : TAGPU_PRECISION_FP64;
  c.slices = opts && opts->slices > 0 ? opts->slices : 7;
  const float cthr = opts && opts->threshold >= 0 ? opts->threshold : ctx->threshold;
  if (c.precision != TAGPU_PRECISION_FP64 && c.precision != TAGPU_PRECISION_OZAKI)
    return fail(ctx, TAGPU_ERR_INVALID, "unknown precision %d", c.precision);
  if (c.precision == TAGPU_PRECISION_OZAKI && (c.slices < 2 || c.slices > 7))
    return fail(ctx, TAGPU_ERR_INVALID, "slices must be 2..7");
  tagpu_status e;
  std::string err;
  if ((e = plan_contraction(c, c_idx, alpha, A, a_idx, B, b_idx, cthr))) return e;
  if ((e = run_shape_and_pairs(c))) return e;
  if ((e = make_result(c, A, B))) return e;
  if ((e = prepare_operands(c, A, B))) return e;
  c.view = gemm_view(c);
  const bool emul = c.precision == TAGPU_PRECISION_OZAKI && c.npairs > 0 && c.C->elements > 0;
  if (c.nfused > 0 && (e = build_general_items(c, !emul))) return e;
  if (emul) {
    // one plan per GEMM view: the contraction, or every fused element of a
    // general product (its matrices inside the slab's tiles)
    const std::vector<GemmView> one(1, c.view);
    const std::vector<GemmView>& vs = c.nfused > 0 ? c.gviews : one;
    c.st.gemm_blocks = 0;
    for (const GemmView& v : vs) {
      OzakiPlan* pl = nullptr;
      e = ozaki_plan(ctx->stream, v, c.msz.data(), c.nsz.data(), c.ksz.data(), c.slices, &pl,
                     &err);
      if (e) return fail(ctx, e, "%s", err.c_str());
      ozaki_set_wait(pl, ctx->wait_ns);
      c.ozs.push_back(pl);
      const size_t b = ozaki_scratch_bytes(pl);
      c.oz_bytes += b;
      ctx->used += b;
      c.st.gemm_blocks += 2 * ozaki_units(pl);   // a unit is a pair of output blocks
      if (ctx->budget && ctx->used.load() > ctx->budget)
        return fail(ctx, TAGPU_ERR_NOMEM, "emulated-form scratch (%zu bytes) exceeds the budget",
                    c.oz_bytes);
    }
    const char* env_tune = getenv("TAGPU_AUTOTUNE");
    if (c.ozs.size() == 1 && ((opts && opts->autotune) || (env_tune && atoi(env_tune) != 0))) {
      std::string log;
      const char* cache = getenv("TAGPU_TUNE_CACHE");
      e = ozaki_autotune(c.ozs[0], ctx->sm_count, ctx->stream, cache, &log, &err);
      if (e) return fail(ctx, e, "%s", err.c_str());
      c.tune_log = log;
    }
  } else if (c.nfused == 0) {
    if ((e = build_dmma_items(c, 0))) return e;
  }
  if (c.post) {
    c.post_in = c.C->data;
    c.post_out = c.Cfinal->data;
  }
  return TAGPU_OK;
}

void fill_stats(Contraction& c) {
  tagpu_contract_stats& st = c.st;
  st.result_tiles = c.Ht * c.Mt * c.Nt;
  int64_t nz = 0;
  for (auto o : c.result()->off) nz += o >= 0;
  st.nonzero_result_tiles = nz;
  st.zero_tiles = c.zero_count;
  st.pairs = c.npairs;
  st.flops = c.flops;
  st.left_permtype = c.po.lop;
  st.right_permtype = c.po.rop;
  st.precision = c.precision;
  st.slices = c.precision == TAGPU_PRECISION_OZAKI ? c.slices : 0;
}

// Move the contents of `src` into the caller-visible handle `dst`.
void move_into(tagpu_array* dst, tagpu_array* src) {
  if (dst->data) dev_free(dst->ctx, dst->data, dst->bytes);
  dst->rank = src->rank;
  dst->hm = std::move(src->hm);
  dst->nt = std::move(src->nt);
  dst->dense = src->dense;
  dst->norms = std::move(src->norms);
  dst->threshold = src->threshold;
  dst->zero_count = src->zero_count;
  dst->off = std::move(src->off);
  dst->elements = src->elements;
  dst->data = src->data;
  dst->bytes = src->bytes;
  src->data = nullptr;
  src->bytes = 0;
}

}  // namespace

namespace tagpu {

// Device-side work lists of one launch set (kept alive while it may replay).
struct LaunchBufs {
  DBuf views, items;            // DMMA contraction views and 64x64 work items
  DBuf derr;                    // DMMA error flag (a bounded stage wait ran out)
  DBuf ozp[8], ozv[8];          // emulated form: parameter blocks, block offsets
  int64_t oz_nblk[8] = {0};
  int64_t oz_nkb[8] = {0};   // 32-k stages of the group's units
  // emulated form, per digit count: job tables of the grouped zeroing,
  // frame and split launches
  DBuf gz[8], gf[8], gsa[8], gsb[8];
  OzGroupDims gdims[8];
  // plans whose error flag an emulated GEMM launch of this set writes (a
  // grouped launch writes its first plan's flag for all of its views)
  std::vector<OzakiPlan*> err_owners;
  bool any_error() const {
    for (OzakiPlan* p : err_owners)
      if (ozaki_error(p)) return true;
    if (derr.p) {
      int e = 0;
      if (cudaMemcpy(&e, derr.p, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) {
        cudaGetLastError();
        return true;
      }
      if (e) return true;
    }
    return false;
  }
  explicit LaunchBufs(tagpu_ctx* c) : views(c), items(c), derr(c) {
    for (int i = 0; i < 8; ++i) {
      ozp[i].ctx = c;
      ozv[i].ctx = c;
      gz[i].ctx = gf[i].ctx = gsa[i].ctx = gsb[i].ctx = c;
    }
  }
};

// Kernel (d) and the post-permutation for a set of planned contractions;
// no host synchronisation, so the sequence can be captured in a graph.
// upload: (re)build the device work lists first (outside any capture).
tagpu_status enqueue_gemms(tagpu_ctx* ctx, std::vector<Contraction*>& cs, LaunchBufs& lb,
                           bool upload, cudaStream_t stream = nullptr) {
  if (!stream) stream = ctx->stream;
  DBuf& d_views = lb.views;
  DBuf& d_items = lb.items;
  std::vector<GemmView> views;
  std::vector<WorkItem> items;
  for (auto* c : cs) {
    if (c->view.C == nullptr || c->emulated()) continue;
    {
      const int32_t base = (int32_t)views.size();
      if (c->gviews.empty())
        views.push_back(c->view);
      else
        views.insert(views.end(), c->gviews.begin(), c->gviews.end());
      for (WorkItem w : c->items) {
        w.view += base;
        items.push_back(w);
      }
    }
  }
  // the DMMA loader's bulk copies start up to 8 bytes before a row and rely
  // on 16-byte aligned operand allocations (device allocations are 256-byte
  // aligned)
  for (const GemmView& v : views)
    if (((uintptr_t)v.A | (uintptr_t)v.B) & 15)
      return fail(ctx, TAGPU_ERR_INVALID, "plain GEMM: operand storage not 16-byte aligned");
  if (upload) {
    tagpu_status e;
    if ((e = upload_vec(ctx, d_views, views)) || (e = upload_vec(ctx, d_items, items))) return e;
    if (stream != ctx->stream) CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  }
  // emulated form: frames and splitting per contraction, then one GEMM launch
  // per slice count over the output blocks of all of them
  lb.err_owners.clear();
  std::vector<OzakiPlan*> by_s[8];
  for (auto* c : cs) {
    if (!c->emulated()) continue;
    for (OzakiPlan* pl : c->ozs) by_s[ozaki_slices(pl)].push_back(pl);
    c->st.gemm_launches = 5;
  }
  // frames and splits: row-chunked plans and lone plans on their own, the
  // rest of each digit count in one launch per step
  for (int S = 2; S < 8; ++S) {
    std::vector<OzakiPlan*> grp;
    for (OzakiPlan* pl : by_s[S]) {
      if (ozaki_chunks(pl) > 1)
        ozaki_enqueue(pl, ctx->sm_count, stream);
      else
        grp.push_back(pl);
    }
    if (grp.size() == 1) ozaki_enqueue(grp[0], ctx->sm_count, stream);
    if (grp.size() < 2) continue;
    if (upload) {
      std::vector<uint8_t> z, f, a, b;
      ozaki_group_tables(grp.data(), (int)grp.size(), &z, &f, &a, &b, &lb.gdims[S]);
      tagpu_status e;
      if ((e = upload_vec(ctx, lb.gz[S], z)) || (e = upload_vec(ctx, lb.gf[S], f)) ||
          (e = upload_vec(ctx, lb.gsa[S], a)) || (e = upload_vec(ctx, lb.gsb[S], b)))
        return e;
      if (stream != ctx->stream) CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    }
    ozaki_group_enqueue(lb.gz[S].p, lb.gf[S].p, lb.gsa[S].p, lb.gsb[S].p, lb.gdims[S], S,
                        ctx->sm_count, stream);
  }
  for (int S = 2; S < 8; ++S) {
    std::vector<OzakiPlan*> g;
    for (OzakiPlan* pl : by_s[S]) {
      if (ozaki_chunks(pl) > 1) {
        ozaki_enqueue_gemm(pl, ctx->sm_count, stream);
        lb.err_owners.push_back(pl);
      } else {
        g.push_back(pl);
      }
    }
    if (g.empty()) continue;
    lb.err_owners.push_back(g[0]);
    if (g.size() == 1) {
      ozaki_enqueue_gemm(g[0], ctx->sm_count, stream);
      continue;
    }
    if (upload) {
      const size_t psz = ozaki_params_size();
      std::vector<uint8_t> params(psz * g.size());
      std::vector<int64_t> vstart(1, 0);
      for (size_t i = 0; i < g.size(); ++i) {
        ozaki_params(g[i], params.data() + i * psz);
        vstart.push_back(vstart.back() + ozaki_units(g[i]));
      }
      tagpu_status e;
      if ((e = upload_vec(ctx, lb.ozp[S], params)) || (e = upload_vec(ctx, lb.ozv[S], vstart)))
        return e;
      lb.oz_nblk[S] = vstart.back();
      lb.oz_nkb[S] = 0;
      for (OzakiPlan* pl : g) lb.oz_nkb[S] += ozaki_stages(pl);
      if (stream != ctx->stream) CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    }
    ozaki_enqueue_gemm_views(lb.ozp[S].p, lb.ozv[S].as<int64_t>(), (int)g.size(), lb.oz_nblk[S],
                             lb.oz_nkb[S], S, ozaki_error_flag(g[0]), ctx->sm_count, ctx->wait_ns,
                             stream);
  }
  if (!items.empty()) {
    if (!lb.derr.p) {
      tagpu_status e = lb.derr.alloc(sizeof(int));
      if (e) return e;
    }
    CUDA_TRY(ctx, cudaMemsetAsync(lb.derr.p, 0, sizeof(int), stream));
    launch_dmma_gemm(stream, d_views.as<GemmView>(), d_items.as<WorkItem>(),
                     (int64_t)items.size(), lb.derr.as<int>(), ctx->wait_ns, ctx->sm_count);
    for (auto* c : cs) {
      if (c->emulated()) continue;
      c->st.gemm_blocks = (int64_t)c->items.size();
      c->st.gemm_launches = c->items.empty() ? 0 : 1;
    }
  }
  for (auto* c : cs)
    if (c->post) c->post->enqueue(stream, c->post_in, c->post_out);
  CUDA_TRY(ctx, cudaGetLastError());
  return TAGPU_OK;
}

tagpu_status contract_impl(tagpu_ctx* ctx, const char* c_idx, double alpha, tagpu_array* A,
                           const char* a_idx, tagpu_array* B, const char* b_idx,
                           const tagpu_contract_opts* opts, tagpu_array** out,
                           tagpu_contract_stats* stats) {
  const auto t0 = std::chrono::steady_clock::now();
  const int64_t launches0 = launch_count();
  Contraction c(ctx);
  tagpu_status e = plan_all(c, c_idx, alpha, A, a_idx, B, b_idx, opts);
  if (e) return e;
  LaunchBufs lbuf(ctx);
  std::vector<Contraction*> cs{&c};
  if (c.emulated() && c.ozs.size() > 1) {
    // general product: the fused elements' plans in grouped launches
    EventTimer tm(ctx->stream);
    if ((e = enqueue_gemms(ctx, cs, lbuf, true))) return e;
    tm.stop();
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    c.st.ms_gemm = tm.ms();
    if (lbuf.any_error())
      return fail(ctx, TAGPU_ERR_TIMEOUT,
                  "emulated GEMM: a bounded wait ran out; results invalid");
  } else if (c.emulated()) {
    OzakiPlan* oz = c.ozs[0];
    EventTimer t_split(ctx->stream);
    ozaki_enqueue(oz, ctx->sm_count, ctx->stream);
    t_split.stop();
    EventTimer t_gemm(ctx->stream);
    ozaki_enqueue_gemm(oz, ctx->sm_count, ctx->stream);
    t_gemm.stop();
    if (c.post) c.post->enqueue(ctx->stream, c.post_in, c.post_out);
    CUDA_TRY(ctx, cudaGetLastError());
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    c.st.ms_split = t_split.ms();
    c.st.ms_gemm = t_gemm.ms();
    c.st.gemm_launches = 5;
    const int oe = ozaki_error(oz);
    if (oe)
      return fail(ctx, TAGPU_ERR_TIMEOUT,
                  "emulated GEMM: a bounded wait ran out (role code %d); results invalid", oe);
  } else {
    EventTimer tm(ctx->stream);
    if ((e = enqueue_gemms(ctx, cs, lbuf, true))) return e;
    tm.stop();
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    c.st.ms_gemm = tm.ms();
    if (lbuf.any_error())
      return fail(ctx, TAGPU_ERR_TIMEOUT, "plain GEMM: a bounded stage wait ran out; results invalid");
  }
  fill_stats(c);
  for (OzakiPlan* pl : c.ozs) c.st.mma_flops += ozaki_mma_flops(pl);
  c.st.kernel_launches = launch_count() - launches0;
  c.st.ms_total =
      std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (stats) *stats = c.st;
  *out = c.Cfinal ? c.Cfinal.release() : c.C.release();
  return TAGPU_OK;
}

}  // namespace tagpu

// ---------------------------------------------------------------------------
// batches: many contractions, one persistent GEMM launch, captured in a graph
// ---------------------------------------------------------------------------

struct tagpu_batch {
  tagpu_ctx* ctx;
  struct Entry {
    std::string c, a, b;
    double alpha;
    tagpu_array *A, *B, *C;
    tagpu_contract_opts opts;
    std::unique_ptr<Contraction> plan;
  };
  std::vector<Entry> entries;
  bool planned = false;
  LaunchBufs lb;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  tagpu_contract_stats stats{};
  explicit tagpu_batch(tagpu_ctx* c) : ctx(c), lb(c) {}
  ~tagpu_batch() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
  }
};

extern "C" {

tagpu_status tagpu_contract(tagpu_ctx* ctx, const char* c_idx, double alpha, tagpu_array* A,
                            const char* a_idx, tagpu_array* B, const char* b_idx,
                            const tagpu_contract_opts* opts, tagpu_array** c) {
  if (!ctx || !A || !B || !c) return ctx ? fail(ctx, TAGPU_ERR_INVALID, "null argument")
                                         : TAGPU_ERR_INVALID;
  if (A->ctx != ctx || B->ctx != ctx)
    return fail(ctx, TAGPU_ERR_INVALID, "arrays belong to another context");
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  *c = nullptr;
  return contract_impl(ctx, c_idx, alpha, A, a_idx, B, b_idx, opts, c, &ctx->last);
}

tagpu_status tagpu_contract_accumulate(tagpu_ctx* ctx, const char* c_idx, double alpha,
                                       tagpu_array* A, const char* a_idx, tagpu_array* B,
                                       const char* b_idx, const tagpu_contract_opts* opts,
                                       tagpu_array* C) {
  if (!ctx || !A || !B || !C) return ctx ? fail(ctx, TAGPU_ERR_INVALID, "null argument")
                                         : TAGPU_ERR_INVALID;
  if (A->ctx != ctx || B->ctx != ctx || C->ctx != ctx)
    return fail(ctx, TAGPU_ERR_INVALID, "arrays belong to another context");
  if (C == A || C == B)
    return fail(ctx, TAGPU_ERR_INVALID, "accumulate: the target may not be an argument");
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  tagpu_array* p = nullptr;
  if (tagpu_status st = materialize(C)) return st;
  tagpu_status st = contract_impl(ctx, c_idx, alpha, A, a_idx, B, b_idx, opts, &p, &ctx->last);
  if (st) return st;
  std::unique_ptr<tagpu_array> P(p);
  if (P->rank != C->rank || P->hm != C->hm)
    return fail(ctx, TAGPU_ERR_INVALID, "accumulate: the target's tiling differs from the product's");
  if (P->dense != C->dense)
    return fail(ctx, TAGPU_ERR_UNSUPPORTED, "accumulate: dense and sparse policies mixed");
  // result shape: SparseShape::add (sparse_shape.h:1309-1328), float sum of the
  // scaled norms, zeroed below the threshold in force
  tagpu_array R;   // the result: C's tiling and policy, storage of its own
  R.ctx = ctx;
  R.rank = C->rank;
  R.hm = C->hm;
  R.nt = C->nt;
  R.dense = C->dense;
  if (!C->dense) {
    const int64_t n = C->ntiles();
    R.threshold = ctx->threshold;
    R.norms.assign(n, 0.0f);
    R.zero_count = 0;
    for (int64_t t = 0; t < n; ++t) {
      float v = C->norms[t] + P->norms[t];
      if (v < R.threshold) {
        v = 0.0f;
        ++R.zero_count;
      }
      R.norms[t] = v;
    }
  }
  pack_offsets(&R);
  if ((st = ensure_storage(&R))) return st;
  std::vector<AddChunk> chunks;
  const int64_t kChunk = 1 << 14;
  for (int64_t t = 0; t < (int64_t)R.off.size(); ++t) {
    if (R.off[t] < 0) continue;
    const int64_t c = C->off[t], q = P->off[t], vol = R.tile_volume(t);
    if (c < 0 && q < 0) {
      CUDA_TRY(ctx, cudaMemsetAsync(R.data + R.off[t], 0, vol * sizeof(double), ctx->stream));
      continue;
    }
    for (int64_t x = 0; x < vol; x += kChunk)
      chunks.push_back({R.off[t] + x, c < 0 ? -1 : c + x, q < 0 ? -1 : q + x,
                        std::min(kChunk, vol - x)});
  }
  DBuf dch(ctx);
  if ((st = upload_vec(ctx, dch, chunks))) return st;
  launch_add_tiles(ctx->stream, dch.as<AddChunk>(), (int64_t)chunks.size(), C->data, P->data,
                   R.data);
  CUDA_TRY(ctx, cudaGetLastError());
  CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  // C takes the result; its old storage leaves with R
  std::swap(C->norms, R.norms);
  std::swap(C->threshold, R.threshold);
  std::swap(C->zero_count, R.zero_count);
  std::swap(C->off, R.off);
  std::swap(C->elements, R.elements);
  std::swap(C->data, R.data);
  std::swap(C->bytes, R.bytes);
  return TAGPU_OK;
}

tagpu_status tagpu_batch_create(tagpu_ctx* ctx, tagpu_batch** out) {
  if (!ctx || !out) return TAGPU_ERR_INVALID;
  *out = new tagpu_batch(ctx);
  return TAGPU_OK;
}

tagpu_status tagpu_batch_add(tagpu_batch* b, const char* c_idx, double alpha, tagpu_array* A,
                             const char* a_idx, tagpu_array* B, const char* b_idx,
                             const tagpu_contract_opts* opts, tagpu_array** c) {
  if (!b || !A || !B || !c || !c_idx || !a_idx || !b_idx) return TAGPU_ERR_INVALID;
  tagpu_ctx* ctx = b->ctx;
  if (b->planned) return fail(ctx, TAGPU_ERR_STATE, "batch already ran; create a new one");
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  tagpu_batch::Entry e;
  e.c = c_idx;
  e.a = a_idx;
  e.b = b_idx;
  e.alpha = alpha;
  e.A = A;
  e.B = B;
  e.opts = opts ? *opts : tagpu_contract_opts{TAGPU_PRECISION_FP64, 0, -1.0f, 0};
  e.C = new_array(ctx, {});
  b->entries.push_back(std::move(e));
  *c = b->entries.back().C;
  return TAGPU_OK;
}

tagpu_status tagpu_batch_run(tagpu_batch* b) {
  if (!b) return TAGPU_ERR_INVALID;
  tagpu_ctx* ctx = b->ctx;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  const auto t0 = std::chrono::steady_clock::now();
  tagpu_status e;
  if (!b->planned) {
    std::vector<Contraction*> cs;
    for (auto& en : b->entries) {
      en.plan.reset(new Contraction(ctx));
      if ((e = plan_all(*en.plan, en.c.c_str(), en.alpha, en.A, en.a.c_str(), en.B,
                        en.b.c_str(), &en.opts)))
        return e;
      cs.push_back(en.plan.get());
    }
    // hand the result storage to the caller-visible handles now: the device
    // pointers the graph captures stay valid as long as the handles live
    for (auto& en : b->entries) {
      Contraction& c = *en.plan;
      fill_stats(c);
    }
    // run once eagerly (uploads the work lists), then capture the launches
    if ((e = enqueue_gemms(ctx, cs, b->lb, true))) return e;
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    if (b->lb.any_error())
      return fail(ctx, TAGPU_ERR_TIMEOUT, "emulated GEMM: a bounded wait ran out");
    CUDA_TRY(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    e = enqueue_gemms(ctx, cs, b->lb, false);
    cudaGraph_t g = nullptr;
    cudaError_t ce = cudaStreamEndCapture(ctx->stream, &g);
    if (e) return e;
    if (ce != cudaSuccess)
      return fail(ctx, TAGPU_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(ce));
    b->graph = g;
    CUDA_TRY(ctx, cudaGraphInstantiate(&b->exec, g, 0));
    // results move into the caller-visible handles; the captured launches
    // keep writing the same device buffers, so a result handle must outlive
    // the runs of its batch
    for (auto& en : b->entries) move_into(en.C, en.plan->result());
    b->planned = true;
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  } else {
    CUDA_TRY(ctx, cudaGraphLaunch(b->exec, ctx->stream));
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    if (b->lb.any_error())
      return fail(ctx, TAGPU_ERR_TIMEOUT, "emulated GEMM: a bounded wait ran out");
  }
  tagpu_contract_stats& s = b->stats;
  s = tagpu_contract_stats{};
  for (auto& en : b->entries) {
    const auto& c = en.plan->st;
    s.result_tiles += c.result_tiles;
    s.nonzero_result_tiles += c.nonzero_result_tiles;
    s.zero_tiles += c.zero_tiles;
    s.pairs += c.pairs;
    s.flops += c.flops;
    s.ms_shape += c.ms_shape;
    s.ms_pairs += c.ms_pairs;
    s.ms_permute += c.ms_permute;
    s.ms_split += c.ms_split;
    s.gemm_blocks += c.gemm_blocks;
  }
  s.gemm_launches = b->exec ? 1 : 0;
  s.ms_total =
      std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return TAGPU_OK;
}

tagpu_status tagpu_batch_stats(const tagpu_batch* b, tagpu_contract_stats* st) {
  if (!b || !st) return TAGPU_ERR_INVALID;
  *st = b->stats;
  // the digit-slice products of the last run, read from the plans' counters
  std::lock_guard<std::recursive_mutex> lk(b->ctx->mu);
  cudaSetDevice(b->ctx->device);
  st->mma_flops = 0;
  for (const auto& en : b->entries)
    if (en.plan)
      for (OzakiPlan* pl : en.plan->ozs) st->mma_flops += ozaki_mma_flops(pl);
  return TAGPU_OK;
}

tagpu_status tagpu_batch_destroy(tagpu_batch* b) {
  if (!b) return TAGPU_ERR_INVALID;
  std::lock_guard<std::recursive_mutex> lk(b->ctx->mu);
  cudaSetDevice(b->ctx->device);
  cudaStreamSynchronize(b->ctx->stream);
  delete b;
  return TAGPU_OK;
}

tagpu_status tagpu_last_stats(const tagpu_ctx* ctx, tagpu_contract_stats* st) {
  if (!ctx || !st) return TAGPU_ERR_INVALID;
  *st = ctx->last;
  return TAGPU_OK;
}

tagpu_status tagpu_shape_gemm(tagpu_ctx* ctx, int64_t M, int64_t N, int64_t K,
                              const float* left, const float* right, const float* k_sizes,
                              double factor, float threshold, float* result,
                              int64_t* zero_count) {
  if (!ctx || M < 0 || N < 0 || K < 0 || (M * N != 0 && !result))
    return ctx ? fail(ctx, TAGPU_ERR_INVALID, "shape_gemm: bad arguments") : TAGPU_ERR_INVALID;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  const bool outer = k_sizes == nullptr;
  const int64_t Kl = outer ? 1 : K;
  std::vector<float> l(left, left + M * Kl), r(right, right + Kl * N);
  std::vector<float> ks;
  if (!outer) ks.assign(k_sizes, k_sizes + K);
  DBuf dL(ctx), dR(ctx), dK(ctx), dC(ctx), dz(ctx);
  tagpu_status e;
  if ((e = upload_vec(ctx, dL, l)) || (e = upload_vec(ctx, dR, r)) || (e = upload_vec(ctx, dK, ks)) ||
      (e = dC.alloc(std::max<int64_t>(1, M * N) * sizeof(float))) ||
      (e = dz.alloc(sizeof(unsigned long long))))
    return e;
  CUDA_TRY(ctx, cudaMemsetAsync(dz.p, 0, sizeof(unsigned long long), ctx->stream));
  if (!outer && K == 0) {
    CUDA_TRY(ctx, cudaMemsetAsync(dC.p, 0, std::max<int64_t>(1, M * N) * sizeof(float),
                                  ctx->stream));
    unsigned long long z = (unsigned long long)(M * N);
    CUDA_TRY(ctx, cudaMemcpyAsync(dz.p, &z, sizeof(z), cudaMemcpyHostToDevice, ctx->stream));
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
    // 0 < threshold for any positive threshold: every tile is zero
    if (!(0.0f < threshold)) {
      z = 0;
      CUDA_TRY(ctx, cudaMemcpyAsync(dz.p, &z, sizeof(z), cudaMemcpyHostToDevice, ctx->stream));
    }
  } else {
    launch_shape_gemm(ctx->stream, M, N, outer ? 0 : K, dL.as<float>(), dR.as<float>(),
                      dK.as<float>(), (float)std::fabs(factor), threshold, dC.as<float>(),
                      dz.as<unsigned long long>());
    CUDA_TRY(ctx, cudaGetLastError());
  }
  unsigned long long z = 0;
  if (M * N != 0)
    CUDA_TRY(ctx, cudaMemcpyAsync(result, dC.p, M * N * sizeof(float), cudaMemcpyDeviceToHost,
                                  ctx->stream));
  CUDA_TRY(ctx, cudaMemcpyAsync(&z, dz.p, sizeof(z), cudaMemcpyDeviceToHost, ctx->stream));
  CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  if (zero_count) *zero_count = (int64_t)z;
  return TAGPU_OK;
}

tagpu_status tagpu_pair_list(tagpu_ctx* ctx, int64_t M, int64_t N, int64_t K,
                             const float* cnorm, float c_thr, const float* lnorm, float l_thr,
                             const float* rnorm, float r_thr, int64_t* offsets, int32_t* kidx,
                             int64_t kidx_cap, int64_t* npairs) {
  if (!ctx || M < 0 || N < 0 || K < 0 || !offsets)
    return ctx ? fail(ctx, TAGPU_ERR_INVALID, "pair_list: bad arguments") : TAGPU_ERR_INVALID;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  const int64_t MN = M * N;
  std::vector<float> c(cnorm, cnorm + MN), l(lnorm, lnorm + M * K), r(rnorm, rnorm + K * N);
  std::vector<int32_t> ones_m(std::max<int64_t>(1, M), 1), ones_n(std::max<int64_t>(1, N), 1),
      ones_k(std::max<int64_t>(1, K), 1);
  DBuf dC(ctx), dL(ctx), dR(ctx), dm(ctx), dn(ctx), dk(ctx), dcnt(ctx), doff(ctx), dki(ctx),
      dfl(ctx);
  tagpu_status e;
  if ((e = upload_vec(ctx, dC, c)) || (e = upload_vec(ctx, dL, l)) || (e = upload_vec(ctx, dR, r)) ||
      (e = upload_vec(ctx, dm, ones_m)) || (e = upload_vec(ctx, dn, ones_n)) ||
      (e = upload_vec(ctx, dk, ones_k)) ||
      (e = dcnt.alloc(std::max<int64_t>(1, MN) * sizeof(int64_t))) ||
      (e = doff.alloc((MN + 1) * sizeof(int64_t))) || (e = dfl.alloc(sizeof(double))))
    return e;
  CUDA_TRY(ctx, cudaMemsetAsync(dfl.p, 0, sizeof(double), ctx->stream));
  launch_pair_count(ctx->stream, M, N, K, dC.as<float>(), c_thr, dL.as<float>(), l_thr,
                    dR.as<float>(), r_thr, dm.as<int32_t>(), dn.as<int32_t>(), dk.as<int32_t>(),
                    dcnt.as<int64_t>(), dfl.as<double>());
  launch_exclusive_scan(ctx->stream, dcnt.as<int64_t>(), MN, doff.as<int64_t>());
  CUDA_TRY(ctx, cudaGetLastError());
  CUDA_TRY(ctx, cudaMemcpyAsync(offsets, doff.p, (MN + 1) * sizeof(int64_t),
                                cudaMemcpyDeviceToHost, ctx->stream));
  CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  const int64_t np = offsets[MN];
  if (npairs) *npairs = np;
  if (kidx) {
    if (kidx_cap < np) return fail(ctx, TAGPU_ERR_INVALID, "pair_list: kidx capacity too small");
    if ((e = dki.alloc(std::max<int64_t>(1, np) * sizeof(int32_t)))) return e;
    launch_pair_emit(ctx->stream, M, N, K, dC.as<float>(), c_thr, dL.as<float>(), l_thr,
                     dR.as<float>(), r_thr, doff.as<int64_t>(), dki.as<int32_t>());
    CUDA_TRY(ctx, cudaGetLastError());
    if (np)
      CUDA_TRY(ctx, cudaMemcpyAsync(kidx, dki.p, np * sizeof(int32_t), cudaMemcpyDeviceToHost,
                                    ctx->stream));
    CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  }
  return TAGPU_OK;
}

tagpu_status tagpu_permute(tagpu_ctx* ctx, int rank, const int64_t* extents, const int32_t* perm,
                           const double* in, double* out) {
  if (!ctx || rank < 1 || rank > 8 || !extents || !perm)
    return ctx ? fail(ctx, TAGPU_ERR_INVALID, "permute: bad arguments") : TAGPU_ERR_INVALID;
  std::vector<bool> seen(rank, false);
  for (int d = 0; d < rank; ++d) {
    if (perm[d] < 0 || perm[d] >= rank || seen[perm[d]])
      return fail(ctx, TAGPU_ERR_INVALID, "permute: not a permutation");
    seen[perm[d]] = true;
  }
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  cudaSetDevice(ctx->device);
  int64_t vol = 1;
  for (int d = 0; d < rank; ++d) vol *= extents[d];
  if (vol == 0) return TAGPU_OK;
  if (!in || !out) return fail(ctx, TAGPU_ERR_INVALID, "permute: null buffer");
  PermuteDesc pd{};
  pd.rank = rank;
  for (int d = 0; d < rank; ++d) pd.perm[d] = perm[d];
  std::vector<int32_t> ext(extents, extents + rank);
  std::vector<int64_t> zero(1, 0), items = {0, permute_items(pd, extents)};
  DBuf dext(ctx), dio(ctx), dis(ctx), din(ctx), dout(ctx);
  tagpu_status e;
  if ((e = upload_vec(ctx, dext, ext)) || (e = upload_vec(ctx, dio, zero)) ||
      (e = upload_vec(ctx, dis, items)) || (e = din.alloc(vol * sizeof(double))) ||
      (e = dout.alloc(vol * sizeof(double))))
    return e;
  CUDA_TRY(ctx, cudaMemcpyAsync(din.p, in, vol * sizeof(double), cudaMemcpyHostToDevice,
                                ctx->stream));
  launch_permute(ctx->stream, pd, 1, dext.as<int32_t>(), dio.as<int64_t>(), dio.as<int64_t>(),
                 dis.as<int64_t>(), items[1], din.as<double>(), dout.as<double>());
  CUDA_TRY(ctx, cudaGetLastError());
  CUDA_TRY(ctx, cudaMemcpyAsync(out, dout.p, vol * sizeof(double), cudaMemcpyDeviceToHost,
                                ctx->stream));
  CUDA_TRY(ctx, cudaStreamSynchronize(ctx->stream));
  return TAGPU_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// serving: admission by HBM footprint, continuous batching, two-stage pipeline
// (plan the next batch on the context stream while the GEMMs of the current
// batch run on the server's own stream)
// ---------------------------------------------------------------------------

struct tagpu_server {
  struct Req {
    uint64_t id = 0;
    std::string c, a, b;
    double alpha = 1.0;
    tagpu_array *A = nullptr, *B = nullptr;
    tagpu_contract_opts opts{};
    size_t bound = 0;        // footprint reserved at admission
    size_t held = 0;         // result bytes kept for the client until it takes them
    double t_submit = 0, t_admit = 0;
    bool done = false;
    tagpu_array* C = nullptr;
    tagpu_request_result res{};
    std::unique_ptr<Contraction> plan;
    cudaEvent_t prep = nullptr;   // served: the preparation kernels are done
    std::vector<int> jobs;        // served: job ids of its plans
    ~Req() {
      if (prep) cudaEventDestroy(prep);
    }
  };
  tagpu_ctx* ctx = nullptr;
  tagpu_server_config cfg{};
  cudaStream_t gemm_stream = nullptr;   // the persistent served GEMM
  OzakiServe* served = nullptr;
  std::thread worker;
  std::mutex m;
  std::condition_variable cv, done_cv;
  bool stopping = false;
  std::deque<std::shared_ptr<Req>> queue;
  std::unordered_map<uint64_t, std::shared_ptr<Req>> all;
  uint64_t next_id = 1, next_batch = 1;
  size_t in_use = 0, peak = 0;
  int64_t submitted = 0, completed = 0, rejected = 0, failed = 0, batches = 0;
  double flops = 0, t_first = -1, t_last = 0;
  std::vector<double> lat;
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
  double now_ms() const {
    return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0)
        .count();
  }
  void run();
};

namespace {

// Upper bound of the device bytes a request can need: the dense result, the
// pair list, permuted operand copies and the emulated form's digit bricks.
size_t footprint_bound(tagpu_array* A, const std::vector<std::string>& ai, tagpu_array* B,
                       const std::vector<std::string>& bi, const tagpu_contract_opts& o) {
  double m = 1, n = 1, k = 1, mt = 1, nt = 1, kt = 1;
  for (size_t d = 0; d < ai.size(); ++d) {
    const double ext = (double)(A->hm[d].back() - A->hm[d][0]);
    if (find_idx(bi, ai[d]) >= 0) {
      k *= ext;
      kt *= (double)A->nt[d];
    } else {
      m *= ext;
      mt *= (double)A->nt[d];
    }
  }
  for (size_t d = 0; d < bi.size(); ++d)
    if (find_idx(ai, bi[d]) < 0) {
      n *= (double)(B->hm[d].back() - B->hm[d][0]);
      nt *= (double)B->nt[d];
    }
  double bytes = 2.0 * m * n * 8;                 // result (+ permuted copy)
  bytes += mt * nt * kt * 4 + mt * nt * 32;       // pair list, offsets
  bytes += (double)A->bytes + (double)B->bytes;   // explicit permutations
  if (o.precision == TAGPU_PRECISION_OZAKI) {
    const int S = o.slices > 0 ? o.slices : 7;
    const double kk = std::ceil(k / 32.0) * 32.0;
    bytes += (std::ceil(m / 128.0) * 128.0 + std::ceil(n / 64.0) * 64.0) * kk * 2.0 * S;
    bytes += (m + n) * 24 + (m / 128.0 + n / 64.0 + 2) * (k / 32.0 + 1) * 32;
  }
  return (size_t)bytes + (1u << 20);
}

}  // namespace

// The request loop.  Admitted emulated requests are planned and prepared
// (screening, pair list, frames, digit bricks, stage shifts) on the
// context's stream, then published as jobs into the persistent served GEMM's
// work queue: short jobs into the lane its clusters take first, so a small
// request admitted while a large one runs starts as soon as any cluster
// finishes its current unit.  A request completes when all its jobs are
// counted done (and its post-permutation, if any, has run).  Other requests
// (plain FP64, emulated plans built in row chunks or with another slice
// count) run alone on the whole GPU: publication pauses, the served jobs out
// finish, the served kernel stops, and they run on the context's stream one
// after another; then publication resumes.  (Run beside the served kernel,
// they would get only the few clusters it leaves free for the preparation
// kernels.)
void tagpu_server::run() {
  std::deque<std::shared_ptr<Req>> prepping, serving, exclusive;
  LaunchBufs lb(ctx);
  const int S = cfg.slices;
  // jobs of at most this many (unit, k block) stages go to the first lane:
  // about 0.3 ms of the whole GPU
  constexpr int kShortStages = 76 * 256;
  constexpr int kReserve = 4;   // clusters left free for other kernels
  std::string err;
  int64_t wave = 0;   // requests published so far (batch ids of served requests)
  auto finish = [&](const std::shared_ptr<Req>& r, tagpu_status st) {
    const double t = now_ms();
    std::lock_guard<std::mutex> lk(m);
    r->res.status = st;
    if (st == TAGPU_OK) {
      Contraction& c = *r->plan;
      fill_stats(c);
      r->C = c.Cfinal ? c.Cfinal.release() : c.C.release();
      r->res.flops = c.flops;
      r->res.pairs = c.npairs;
      flops += c.flops;
      ++completed;
      lat.push_back(t - r->t_submit);
    } else {
      ++failed;
    }
    r->res.latency_ms = t - r->t_submit;
    {
      std::lock_guard<std::recursive_mutex> lk2(ctx->mu);
      r->plan.reset();
    }
    // the result stays in HBM until the client takes it: it keeps its bytes
    // of the admission budget until then
    r->held = r->C ? r->C->bytes : 0;
    in_use -= r->bound;
    in_use += r->held;
    r->done = true;
    t_last = t;
    done_cv.notify_all();
    cv.notify_all();
  };
  for (;;) {
    std::vector<std::shared_ptr<Req>> batch;
    {
      std::unique_lock<std::mutex> lk(m);
      const bool busy = !prepping.empty() || !serving.empty() || !exclusive.empty();
      if (!busy) {
        cv.wait(lk, [&] { return stopping || !queue.empty(); });
        if (stopping && queue.empty()) break;
      }
      const size_t budget = cfg.hbm_budget_bytes;
      const int maxb = cfg.max_batch > 0 ? cfg.max_batch : 64;
      for (auto it = queue.begin(); it != queue.end() && (int)batch.size() < maxb;) {
        if (budget == 0 || in_use + (*it)->bound <= budget) {
          in_use += (*it)->bound;
          peak = std::max(peak, in_use);
          (*it)->t_admit = now_ms();
          batch.push_back(*it);
          it = queue.erase(it);
        } else {
          ++it;
        }
      }
      if (batch.empty() && !busy && !queue.empty()) {
        if (stopping) {
          // results nobody took hold the budget: the queue can never run
          for (auto& r : queue) {
            r->res.status = TAGPU_ERR_STATE;
            r->res.latency_ms = now_ms() - r->t_submit;
            r->done = true;
            ++failed;
          }
          queue.clear();
          done_cv.notify_all();
          break;
        }
        // nothing fits until a client takes a result
        cv.wait_for(lk, std::chrono::milliseconds(5));
        continue;
      }
    }
    // plan and prepare the admitted requests
    for (auto& r : batch) {
      r->res.queue_ms = r->t_admit - r->t_submit;
      tagpu_status e;
      bool servable = false;
      {
        std::lock_guard<std::recursive_mutex> lk(ctx->mu);
        cudaSetDevice(ctx->device);
        r->plan.reset(new Contraction(ctx));
        e = plan_all(*r->plan, r->c.c_str(), r->alpha, r->A, r->a.c_str(), r->B, r->b.c_str(),
                     &r->opts);
        Contraction& c = *r->plan;
        if (!e && c.emulated()) {
          servable = true;
          for (OzakiPlan* pl : c.ozs)
            servable = servable && ozaki_chunks(pl) == 1 && ozaki_slices(pl) == S;
        }
        if (!e && servable && !served) {
          e = ozaki_serve_create(S, ctx->sm_count, kReserve, ctx->wait_ns, gemm_stream, &served,
                                 &err);
          if (e) fail(ctx, e, "%s", err.c_str());
        }
        if (!e && servable) {
          for (OzakiPlan* pl : c.ozs) ozaki_prepare_served(pl, ctx->sm_count, ctx->stream);
          if (cudaEventCreateWithFlags(&r->prep, cudaEventDisableTiming) != cudaSuccess ||
              cudaEventRecord(r->prep, ctx->stream) != cudaSuccess) {
            cudaGetLastError();
            e = TAGPU_ERR_CUDA;
          }
        }
      }
      if (e) {
        finish(r, e);
        continue;
      }
      if (!servable) {
        exclusive.push_back(r);   // runs alone once the served jobs out are done
        continue;
      }
      prepping.push_back(r);
    }
    // requests that run alone: once no served job is out
    if (!exclusive.empty() && serving.empty()) {
      if (served) {
        std::lock_guard<std::recursive_mutex> lk(ctx->mu);
        ozaki_serve_reset(served, &err);   // stops the served kernel
      }
      while (!exclusive.empty()) {
        auto r = exclusive.front();
        exclusive.pop_front();
        tagpu_status e;
        {
          std::lock_guard<std::recursive_mutex> lk(ctx->mu);
          cudaSetDevice(ctx->device);
          Contraction& c = *r->plan;
          std::vector<Contraction*> one{&c};
          e = enqueue_gemms(ctx, one, lb, true, ctx->stream);
          if (!e && c.post) c.post->enqueue(ctx->stream, c.post_in, c.post_out);
          if (!e && cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
            cudaGetLastError();
            e = TAGPU_ERR_CUDA;
          }
          if (!e && lb.any_error()) e = TAGPU_ERR_TIMEOUT;
        }
        ++batches;
        r->res.batch_size = 1;
        r->res.batch_id = next_batch++;
        finish(r, e);
      }
    }
    // publish the requests whose preparation has finished (in admission
    // order), unless requests wait to run alone
    bool published = false;
    while (!prepping.empty() && exclusive.empty()) {
      auto& r = prepping.front();
      const cudaError_t q = cudaEventQuery(r->prep);
      if (q == cudaErrorNotReady) break;
      if (q != cudaSuccess) {
        cudaGetLastError();
        auto rr = r;
        prepping.pop_front();
        finish(rr, TAGPU_ERR_CUDA);
        continue;
      }
      Contraction& c = *r->plan;
      std::vector<int> ids;
      bool full = false;
      for (OzakiPlan* pl : c.ozs) {
        const int lane = ozaki_stage_count(pl) <= kShortStages ? 0 : 1;
        const int id = ozaki_serve_publish(served, pl, lane);
        if (id == -1) {
          full = true;   // tables full: published jobs of this request stay valid
          break;
        }
        ids.push_back(id);
      }
      r->jobs.insert(r->jobs.end(), ids.begin(), ids.end());
      if (full) break;   // the rest after the next reset
      r->res.batch_id = (uint64_t)++wave;
      serving.push_back(r);
      prepping.pop_front();
      published = true;
    }
    // keep the served kernel running while jobs are out
    if (!serving.empty() && served) {
      int exited_error = 0;
      tagpu_status e = ozaki_serve_kick(served, &exited_error, &err);
      if (e || exited_error) {
        // a bounded wait ran out (or the launch failed): the jobs out are lost
        while (!serving.empty()) {
          auto r = serving.front();
          serving.pop_front();
          finish(r, e ? e : TAGPU_ERR_TIMEOUT);
        }
        ozaki_serve_reset(served, &err);
      }
    }
    (void)published;
    // completions
    for (auto it = serving.begin(); it != serving.end();) {
      auto r = *it;
      bool all = true;
      for (int id : r->jobs) all = all && ozaki_serve_done(served, id);
      if (!all) {
        ++it;
        continue;
      }
      tagpu_status e = TAGPU_OK;
      {
        std::lock_guard<std::recursive_mutex> lk(ctx->mu);
        cudaSetDevice(ctx->device);
        Contraction& c = *r->plan;
        if (c.post) {
          c.post->enqueue(ctx->stream, c.post_in, c.post_out);
          if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) {
            cudaGetLastError();
            e = TAGPU_ERR_CUDA;
          }
        }
      }
      r->res.batch_size = (int)serving.size();   // requests on the GPU together
      it = serving.erase(it);
      finish(r, e);
    }
    // with nothing out, the job tables start over
    if (served && serving.empty() && prepping.empty()) {
      std::lock_guard<std::recursive_mutex> lk(ctx->mu);
      ozaki_serve_reset(served, &err);
      ++batches;
    }
    if (!serving.empty() || !prepping.empty()) {
      // poll the completion flags; new arrivals wake the loop at once
      std::unique_lock<std::mutex> lk(m);
      cv.wait_for(lk, std::chrono::microseconds(50));
    }
  }
  if (served) {
    ozaki_serve_destroy(served);
    served = nullptr;
  }
}

extern "C" {

tagpu_status tagpu_server_start(tagpu_ctx* ctx, const tagpu_server_config* cfg,
                                tagpu_server** out) {
  if (!ctx || !out) return TAGPU_ERR_INVALID;
  auto* s = new tagpu_server;
  s->ctx = ctx;
  if (cfg) s->cfg = *cfg;
  if (s->cfg.slices <= 0) s->cfg.slices = 7;
  cudaSetDevice(ctx->device);
  if (cudaStreamCreateWithFlags(&s->gemm_stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete s;
    return fail(ctx, TAGPU_ERR_CUDA, "server stream creation failed");
  }
  s->worker = std::thread([s] {
    cudaSetDevice(s->ctx->device);
    s->run();
  });
  *out = s;
  return TAGPU_OK;
}

tagpu_status tagpu_server_submit(tagpu_server* s, const tagpu_request* req, uint64_t* id) {
  if (!s || !req || !req->A || !req->B || !req->c_idx || !req->a_idx || !req->b_idx)
    return TAGPU_ERR_INVALID;
  auto r = std::make_shared<tagpu_server::Req>();
  r->c = req->c_idx;
  r->a = req->a_idx;
  r->b = req->b_idx;
  r->alpha = req->alpha;
  r->A = req->A;
  r->B = req->B;
  r->opts.precision = req->precision >= 0 ? req->precision : s->cfg.precision;
  r->opts.slices = req->slices > 0 ? req->slices : s->cfg.slices;
  r->opts.threshold = -1.0f;
  r->opts.autotune = 0;
  std::vector<std::string> ai, bi;
  if (!parse_indices(req->a_idx, ai) || !parse_indices(req->b_idx, bi) ||
      (int)ai.size() != req->A->rank || (int)bi.size() != req->B->rank)
    return fail(s->ctx, TAGPU_ERR_INVALID, "server: malformed request indices");
  r->bound = footprint_bound(req->A, ai, req->B, bi, r->opts);
  std::lock_guard<std::mutex> lk(s->m);
  ++s->submitted;
  if (s->cfg.hbm_budget_bytes && r->bound > s->cfg.hbm_budget_bytes) {
    ++s->rejected;
    return fail(s->ctx, TAGPU_ERR_REJECTED,
                "request footprint bound %.3g GB exceeds the budget %.3g GB", r->bound / 1e9,
                s->cfg.hbm_budget_bytes / 1e9);
  }
  if (s->stopping) return fail(s->ctx, TAGPU_ERR_STATE, "server is stopping");
  r->id = s->next_id++;
  r->t_submit = s->now_ms();
  if (s->t_first < 0) s->t_first = r->t_submit;
  s->queue.push_back(r);
  s->all[r->id] = r;
  if (id) *id = r->id;
  s->cv.notify_all();
  return TAGPU_OK;
}

static tagpu_status server_take(tagpu_server* s, uint64_t id, tagpu_array** c,
                                tagpu_request_result* res) {
  auto it = s->all.find(id);
  if (it == s->all.end()) return TAGPU_ERR_INVALID;
  auto r = it->second;
  if (!r->done) return TAGPU_ERR_NOT_READY;
  if (res) *res = r->res;
  if (c) {
    *c = r->C;
  } else if (r->C) {
    std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
    delete r->C;
  }
  r->C = nullptr;
  s->in_use -= r->held;
  r->held = 0;
  s->cv.notify_all();   // the freed bytes may admit queued requests
  s->all.erase(it);
  return TAGPU_OK;
}

tagpu_status tagpu_server_poll(tagpu_server* s, uint64_t id, tagpu_array** c,
                               tagpu_request_result* res) {
  if (!s) return TAGPU_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->m);
  return server_take(s, id, c, res);
}

tagpu_status tagpu_server_wait(tagpu_server* s, uint64_t id, double timeout_ms, tagpu_array** c,
                               tagpu_request_result* res) {
  if (!s) return TAGPU_ERR_INVALID;
  std::unique_lock<std::mutex> lk(s->m);
  auto ready = [&] {
    auto it = s->all.find(id);
    return it == s->all.end() || it->second->done;
  };
  if (timeout_ms < 0) {
    s->done_cv.wait(lk, ready);
  } else if (!s->done_cv.wait_for(lk, std::chrono::duration<double, std::milli>(timeout_ms),
                                  ready)) {
    return TAGPU_ERR_TIMEOUT;
  }
  return server_take(s, id, c, res);
}

tagpu_status tagpu_server_get_stats(tagpu_server* s, tagpu_server_stats* st) {
  if (!s || !st) return TAGPU_ERR_INVALID;
  std::lock_guard<std::mutex> lk(s->m);
  *st = tagpu_server_stats{};
  st->submitted = s->submitted;
  st->completed = s->completed;
  st->rejected = s->rejected;
  st->failed = s->failed;
  st->batches = s->batches;
  st->flops = s->flops;
  st->wall_ms = s->t_first >= 0 ? s->t_last - s->t_first : 0;
  st->bytes_in_use = s->in_use;
  st->peak_bytes = s->peak;
  if (!s->lat.empty()) {
    std::vector<double> v = s->lat;
    std::sort(v.begin(), v.end());
    auto pct = [&](double p) {
      const double x = p * (v.size() - 1);
      const size_t i = (size_t)x;
      const double f = x - i;
      return i + 1 < v.size() ? v[i] * (1 - f) + v[i + 1] * f : v[i];
    };
    st->p50_ms = pct(0.50);
    st->p99_ms = pct(0.99);
    double sum = 0;
    for (double x : v) sum += x;
    st->mean_ms = sum / v.size();
  }
  return TAGPU_OK;
}

tagpu_status tagpu_server_stop(tagpu_server* s) {
  if (!s) return TAGPU_ERR_INVALID;
  {
    std::lock_guard<std::mutex> lk(s->m);
    s->stopping = true;
  }
  s->cv.notify_all();
  if (s->worker.joinable()) s->worker.join();
  {
    std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
    for (auto& kv : s->all)
      if (kv.second->C) delete kv.second->C;
    s->all.clear();
  }
  cudaStreamDestroy(s->gemm_stream);
  delete s;
  return TAGPU_OK;
}

}  // extern "C"
