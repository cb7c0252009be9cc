// C++ façade over the tagpu C ABI with TiledArray's user-facing names, so
// that contraction code such as
//
//   TA::TSpArrayD C;
//   C("i,j") = A("i,k") * B("k,j");
//   R("a,b,i,j") = 0.5 * (V("a,b,c,d") * T("c,d,i,j"));
//
// compiles unchanged against tagpu (namespace alias TA = tagpu::ta).
// Mirrors (paths relative to the TiledArray source tree): TiledRange1
// (tiled_range1.h:47), TiledRange (tiled_range.h:33), SparseShape
// (sparse_shape.h:75), DistArray (dist_array.h:63, operator()(std::string)
// :1311-1325), TsrExpr::operator= (expressions/tsr_expr.h:132-138),
// scaled expressions (expressions/scal_expr.h).  Errors throw tagpu::Exception
// (TiledArray throws TiledArray::Exception).  Header-only; link libtagpu.so.
#pragma once

#include <cstdint>
#include <initializer_list>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../tagpu.h"

namespace tagpu {
namespace ta {

class Exception : public std::runtime_error {
 public:
  Exception(tagpu_status s, const std::string& m) : std::runtime_error(m), status(s) {}
  tagpu_status status;
};

// TA::initialize / default World: one context on one GPU.
class World {
 public:
  explicit World(int device = 0, size_t hbm_budget_bytes = 0) {
    tagpu_config cfg{device, hbm_budget_bytes};
    tagpu_status s = tagpu_init(&cfg, &ctx_);
    if (s != TAGPU_OK) throw Exception(s, "tagpu_init failed");
  }
  ~World() {
    if (ctx_) tagpu_shutdown(ctx_);
  }
  World(const World&) = delete;
  World& operator=(const World&) = delete;
  tagpu_ctx* ctx() const { return ctx_; }
  void check(tagpu_status s) const {
    if (s != TAGPU_OK) throw Exception(s, tagpu_last_error(ctx_));
  }
  void fence() const { check(tagpu_sync(ctx_)); }
  static World*& default_world() {
    static World* w = nullptr;
    return w;
  }

 private:
  tagpu_ctx* ctx_ = nullptr;
};

inline World& get_default_world() {
  if (!World::default_world()) throw Exception(TAGPU_ERR_STATE, "call initialize() first");
  return *World::default_world();
}
inline World& initialize(int device = 0) {
  if (!World::default_world()) World::default_world() = new World(device);
  return *World::default_world();
}
inline void finalize() {
  delete World::default_world();
  World::default_world() = nullptr;
}

class TiledRange1 {
 public:
  TiledRange1() : h_{0} {}
  TiledRange1(std::initializer_list<int64_t> h) : h_(h) {}
  template <typename It>
  TiledRange1(It b, It e) : h_(b, e) {}
  explicit TiledRange1(std::vector<int64_t> h) : h_(std::move(h)) {}
  const std::vector<int64_t>& hashmarks() const { return h_; }
  int64_t tile_count() const { return (int64_t)h_.size() - 1; }
  int64_t extent() const { return h_.back() - h_.front(); }
  bool operator==(const TiledRange1& o) const { return h_ == o.h_; }

 private:
  std::vector<int64_t> h_;
};

class TiledRange {
 public:
  TiledRange() = default;
  TiledRange(std::initializer_list<TiledRange1> d) : d_(d) {}
  TiledRange(std::initializer_list<std::initializer_list<int64_t>> d) {
    for (auto& x : d) d_.emplace_back(x);
  }
  explicit TiledRange(std::vector<TiledRange1> d) : d_(std::move(d)) {}
  int rank() const { return (int)d_.size(); }
  const TiledRange1& dim(int i) const { return d_[i]; }
  int64_t tile_volume() const {
    int64_t v = 1;
    for (auto& x : d_) v *= x.tile_count();
    return v;
  }

 private:
  std::vector<TiledRange1> d_;
};

// SparseShape<float>: per-tile Frobenius norms (unscaled unless
// do_not_scale), scaled by the inverse tile volume when attached.
template <typename T = float>
class SparseShape {
 public:
  SparseShape() = default;
  SparseShape(std::vector<float> norms, const TiledRange& tr, bool do_not_scale = false)
      : norms_(std::move(norms)), do_not_scale_(do_not_scale) {
    (void)tr;
  }
  const std::vector<float>& norms() const { return norms_; }
  bool do_not_scale() const { return do_not_scale_; }
  static T threshold() { return threshold_; }
  static void threshold(T t) {
    threshold_ = t;
    if (World::default_world()) tagpu_threshold_set(World::default_world()->ctx(), (float)t);
  }

 private:
  std::vector<float> norms_;
  bool do_not_scale_ = false;
  static inline T threshold_ = (T)1.1920928955078125e-7;
};

class DistArray;

struct TsrExpr {
  DistArray* array;
  std::string idx;
  double factor;
  TsrExpr& operator=(const struct MultExpr& e);
  // C("i,j") += A("i,k") * B("k,j") (expressions/tsr_expr.h:146-152)
  TsrExpr& operator+=(const struct MultExpr& e);
};

struct MultExpr {
  TsrExpr left, right;
  double factor;
};

inline MultExpr operator*(const TsrExpr& l, const TsrExpr& r) {
  return MultExpr{l, r, l.factor * r.factor};
}
inline TsrExpr operator*(double s, TsrExpr e) {
  e.factor *= s;
  return e;
}
inline MultExpr operator*(double s, MultExpr e) {
  e.factor *= s;
  return e;
}

// DistArray<Tensor<double>, SparsePolicy|DensePolicy>: shallow-copy handle
// to device-resident tiles.
class DistArray {
 public:
  DistArray() : world_(World::default_world()) {}
  DistArray(World& w, const TiledRange& tr) : world_(&w) { create(tr); }
  DistArray(World& w, const TiledRange& tr, const SparseShape<float>& shape) : world_(&w) {
    create(tr);
    set_shape(shape);
  }
  explicit DistArray(const TiledRange& tr) : DistArray(get_default_world(), tr) {}
  DistArray(const TiledRange& tr, const SparseShape<float>& s)
      : DistArray(get_default_world(), tr, s) {}

  void set_shape(const SparseShape<float>& s) {
    world_->check(tagpu_array_set_shape(h(), s.norms().data(), s.do_not_scale() ? 1 : 0, -1.0f));
  }
  // tiles: the nonzero tiles in ordinal order, row-major each, concatenated
  void set_tiles(const std::vector<double>& packed) {
    world_->check(tagpu_array_upload(h(), packed.data(), (int64_t)packed.size()));
  }
  std::vector<double> tiles() const {
    tagpu_array_info i{};
    world_->check(tagpu_array_get_info(h(), &i));
    std::vector<double> out(i.elements);
    world_->check(tagpu_array_download(h(), out.data(), i.elements));
    return out;
  }
  std::vector<int64_t> tile_offsets() const {
    tagpu_array_info i{};
    world_->check(tagpu_array_get_info(h(), &i));
    std::vector<int64_t> o(i.ntiles_total);
    world_->check(tagpu_array_get_tile_offsets(h(), o.data()));
    return o;
  }
  std::vector<float> shape_norms() const {
    tagpu_array_info i{};
    world_->check(tagpu_array_get_info(h(), &i));
    std::vector<float> n(i.ntiles_total);
    world_->check(tagpu_array_get_norms(h(), n.data()));
    return n;
  }
  // TiledArray::truncate (conversions/truncate.h:52-80): the shape rebuilt
  // from the stored tiles' norms; threshold < 0 means the context default
  void truncate(float threshold = -1.0f) {
    world_->check(tagpu_array_truncate(h(), threshold));
  }
  // is_zero(ordinal) of the shape (a tile absent from storage)
  bool is_zero(int64_t ordinal) const { return tile_offsets().at(ordinal) < 0; }
  // DistArray::find(ordinal).get() of a nonzero tile, row-major over its range
  std::vector<double> find(int64_t ordinal) const {
    tagpu_array_info i{};
    world_->check(tagpu_array_get_info(h(), &i));
    if (ordinal < 0 || ordinal >= i.ntiles_total)
      throw Exception(TAGPU_ERR_INVALID, "tile ordinal out of range");
    int64_t vol = 1, o = ordinal;
    for (int d = i.rank - 1; d >= 0; --d) {
      std::vector<int64_t> hm(i.ntiles[d] + 1);
      world_->check(tagpu_array_get_hashmarks(h(), d, hm.data()));
      const int64_t x = o % i.ntiles[d];
      o /= i.ntiles[d];
      vol *= hm[x + 1] - hm[x];
    }
    std::vector<double> t(vol);
    world_->check(tagpu_array_get_tile(h(), ordinal, t.data(), vol));
    return t;
  }
  // archive I/O in DistArray::serialize order (single rank)
  void save(const std::string& path) const {
    world_->check(tagpu_array_save(h(), path.c_str()));
  }
  static DistArray load(World& w, const std::string& path) {
    tagpu_array* a = nullptr;
    w.check(tagpu_array_load(w.ctx(), path.c_str(), &a));
    DistArray r;
    r.reset(a, &w);
    return r;
  }
  // make_array with synthetic tiles generated on the device
  void fill_random(uint64_t seed, uint64_t stream, int kind = 0,
                   const std::vector<double>* tile_scale = nullptr, float threshold = -1.0f) {
    world_->check(tagpu_array_generate(h(), seed, stream, kind,
                                       tile_scale ? tile_scale->data() : nullptr, 1, threshold));
  }
  TsrExpr operator()(const std::string& idx) { return TsrExpr{this, idx, 1.0}; }
  tagpu_array* handle() const { return h_ ? h_.get() : nullptr; }
  World& world() const { return *world_; }
  void set_precision(tagpu_precision p, int slices = 0) {
    precision_ = p;
    slices_ = slices;
  }
  tagpu_contract_opts opts() const {
    return tagpu_contract_opts{precision_, slices_, -1.0f, 0};
  }
  void reset(tagpu_array* a, World* w = nullptr) {
    if (w) world_ = w;
    h_.reset(a, [](tagpu_array* x) { tagpu_array_destroy(x); });
  }

 private:
  void create(const TiledRange& tr) {
    std::vector<int64_t> nt;
    std::vector<const int64_t*> hm;
    for (int d = 0; d < tr.rank(); ++d) {
      nt.push_back(tr.dim(d).tile_count());
      hm.push_back(tr.dim(d).hashmarks().data());
    }
    tagpu_array* a = nullptr;
    world_->check(tagpu_array_create(world_->ctx(), tr.rank(), nt.data(), hm.data(), &a));
    reset(a);
  }
  tagpu_array* h() const {
    if (!h_) throw Exception(TAGPU_ERR_STATE, "uninitialized DistArray");
    return h_.get();
  }
  World* world_ = nullptr;
  std::shared_ptr<tagpu_array> h_;
  int precision_ = TAGPU_PRECISION_FP64;
  int slices_ = 0;
};

inline TsrExpr& TsrExpr::operator=(const MultExpr& e) {
  World& w = e.left.array->world();
  tagpu_contract_opts o = array->opts();
  tagpu_array* c = nullptr;
  w.check(tagpu_contract(w.ctx(), idx.c_str(), e.factor * factor, e.left.array->handle(),
                         e.left.idx.c_str(), e.right.array->handle(), e.right.idx.c_str(), &o,
                         &c));
  array->reset(c, &w);
  return *this;
}

inline TsrExpr& TsrExpr::operator+=(const MultExpr& e) {
  World& w = e.left.array->world();
  tagpu_contract_opts o = array->opts();
  w.check(tagpu_contract_accumulate(w.ctx(), idx.c_str(), e.factor * factor,
                                    e.left.array->handle(), e.left.idx.c_str(),
                                    e.right.array->handle(), e.right.idx.c_str(), &o,
                                    array->handle()));
  return *this;
}

using TSpArrayD = DistArray;
using TArrayD = DistArray;

}  // namespace ta
}  // namespace tagpu
