// Drop-in check of the C++ façade: TiledArray-style expressions compile
// unchanged and give the same result as a naive host loop (integer data, so
// the comparison is exact).  Built and run by tests/test_gpu_facade.py.
#include <cstdio>
#include <vector>

#include "tagpu/tiledarray.hpp"

namespace TA = tagpu::ta;

static int check(const char* what, const std::vector<double>& got, const std::vector<double>& ref) {
  if (got.size() != ref.size()) {
    std::printf("FAIL %s: size %zu vs %zu\n", what, got.size(), ref.size());
    return 1;
  }
  for (size_t i = 0; i < got.size(); ++i)
    if (got[i] != ref[i]) {
      std::printf("FAIL %s: element %zu: %g vs %g\n", what, i, got[i], ref[i]);
      return 1;
    }
  std::printf("ok %s (%zu elements)\n", what, got.size());
  return 0;
}

int main() {
  TA::World& world = TA::initialize(0);
  // A: 2 x 3 tiles over (0,3,7) x (0,2,5,9); B: (0,2,5,9) x (0,4,6)
  TA::TiledRange trA{{0, 3, 7}, {0, 2, 5, 9}};
  TA::TiledRange trB{{0, 2, 5, 9}, {0, 4, 6}};
  TA::TSpArrayD A(world, trA), B(world, trB);
  A.fill_random(5, 0, 1);  // integer data 0..100, shape from the tile norms
  B.fill_random(5, 1, 1);
  TA::TSpArrayD C;
  C("i,j") = A("i,k") * B("k,j");
  TA::TSpArrayD D;
  D("j,i") = 2.0 * (A("i,k") * B("k,j"));

  // naive reference on the host from the downloaded tiles
  auto dense = [](const TA::DistArray& X, const std::vector<std::vector<int64_t>>& hm) {
    const int64_t R = hm[0].back(), Cc = hm[1].back();
    std::vector<double> out(R * Cc, 0.0);
    auto data = X.tiles();
    auto offs = X.tile_offsets();
    const int64_t nc = (int64_t)hm[1].size() - 1;
    for (size_t t = 0; t < offs.size(); ++t) {
      if (offs[t] < 0) continue;
      const int64_t ti = t / nc, tj = t % nc;
      const int64_t r0 = hm[0][ti], r1 = hm[0][ti + 1], c0 = hm[1][tj], c1 = hm[1][tj + 1];
      for (int64_t r = r0; r < r1; ++r)
        for (int64_t c = c0; c < c1; ++c)
          out[r * Cc + c] = data[offs[t] + (r - r0) * (c1 - c0) + (c - c0)];
    }
    return out;
  };
  auto a = dense(A, {{0, 3, 7}, {0, 2, 5, 9}});
  auto b = dense(B, {{0, 2, 5, 9}, {0, 4, 6}});
  std::vector<double> ref(7 * 6, 0.0), reft(6 * 7, 0.0);
  for (int i = 0; i < 7; ++i)
    for (int j = 0; j < 6; ++j) {
      double s = 0;
      for (int k = 0; k < 9; ++k) s += a[i * 9 + k] * b[k * 6 + j];
      ref[i * 6 + j] = s;
      reft[j * 7 + i] = 2.0 * s;
    }
  int fails = 0;
  fails += check("C(i,j) = A(i,k) * B(k,j)", dense(C, {{0, 3, 7}, {0, 4, 6}}), ref);
  fails += check("D(j,i) = 2 * A(i,k) * B(k,j)", dense(D, {{0, 4, 6}, {0, 3, 7}}), reft);
  // emulated FP64 through the same expression
  TA::TSpArrayD E;
  E.set_precision(TAGPU_PRECISION_OZAKI);
  E("i,j") = A("i,k") * B("k,j");
  fails += check("emulated C(i,j)", dense(E, {{0, 3, 7}, {0, 4, 6}}), ref);
  // accumulate: C already holds A*B, so C += 0.5 * A*B gives 1.5 * A*B
  C("i,j") += 0.5 * (A("i,k") * B("k,j"));
  std::vector<double> ref15(ref);
  for (auto& v : ref15) v *= 1.5;
  fails += check("C(i,j) += 0.5 * A(i,k) * B(k,j)", dense(C, {{0, 3, 7}, {0, 4, 6}}), ref15);
  C = TA::TSpArrayD();
  D = TA::TSpArrayD();
  E = TA::TSpArrayD();
  A = TA::TSpArrayD();
  B = TA::TSpArrayD();
  TA::finalize();
  return fails;
}
