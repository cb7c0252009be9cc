// Compile-only check of the façade's array services (truncate, tile access,
// archive I/O) as a TiledArray user would write them; not executed.
#include <tagpu/tiledarray.hpp>

#include <string>
#include <vector>

namespace ta = tagpu::ta;

double use_services(ta::World& world, ta::TSpArrayD& a, const std::string& path) {
  a.truncate();
  a.truncate(1e-6f);
  double s = 0;
  if (!a.is_zero(0)) {
    std::vector<double> t = a.find(0);
    for (double x : t) s += x;
  }
  a.save(path);
  ta::TSpArrayD b = ta::TSpArrayD::load(world, path);
  ta::TSpArrayD c;
  c("i,j") = b("i,k") * a("k,j");
  c("i,j") += 0.5 * (b("i,k") * a("k,j"));
  return s + (double)c.tiles().size();
}
