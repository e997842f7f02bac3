// `<<=` on FP32 fields through the drop-in headers, against the same expressions on FP64 fields
// (the FP32 inputs are the FP64 ones rounded).  Exercises the lowering passes on float: the
// constant factoring (signed pairs, FMA sums, factors applied at the root), its fallback for a
// pair with unequal coefficients, and the composition of nested linear stencils.
//
//   float_assign [n]      (default 20)
//
// The expressions: the heat update (factored), a pair with unequal coefficients (kept as
// written), a nested chain (composed), and a factored operand minus an unfactored one.
//
// Prints one JSON object: per expression the relative max-norm difference between the FP32 and
// the FP64 results over the written cells.
#include <spatialops/Nebo.h>
#include <spatialops/structured/FVStaggered.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "catalog_support.h"

using namespace SpatialOps;

template <typename T>
using SF = SpatialField<SVol, T>;

template <typename T>
static SF<T> make_field(int n, uint64_t stream, double lo, double hi) {
  const IntVec N(n, n - 2, n - 4);
  const GhostData g(1);
  const BoundaryCellInfo bc = BoundaryCellInfo::build<SF<T>>(false, false, false);
  const MemoryWindow w = get_window_with_ghost(N, g, bc);
  std::vector<T> v(w.glob_npts());
  for (size_t i = 0; i < v.size(); ++i) v[i] = (T)(lo + (hi - lo) * 0.5 * (catalog::uniform_pm1(stream, i) + 1.0));
  return SF<T>(w, bc, g, v.data());
}

template <typename T>
static SF<T> sentinel_field(int n) {
  SF<T> f = make_field<T>(n, 1, 0.0, 0.0);
  f <<= (T)-7777.25;
  return f;
}

// SVol -> SVol stencils (the algebra of the staggered operators on one location)
typedef NEBO_FIRST_IJK(-1, 0, 0)::NEBO_ADD_IJK(0, 0, 0) LoX;
typedef NEBO_FIRST_IJK(0, 0, 0)::NEBO_ADD_IJK(1, 0, 0) HiX;
typedef NEBO_FIRST_IJK(0, -1, 0)::NEBO_ADD_IJK(0, 0, 0) LoY;
typedef NEBO_FIRST_IJK(0, 0, 0)::NEBO_ADD_IJK(0, 1, 0) HiY;
typedef NEBO_FIRST_IJK(0, 0, -1)::NEBO_ADD_IJK(0, 0, 0) LoZ;
typedef NEBO_FIRST_IJK(0, 0, 0)::NEBO_ADD_IJK(0, 0, 1) HiZ;

template <typename T>
struct Ops {
  typedef SF<T> F;
  NeboStencilBuilder<Interpolant, LoX, F, F> ix{build_two_point_coef_collection(0.5, 0.5)};
  NeboStencilBuilder<Interpolant, LoY, F, F> iy{build_two_point_coef_collection(0.5, 0.5)};
  NeboStencilBuilder<Interpolant, LoZ, F, F> iz{build_two_point_coef_collection(0.5, 0.5)};
  NeboStencilBuilder<Gradient, LoX, F, F> gx{build_two_point_coef_collection(-1.25, 1.25)};
  NeboStencilBuilder<Gradient, LoY, F, F> gy{build_two_point_coef_collection(-1.25, 1.25)};
  NeboStencilBuilder<Gradient, LoZ, F, F> gz{build_two_point_coef_collection(-1.25, 1.25)};
  NeboStencilBuilder<Divergence, HiX, F, F> dx{build_two_point_coef_collection(-1.25, 1.25)};
  NeboStencilBuilder<Divergence, HiY, F, F> dy{build_two_point_coef_collection(-1.25, 1.25)};
  NeboStencilBuilder<Divergence, HiZ, F, F> dz{build_two_point_coef_collection(-1.25, 1.25)};
  NeboStencilBuilder<Gradient, HiX, F, F> uneq{build_two_point_coef_collection(0.25, 0.75)};
};

template <typename T>
struct Results {
  std::vector<std::vector<double>> out;
};

template <typename T>
static Results<T> run(int n) {
  Ops<T> o;
  SF<T> a = make_field<T>(n, 11, -1.0, 1.0), lam = make_field<T>(n, 12, 0.5, 1.5);
  Results<T> r;
  auto keep = [&](SF<T>& f) {
    const T* v = f.field_values(CPU_INDEX);
    r.out.emplace_back(v, v + f.window_with_ghost().glob_npts());
  };
  {  // the heat update (factored)
    SF<T> out = sentinel_field<T>(n);
    out <<= a + (T)0.05 * (o.dx(o.ix(lam) * o.gx(a)) + o.dy(o.iy(lam) * o.gy(a)) + o.dz(o.iz(lam) * o.gz(a)));
    keep(out);
  }
  {  // a pair with unequal coefficients (kept as written)
    SF<T> out = sentinel_field<T>(n);
    out <<= o.uneq(a) * lam - (T)2 * a;
    keep(out);
  }
  {  // a nested chain (composed into one stencil)
    SF<T> out = sentinel_field<T>(n);
    out <<= o.ix(o.gx(o.ix(a))) * lam;
    keep(out);
  }
  {  // a factored left operand minus an unfactored one (r * x - y in one FMA)
    SF<T> out = sentinel_field<T>(n);
    out <<= o.gx(a) * lam - a;
    keep(out);
  }
  return r;
}

int main(int argc, char** argv) {
  const int n = argc > 1 ? std::atoi(argv[1]) : 20;
  if (n < 8) return 1;
  const Results<double> d = run<double>(n);
  const Results<float> f = run<float>(n);
  const char* names[] = {"heat_update", "unequal_pair", "composed_chain", "left_factor_difference"};
  std::string json = "{";
  for (size_t e = 0; e < d.out.size(); ++e) {
    double diff = 0.0, mag = 0.0;
    long written = 0, mismatched_writes = 0;
    for (size_t i = 0; i < d.out[e].size(); ++i) {
      const bool wd = d.out[e][i] != -7777.25, wf = f.out[e][i] != -7777.25f;
      if (wd != wf) ++mismatched_writes;
      if (!wd) continue;
      ++written;
      diff = std::fmax(diff, std::fabs((double)f.out[e][i] - d.out[e][i]));
      mag = std::fmax(mag, std::fabs(d.out[e][i]));
    }
    char buf[256];
    std::snprintf(buf, sizeof buf, "%s\"%s\": {\"rel_diff\": %.3e, \"written\": %ld, \"write_set_mismatch\": %ld}",
                  e ? ", " : "", names[e], mag > 0 ? diff / mag : diff, written, mismatched_writes);
    json += buf;
  }
  json += "}";
  std::printf("%s\n", json.c_str());
  return 0;
}
