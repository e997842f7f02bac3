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
// the FP64 results over the written cells, and between the FP64 results and direct host loops of
// the same expressions (an algebra check of the lowering passes).
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
  std::vector<double> a, lam;  // the inputs as the fields hold them
  int gx = 0, gy = 0;          // window pitches
};

// The expressions by direct loops on the host, at window cell i (FP64).
static double host_value(int e, const std::vector<double>& a, const std::vector<double>& lam, int gx, int gy, long i) {
  const long sx = 1, sy = gx, sz = (long)gx * gy;
  auto I = [&](const std::vector<double>& f, long c, long s) { return 0.5 * f[c - s] + 0.5 * f[c]; };
  auto G = [&](const std::vector<double>& f, long c, long s) { return -1.25 * f[c - s] + 1.25 * f[c]; };
  auto flux = [&](long c, long s) { return I(lam, c, s) * G(a, c, s); };
  auto D = [&](long c, long s) { return -1.25 * flux(c, s) + 1.25 * flux(c + s, s); };
  switch (e) {
    case 0:
      return a[i] + 0.05 * (D(i, sx) + D(i, sy) + D(i, sz));
    case 1:
      return (0.25 * a[i] + 0.75 * a[i + sx]) * lam[i] - 2.0 * a[i];
    case 2: {
      auto ia = [&](long c) { return I(a, c, sx); };
      auto gia = [&](long c) { return -1.25 * ia(c - sx) + 1.25 * ia(c); };
      return (0.5 * gia(i - sx) + 0.5 * gia(i)) * lam[i];
    }
    default:
      return G(a, i, sx) * lam[i] - a[i];
  }
}

template <typename T>
static Results<T> run(int n) {
  Ops<T> o;
  SF<T> a = make_field<T>(n, 11, -1.0, 1.0), lam = make_field<T>(n, 12, 0.5, 1.5);
  Results<T> r;
  {
    const size_t np = a.window_with_ghost().glob_npts();
    const T* va = a.field_values(CPU_INDEX);
    const T* vl = lam.field_values(CPU_INDEX);
    r.a.assign(va, va + np);
    r.lam.assign(vl, vl + np);
    r.gx = (int)a.window_with_ghost().glob_dim(0);
    r.gy = (int)a.window_with_ghost().glob_dim(1);
  }
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
    // the FP64 results against the host loops
    double hdiff = 0.0, hmag = 0.0;
    for (size_t i = 0; i < d.out[e].size(); ++i) {
      if (d.out[e][i] == -7777.25) continue;
      const double h = host_value((int)e, d.a, d.lam, d.gx, d.gy, (long)i);
      hdiff = std::fmax(hdiff, std::fabs(d.out[e][i] - h));
      hmag = std::fmax(hmag, std::fabs(h));
    }
    char buf[320];
    std::snprintf(buf, sizeof buf,
                  "%s\"%s\": {\"rel_diff\": %.3e, \"fp64_rel_diff_host\": %.3e, \"written\": %ld, "
                  "\"write_set_mismatch\": %ld}",
                  e ? ", " : "", names[e], mag > 0 ? diff / mag : diff, hmag > 0 ? hdiff / hmag : hdiff, written,
                  mismatched_writes);
    json += buf;
  }
  json += "}";
  std::printf("%s\n", json.c_str());
  return 0;
}
