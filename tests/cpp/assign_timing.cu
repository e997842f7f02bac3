// Times `<<=` through the drop-in headers against the library's hand-fused kernels at one size.
//
//   assign_timing [n] [reps] [which]      (defaults 256, 20, all; which: deep | filter | heat | all)
//
// Expressions (written as the reference's users write them):
//   deep    out <<= cond(mask, 0.0)(Interp_SX(Grad_XS(Interp_SX(a))) * exp(b) + sin(c))
//           (the deep-chain workload; test/StencilTestDeepChain.cpp's chain with a mask)
//   filter  f <<= BoxFilter_XX(out)
//   heat    Tn <<= T + dt * (DivX(InterpX(lam) * GradX(T)) + DivY(...) + DivZ(...))
//           (examples/heat_equation.cpp:216-220 folded into the Euler update)
//   next    the drop-in's widened rows at the same size:
//           masked_assign(mask, out, a * b) over 5 % of the cells (a point list) and the same
//           values by a full-sweep cond(mask, a * b)(out);
//           out <<= apply_pointwise<F>(a, b, c, d), F = (a + b) * c + d, and the same as an
//           expression;
//           NeboBoundaryConditionBuilder<GradX> on the x = -1 face (one 256 x 256 plane);
// and, through the C ABI on the same fields, nebo_deep_chain (out and filt), nebo_box_filter and
// nebo_heat_step.  Prints one JSON object: per expression the milliseconds per launch (CUDA
// events around `reps` launches after 3 warm-up launches; every input is larger than L2), the
// cell updates per second, the algorithmic GB/s and the largest difference from the hand
// kernel's result relative to its largest magnitude.
//
// Built in three variants (spatialops-threadfix_gb300/build.py): the default (tiled lowering,
// fixed-point exp/sin), NEBO_UNTILED + NEBO_CUDA_LIBM (one thread per column with CUDA's
// functions: the reference GPU kernel's design) and NEBO_CUDA_LIBM alone.
#include <spatialops/Nebo.h>
#include <spatialops/OperatorDatabase.h>
#include <spatialops/structured/FVStaggered.h>
#include <spatialops/structured/stencil/StencilBuilder.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "catalog_support.h"

using namespace SpatialOps;

#ifdef NEBO_UNTILED
static const char* kLowering = "one thread per column (untiled)";
#else
static const char* kLowering = "tiled (linear stencil chains composed, other inner stencil levels in shared memory)";
#endif
#ifdef NEBO_CUDA_LIBM
static const char* kMath = "CUDA exp/sin";
#else
static const char* kMath = "fixed-point exp/sin";
#endif

struct TimingSum4 {
  NEBO_HD double operator()(double a, double b, double c, double d) const { return (a + b) * c + d; }
};

static void check(int rc, const char* what) {
  if (rc != 0) {
    std::fprintf(stderr, "%s failed: %s\n", what, nebo_last_error());
    std::exit(1);
  }
}
static void check_cuda(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    std::fprintf(stderr, "%s failed: %s\n", what, cudaGetErrorString(e));
    std::exit(1);
  }
}

template <typename F>
static F make_field(int n, uint64_t stream, double lo, double hi) {
  const IntVec N(n, n, n);
  const GhostData g(1);
  const BoundaryCellInfo bc = BoundaryCellInfo::build<F>(false, false, false);
  const MemoryWindow w = get_window_with_ghost(N, g, bc);
  std::vector<double> v(w.glob_npts());
  for (size_t i = 0; i < v.size(); ++i) v[i] = lo + (hi - lo) * 0.5 * (catalog::uniform_pm1(stream, i) + 1.0);
  return F(w, bc, g, v.data());
}

template <typename F>
static F zero_field(int n) {
  const IntVec N(n, n, n);
  const GhostData g(1);
  const BoundaryCellInfo bc = BoundaryCellInfo::build<F>(false, false, false);
  return F(get_window_with_ghost(N, g, bc), bc, g, NULL);
}

// milliseconds per call of f over reps calls (3 warm-up calls first)
template <class Fn>
static double time_ms(Fn f, int reps) {
  for (int i = 0; i < 3; ++i) f();
  check_cuda(cudaDeviceSynchronize(), "warm-up");
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, 0);
  for (int i = 0; i < reps; ++i) f();
  cudaEventRecord(e1, 0);
  check_cuda(cudaEventSynchronize(e1), "timed calls");
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return ms / reps;
}

template <typename F>
static double max_rel_diff(const F& a, const F& b) {
  const double* x = a.field_values(CPU_INDEX);
  const double* y = b.field_values(CPU_INDEX);
  const size_t n = a.window_with_ghost().glob_npts();
  double d = 0.0, m = 0.0;
  for (size_t i = 0; i < n; ++i) {
    d = std::fmax(d, std::fabs(x[i] - y[i]));
    m = std::fmax(m, std::fabs(y[i]));
  }
  return m > 0 ? d / m : d;
}

struct Line {
  std::string s;
  void add(const char* name, double ms, double cells, double bytes_per_cell, double diff) {
    char buf[512];
    std::snprintf(buf, sizeof buf,
                  "%s\"%s\": {\"ms\": %.5f, \"gcells_per_s\": %.3f, \"alg_gbs\": %.1f, \"bytes_per_cell\": %.3f, "
                  "\"rel_diff_vs_hand\": %.3e}",
                  s.empty() ? "" : ", ", name, ms, cells / (ms * 1e-3) / 1e9, cells * bytes_per_cell / (ms * 1e-3) / 1e9,
                  bytes_per_cell, diff);
    s += buf;
  }
};

int main(int argc, char** argv) {
  const int n = argc > 1 ? std::atoi(argv[1]) : 256;
  const int reps = argc > 2 ? std::atoi(argv[2]) : 20;
  const std::string which = argc > 3 ? argv[3] : "all";
  const bool all = which == "all";
  if (n < 4 || reps < 1) return 1;
  OperatorDatabase opdb;
  build_stencils(n, n, n, (double)n, (double)n, (double)n, opdb);
  const double cells = (double)n * n * n;
  Line out;

  if (all || which == "deep" || which == "filter") {
    typedef OperatorTypeBuilder<Interpolant, SVolField, XVolField>::type IS2X;
    typedef OperatorTypeBuilder<Gradient, XVolField, SVolField>::type GX2S;
    typedef OperatorTypeBuilder<Filter, XVolField, XVolField>::type BoxX;
    const IS2X& is2x = *opdb.retrieve_operator<IS2X>();
    const GX2S& gx2s = *opdb.retrieve_operator<GX2S>();
    const BoxX& boxx = *opdb.retrieve_operator<BoxX>();
    SVolField a = make_field<SVolField>(n, 3, -1.0, 1.0);
    XVolField b = make_field<XVolField>(n, 4, -1.0, 1.0), c = make_field<XVolField>(n, 5, -1.0, 1.0);
    XVolField o1 = zero_field<XVolField>(n), o2 = zero_field<XVolField>(n);
    XVolField f1 = zero_field<XVolField>(n), f2 = zero_field<XVolField>(n);
    // mask: 5 % of the cells (hashed) plus every interior cell with an index at 0 or n-1
    std::vector<IntVec> pts;
    const uint64_t ms = 6;
    for (int z = 0; z < n; ++z)
      for (int y = 0; y < n; ++y)
        for (int x = 0; x < n; ++x) {
          const bool edge = x == 0 || y == 0 || z == 0 || x == n - 1 || y == n - 1 || z == n - 1;
          if (edge || catalog::uniform_pm1(ms, (uint64_t)((z * n + y) * n + x)) < -0.9) pts.push_back(IntVec(x, y, z));
        }
    SpatialMask<XVolField> m(o1, pts);
    const double t_deep = time_ms([&] { o1 <<= cond(m, 0.0)(is2x(gx2s(is2x(a))) * exp(b) + sin(c)); }, reps);
    const double t_filt = time_ms([&] { f1 <<= boxx(o1); }, reps);
    const nebo_field da = a.descriptor(), db = b.descriptor(), dc = c.descriptor();
    const nebo_field do2 = o2.descriptor(), df2 = f2.descriptor();
    const uint32_t* words = m.mask_values(GPU_INDEX);
    nebo_profile_enable(1);
    nebo_profile_report(nullptr, 0, 1);
    const double t_hand = time_ms([&] { check(nebo_deep_chain(&da, &db, &dc, words, &do2, &df2, 1.0, nullptr), "nebo_deep_chain"); },
                                  reps);
    char rep[4096];
    nebo_profile_report(rep, sizeof rep, 1);
    nebo_profile_enable(0);
    // the hand kernels' per-launch times (chain and filter) from the library's own events
    double hand_chain = 0, hand_filter = 0;
    if (const char* p = std::strstr(rep, "\"deep_chain\"")) {
      const char* q = std::strstr(p, "\"ms\":");
      const char* l = std::strstr(p, "\"launches\":");
      if (q && l) hand_chain = std::atof(q + 5) / std::atof(l + 11);
    }
    if (const char* p = std::strstr(rep, "\"box_filter\"")) {
      const char* q = std::strstr(p, "\"ms\":");
      const char* l = std::strstr(p, "\"launches\":");
      if (q && l) hand_filter = std::atof(q + 5) / std::atof(l + 11);
    }
    const nebo_field dsrc = o1.descriptor(), ddst = f2.descriptor();
    const double t_hand_filter = time_ms([&] { check(nebo_box_filter(&dsrc, &ddst, 0, nullptr, nullptr), "nebo_box_filter"); }, reps);
    const double d_out = max_rel_diff(o1, o2);
    check(nebo_box_filter(&dsrc, &ddst, 0, nullptr, nullptr), "nebo_box_filter");
    check_cuda(cudaDeviceSynchronize(), "filter");
    const double d_filt = max_rel_diff(f1, f2);
    out.add("deep_assign", t_deep, cells, 32.125, d_out);
    out.add("filter_assign", t_filt, cells, 16.0, d_filt);
    out.add("deep_hand_chain", hand_chain > 0 ? hand_chain : t_hand, cells, 32.125, 0.0);
    out.add("deep_hand_chain_and_filter", t_hand, cells, 48.125, 0.0);
    out.add("filter_hand", t_hand_filter, cells, 16.0, 0.0);
    (void)hand_filter;
  }

  if (all || which == "heat") {
    typedef BasicOpTypes<SVolField> OS;
    const OS::InterpC2FX& ix = *opdb.retrieve_operator<OS::InterpC2FX>();
    const OS::InterpC2FY& iy = *opdb.retrieve_operator<OS::InterpC2FY>();
    const OS::InterpC2FZ& iz = *opdb.retrieve_operator<OS::InterpC2FZ>();
    const OS::GradX& gx = *opdb.retrieve_operator<OS::GradX>();
    const OS::GradY& gy = *opdb.retrieve_operator<OS::GradY>();
    const OS::GradZ& gz = *opdb.retrieve_operator<OS::GradZ>();
    const OS::DivX& dx = *opdb.retrieve_operator<OS::DivX>();
    const OS::DivY& dy = *opdb.retrieve_operator<OS::DivY>();
    const OS::DivZ& dz = *opdb.retrieve_operator<OS::DivZ>();
    SVolField T = make_field<SVolField>(n, 1, -1.0, 1.0), lam = make_field<SVolField>(n, 2, 0.5, 1.5);
    SVolField Tn = zero_field<SVolField>(n), Th = zero_field<SVolField>(n);
    const double dt = 0.15 / 1.5;
    const double t_heat = time_ms([&] { Tn <<= T + dt * (dx(ix(lam) * gx(T)) + dy(iy(lam) * gy(T)) + dz(iz(lam) * gz(T))); },
                                  reps);
    const nebo_field dT = T.descriptor(), dTh = Th.descriptor(), dl = lam.descriptor();
    const double sp[3] = {1.0, 1.0, 1.0};
    const double t_hand = time_ms([&] { check(nebo_heat_step(&dT, &dTh, &dl, dt, sp, nullptr), "nebo_heat_step"); }, reps);
    // compare interiors only (the hand kernel also writes periodic ghost images)
    const double* x = Tn.field_values(CPU_INDEX);
    const double* y = Th.field_values(CPU_INDEX);
    const int g = n + 2;
    double d = 0, mm = 0;
    for (int k = 1; k <= n; ++k)
      for (int j = 1; j <= n; ++j)
        for (int i = 1; i <= n; ++i) {
          const size_t q = (size_t)i + (size_t)g * (j + (size_t)g * k);
          d = std::fmax(d, std::fabs(x[q] - y[q]));
          mm = std::fmax(mm, std::fabs(y[q]));
        }
    out.add("heat_assign", t_heat, cells, 24.0, mm > 0 ? d / mm : d);
    out.add("heat_hand", t_hand, cells, 24.0, 0.0);
  }
  if (all || which == "next") {
    typedef BasicOpTypes<SVolField> OS;
    SVolField a = make_field<SVolField>(n, 7, -1.0, 1.0), b = make_field<SVolField>(n, 8, -1.0, 1.0);
    SVolField c = make_field<SVolField>(n, 9, -1.0, 1.0), d = make_field<SVolField>(n, 10, -1.0, 1.0);
    SVolField o1 = zero_field<SVolField>(n), o2 = zero_field<SVolField>(n);
    std::vector<IntVec> pts;
    for (int z = 0; z < n; ++z)
      for (int y = 0; y < n; ++y)
        for (int x = 0; x < n; ++x)
          if (catalog::uniform_pm1(12, (uint64_t)((z * n + y) * n + x)) < -0.9) pts.push_back(IntVec(x, y, z));
    SpatialMask<SVolField> m(o1, pts);
    const double npts = (double)pts.size();
    // point list: per point a, b read, out written (24 B) and its 3 ints (12 B)
    const double t_masked = time_ms([&] { masked_assign(m, o1, a * b); }, reps);
    const double t_sweep = time_ms([&] { o2 <<= cond(m, a * b)(o2); }, reps);
    const double d_mask = max_rel_diff(o1, o2);
    out.add("masked_assign_5pct", t_masked, npts, 36.0, d_mask);
    out.add("masked_full_sweep_cond", t_sweep, cells, 16.0 + 1.0 / 8.0 + 2.0 * npts / cells * 8.0, 0.0);
    const double t_apply = time_ms([&] { o1 <<= apply_pointwise<TimingSum4>(a, b, c, d); }, reps);
    const double t_expr = time_ms([&] { o2 <<= (a + b) * c + d; }, reps);
    out.add("apply_pointwise_4", t_apply, cells, 40.0, max_rel_diff(o1, o2));
    out.add("apply_pointwise_as_expression", t_expr, cells, 40.0, 0.0);
    // a boundary condition on one face: 256 x 256 points, phi read at the stencil's two points
    // and written at one, gamma read (32 B per point)
    typedef OS::GradX Op;
    typedef Op::DestFieldType SX;
    NeboBoundaryConditionBuilder<Op> bc(*opdb.retrieve_operator<Op>());
    SX gamma = make_field<SX>(n, 11, -1.0, 1.0), proto = zero_field<SX>(n);
    std::vector<IntVec> face;
    for (int z = 0; z < n; ++z)
      for (int y = 0; y < n; ++y) face.push_back(IntVec(0, y, z));
    SpatialMask<SX> fm(proto, face);
    const double t_bc = time_ms([&] { bc(fm, a, gamma, true); }, reps);
    out.add("bc_gradx_face", t_bc, (double)face.size(), 32.0, 0.0);
  }
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceProp prop;
  cudaGetDeviceProperties(&prop, dev);
  std::printf("{\"n\": %d, \"reps\": %d, \"lowering\": \"%s\", \"math\": \"%s\", \"device\": \"%s\", %s}\n", n, reps, kLowering,
              kMath, prop.name, out.s.c_str());
  return 0;
}
