// Golden-vector generator built from the reference's own headers.
//
// oracle/Makefile compiles this file with the reference tree on the include path (serial Nebo,
// no CUDA; Boost names come from oracle/compat).  The binary it makes, oracle/_ref/ref_driver,
// is the reference itself evaluating the workloads below; tests/golden/make_golden.py runs it
// and stores small input/output fixtures under tests/golden/.  It is test infrastructure: the
// product never links or runs it.
//
// Commands
//   catalog <domain> <out.bin>
//       every case of tests/cpp/catalog_cases.inc on one of three small domains
//   heat <nx> <ny> <nz> <steps> <dt> <lambda.bin> <T0.bin> <out.bin>
//       explicit Euler heat equation, periodic ghosts, one ghost layer
//       (rhs as in examples/heat_equation.cpp:216-220, update as test/heatEqn/main.cpp:234-273)
//   deep <nx> <ny> <nz> <a.bin> <b.bin> <c.bin> <maskpts.bin> <out.bin>
//       out <<= cond(mask,0)(Interp(Grad(Interp(a)))*exp(b)+sin(c)); f <<= BoxFilter(out)
//   transport <n> <steps> <dt> <nu> <phi.bin> <u.bin> <v.bin> <w.bin> <lambda.bin> <out.bin>
//       upwind advection + 4th-order diffusion, Heun RK2, two ghost layers, periodic
//   ghosts <out.bin>
//       write regions of a family of expressions on fields with BC cells (sentinel bitmaps)

#include <spatialops/structured/FVStaggered.h>
#include <spatialops/structured/Grid.h>
#include <spatialops/structured/stencil/StencilBuilder.h>
#include <spatialops/NeboStencilBuilder.h>
#include <spatialops/Nebo.h>

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <thread>
#include <typeinfo>
#include <vector>

#include "../../tests/cpp/catalog_ctx.h"

// ----------------------------------------------------------------------------- periodic fill
template <typename F>
static void fill_periodic(F& f, const int n[3], int g) {
  const MemoryWindow& w = f.window_with_ghost();
  const int gx = (int)w.glob_dim(0), gy = (int)w.glob_dim(1), gz = (int)w.glob_dim(2);
  double* v = f.field_values(CPU_INDEX);
  for (int z = -g; z < n[2] + g; ++z)
    for (int y = -g; y < n[1] + g; ++y)
      for (int x = -g; x < n[0] + g; ++x) {
        const bool inside = x >= 0 && x < n[0] && y >= 0 && y < n[1] && z >= 0 && z < n[2];
        if (inside) continue;
        const int sx = ((x % n[0]) + n[0]) % n[0];
        const int sy = ((y % n[1]) + n[1]) % n[1];
        const int sz = ((z % n[2]) + n[2]) % n[2];
        v[(x + g) + gx * ((y + g) + gy * (z + g))] = v[(sx + g) + gx * ((sy + g) + gy * (sz + g))];
      }
  (void)gz;
}

template <typename F>
static F make_field(const int n[3], int g) {
  const BoundaryCellInfo bc = BoundaryCellInfo::build<F>(false, false, false);
  const MemoryWindow w = get_window_with_ghost(IntVec(n[0], n[1], n[2]), GhostData(g), bc);
  return F(w, bc, GhostData(g), NULL);
}

template <typename F>
static void load(F& f, const std::vector<double>& v) {
  double* p = f.field_values(CPU_INDEX);
  for (size_t i = 0; i < v.size(); ++i) p[i] = v[i];
}

// ----------------------------------------------------------------------------- heat
// With NEBO_REF_TIMING set, the wall time of a driver's `<<=` evaluations goes to stderr (it is
// not a record: the golden vectors do not change).
static void report_seconds(const char* what, std::chrono::steady_clock::time_point t0) {
  if (!std::getenv("NEBO_REF_TIMING")) return;
  const double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  std::fprintf(stderr, "seconds %s %.6f\n", what, s);
}

static int run_heat(int argc, char** argv) {
  if (argc < 10) return 1;
  int n[3] = {std::atoi(argv[2]), std::atoi(argv[3]), std::atoi(argv[4])};
  const int steps = std::atoi(argv[5]);
  const double dt = std::strtod(argv[6], NULL);
  const size_t npts = (size_t)(n[0] + 2) * (n[1] + 2) * (n[2] + 2);
  SVolField lam = make_field<SVolField>(n, 1);
  SVolField T0 = make_field<SVolField>(n, 1);
  SVolField T1 = make_field<SVolField>(n, 1);
  load(lam, read_doubles(argv[7], npts));
  load(T0, read_doubles(argv[8], npts));
  load(T1, std::vector<double>(npts, 0.0));
  OperatorDatabase opdb;
  build_stencils(n[0], n[1], n[2], (double)n[0], (double)n[1], (double)n[2], opdb);
  typedef BasicOpTypes<SVolField> OT;
  const OT::InterpC2FX& ix = *opdb.retrieve_operator<OT::InterpC2FX>();
  const OT::InterpC2FY& iy = *opdb.retrieve_operator<OT::InterpC2FY>();
  const OT::InterpC2FZ& iz = *opdb.retrieve_operator<OT::InterpC2FZ>();
  const OT::GradX& gx = *opdb.retrieve_operator<OT::GradX>();
  const OT::GradY& gy = *opdb.retrieve_operator<OT::GradY>();
  const OT::GradZ& gz = *opdb.retrieve_operator<OT::GradZ>();
  const OT::DivX& dx = *opdb.retrieve_operator<OT::DivX>();
  const OT::DivY& dy = *opdb.retrieve_operator<OT::DivY>();
  const OT::DivZ& dz = *opdb.retrieve_operator<OT::DivZ>();
  fill_periodic(lam, n, 1);
  SVolField* cur = &T0;
  SVolField* nxt = &T1;
  Out o(argv[9]);
  const auto t0 = std::chrono::steady_clock::now();
  for (int s = 0; s < steps; ++s) {
    fill_periodic(*cur, n, 1);
    *nxt <<= *cur + dt * (dx(ix(lam) * gx(*cur)) + dy(iy(lam) * gy(*cur)) + dz(iz(lam) * gz(*cur)));
    std::swap(cur, nxt);
  }
  report_seconds("heat", t0);
  fill_periodic(*cur, n, 1);
  dump(o, "T", *cur);
  o.value("sum", nebo_sum(*cur));
  o.value("max", nebo_max(*cur));
  o.value("norm", nebo_norm(*cur));
  return 0;
}

// ----------------------------------------------------------------------------- deep chain
static int run_deep(int argc, char** argv) {
  if (argc < 10) return 1;
  int n[3] = {std::atoi(argv[2]), std::atoi(argv[3]), std::atoi(argv[4])};
  SVolField a = make_field<SVolField>(n, 1);
  XVolField b = make_field<XVolField>(n, 1);
  XVolField c = make_field<XVolField>(n, 1);
  XVolField out = make_field<XVolField>(n, 1);
  XVolField filt = make_field<XVolField>(n, 1);
  const size_t ns = a.window_with_ghost().glob_npts();
  const size_t nx = b.window_with_ghost().glob_npts();
  load(a, read_doubles(argv[5], ns));
  load(b, read_doubles(argv[6], nx));
  load(c, read_doubles(argv[7], nx));
  std::vector<int32_t> p = read_ints(argv[8]);
  std::vector<IntVec> pts;
  for (size_t i = 0; i + 2 < p.size(); i += 3) pts.push_back(IntVec(p[i], p[i + 1], p[i + 2]));
  SpatialMask<XVolField> mask(out, pts);
  OperatorDatabase opdb;
  build_stencils(n[0], n[1], n[2], (double)n[0], (double)n[1], (double)n[2], opdb);
  typedef OperatorTypeBuilder<Interpolant, SVolField, XVolField>::type IS2X;
  typedef OperatorTypeBuilder<Gradient, XVolField, SVolField>::type GX2S;
  typedef OperatorTypeBuilder<Filter, XVolField, XVolField>::type Box;
  const IS2X& is2x = *opdb.retrieve_operator<IS2X>();
  const GX2S& gx2s = *opdb.retrieve_operator<GX2S>();
  const Box& box = *opdb.retrieve_operator<Box>();
  Out o(argv[9]);
  const auto t0 = std::chrono::steady_clock::now();
  out <<= 0.0;
  out <<= cond(mask, 0.0)(is2x(gx2s(is2x(a))) * exp(b) + sin(c));
  filt <<= 0.0;
  filt <<= box(out);
  report_seconds("deep", t0);
  dump(o, "out", out);
  dump(o, "filt", filt);
  o.value("sum", nebo_sum(filt));
  o.value("max", nebo_max(filt));
  o.value("norm", nebo_norm(filt));
  return 0;
}

// ----------------------------------------------------------------------------- transport
// Staggered-velocity scalar transport on SVol phi with two ghost layers.
// Face flux (XVol): F = nu*Interp(lambda)*G4(phi) - u*cond(u>0, phi[i-1])(phi[i]);
// rhs = Grad_{X->S}(Fx) + Grad_{Y->S}(Fy) + Grad_{Z->S}(Fz); Heun's RK2.
struct UpLoX { typedef NeboStencilPointCollection<IndexTriplet<-1, 0, 0>, NeboNil> StPtCollection; };
struct UpHiX { typedef NeboStencilPointCollection<IndexTriplet<0, 0, 0>, NeboNil> StPtCollection; };
struct UpLoY { typedef NeboStencilPointCollection<IndexTriplet<0, -1, 0>, NeboNil> StPtCollection; };
struct UpHiY { typedef NeboStencilPointCollection<IndexTriplet<0, 0, 0>, NeboNil> StPtCollection; };
struct UpLoZ { typedef NeboStencilPointCollection<IndexTriplet<0, 0, -1>, NeboNil> StPtCollection; };
struct UpHiZ { typedef NeboStencilPointCollection<IndexTriplet<0, 0, 0>, NeboNil> StPtCollection; };
struct G4X { typedef NEBO_FIRST_IJK(-2, 0, 0)::NEBO_ADD_IJK(-1, 0, 0)::NEBO_ADD_IJK(0, 0, 0)::NEBO_ADD_IJK(1, 0, 0) StPtCollection; };
struct G4Y { typedef NEBO_FIRST_IJK(0, -2, 0)::NEBO_ADD_IJK(0, -1, 0)::NEBO_ADD_IJK(0, 0, 0)::NEBO_ADD_IJK(0, 1, 0) StPtCollection; };
struct G4Z { typedef NEBO_FIRST_IJK(0, 0, -2)::NEBO_ADD_IJK(0, 0, -1)::NEBO_ADD_IJK(0, 0, 0)::NEBO_ADD_IJK(0, 0, 1) StPtCollection; };

static int run_transport(int argc, char** argv) {
  if (argc < 12) return 1;
  const int N = std::atoi(argv[2]);
  int n[3] = {N, N, N};
  const int steps = std::atoi(argv[3]);
  const double dt = std::strtod(argv[4], NULL);
  const double nu = std::strtod(argv[5], NULL);
  const int G = 2;
  SVolField phi = make_field<SVolField>(n, G), phi1 = make_field<SVolField>(n, G), phin = make_field<SVolField>(n, G);
  SVolField lam = make_field<SVolField>(n, G);
  XVolField u = make_field<XVolField>(n, G);
  YVolField v = make_field<YVolField>(n, G);
  ZVolField w = make_field<ZVolField>(n, G);
  const size_t np = phi.window_with_ghost().glob_npts();
  load(phi, read_doubles(argv[6], np));
  load(u, read_doubles(argv[7], np));
  load(v, read_doubles(argv[8], np));
  load(w, read_doubles(argv[9], np));
  load(lam, read_doubles(argv[10], np));
  load(phi1, std::vector<double>(np, 0.0));
  load(phin, std::vector<double>(np, 0.0));
  fill_periodic(lam, n, G);
  fill_periodic(u, n, G);
  fill_periodic(v, n, G);
  fill_periodic(w, n, G);
  OperatorDatabase opdb;
  build_stencils(n[0], n[1], n[2], (double)n[0], (double)n[1], (double)n[2], opdb);
  typedef OperatorTypeBuilder<Interpolant, SVolField, XVolField>::type IX;
  typedef OperatorTypeBuilder<Interpolant, SVolField, YVolField>::type IY;
  typedef OperatorTypeBuilder<Interpolant, SVolField, ZVolField>::type IZ;
  typedef OperatorTypeBuilder<Gradient, XVolField, SVolField>::type DX;
  typedef OperatorTypeBuilder<Gradient, YVolField, SVolField>::type DY;
  typedef OperatorTypeBuilder<Gradient, ZVolField, SVolField>::type DZ;
  const IX& ix = *opdb.retrieve_operator<IX>();
  const IY& iy = *opdb.retrieve_operator<IY>();
  const IZ& iz = *opdb.retrieve_operator<IZ>();
  const DX& dx = *opdb.retrieve_operator<DX>();
  const DY& dy = *opdb.retrieve_operator<DY>();
  const DZ& dz = *opdb.retrieve_operator<DZ>();
  NeboStencilBuilder<Interpolant, UpLoX::StPtCollection, SVolField, XVolField> lox(build_coef_collection(1.0));
  NeboStencilBuilder<Interpolant, UpHiX::StPtCollection, SVolField, XVolField> hix(build_coef_collection(1.0));
  NeboStencilBuilder<Interpolant, UpLoY::StPtCollection, SVolField, YVolField> loy(build_coef_collection(1.0));
  NeboStencilBuilder<Interpolant, UpHiY::StPtCollection, SVolField, YVolField> hiy(build_coef_collection(1.0));
  NeboStencilBuilder<Interpolant, UpLoZ::StPtCollection, SVolField, ZVolField> loz(build_coef_collection(1.0));
  NeboStencilBuilder<Interpolant, UpHiZ::StPtCollection, SVolField, ZVolField> hiz(build_coef_collection(1.0));
  const double h = 1.0 / 24.0;  // unit spacing
  NeboStencilBuilder<Gradient, G4X::StPtCollection, SVolField, XVolField> g4x(build_four_point_coef_collection(h, -27.0 * h, 27.0 * h, -h));
  NeboStencilBuilder<Gradient, G4Y::StPtCollection, SVolField, YVolField> g4y(build_four_point_coef_collection(h, -27.0 * h, 27.0 * h, -h));
  NeboStencilBuilder<Gradient, G4Z::StPtCollection, SVolField, ZVolField> g4z(build_four_point_coef_collection(h, -27.0 * h, 27.0 * h, -h));

#define TRANSPORT_RHS(P)                                                              \
  (dx(nu * ix(lam) * g4x(P) - u * cond(u > 0.0, lox(P))(hix(P))) +                     \
   dy(nu * iy(lam) * g4y(P) - v * cond(v > 0.0, loy(P))(hiy(P))) +                     \
   dz(nu * iz(lam) * g4z(P) - w * cond(w > 0.0, loz(P))(hiz(P))))

  Out o(argv[11]);
  for (int s = 0; s < steps; ++s) {
    fill_periodic(phi, n, G);
    phi1 <<= phi + dt * TRANSPORT_RHS(phi);
    fill_periodic(phi1, n, G);
    phin <<= 0.5 * phi + 0.5 * (phi1 + dt * TRANSPORT_RHS(phi1));
    phi <<= phin;
  }
  fill_periodic(phi, n, G);
  dump(o, "phi", phi);
  o.value("sum", nebo_sum_interior(phi));
  o.value("max", nebo_max_interior(phi));
  o.value("norm", nebo_norm_interior(phi));
  return 0;
}

int main(int argc, char** argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: ref_driver catalog|heat|deep|transport ...\n");
    return 1;
  }
  const std::string cmd = argv[1];
  int rc = 1;
#ifdef ENABLE_THREADS
  // the Threading build's pool (spatialops/Threading.h:17-19): NEBO_THREADS threads, else one per
  // host core
  {
    const char* nt = std::getenv("NEBO_THREADS");
    const int n = nt ? std::atoi(nt) : (int)std::thread::hardware_concurrency();
    Threading::setup(n > 0 ? n : 1);
  }
#endif
  if (cmd == "catalog" && argc >= 4) {
    const int id = std::atoi(argv[2]);
    Out o(argv[3]);
    CatalogCtx C(id, o);
    nebo_catalog(C);
    rc = 0;
  } else if (cmd == "heat") {
    rc = run_heat(argc, argv);
  } else if (cmd == "deep") {
    rc = run_deep(argc, argv);
  } else if (cmd == "transport") {
    rc = run_transport(argc, argv);
  }
  if (rc) std::fprintf(stderr, "bad arguments for %s\n", cmd.c_str());
  std::fflush(NULL);
  std::_Exit(rc);
}
