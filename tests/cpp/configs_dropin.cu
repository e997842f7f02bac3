// Three of the configurations written in Nebo, as the reference's users write them, through the
// drop-in headers: the code that generated tests/golden/heat.npz, deep.npz and transport.npz
// from the reference's own Nebo.
//   heat       T' <<= T + dt * (DivX(InterpX(lambda) * GradX(T)) + DivY(...) + DivZ(...)) with the
//              operator database's operators, periodic ghost fills, then nebo_sum/max/norm(T)
//   deep       out <<= cond(mask, 0.0)(Interp_SX(Grad_XS(Interp_SX(a))) * exp(b) + sin(c)),
//              filt <<= BoxFilter(out), then nebo_sum/max/norm(filt)
//   transport  per direction the face flux nu * Interp(lambda) * G4(phi) - u * cond(u > 0,
//              phi[i-1])(phi[i]) with user stencil builders (the 4th-order gradient
//              {1, -27, 27, -1}/24 and the one-point upwind reads), its divergence by the Gradient
//              operators, Heun's RK2 with periodic ghost fills
//
//   configs_dropin heat <nx> <ny> <nz> <steps> <dt> <lam> <T0> <out>
//       whole FP64 windows (1 ghost layer) as raw little-endian doubles; prints the reductions
//   configs_dropin deep <nx> <ny> <nz> <a> <b> <c> <points> <out> <filt>
//       a SVol, b, c XVol windows (1 ghost layer); points: int32 (x, y, z) triples
//   configs_dropin transport <n> <steps> <dt> <nu> <phi> <u> <v> <w> <lam> <out>
//       whole FP64 windows (2 ghost layers)
//   configs_dropin transport-time <n> <reps>
//       one RK2 step through `<<=` against nebo_transport_run (the hand-fused FP64 stages) on the
//       same fields; prints one JSON object
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

static void check(int rc, const char* what) {
  if (rc != 0) {
    std::fprintf(stderr, "%s failed: %s\n", what, nebo_last_error());
    std::exit(1);
  }
}

template <typename F>
static F make_field(IntVec N, int ghost, const std::vector<double>* v) {
  const GhostData g(ghost);
  const BoundaryCellInfo bc = BoundaryCellInfo::build<F>(false, false, false);
  const MemoryWindow w = get_window_with_ghost(N, g, bc);
  std::vector<double> zero;
  if (!v) zero.assign(w.glob_npts(), 0.0);
  return F(w, bc, g, const_cast<double*>(v ? v->data() : zero.data()));
}

// periodic images of the interior in the ghost layers, on the device copy
template <typename F>
static void fill_periodic(F& f) {
  f.device_values_for_write();
  const nebo_field d = f.descriptor();
  check(nebo_fill_periodic(&d, nullptr), "nebo_fill_periodic");
}

static std::vector<double> read_doubles(const char* path, size_t n) {
  std::vector<double> v(n);
  FILE* fp = std::fopen(path, "rb");
  if (!fp || std::fread(v.data(), sizeof(double), n, fp) != n) {
    std::fprintf(stderr, "cannot read %zu doubles from %s\n", n, path);
    std::exit(1);
  }
  std::fclose(fp);
  return v;
}

typedef NeboStencilPointCollection<IndexTriplet<-1, 0, 0>, NeboNil> UpLoX;
typedef NeboStencilPointCollection<IndexTriplet<0, 0, 0>, NeboNil> UpHi;
typedef NeboStencilPointCollection<IndexTriplet<0, -1, 0>, NeboNil> UpLoY;
typedef NeboStencilPointCollection<IndexTriplet<0, 0, -1>, NeboNil> UpLoZ;
typedef NEBO_FIRST_IJK(-2, 0, 0)::NEBO_ADD_IJK(-1, 0, 0)::NEBO_ADD_IJK(0, 0, 0)::NEBO_ADD_IJK(1, 0, 0) G4X;
typedef NEBO_FIRST_IJK(0, -2, 0)::NEBO_ADD_IJK(0, -1, 0)::NEBO_ADD_IJK(0, 0, 0)::NEBO_ADD_IJK(0, 1, 0) G4Y;
typedef NEBO_FIRST_IJK(0, 0, -2)::NEBO_ADD_IJK(0, 0, -1)::NEBO_ADD_IJK(0, 0, 0)::NEBO_ADD_IJK(0, 0, 1) G4Z;

struct Transport {
  int n;
  double dt, nu;
  OperatorDatabase opdb;
  SVolField phi, phi1, phin, lam;
  XVolField u;
  YVolField v;
  ZVolField w;
  Transport(int n_, double dt_, double nu_, const std::vector<double>* in[5])
      : n(n_), dt(dt_), nu(nu_), phi(make_field<SVolField>(IntVec(n_, n_, n_), 2, in[0])),
        phi1(make_field<SVolField>(IntVec(n_, n_, n_), 2, nullptr)),
        phin(make_field<SVolField>(IntVec(n_, n_, n_), 2, nullptr)),
        lam(make_field<SVolField>(IntVec(n_, n_, n_), 2, in[4])), u(make_field<XVolField>(IntVec(n_, n_, n_), 2, in[1])),
        v(make_field<YVolField>(IntVec(n_, n_, n_), 2, in[2])), w(make_field<ZVolField>(IntVec(n_, n_, n_), 2, in[3])) {
    build_stencils(n, n, n, (double)n, (double)n, (double)n, opdb);
    fill_periodic(lam);
    fill_periodic(u);
    fill_periodic(v);
    fill_periodic(w);
  }
  void step() {
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
    const NeboStencilBuilder<Interpolant, UpLoX, SVolField, XVolField> lox(build_coef_collection(1.0));
    const NeboStencilBuilder<Interpolant, UpHi, SVolField, XVolField> hix(build_coef_collection(1.0));
    const NeboStencilBuilder<Interpolant, UpLoY, SVolField, YVolField> loy(build_coef_collection(1.0));
    const NeboStencilBuilder<Interpolant, UpHi, SVolField, YVolField> hiy(build_coef_collection(1.0));
    const NeboStencilBuilder<Interpolant, UpLoZ, SVolField, ZVolField> loz(build_coef_collection(1.0));
    const NeboStencilBuilder<Interpolant, UpHi, SVolField, ZVolField> hiz(build_coef_collection(1.0));
    const double h = 1.0 / 24.0;  // unit spacing
    const NeboStencilBuilder<Gradient, G4X, SVolField, XVolField> g4x(build_four_point_coef_collection(h, -27.0 * h, 27.0 * h, -h));
    const NeboStencilBuilder<Gradient, G4Y, SVolField, YVolField> g4y(build_four_point_coef_collection(h, -27.0 * h, 27.0 * h, -h));
    const NeboStencilBuilder<Gradient, G4Z, SVolField, ZVolField> g4z(build_four_point_coef_collection(h, -27.0 * h, 27.0 * h, -h));
#define TRANSPORT_RHS(P)                                                          \
  (dx(nu * ix(lam) * g4x(P) - u * cond(u > 0.0, lox(P))(hix(P))) +                 \
   dy(nu * iy(lam) * g4y(P) - v * cond(v > 0.0, loy(P))(hiy(P))) +                 \
   dz(nu * iz(lam) * g4z(P) - w * cond(w > 0.0, loz(P))(hiz(P))))
    fill_periodic(phi);
    phi1 <<= phi + dt * TRANSPORT_RHS(phi);
    fill_periodic(phi1);
    phin <<= 0.5 * phi + 0.5 * (phi1 + dt * TRANSPORT_RHS(phi1));
    phi <<= phin;
#undef TRANSPORT_RHS
  }
};

static int run_heat(int argc, char** argv) {
  const IntVec N(std::atoi(argv[2]), std::atoi(argv[3]), std::atoi(argv[4]));
  const int steps = std::atoi(argv[5]);
  const double dt = std::strtod(argv[6], NULL);
  const size_t np = (size_t)(N[0] + 2) * (N[1] + 2) * (N[2] + 2);
  const std::vector<double> vl = read_doubles(argv[7], np), vt = read_doubles(argv[8], np);
  SVolField lam = make_field<SVolField>(N, 1, &vl), T0 = make_field<SVolField>(N, 1, &vt);
  SVolField T1 = make_field<SVolField>(N, 1, nullptr);
  OperatorDatabase opdb;
  build_stencils(N[0], N[1], N[2], (double)N[0], (double)N[1], (double)N[2], opdb);
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
  fill_periodic(lam);
  SVolField* cur = &T0;
  SVolField* nxt = &T1;
  for (int s = 0; s < steps; ++s) {
    fill_periodic(*cur);
    *nxt <<= *cur + dt * (dx(ix(lam) * gx(*cur)) + dy(iy(lam) * gy(*cur)) + dz(iz(lam) * gz(*cur)));
    std::swap(cur, nxt);
  }
  fill_periodic(*cur);
  const double* p = cur->field_values(CPU_INDEX);
  FILE* fp = std::fopen(argv[9], "wb");
  if (!fp || std::fwrite(p, sizeof(double), np, fp) != np) return 1;
  std::fclose(fp);
  std::printf("{\"sum\": %.17g, \"max\": %.17g, \"norm\": %.17g}\n", nebo_sum(*cur), nebo_max(*cur),
              nebo_norm(*cur));
  return 0;
}

static void write_doubles(const char* path, const double* p, size_t n) {
  FILE* fp = std::fopen(path, "wb");
  if (!fp || std::fwrite(p, sizeof(double), n, fp) != n) {
    std::fprintf(stderr, "cannot write %s\n", path);
    std::exit(1);
  }
  std::fclose(fp);
}

static int run_deep(int argc, char** argv) {
  const IntVec N(std::atoi(argv[2]), std::atoi(argv[3]), std::atoi(argv[4]));
  const size_t ns = (size_t)(N[0] + 2) * (N[1] + 2) * (N[2] + 2);
  SVolField a = make_field<SVolField>(N, 1, nullptr);
  XVolField b = make_field<XVolField>(N, 1, nullptr);
  const size_t nx = b.window_with_ghost().glob_npts();
  const std::vector<double> va = read_doubles(argv[5], ns), vb = read_doubles(argv[6], nx), vc = read_doubles(argv[7], nx);
  a = make_field<SVolField>(N, 1, &va);
  b = make_field<XVolField>(N, 1, &vb);
  XVolField c = make_field<XVolField>(N, 1, &vc);
  XVolField out = make_field<XVolField>(N, 1, nullptr), filt = make_field<XVolField>(N, 1, nullptr);
  FILE* fp = std::fopen(argv[8], "rb");
  std::vector<int32_t> p;
  int32_t q;
  while (fp && std::fread(&q, sizeof q, 1, fp) == 1) p.push_back(q);
  if (fp) std::fclose(fp);
  std::vector<IntVec> pts;
  for (size_t i = 0; i + 2 < p.size(); i += 3) pts.push_back(IntVec(p[i], p[i + 1], p[i + 2]));
  SpatialMask<XVolField> mask(out, pts);
  OperatorDatabase opdb;
  build_stencils(N[0], N[1], N[2], (double)N[0], (double)N[1], (double)N[2], opdb);
  typedef OperatorTypeBuilder<Interpolant, SVolField, XVolField>::type IS2X;
  typedef OperatorTypeBuilder<Gradient, XVolField, SVolField>::type GX2S;
  typedef OperatorTypeBuilder<Filter, XVolField, XVolField>::type Box;
  const IS2X& is2x = *opdb.retrieve_operator<IS2X>();
  const GX2S& gx2s = *opdb.retrieve_operator<GX2S>();
  const Box& box = *opdb.retrieve_operator<Box>();
  out <<= 0.0;
  out <<= cond(mask, 0.0)(is2x(gx2s(is2x(a))) * exp(b) + sin(c));
  filt <<= 0.0;
  filt <<= box(out);
  write_doubles(argv[9], out.field_values(CPU_INDEX), nx);
  write_doubles(argv[10], filt.field_values(CPU_INDEX), nx);
  std::printf("{\"sum\": %.17g, \"max\": %.17g, \"norm\": %.17g}\n", nebo_sum(filt), nebo_max(filt), nebo_norm(filt));
  return 0;
}

int main(int argc, char** argv) {
  const std::string mode = argc > 1 ? argv[1] : "";
  if (mode == "heat" && argc >= 10) return run_heat(argc, argv);
  if (mode == "deep" && argc >= 11) return run_deep(argc, argv);
  if (mode == "transport" && argc >= 12) {
    const int n = std::atoi(argv[2]), steps = std::atoi(argv[3]);
    const double dt = std::strtod(argv[4], NULL), nu = std::strtod(argv[5], NULL);
    const size_t np = (size_t)(n + 4) * (n + 4) * (n + 4);
    std::vector<double> vals[5];
    const std::vector<double>* in[5];
    for (int i = 0; i < 5; ++i) {
      vals[i] = read_doubles(argv[6 + i], np);
      in[i] = &vals[i];
    }
    Transport t(n, dt, nu, in);
    for (int s = 0; s < steps; ++s) t.step();
    fill_periodic(t.phi);
    const double* p = t.phi.field_values(CPU_INDEX);
    FILE* fp = std::fopen(argv[11], "wb");
    if (!fp || std::fwrite(p, sizeof(double), np, fp) != np) return 1;
    std::fclose(fp);
    return 0;
  }
  if (mode == "transport-time" && argc >= 4) {
    const int n = std::atoi(argv[2]), reps = std::atoi(argv[3]);
    const size_t np = (size_t)(n + 4) * (n + 4) * (n + 4);
    std::vector<double> vals[5];
    const std::vector<double>* in[5];
    for (int i = 0; i < 5; ++i) {
      vals[i].resize(np);
      for (size_t j = 0; j < np; ++j)
        vals[i][j] = i == 4 ? 1.0 + 0.5 * catalog::uniform_pm1(40 + i, j) : catalog::uniform_pm1(40 + i, j);
      in[i] = &vals[i];
    }
    Transport t(n, 0.05, 0.01, in);
    auto time_ms = [&](auto f) {
      for (int i = 0; i < 2; ++i) f();
      cudaDeviceSynchronize();
      cudaEvent_t e0, e1;
      cudaEventCreate(&e0);
      cudaEventCreate(&e1);
      cudaEventRecord(e0, 0);
      for (int i = 0; i < reps; ++i) f();
      cudaEventRecord(e1, 0);
      cudaEventSynchronize(e1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      return (double)ms / reps;
    };
    const double t_assign = time_ms([&] { t.step(); });
    // the hand-fused stages on the same fields (FP64 storage)
    void* work = nullptr;
    check(nebo_alloc(nebo_transport_work_bytes(n, NEBO_F64), &work, nullptr), "nebo_alloc");
    double* ph = t.phi.device_values_for_write();
    const double* pu = t.u.device_values_for_read();
    const double* pv = t.v.device_values_for_read();
    const double* pw = t.w.device_values_for_read();
    const double* pl = t.lam.device_values_for_read();
    const double t_hand = time_ms([&] {
      check(nebo_transport_run(ph, pu, pv, pw, pl, n, 1, 0.05, 0.01, NEBO_F64, work, nullptr), "nebo_transport_run");
    });
    check(nebo_free(work, nullptr), "nebo_free");
    const double cells = (double)n * n * n;
    std::printf("{\"n\": %d, \"reps\": %d, \"transport_assign\": {\"ms_per_rk2_step\": %.4f, \"gcells_per_s\": %.3f}, "
                "\"transport_hand\": {\"ms_per_rk2_step\": %.4f, \"gcells_per_s\": %.3f}}\n",
                n, reps, t_assign, cells / (t_assign * 1e-3) / 1e9, t_hand, cells / (t_hand * 1e-3) / 1e9);
    return 0;
  }
  std::fprintf(stderr, "usage: configs_dropin heat|deep|transport|transport-time ...\n");
  return 1;
}
