// Context shared by the programs that run the expression catalog (tests/cpp/catalog_cases.inc):
// the reference-built golden generator (oracle/ref/ref_driver.cpp) and the GPU catalog program
// (tests/cpp/catalog_gpu.cu).  It uses only names that the reference's headers and the drop-in
// headers both define, so the same code drives both.  The including file includes its SpatialOps
// headers first.
#pragma once

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "catalog_support.h"

using namespace SpatialOps;

// ----------------------------------------------------------------------------- output
struct Out {
  FILE* f;
  explicit Out(const char* path) {
    f = std::fopen(path, "wb");
    if (!f) { std::perror(path); std::exit(2); }
    std::fwrite("NEBOCAT1", 1, 8, f);
  }
  ~Out() { std::fclose(f); }
  void head(uint32_t kind, const std::string& name) {
    uint32_t n = (uint32_t)name.size();
    std::fwrite(&kind, 4, 1, f);
    std::fwrite(&n, 4, 1, f);
    std::fwrite(name.data(), 1, n, f);
  }
  void field(const std::string& name, int type_code, const int glob[3], const double* v) {
    head(0, name);
    int32_t hdr[4] = {glob[0], glob[1], glob[2], type_code};
    std::fwrite(hdr, 4, 4, f);
    std::fwrite(v, 8, (size_t)glob[0] * glob[1] * glob[2], f);
  }
  void value(const std::string& name, double v) {
    head(1, name);
    std::fwrite(&v, 8, 1, f);
  }
  void error(const std::string& name, const std::string& msg) {
    head(2, name);
    uint32_t n = (uint32_t)msg.size();
    std::fwrite(&n, 4, 1, f);
    std::fwrite(msg.data(), 1, n, f);
  }
};

static std::vector<double> read_doubles(const char* path, size_t n) {
  std::vector<double> v(n);
  FILE* f = std::fopen(path, "rb");
  if (!f) { std::perror(path); std::exit(2); }
  if (std::fread(v.data(), 8, n, f) != n) { std::fprintf(stderr, "short read %s\n", path); std::exit(2); }
  std::fclose(f);
  return v;
}

static std::vector<int32_t> read_ints(const char* path) {
  std::vector<int32_t> v;
  FILE* f = std::fopen(path, "rb");
  if (!f) { std::perror(path); std::exit(2); }
  int32_t x;
  while (std::fread(&x, 4, 1, f) == 1) v.push_back(x);
  std::fclose(f);
  return v;
}

// ----------------------------------------------------------------------------- type codes
template <typename F> struct TypeCode;
#define TYPE_CODE(F, C) template <> struct TypeCode<F> { enum { value = C }; };
TYPE_CODE(SVolField, 1) TYPE_CODE(XVolField, 2) TYPE_CODE(YVolField, 3) TYPE_CODE(ZVolField, 4)
TYPE_CODE(SSurfXField, 5) TYPE_CODE(SSurfYField, 6) TYPE_CODE(SSurfZField, 7)
TYPE_CODE(XSurfXField, 8) TYPE_CODE(XSurfYField, 9) TYPE_CODE(XSurfZField, 10)
TYPE_CODE(YSurfXField, 11) TYPE_CODE(YSurfYField, 12) TYPE_CODE(YSurfZField, 13)
TYPE_CODE(ZSurfXField, 14) TYPE_CODE(ZSurfYField, 15) TYPE_CODE(ZSurfZField, 16)
TYPE_CODE(SingleValueField, 17)

template <typename F>
static void dump(Out& o, const std::string& name, const F& f) {
  const MemoryWindow& w = f.window_with_ghost();
  int glob[3] = {(int)w.glob_dim(0), (int)w.glob_dim(1), (int)w.glob_dim(2)};
  o.field(name, TypeCode<F>::value, glob, f.field_values(CPU_INDEX));
}

// ----------------------------------------------------------------------------- catalog context
struct Domain { int n[3]; int ghost; int bc[3]; double L[3]; };
static const Domain DOMAINS[3] = {
    {{7, 6, 5}, 1, {0, 0, 0}, {9.1, 5.4, 5.5}},
    {{6, 5, 4}, 1, {1, 1, 1}, {6.0, 6.5, 3.2}},
    {{6, 6, 6}, 2, {0, 0, 0}, {6.0, 7.2, 4.8}},
};

struct CatalogCtx {
  Domain d;
  int domain_id;
  Out& out;
  OperatorDatabase opdb;
  std::map<std::pair<int, int>, std::shared_ptr<void> > inputs;

  CatalogCtx(int id, Out& o) : d(DOMAINS[id]), domain_id(id), out(o) {
    build_stencils(d.n[0], d.n[1], d.n[2], d.L[0], d.L[1], d.L[2], opdb);
  }

  template <typename F> F make() {
    const IntVec n(d.n[0], d.n[1], d.n[2]);
    const GhostData g(d.ghost);
    const BoundaryCellInfo bc = BoundaryCellInfo::build<F>(d.bc[0] != 0, d.bc[1] != 0, d.bc[2] != 0);
    const MemoryWindow w = get_window_with_ghost(n, g, bc);
    return F(w, bc, g, NULL);
  }

  template <typename F> F& in(int k) {
    std::pair<int, int> key(TypeCode<F>::value, k);
    if (!inputs.count(key)) {
      std::shared_ptr<F> f(new F(make<F>()));
      const uint64_t stream = catalog::field_stream(TypeCode<F>::value, k, domain_id);
      const size_t n = f->window_with_ghost().glob_npts();
      double* v = f->field_values(CPU_INDEX);
      for (size_t i = 0; i < n; ++i) v[i] = catalog::uniform_pm1(stream, i);
      inputs[key] = f;
    }
    return *static_cast<F*>(inputs[key].get());
  }

  // SingleValue fields: a 1x1x1 window without ghosts (test/NeboTest.cpp's SVwindow); the value
  // 2u + 0.25 rounds once however the compiler contracts it
  SingleValueField make_sv() {
    const GhostData g(0);
    const BoundaryCellInfo bc = BoundaryCellInfo::build<SingleValueField>(false, false, false);
    const MemoryWindow w = get_window_with_ghost(IntVec(1, 1, 1), g, bc);
    return SingleValueField(w, bc, g, NULL);
  }
  SingleValueField& sv(int k) {
    std::pair<int, int> key(TypeCode<SingleValueField>::value, k);
    if (!inputs.count(key)) {
      std::shared_ptr<SingleValueField> f(new SingleValueField(make_sv()));
      f->field_values(CPU_INDEX)[0] = 2.0 * catalog::uniform_pm1(catalog::field_stream(17, k, domain_id), 0) + 0.25;
      inputs[key] = f;
    }
    return *static_cast<SingleValueField*>(inputs[key].get());
  }
  SingleValueField fresh_sv() {
    SingleValueField f = make_sv();
    f.field_values(CPU_INDEX)[0] = catalog::CATALOG_SENTINEL_VALUE;
    return f;
  }

  template <typename F> F fresh() {
    F f = make<F>();
    const size_t n = f.window_with_ghost().glob_npts();
    double* v = f.field_values(CPU_INDEX);
    for (size_t i = 0; i < n; ++i) v[i] = catalog::CATALOG_SENTINEL_VALUE;
    return f;
  }

  std::vector<IntVec> plane_points(int axis, int i) const {
    std::vector<IntVec> pts;
    const int a1 = (axis + 1) % 3, a2 = (axis + 2) % 3;
    for (int v = 0; v < d.n[a2]; ++v)
      for (int u = 0; u < d.n[a1]; ++u) {
        int q[3];
        q[axis] = i;
        q[a1] = u;
        q[a2] = v;
        pts.push_back(IntVec(q[0], q[1], q[2]));
      }
    return pts;
  }
  template <typename F> SpatialMask<F> plane_mask(int axis, int i) {
    F proto = make<F>();
    return SpatialMask<F>(proto, plane_points(axis, i));
  }
  template <typename F> SpatialMask<F> mask(int k) {
    std::vector<int> p = catalog::mask_points(k, domain_id, d.n, d.ghost);
    std::vector<IntVec> pts;
    for (size_t i = 0; i < p.size(); i += 3) pts.push_back(IntVec(p[i], p[i + 1], p[i + 2]));
    F proto = make<F>();
    return SpatialMask<F>(proto, pts);
  }

  template <typename F> void rec(const char* name, const F& f) { dump(out, name, f); }
  void val(const char* name, double v) { out.value(name, v); }
  void err(const char* name, const char* msg) { out.error(name, msg); }
};

#define CATALOG_CASE(NAME, ...)                  \
  try {                                          \
    __VA_ARGS__                                  \
  } catch (std::runtime_error & e) {             \
    C.err(NAME, e.what());                       \
  }

#include "catalog_cases.inc"

