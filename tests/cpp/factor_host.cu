// Host check of the constant-factor pass of the `<<=` lowering (Factor / FactorRoot in
// include/spatialops/NeboFactor.h), built for the host by nvcc from the same header (no GPU
// needed).  Prints "<case> <ok> <factor-or-ratio>..." lines; exits 1 when a functor type is not
// the expected one.
#include <spatialops/NeboFactor.h>

#include <cstdio>
#include <type_traits>

using namespace SpatialOps;
using namespace SpatialOps::nebo_detail;

typedef DField<double> F;
typedef DScalar<double> S;
typedef NEBO_FIRST_IJK(-1, 0, 0)::NEBO_ADD_IJK(0, 0, 0) IX;  // Interp {1/2, 1/2}
typedef NEBO_FIRST_IJK(0, 0, 0)::NEBO_ADD_IJK(1, 0, 0) GX;   // Grad / Div {-g, g}
typedef NEBO_FIRST_IJK(-2, 0, 0)::NEBO_ADD_IJK(-1, 0, 0)::NEBO_ADD_IJK(0, 0, 0)::NEBO_ADD_IJK(1, 0, 0) G4;

template <class Pts, class A>
DStencil<double, Pts, A> st(const A& a, std::initializer_list<double> c) {
  DStencil<double, Pts, A> d;
  d.a = a;
  int i = 0;
  for (double v : c) d.c[i++] = v;
  return d;
}

template <class Want, class Got>
bool is_type(const Got&) {
  return std::is_same<Want, Got>::value;
}
#define EXPECT_TYPE(X, ...)                        \
  if (!is_type<__VA_ARGS__>(X)) {                  \
    std::printf("error type of %s\n", #X);         \
    return 1;                                      \
  }

int main() {
  const F T{nullptr, 10, 100}, L{nullptr, 10, 100};
  const double g = 1.0 / 3.0;
  // face flux Interp(L) * Grad(T): two signed pairs, factor 1/2 * g
  auto flux = DBin<OpMul, double, decltype(st<IX>(L, {0.5, 0.5})), decltype(st<GX>(T, {-g, g}))>{
      st<IX>(L, {0.5, 0.5}), st<GX>(T, {-g, g})};
  {
    double s;
    bool ok = true;
    auto f = Factor<decltype(flux)>::make(flux, s, ok);
    EXPECT_TYPE(f, DBin<OpMul, double, DSignedStencil<double, IX, F>, DSignedStencil<double, GX, F>>);
    std::printf("flux %d %.17g %g %g %g %g\n", (int)ok, s, f.a.c[0], f.a.c[1], f.b.c[0], f.b.c[1]);
  }
  // T + dt * Div(flux): the root is an FMA with factor 1, ratio dt * g * (g / 2)
  const double dt = 0.125;
  auto div = st<GX>(flux, {-g, g});
  auto scaled = DBin<OpMul, double, S, decltype(div)>{S{dt}, div};
  auto root = DBin<OpAdd, double, F, decltype(scaled)>{T, scaled};
  {
    bool ok = true;
    typedef FactorRoot<double, decltype(root)> FR;
    static_assert(FR::changes, "the heat update must be factored");
    auto f = FR::make(root, ok);
    EXPECT_TYPE(f.a, F);
    EXPECT_TYPE(f.b, DSignedStencil<double, GX, DBin<OpMul, double, DSignedStencil<double, IX, F>,
                                                     DSignedStencil<double, GX, F>>>);
    std::printf("heat %d %.17g\n", (int)ok, f.r);
  }
  // unequal magnitudes: the 2-point assumption fails, the launch keeps the expression as written
  {
    auto odd = st<IX>(L, {0.25, 0.75});
    bool ok = true;
    FactorRoot<double, decltype(odd)>::make(odd, ok);
    std::printf("unequal %d\n", (int)ok);
  }
  // a zero scalar factor: refused
  {
    auto z = DBin<OpMul, double, S, decltype(div)>{S{0.0}, div};
    bool ok = true;
    FactorRoot<double, decltype(z)>::make(z, ok);
    std::printf("zero %d\n", (int)ok);
  }
  // a 4-point stencil takes its argument's factor into its weights: factor 1
  {
    auto fd = st<G4>(st<IX>(L, {0.5, 0.5}), {1.0 / 24, -27.0 / 24, 27.0 / 24, -1.0 / 24});
    double s;
    bool ok = true;
    auto f = Factor<decltype(fd)>::make(fd, s, ok);
    EXPECT_TYPE(f, DStencil<double, G4, DSignedStencil<double, IX, F>>);
    std::printf("fd4 %d %.17g %.17g %.17g\n", (int)ok, s, f.c[0], f.c[1]);
  }
  return 0;
}
