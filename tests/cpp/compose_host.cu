// Host check of the stencil composition of the `<<=` lowering (Compose / StencilMerge in
// include/spatialops/NeboTiled.h): the composed point lists and coefficients, built for the host
// by nvcc from the same header (no GPU needed).  Prints one line per case,
//   <case> <points> then "x y z coefficient" per point in listed order,
// or "nested <case>" when a case is (correctly) left uncomposed; exits 1 on a type mismatch.
#include <spatialops/NeboTiled.h>

#include <cstdio>
#include <type_traits>

using namespace SpatialOps;
using namespace SpatialOps::nebo_detail;

typedef DField<double> F;
// Interp SVol -> XVol {1/2, 1/2} at (-1, 0), Grad XVol -> SVol {-g, g} at (0, +1)
typedef NEBO_FIRST_IJK(-1, 0, 0)::NEBO_ADD_IJK(0, 0, 0) IX;
typedef NEBO_FIRST_IJK(0, 0, 0)::NEBO_ADD_IJK(1, 0, 0) GX;
// the same two along y
typedef NEBO_FIRST_IJK(0, -1, 0)::NEBO_ADD_IJK(0, 0, 0) IY;
// a 27-point box with weights, and a 2-point x stencil
typedef NEBO_FIRST_IJK(-1, -1, -1)::NEBO_ADD_IJK(0, -1, -1)::NEBO_ADD_IJK(1, -1, -1)::NEBO_ADD_IJK(-1, 0, -1)::
    NEBO_ADD_IJK(0, 0, -1)::NEBO_ADD_IJK(1, 0, -1)::NEBO_ADD_IJK(-1, 1, -1)::NEBO_ADD_IJK(0, 1, -1)::NEBO_ADD_IJK(
        1, 1, -1)::NEBO_ADD_IJK(-1, -1, 0)::NEBO_ADD_IJK(0, -1, 0)::NEBO_ADD_IJK(1, -1, 0)::NEBO_ADD_IJK(-1, 0, 0)::
        NEBO_ADD_IJK(0, 0, 0)::NEBO_ADD_IJK(1, 0, 0)::NEBO_ADD_IJK(-1, 1, 0)::NEBO_ADD_IJK(0, 1, 0)::NEBO_ADD_IJK(
            1, 1, 0)::NEBO_ADD_IJK(-1, -1, 1)::NEBO_ADD_IJK(0, -1, 1)::NEBO_ADD_IJK(1, -1, 1)::NEBO_ADD_IJK(-1, 0, 1)::
            NEBO_ADD_IJK(0, 0, 1)::NEBO_ADD_IJK(1, 0, 1)::NEBO_ADD_IJK(-1, 1, 1)::NEBO_ADD_IJK(0, 1, 1)::NEBO_ADD_IJK(
                1, 1, 1) Box27;

template <class Pts, class A>
DStencil<double, Pts, A> stencil(const A& a, std::initializer_list<double> c) {
  DStencil<double, Pts, A> d;
  d.a = a;
  int i = 0;
  for (double v : c) d.c[i++] = v;
  return d;
}

template <class Pts, class A>
void print_stencil(const char* name, const DStencil<double, Pts, A>& d) {
  std::printf("%s %d", name, (int)Pts::length);
  for (int i = 0; i < Pts::length; ++i)
    std::printf(" %d %d %d %.17g", PtsAt<Pts>::x(i), PtsAt<Pts>::y(i), PtsAt<Pts>::z(i), d.c[i]);
  std::printf("\n");
}

int main() {
  F a{nullptr, 10, 100};
  const double g = 1.0 / 3.0;  // 1/dx
  // Interp(Grad(Interp(a))): one 4-point stencil of the field
  auto chain = stencil<IX>(stencil<GX>(stencil<IX>(a, {0.5, 0.5}), {-g, g}), {0.5, 0.5});
  typedef Compose<decltype(chain)> C1;
  const auto c1 = C1::make(chain);
  if (!std::is_same<typename std::decay<decltype(c1.a)>::type, F>::value) {
    std::printf("error chain not composed to a stencil of the field\n");
    return 1;
  }
  print_stencil("chain", c1);
  // Grad_x(Interp_y(a)): points in the x-y plane
  auto xy = stencil<GX>(stencil<IY>(a, {0.25, 0.75}), {-2.0, 2.0});
  const auto c2 = Compose<decltype(xy)>::make(xy);
  print_stencil("xy", c2);
  // a weighted 27-point box of a 27-point box: 125 points, left nested
  typedef DStencil<double, Box27, DStencil<double, Box27, F>> Big;
  typedef typename Compose<Big>::type B;
  if (std::is_same<typename std::decay<decltype(B().a)>::type, F>::value) {
    std::printf("error 125-point composition not left nested\n");
    return 1;
  }
  std::printf("nested box_of_box\n");
  return 0;
}
