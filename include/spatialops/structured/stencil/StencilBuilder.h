// build_stencils: registers every standard operator with its coefficients
// (drop-in for spatialops/structured/stencil/StencilBuilder.{h,cpp}:52-220).  dx = L/n per axis;
// interpolants {1/2, 1/2}, gradients and divergences {-1/dx, 1/dx}, 4-point interpolants
// {1/4 x 4}, finite-difference gradients {-1/(2dx), 1/(2dx)}, box filters 1/27.
#ifndef SpatialOps_StencilBuilder_h
#define SpatialOps_StencilBuilder_h

#include <spatialops/OperatorDatabase.h>
#include <spatialops/structured/stencil/FVStaggeredOperatorTypes.h>

namespace SpatialOps {

class Grid;

inline void build_stencils(const unsigned int nx, const unsigned int ny, const unsigned int nz, const double Lx,
                           const double Ly, const double Lz, OperatorDatabase& opdb) {
  const double dx = Lx / nx, dy = Ly / ny, dz = Lz / nz;
  const NeboStencilCoefCollection<2> half = build_two_point_coef_collection(0.5, 0.5);
  const NeboStencilCoefCollection<2> cdx = build_two_point_coef_collection(-1.0 / dx, 1.0 / dx);
  const NeboStencilCoefCollection<2> cdy = build_two_point_coef_collection(-1.0 / dy, 1.0 / dy);
  const NeboStencilCoefCollection<2> cdz = build_two_point_coef_collection(-1.0 / dz, 1.0 / dz);
  const NeboStencilCoefCollection<4> quarter = build_four_point_coef_collection(0.25, 0.25, 0.25, 0.25);
  const NeboStencilCoefCollection<2> hdx = build_two_point_coef_collection(-0.5 / dx, 0.5 / dx);
  const NeboStencilCoefCollection<2> hdy = build_two_point_coef_collection(-0.5 / dy, 0.5 / dy);
  const NeboStencilCoefCollection<2> hdz = build_two_point_coef_collection(-0.5 / dz, 0.5 / dz);

#define NEBO_REG(OP, SRC, DEST, C) opdb.register_new_operator(new OperatorTypeBuilder<OP, SRC, DEST>::type(C));
#define NEBO_REG0(OP, SRC, DEST) opdb.register_new_operator(new OperatorTypeBuilder<OP, SRC, DEST>::type());
#define NEBO_REG_BASIC(VOL)                                                            \
  {                                                                                    \
    typedef BasicOpTypes<VOL> O;                                                       \
    opdb.register_new_operator(new O::InterpC2FX(half));                               \
    opdb.register_new_operator(new O::InterpC2FY(half));                               \
    opdb.register_new_operator(new O::InterpC2FZ(half));                               \
    opdb.register_new_operator(new O::InterpF2CX(half));                               \
    opdb.register_new_operator(new O::InterpF2CY(half));                               \
    opdb.register_new_operator(new O::InterpF2CZ(half));                               \
    opdb.register_new_operator(new O::GradX(cdx));                                     \
    opdb.register_new_operator(new O::GradY(cdy));                                     \
    opdb.register_new_operator(new O::GradZ(cdz));                                     \
    opdb.register_new_operator(new O::DivX(cdx));                                      \
    opdb.register_new_operator(new O::DivY(cdy));                                      \
    opdb.register_new_operator(new O::DivZ(cdz));                                      \
  }
  NEBO_REG_BASIC(SVolField)
  NEBO_REG_BASIC(XVolField)
  NEBO_REG_BASIC(YVolField)
  NEBO_REG_BASIC(ZVolField)

  NEBO_REG(Interpolant, XVolField, YSurfXField, half) NEBO_REG(Gradient, XVolField, YSurfXField, cdy)
  NEBO_REG(Interpolant, XVolField, ZSurfXField, half) NEBO_REG(Gradient, XVolField, ZSurfXField, cdz)
  NEBO_REG(Interpolant, YVolField, XSurfYField, half) NEBO_REG(Gradient, YVolField, XSurfYField, cdx)
  NEBO_REG(Interpolant, YVolField, ZSurfYField, half) NEBO_REG(Gradient, YVolField, ZSurfYField, cdz)
  NEBO_REG(Interpolant, ZVolField, XSurfZField, half) NEBO_REG(Gradient, ZVolField, XSurfZField, cdx)
  NEBO_REG(Interpolant, ZVolField, YSurfZField, half) NEBO_REG(Gradient, ZVolField, YSurfZField, cdy)

  NEBO_REG(Interpolant, SVolField, XVolField, half) NEBO_REG(Gradient, SVolField, XVolField, cdx)
  NEBO_REG(Interpolant, SVolField, YVolField, half) NEBO_REG(Gradient, SVolField, YVolField, cdy)
  NEBO_REG(Interpolant, SVolField, ZVolField, half) NEBO_REG(Gradient, SVolField, ZVolField, cdz)
  NEBO_REG(Interpolant, XVolField, SVolField, half) NEBO_REG(Gradient, XVolField, SVolField, cdx)
  NEBO_REG(Interpolant, YVolField, SVolField, half) NEBO_REG(Gradient, YVolField, SVolField, cdy)
  NEBO_REG(Interpolant, ZVolField, SVolField, half) NEBO_REG(Gradient, ZVolField, SVolField, cdz)

  NEBO_REG0(Interpolant, SVolField, SVolField) NEBO_REG0(Interpolant, XVolField, XVolField)
  NEBO_REG0(Interpolant, YVolField, YVolField) NEBO_REG0(Interpolant, ZVolField, ZVolField)
  NEBO_REG0(Interpolant, XVolField, SSurfXField) NEBO_REG0(Interpolant, YVolField, SSurfYField)
  NEBO_REG0(Interpolant, ZVolField, SSurfZField) NEBO_REG0(Interpolant, SVolField, XSurfXField)
  NEBO_REG0(Interpolant, SVolField, YSurfYField) NEBO_REG0(Interpolant, SVolField, ZSurfZField)
  NEBO_REG0(Interpolant, XSurfXField, SVolField) NEBO_REG0(Interpolant, YSurfYField, SVolField)
  NEBO_REG0(Interpolant, ZSurfZField, SVolField)

  NEBO_REG(Interpolant, SVolField, XSurfYField, quarter) NEBO_REG(Interpolant, SVolField, XSurfZField, quarter)
  NEBO_REG(Interpolant, SVolField, YSurfXField, quarter) NEBO_REG(Interpolant, SVolField, YSurfZField, quarter)
  NEBO_REG(Interpolant, SVolField, ZSurfXField, quarter) NEBO_REG(Interpolant, SVolField, ZSurfYField, quarter)
  NEBO_REG(Interpolant, XSurfYField, SVolField, quarter) NEBO_REG(Interpolant, XSurfZField, SVolField, quarter)
  NEBO_REG(Interpolant, YSurfXField, SVolField, quarter) NEBO_REG(Interpolant, YSurfZField, SVolField, quarter)
  NEBO_REG(Interpolant, ZSurfXField, SVolField, quarter) NEBO_REG(Interpolant, ZSurfYField, SVolField, quarter)
  NEBO_REG(Interpolant, XVolField, YVolField, quarter) NEBO_REG(Interpolant, XVolField, ZVolField, quarter)
  NEBO_REG(Interpolant, YVolField, XVolField, quarter) NEBO_REG(Interpolant, YVolField, ZVolField, quarter)
  NEBO_REG(Interpolant, ZVolField, XVolField, quarter) NEBO_REG(Interpolant, ZVolField, YVolField, quarter)

  NEBO_REG0(Filter, SVolField, SVolField) NEBO_REG0(Filter, XVolField, XVolField)
  NEBO_REG0(Filter, YVolField, YVolField) NEBO_REG0(Filter, ZVolField, ZVolField)
  NEBO_REG0(Filter, XSurfXField, XSurfXField) NEBO_REG0(Filter, XSurfYField, XSurfYField)
  NEBO_REG0(Filter, XSurfZField, XSurfZField) NEBO_REG0(Filter, YSurfXField, YSurfXField)
  NEBO_REG0(Filter, YSurfYField, YSurfYField) NEBO_REG0(Filter, YSurfZField, YSurfZField)
  NEBO_REG0(Filter, ZSurfXField, ZSurfXField) NEBO_REG0(Filter, ZSurfYField, ZSurfYField)
  NEBO_REG0(Filter, ZSurfZField, ZSurfZField)

#define NEBO_REG_FD(VOL)                                                                               \
  NEBO_REG(InterpolantX, VOL, VOL, half) NEBO_REG(InterpolantY, VOL, VOL, half)                       \
  NEBO_REG(InterpolantZ, VOL, VOL, half) NEBO_REG(GradientX, VOL, VOL, hdx)                           \
  NEBO_REG(GradientY, VOL, VOL, hdy) NEBO_REG(GradientZ, VOL, VOL, hdz)
  NEBO_REG_FD(SVolField)
  NEBO_REG_FD(XVolField)
  NEBO_REG_FD(YVolField)
  NEBO_REG_FD(ZVolField)
#undef NEBO_REG_FD
#undef NEBO_REG_BASIC
#undef NEBO_REG0
#undef NEBO_REG
}

}  // namespace SpatialOps
#endif
