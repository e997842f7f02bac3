// Operator type table: which stencil builder implements (operator, source field, destination
// field) (drop-in for spatialops/structured/stencil/FVStaggeredOperatorTypes.h:64-293).  The
// table lists the same registered combinations, because user code names operators by these
// types.
#ifndef SpatialOps_FVStaggeredOperatorTypes_h
#define SpatialOps_FVStaggeredOperatorTypes_h

#include <spatialops/Nebo.h>
#include <spatialops/SpatialOpsDefs.h>
#include <spatialops/structured/FVStaggeredFieldTypes.h>

namespace SpatialOps {

template <typename OpT, typename SrcT, typename DestT>
struct OperatorTypeBuilder;

// same-type interpolant: the null stencil
template <typename FieldT>
struct OperatorTypeBuilder<Interpolant, FieldT, FieldT> {
  typedef NeboSumStencilBuilder<NullStencilCollection::StPtCollection, FieldT, FieldT> type;
};

template <typename CellT>
struct BasicOpTypes;

#define NEBO_OP_BUILDER(STYLE, OP, SRC, DEST)                                                       \
  template <>                                                                                       \
  struct OperatorTypeBuilder<OP, SRC, DEST> {                                                       \
    typedef NeboStencilBuilder<OP, STYLE<OP, SRC, DEST>::StPtCollection, SRC, DEST> type;            \
  };
#define NEBO_NULL_OP_BUILDER(OP, SRC, DEST)                                                         \
  template <>                                                                                       \
  struct OperatorTypeBuilder<OP, SRC, DEST> {                                                       \
    typedef NeboSumStencilBuilder<NullStencilCollection::StPtCollection, SRC, DEST> type;            \
  };
#define NEBO_BASIC_OPTYPES(VOL)                                                                     \
  NEBO_OP_BUILDER(Stencil2Collection, Interpolant, VOL, FaceTypes<VOL>::XFace)                      \
  NEBO_OP_BUILDER(Stencil2Collection, Interpolant, VOL, FaceTypes<VOL>::YFace)                      \
  NEBO_OP_BUILDER(Stencil2Collection, Interpolant, VOL, FaceTypes<VOL>::ZFace)                      \
  NEBO_OP_BUILDER(Stencil2Collection, Interpolant, FaceTypes<VOL>::XFace, VOL)                      \
  NEBO_OP_BUILDER(Stencil2Collection, Interpolant, FaceTypes<VOL>::YFace, VOL)                      \
  NEBO_OP_BUILDER(Stencil2Collection, Interpolant, FaceTypes<VOL>::ZFace, VOL)                      \
  NEBO_OP_BUILDER(Stencil2Collection, Gradient, VOL, FaceTypes<VOL>::XFace)                         \
  NEBO_OP_BUILDER(Stencil2Collection, Gradient, VOL, FaceTypes<VOL>::YFace)                         \
  NEBO_OP_BUILDER(Stencil2Collection, Gradient, VOL, FaceTypes<VOL>::ZFace)                         \
  NEBO_OP_BUILDER(Stencil2Collection, Divergence, FaceTypes<VOL>::XFace, VOL)                       \
  NEBO_OP_BUILDER(Stencil2Collection, Divergence, FaceTypes<VOL>::YFace, VOL)                       \
  NEBO_OP_BUILDER(Stencil2Collection, Divergence, FaceTypes<VOL>::ZFace, VOL)                       \
  template <>                                                                                       \
  struct BasicOpTypes<VOL> {                                                                        \
    typedef OperatorTypeBuilder<Interpolant, VOL, FaceTypes<VOL>::XFace>::type InterpC2FX;         \
    typedef OperatorTypeBuilder<Interpolant, VOL, FaceTypes<VOL>::YFace>::type InterpC2FY;         \
    typedef OperatorTypeBuilder<Interpolant, VOL, FaceTypes<VOL>::ZFace>::type InterpC2FZ;         \
    typedef OperatorTypeBuilder<Interpolant, FaceTypes<VOL>::XFace, VOL>::type InterpF2CX;         \
    typedef OperatorTypeBuilder<Interpolant, FaceTypes<VOL>::YFace, VOL>::type InterpF2CY;         \
    typedef OperatorTypeBuilder<Interpolant, FaceTypes<VOL>::ZFace, VOL>::type InterpF2CZ;         \
    typedef OperatorTypeBuilder<Gradient, VOL, FaceTypes<VOL>::XFace>::type GradX;                 \
    typedef OperatorTypeBuilder<Gradient, VOL, FaceTypes<VOL>::YFace>::type GradY;                 \
    typedef OperatorTypeBuilder<Gradient, VOL, FaceTypes<VOL>::ZFace>::type GradZ;                 \
    typedef OperatorTypeBuilder<Divergence, FaceTypes<VOL>::XFace, VOL>::type DivX;                \
    typedef OperatorTypeBuilder<Divergence, FaceTypes<VOL>::YFace, VOL>::type DivY;                \
    typedef OperatorTypeBuilder<Divergence, FaceTypes<VOL>::ZFace, VOL>::type DivZ;                \
  };

NEBO_BASIC_OPTYPES(SVolField)
NEBO_BASIC_OPTYPES(XVolField)
NEBO_BASIC_OPTYPES(YVolField)
NEBO_BASIC_OPTYPES(ZVolField)

NEBO_OP_BUILDER(Stencil2Collection, Interpolant, XVolField, YSurfXField)
NEBO_OP_BUILDER(Stencil2Collection, Gradient, XVolField, YSurfXField)
NEBO_OP_BUILDER(Stencil2Collection, Interpolant, XVolField, ZSurfXField)
NEBO_OP_BUILDER(Stencil2Collection, Gradient, XVolField, ZSurfXField)
NEBO_OP_BUILDER(Stencil2Collection, Interpolant, YVolField, XSurfYField)
NEBO_OP_BUILDER(Stencil2Collection, Gradient, YVolField, XSurfYField)
NEBO_OP_BUILDER(Stencil2Collection, Interpolant, YVolField, ZSurfYField)
NEBO_OP_BUILDER(Stencil2Collection, Gradient, YVolField, ZSurfYField)
NEBO_OP_BUILDER(Stencil2Collection, Interpolant, ZVolField, XSurfZField)
NEBO_OP_BUILDER(Stencil2Collection, Gradient, ZVolField, XSurfZField)
NEBO_OP_BUILDER(Stencil2Collection, Interpolant, ZVolField, YSurfZField)
NEBO_OP_BUILDER(Stencil2Collection, Gradient, ZVolField, YSurfZField)

NEBO_OP_BUILDER(Stencil2Collection, Interpolant, SVolField, XVolField)
NEBO_OP_BUILDER(Stencil2Collection, Gradient, SVolField, XVolField)
NEBO_OP_BUILDER(Stencil2Collection, Interpolant, SVolField, YVolField)
NEBO_OP_BUILDER(Stencil2Collection, Gradient, SVolField, YVolField)
NEBO_OP_BUILDER(Stencil2Collection, Interpolant, SVolField, ZVolField)
NEBO_OP_BUILDER(Stencil2Collection, Gradient, SVolField, ZVolField)
NEBO_OP_BUILDER(Stencil2Collection, Interpolant, XVolField, SVolField)
NEBO_OP_BUILDER(Stencil2Collection, Gradient, XVolField, SVolField)
NEBO_OP_BUILDER(Stencil2Collection, Interpolant, YVolField, SVolField)
NEBO_OP_BUILDER(Stencil2Collection, Gradient, YVolField, SVolField)
NEBO_OP_BUILDER(Stencil2Collection, Interpolant, ZVolField, SVolField)
NEBO_OP_BUILDER(Stencil2Collection, Gradient, ZVolField, SVolField)

NEBO_NULL_OP_BUILDER(Interpolant, XVolField, SSurfXField)
NEBO_NULL_OP_BUILDER(Interpolant, YVolField, SSurfYField)
NEBO_NULL_OP_BUILDER(Interpolant, ZVolField, SSurfZField)
NEBO_NULL_OP_BUILDER(Interpolant, SVolField, XSurfXField)
NEBO_NULL_OP_BUILDER(Interpolant, SVolField, YSurfYField)
NEBO_NULL_OP_BUILDER(Interpolant, SVolField, ZSurfZField)
NEBO_NULL_OP_BUILDER(Interpolant, XSurfXField, SVolField)
NEBO_NULL_OP_BUILDER(Interpolant, YSurfYField, SVolField)
NEBO_NULL_OP_BUILDER(Interpolant, ZSurfZField, SVolField)

NEBO_OP_BUILDER(Stencil4Collection, Interpolant, SVolField, XSurfYField)
NEBO_OP_BUILDER(Stencil4Collection, Interpolant, SVolField, XSurfZField)
NEBO_OP_BUILDER(Stencil4Collection, Interpolant, SVolField, YSurfXField)
NEBO_OP_BUILDER(Stencil4Collection, Interpolant, SVolField, YSurfZField)
NEBO_OP_BUILDER(Stencil4Collection, Interpolant, SVolField, ZSurfXField)
NEBO_OP_BUILDER(Stencil4Collection, Interpolant, SVolField, ZSurfYField)
NEBO_OP_BUILDER(Stencil4Collection, Interpolant, XSurfYField, SVolField)
NEBO_OP_BUILDER(Stencil4Collection, Interpolant, XSurfZField, SVolField)
NEBO_OP_BUILDER(Stencil4Collection, Interpolant, YSurfXField, SVolField)
NEBO_OP_BUILDER(Stencil4Collection, Interpolant, YSurfZField, SVolField)
NEBO_OP_BUILDER(Stencil4Collection, Interpolant, ZSurfXField, SVolField)
NEBO_OP_BUILDER(Stencil4Collection, Interpolant, ZSurfYField, SVolField)
NEBO_OP_BUILDER(Stencil4Collection, Interpolant, XVolField, YVolField)
NEBO_OP_BUILDER(Stencil4Collection, Interpolant, XVolField, ZVolField)
NEBO_OP_BUILDER(Stencil4Collection, Interpolant, YVolField, XVolField)
NEBO_OP_BUILDER(Stencil4Collection, Interpolant, YVolField, ZVolField)
NEBO_OP_BUILDER(Stencil4Collection, Interpolant, ZVolField, XVolField)
NEBO_OP_BUILDER(Stencil4Collection, Interpolant, ZVolField, YVolField)

#define NEBO_FILTER_BUILDER(F)                                                                      \
  template <>                                                                                       \
  struct OperatorTypeBuilder<Filter, F, F> {                                                        \
    typedef NeboAverageStencilBuilder<BoxFilter3DStencilCollection::StPtCollection, F, F> type;     \
  };
NEBO_FILTER_BUILDER(SVolField)
NEBO_FILTER_BUILDER(XVolField)
NEBO_FILTER_BUILDER(YVolField)
NEBO_FILTER_BUILDER(ZVolField)
NEBO_FILTER_BUILDER(XSurfXField)
NEBO_FILTER_BUILDER(XSurfYField)
NEBO_FILTER_BUILDER(XSurfZField)
NEBO_FILTER_BUILDER(YSurfXField)
NEBO_FILTER_BUILDER(YSurfYField)
NEBO_FILTER_BUILDER(YSurfZField)
NEBO_FILTER_BUILDER(ZSurfXField)
NEBO_FILTER_BUILDER(ZSurfYField)
NEBO_FILTER_BUILDER(ZSurfZField)

#define NEBO_FD_BUILDER(OP, F)                                                                      \
  template <>                                                                                       \
  struct OperatorTypeBuilder<OP, F, F> {                                                            \
    typedef NeboStencilBuilder<OP, FDStencilCollection<OP, F, F>::StPtCollection, F, F> type;       \
  };
#define NEBO_FD_ALL(OP) NEBO_FD_BUILDER(OP, SVolField) NEBO_FD_BUILDER(OP, XVolField) \
                        NEBO_FD_BUILDER(OP, YVolField) NEBO_FD_BUILDER(OP, ZVolField)
NEBO_FD_ALL(InterpolantX)
NEBO_FD_ALL(InterpolantY)
NEBO_FD_ALL(InterpolantZ)
NEBO_FD_ALL(GradientX)
NEBO_FD_ALL(GradientY)
NEBO_FD_ALL(GradientZ)

#undef NEBO_FD_ALL
#undef NEBO_FD_BUILDER
#undef NEBO_FILTER_BUILDER
#undef NEBO_BASIC_OPTYPES
#undef NEBO_NULL_OP_BUILDER
#undef NEBO_OP_BUILDER

}  // namespace SpatialOps
#endif
