// Stencil builders and point collections (drop-in for spatialops/NeboStencilBuilder.h:85-501).
//
// The point collections are the staggered-mesh geometry itself (which neighbours an operator
// reads), so they are defined by the same compile-time rules as the reference:
//   Stencil2Collection  low  = -(src offset > dest offset), high = (src offset < dest offset)
//   Stencil4Collection  the 2x2 product of that rule over the two staggered directions
//   FDStencilCollection -unit and +unit along the operator's direction
//   BoxFilter*          the 27/9/3 neighbours, x fastest, then y, then z
#ifndef SpatialOps_NeboStencilBuilder_h
#define SpatialOps_NeboStencilBuilder_h

#include <spatialops/NeboAssignment.h>
#include <spatialops/NeboCore.h>
#include <spatialops/NeboOperators.h>

namespace SpatialOps {

template <typename OperatorType, typename PntCltnT, typename SrcFieldT, typename DestFieldT>
struct NeboStencilBuilder {
  typedef OperatorType type;
  typedef PntCltnT PointCollectionType;
  typedef SrcFieldT SrcFieldType;
  typedef DestFieldT DestFieldType;
  typedef NeboStencilCoefCollection<PointCollectionType::length> CoefCollection;
  typedef typename DestFieldT::value_type T;

  template <typename Arg>
  struct WithArg {
    typedef nebo_detail::StencilNode<T, PointCollectionType, Arg> Stencil;
    typedef NeboExpression<Stencil, DestFieldType> Result;
  };
  typedef nebo_detail::FieldNode<SrcFieldType> FieldArg;
  typedef nebo_detail::StencilNode<T, PointCollectionType, FieldArg> FieldStencil;
  typedef NeboExpression<FieldStencil, DestFieldType> FieldResult;

  explicit NeboStencilBuilder(const CoefCollection& coefs) : coefCollection_(coefs) {}
  const CoefCollection& coefs() const { return coefCollection_; }
  void apply_to_field(const SrcFieldType& src, DestFieldType& dest) const { dest <<= (*this)(src); }
  FieldResult operator()(const SrcFieldType& src) const { return FieldResult(FieldStencil(FieldArg(src), coefCollection_)); }
  template <typename Arg>
  typename WithArg<Arg>::Result operator()(const NeboExpression<Arg, SrcFieldType>& src) const {
    return typename WithArg<Arg>::Result(typename WithArg<Arg>::Stencil(src.expr(), coefCollection_));
  }

 private:
  CoefCollection coefCollection_;
};

// Sum over the points without coefficients (NeboSumStencil, NeboStencils.h:826-1046).
template <typename PntCltnT, typename SrcFieldT, typename DestFieldT>
struct NeboSumStencilBuilder {
  typedef PntCltnT PointCollectionType;
  typedef SrcFieldT SrcFieldType;
  typedef DestFieldT DestFieldType;
  typedef typename DestFieldT::value_type T;
  template <typename Arg>
  struct WithArg {
    typedef nebo_detail::SumStencilNode<T, PointCollectionType, Arg> Stencil;
    typedef NeboExpression<Stencil, DestFieldType> Result;
  };
  typedef nebo_detail::FieldNode<SrcFieldType> FieldArg;
  typedef nebo_detail::SumStencilNode<T, PointCollectionType, FieldArg> FieldStencil;
  typedef NeboExpression<FieldStencil, DestFieldType> FieldResult;

  NeboSumStencilBuilder() {}
  void apply_to_field(const SrcFieldType& src, DestFieldType& dest) const { dest <<= (*this)(src); }
  FieldResult operator()(const SrcFieldType& src) const { return FieldResult(FieldStencil(FieldArg(src))); }
  template <typename Arg>
  typename WithArg<Arg>::Result operator()(const NeboExpression<Arg, SrcFieldType>& src) const {
    return typename WithArg<Arg>::Result(typename WithArg<Arg>::Stencil(src.expr()));
  }
};

// Average = sum stencil * (1/npoints) (NeboStencilBuilder.h:389-452).
template <typename PntCltnT, typename SrcFieldT, typename DestFieldT>
struct NeboAverageStencilBuilder {
  typedef PntCltnT PointCollectionType;
  typedef SrcFieldT SrcFieldType;
  typedef DestFieldT DestFieldType;
  typedef typename DestFieldT::value_type T;
  template <typename Arg>
  struct WithArg {
    typedef nebo_detail::SumStencilNode<T, PointCollectionType, Arg> Stencil;
    typedef nebo_detail::BinNode<nebo_detail::OpMul, Stencil, nebo_detail::ScalarNode<T>> Average;
    typedef NeboExpression<Average, DestFieldType> Result;
  };
  typedef nebo_detail::FieldNode<SrcFieldType> FieldArg;
  typedef typename WithArg<FieldArg>::Stencil FieldStencil;
  typedef typename WithArg<FieldArg>::Average FieldAverage;
  typedef NeboExpression<FieldAverage, DestFieldType> FieldResult;

  NeboAverageStencilBuilder() {}
  void apply_to_field(const SrcFieldType& src, DestFieldType& dest) const { dest <<= (*this)(src); }
  FieldResult operator()(const SrcFieldType& src) const {
    return FieldResult(FieldAverage(FieldStencil(FieldArg(src)), nebo_detail::ScalarNode<T>((T)(1.0 / double(PointCollectionType::length)))));
  }
  template <typename Arg>
  typename WithArg<Arg>::Result operator()(const NeboExpression<Arg, SrcFieldType>& src) const {
    typedef typename WithArg<Arg>::Average Avg;
    return typename WithArg<Arg>::Result(
        Avg(typename WithArg<Arg>::Stencil(src.expr()), nebo_detail::ScalarNode<T>((T)(1.0 / double(PointCollectionType::length)))));
  }
};

template <typename OperatorType, typename SrcFieldType, typename DestFieldType>
struct Stencil2Collection {
  typedef typename SrcFieldType::Location::Offset SrcOffset;
  typedef typename DestFieldType::Location::Offset DestOffset;
  typedef typename GreaterThan<SrcOffset, DestOffset>::result::Negate LowStPt;
  typedef typename LessThan<SrcOffset, DestOffset>::result HighStPt;
  typedef NEBO_FIRST_POINT(LowStPt)::NEBO_ADD_POINT(HighStPt) StPtCollection;
};

template <typename OperatorType, typename SrcFieldType, typename DestFieldType>
struct Stencil4Collection {
  typedef typename SrcFieldType::Location::Offset SrcOffset;
  typedef typename DestFieldType::Location::Offset DestOffset;
  typedef IndexTriplet<1, 0, 0> XUnit;
  typedef IndexTriplet<0, 1, 0> YUnit;
  typedef IndexTriplet<0, 0, 1> ZUnit;
  typedef typename std::conditional<((int)SrcOffset::X != (int)DestOffset::X), XUnit, YUnit>::type FirstDir;
  typedef typename std::conditional<((int)SrcOffset::Z != (int)DestOffset::Z), ZUnit, YUnit>::type SecondDir;
  typedef typename Multiply<SrcOffset, FirstDir>::result SrcInFirstDir;
  typedef typename Multiply<SrcOffset, SecondDir>::result SrcInSecondDir;
  typedef typename Multiply<DestOffset, FirstDir>::result DestInFirstDir;
  typedef typename Multiply<DestOffset, SecondDir>::result DestInSecondDir;
  typedef typename GreaterThan<SrcInFirstDir, DestInFirstDir>::result::Negate LoValInFirstDir;
  typedef typename LessThan<SrcInFirstDir, DestInFirstDir>::result HiValInFirstDir;
  typedef typename GreaterThan<SrcInSecondDir, DestInSecondDir>::result::Negate LoValInSecondDir;
  typedef typename LessThan<SrcInSecondDir, DestInSecondDir>::result HiValInSecondDir;
  typedef typename Add<LoValInFirstDir, LoValInSecondDir>::result StPt1;
  typedef typename Add<HiValInFirstDir, LoValInSecondDir>::result StPt2;
  typedef typename Add<LoValInFirstDir, HiValInSecondDir>::result StPt3;
  typedef typename Add<HiValInFirstDir, HiValInSecondDir>::result StPt4;
  typedef NEBO_FIRST_POINT(StPt1)::NEBO_ADD_POINT(StPt2)::NEBO_ADD_POINT(StPt3)::NEBO_ADD_POINT(StPt4) StPtCollection;
};

template <typename OperatorType, typename SrcFieldType, typename DestFieldType>
struct FDStencilCollection {
  typedef typename OperatorType::DirT DirT;
  typedef typename UnitTriplet<DirT>::type DirVec;
  typedef typename DirVec::Negate LowStPt;
  typedef DirVec HighStPt;
  typedef NEBO_FIRST_POINT(LowStPt)::NEBO_ADD_POINT(HighStPt) StPtCollection;
};

struct NullStencilCollection {
  typedef NEBO_FIRST_IJK(0, 0, 0) StPtCollection;
};

namespace nebo_detail {
// points of a box, x fastest, then y, then z (first point innermost)
template <int X0, int X1, int Y0, int Y1, int Z0, int Z1, int x, int y, int z, class Acc, bool Done = (z > Z1)>
struct BoxPointsImpl {
  typedef NeboStencilPointCollection<IndexTriplet<x, y, z>, Acc> Next;
  typedef typename BoxPointsImpl<X0, X1, Y0, Y1, Z0, Z1, (x < X1 ? x + 1 : X0), (x < X1 ? y : (y < Y1 ? y + 1 : Y0)),
                                 ((x < X1 || y < Y1) ? z : z + 1), Next>::type type;
};
template <int X0, int X1, int Y0, int Y1, int Z0, int Z1, int x, int y, int z, class Acc>
struct BoxPointsImpl<X0, X1, Y0, Y1, Z0, Z1, x, y, z, Acc, true> {
  typedef Acc type;
};
template <int X0, int X1, int Y0, int Y1, int Z0, int Z1>
struct BoxPoints {
  typedef typename BoxPointsImpl<X0, X1, Y0, Y1, Z0, Z1, X0, Y0, Z0, NeboNil>::type type;
};
}  // namespace nebo_detail

struct BoxFilter3DStencilCollection { typedef nebo_detail::BoxPoints<-1, 1, -1, 1, -1, 1>::type StPtCollection; };
struct BoxFilter2DXYStencilCollection { typedef nebo_detail::BoxPoints<-1, 1, -1, 1, 0, 0>::type StPtCollection; };
struct BoxFilter2DXZStencilCollection { typedef nebo_detail::BoxPoints<-1, 1, 0, 0, -1, 1>::type StPtCollection; };
struct BoxFilter2DYZStencilCollection { typedef nebo_detail::BoxPoints<0, 0, -1, 1, -1, 1>::type StPtCollection; };
struct BoxFilter1DXStencilCollection { typedef nebo_detail::BoxPoints<-1, 1, 0, 0, 0, 0>::type StPtCollection; };
struct BoxFilter1DYStencilCollection { typedef nebo_detail::BoxPoints<0, 0, -1, 1, 0, 0>::type StPtCollection; };
struct BoxFilter1DZStencilCollection { typedef nebo_detail::BoxPoints<0, 0, 0, 0, -1, 1>::type StPtCollection; };

}  // namespace SpatialOps
#endif
