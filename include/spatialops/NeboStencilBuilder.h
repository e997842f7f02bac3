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

// ============================================================================ edgeless stencils
// A weighted stencil whose ghost rule keeps only the additive part (NeboEdgelessStencilBuilder,
// NeboStencilBuilder.h:85-148 with NeboStencils.h:526-824).  The first template parameter (the
// reference's operator type slot, NeboNil in its own uses) is not used.
template <typename OperatorType, typename PntCltnT, typename SrcFieldT, typename DestFieldT>
struct NeboEdgelessStencilBuilder {
  typedef PntCltnT PointCollectionType;
  typedef SrcFieldT SrcFieldType;
  typedef DestFieldT DestFieldType;
  typedef NeboStencilCoefCollection<PointCollectionType::length> CoefCollection;
  typedef typename DestFieldT::value_type T;
  template <typename Arg>
  struct WithArg {
    typedef nebo_detail::EdgelessStencilNode<T, PointCollectionType, Arg> Stencil;
    typedef NeboExpression<Stencil, DestFieldType> Result;
  };
  typedef nebo_detail::FieldNode<SrcFieldType> FieldArg;
  typedef nebo_detail::EdgelessStencilNode<T, PointCollectionType, FieldArg> FieldStencil;
  typedef NeboExpression<FieldStencil, DestFieldType> FieldResult;

  explicit NeboEdgelessStencilBuilder(const CoefCollection& coefs) : coefCollection_(coefs) {}
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

// ============================================================================ mask shifts
// Which cell of the destination type sits on the minus / plus side of a source-type mask point
// (NeboStencilBuilder.h:503-526): for staggered pairs from the two locations' offsets, for an
// operator between fields of one type (an FD stencil) from its direction.
template <typename OperatorType, typename SrcFieldType, typename DestFieldType>
struct MaskShiftPoints {
  typedef typename SrcFieldType::Location::Offset SrcOffset;
  typedef typename DestFieldType::Location::Offset DestOffset;
  typedef typename LessThan<SrcOffset, DestOffset>::result MinusPoint;
  typedef typename GreaterThan<SrcOffset, DestOffset>::result::Negate PlusPoint;
};
template <typename OperatorType, typename FieldType>
struct MaskShiftPoints<OperatorType, FieldType, FieldType> {
  typedef typename OperatorType::type OpT;
  typedef FDStencilCollection<OpT, FieldType, FieldType> FDStencil;
  typedef typename FDStencil::DirVec MinusPoint;
  typedef typename FDStencil::DirVec::Negate PlusPoint;
};

// A mask of one field type read as a mask of another, shifted to the minus or plus side
// (NeboMaskShiftBuilder, NeboStencilBuilder.h:528-582).
template <typename OperatorT, typename SrcFieldT, typename DestFieldT>
struct NeboMaskShiftBuilder {
  typedef OperatorT OperatorType;
  typedef SrcFieldT SrcFieldType;
  typedef DestFieldT DestFieldType;
  typedef SpatialMask<SrcFieldType> SrcMask;
  typedef SpatialMask<DestFieldType> DestMask;
  typedef typename MaskShiftPoints<OperatorType, SrcFieldType, DestFieldType>::MinusPoint MinusPoint;
  typedef typename MaskShiftPoints<OperatorType, SrcFieldType, DestFieldType>::PlusPoint PlusPoint;
  typedef nebo_detail::MaskShiftNode<MinusPoint, SrcFieldType> MinusShift;
  typedef nebo_detail::MaskShiftNode<PlusPoint, SrcFieldType> PlusShift;
  typedef NeboBooleanExpression<MinusShift, DestFieldType> MinusResult;
  typedef NeboBooleanExpression<PlusShift, DestFieldType> PlusResult;

  NeboMaskShiftBuilder() {}
  MinusResult minus(const SrcMask& src) const { return MinusResult(MinusShift(src)); }
  PlusResult plus(const SrcMask& src) const { return PlusResult(PlusShift(src)); }
};

// ============================================================================ boundary conditions
namespace nebo_detail {
// every point of a collection minus Pt (ListSubtract)
template <class PC, class Pt>
struct PtsSubtract;
template <class Pt>
struct PtsSubtract<NeboNil, Pt> {
  typedef NeboNil type;
};
template <class P, class C, class Pt>
struct PtsSubtract<NeboStencilPointCollection<P, C>, Pt> {
  typedef NeboStencilPointCollection<typename Subtract<P, Pt>::result, typename PtsSubtract<C, Pt>::type> type;
};

// value(p) of every mask point shifted to the phi cell p = point - shift, into vals (all reads
// see phi as it was), then the values scattered into phi.
template <typename T, class D>
__global__ void __launch_bounds__(256) nebo_bc_eval_kernel(const int32_t* __restrict__ pts, int npts, int sx, int sy_,
                                                           int sz_, D rhs, T* __restrict__ vals) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < npts; i += gridDim.x * blockDim.x)
    vals[i] = rhs.eval(pts[3 * i] - sx, pts[3 * i + 1] - sy_, pts[3 * i + 2] - sz_);
}
template <typename T>
__global__ void __launch_bounds__(256) nebo_bc_scatter_kernel(const int32_t* __restrict__ pts, int npts, int sx, int sy_,
                                                              int sz_, T* __restrict__ out, int sy, long sz,
                                                              const T* __restrict__ vals) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < npts; i += gridDim.x * blockDim.x)
    out[(long)(pts[3 * i] - sx) + (long)sy * (pts[3 * i + 1] - sy_) + sz * (pts[3 * i + 2] - sz_)] = vals[i];
}
}  // namespace nebo_detail

// Inverts an operator at masked points: with gamma the operator's value on the destination
// type and phi its source field, sets the phi cell on the minus (or plus) side of every mask
// point so that the operator applied to phi gives gamma there (NeboBoundaryConditionBuilder,
// NeboStencilBuilder.h:584-764):
//   minus: phi[p] = (gamma[p - Low] - sum_{q != Low} c_q phi[p + q - Low]) / c_Low,  p = point - MinusPoint
//   plus:  phi[p] = (gamma[p - High] - sum_{q != High} c_q phi[p + q - High]) / c_High, p = point - PlusPoint
// (Low/High: the first/last listed stencil points; the sum in the stencil's fold order).
// The reference walks the points in order on the CPU and sweeps the whole field with cond() on a
// GPU; here two kernels run over the mask's point list only: every value is computed from phi as
// it was, then all are written.  The two agree unless one point's stencil reads another point's
// phi cell.  Points whose phi cell or whose reads fall outside the fields' valid windows are
// rejected on the host.
template <typename OperatorT>
struct NeboBoundaryConditionBuilder {
  typedef OperatorT OperatorType;
  typedef typename OperatorType::SrcFieldType PhiFieldType;
  typedef typename OperatorType::DestFieldType GammaFieldType;
  typedef typename OperatorType::PointCollectionType PointCollection;
  typedef typename PointCollection::Last LowPoint;
  typedef typename PointCollection::AllButLast NonLowPoints;
  typedef typename PointCollection::First HighPoint;
  typedef typename PointCollection::AllButFirst NonHighPoints;
  typedef typename Subtract<IndexTriplet<0, 0, 0>, LowPoint>::result LowGammaPoint;
  typedef typename Subtract<IndexTriplet<0, 0, 0>, HighPoint>::result HighGammaPoint;
  typedef typename nebo_detail::PtsSubtract<NonLowPoints, LowPoint>::type NonLowSrcPoints;
  typedef typename nebo_detail::PtsSubtract<NonHighPoints, HighPoint>::type NonHighSrcPoints;
  typedef NeboMaskShiftBuilder<OperatorType, GammaFieldType, PhiFieldType> Shift;
  typedef NeboStencilCoefCollection<PointCollection::length> CoefCollection;
  typedef typename PhiFieldType::value_type T;
  static_assert(PointCollection::length >= 2, "a boundary condition inverts a stencil of two or more points");

  explicit NeboBoundaryConditionBuilder(const OperatorType& op) : coefs_(op.coefs()) {}

  template <typename ExprType>
  void operator()(SpatialMask<GammaFieldType> mask, PhiFieldType& phi,
                  const NeboExpression<ExprType, GammaFieldType>& gamma, bool minus) const {
    if (minus)
      apply<LowGammaPoint, NonLowSrcPoints>(mask, phi, gamma.expr(), Shift::MinusPoint::int_vec(),
                                            coefs_.all_but_last(), coefs_.last());
    else
      apply<HighGammaPoint, NonHighSrcPoints>(mask, phi, gamma.expr(), Shift::PlusPoint::int_vec(), coefs_.others(),
                                              coefs_.coef());
  }
  void operator()(SpatialMask<GammaFieldType> mask, PhiFieldType& phi, const GammaFieldType& gamma, bool minus) const {
    typedef nebo_detail::FieldNode<GammaFieldType> G;
    (*this)(mask, phi, NeboExpression<G, GammaFieldType>(G(gamma)), minus);
  }
  void operator()(SpatialMask<GammaFieldType> mask, PhiFieldType& phi, const double gamma, bool minus) const {
    typedef nebo_detail::ScalarNode<T> G;
    (*this)(mask, phi, NeboExpression<G, GammaFieldType>(G((T)gamma)), minus);
  }

 private:
  // inclusive-exclusive index range of a field window along axis i (interior-relative)
  template <class F>
  static void window_range(const F& f, int i, int& lo, int& hi) {
    lo = -f.get_valid_ghost_data().get_minus(i);
    hi = lo + (int)f.window_with_ghost().extent(i);
  }

  template <class GPt, class PhiPts, class GExpr>
  void apply(const SpatialMask<GammaFieldType>& mask, PhiFieldType& phi, const GExpr& g, const IntVec& shift,
             const NeboStencilCoefCollection<PhiPts::length>& pc, double coef) const {
    const std::vector<IntVec>& pts = mask.points();
    const int np = (int)pts.size();
    if (np == 0) return;
    // valid windows: phi's whole window; gamma's expression where it is valid
    int plo[3], phi_hi[3], glo[3], ghi[3];
    const GhostData gg = g.ghosts_with_bc();
    const IntVec gext = mask.interior_extent() - mask.boundary_info().has_extra();
    for (int i = 0; i < 3; ++i) {
      window_range(phi, i, plo[i], phi_hi[i]);
      glo[i] = -gg.get_minus(i);
      ghi[i] = gext[i] + gg.get_plus(i);
    }
    std::vector<IntVec> reads;
    collect_points<PhiPts>(reads);
    const IntVec gp = GPt::int_vec();
    // every condition bounds one coordinate of one point: the mask's per-axis extremes decide
    // them all, and only a failure walks the points (for the first one that reaches out)
    auto inside = [&](const IntVec& p) {
      bool ok = true;
      for (int i = 0; i < 3; ++i) {
        ok = ok && p[i] >= plo[i] && p[i] < phi_hi[i] && p[i] + gp[i] >= glo[i] && p[i] + gp[i] < ghi[i];
        for (const IntVec& q : reads) ok = ok && p[i] + q[i] >= plo[i] && p[i] + q[i] < phi_hi[i];
      }
      return ok;
    };
    if (!inside(mask.point_min() - shift) || !inside(mask.point_max() - shift)) {
      for (const IntVec& m : pts) {
        if (inside(m - shift)) continue;
        std::ostringstream msg;
        msg << "Nebo error in Nebo Boundary Condition:\nmask point (" << m[0] << "," << m[1] << "," << m[2]
            << ") reaches outside the fields' valid cells";
        throw std::runtime_error(msg.str());
      }
    }
    // (gamma stencil with coefficient 1 - phi stencil) / coefficient, as the reference builds it
    typedef nebo_detail::EdgelessStencilNode<T, NEBO_FIRST_POINT_WO_TN(GPt), GExpr> GS;
    typedef nebo_detail::EdgelessStencilNode<T, PhiPts, nebo_detail::FieldNode<PhiFieldType>> PS;
    typedef nebo_detail::BinNode<nebo_detail::OpSub, GS, PS> Diff;
    typedef nebo_detail::BinNode<nebo_detail::OpDiv, Diff, nebo_detail::ScalarNode<T>> Rhs;
    const Rhs rhs(Diff(GS(g, NeboStencilCoefCollection<1>(1.0)), PS(nebo_detail::FieldNode<PhiFieldType>(phi), pc)),
                  nebo_detail::ScalarNode<T>((T)coef));
    nebo_detail::LaunchStreamScope scope(phi.get_stream());
    const auto dev = rhs.device();  // uploads any input edited on the host; orders other streams' writes
    T* out = phi.device_values_for_write() + phi.interior_origin();
    const int sy = (int)phi.window_with_ghost().glob_dim(0);
    const long sz = (long)phi.window_with_ghost().glob_dim(0) * (long)phi.window_with_ghost().glob_dim(1);
    cudaStream_t s = (cudaStream_t)phi.get_stream();
    T* vals = nullptr;
    nebo_detail::throw_cuda(cudaMallocAsync((void**)&vals, sizeof(T) * np, s), "Nebo Boundary Condition (allocation)");
    const int threads = 256;
    int blocks = (np + threads - 1) / threads;
    if (blocks > 8 * nebo_detail::device_sm_count()) blocks = 8 * nebo_detail::device_sm_count();
    nebo_detail::nebo_bc_eval_kernel<T, typename std::decay<decltype(dev)>::type><<<blocks, threads, 0, s>>>(
        mask.device_points(), np, shift[0], shift[1], shift[2], dev, vals);
    nebo_detail::nebo_bc_scatter_kernel<T><<<blocks, threads, 0, s>>>(mask.device_points(), np, shift[0], shift[1],
                                                                      shift[2], out, sy, sz, vals);
    const cudaError_t e = cudaGetLastError();
    cudaFreeAsync(vals, s);
    nebo_detail::throw_cuda(e, "Nebo Boundary Condition (kernel launch)");
  }

  template <class PC>
  static typename std::enable_if<(PC::length > 0)>::type collect_points(std::vector<IntVec>& v) {
    v.push_back(PC::Point::int_vec());
    collect_points<typename PC::Collection>(v);
  }
  template <class PC>
  static typename std::enable_if<(PC::length == 0)>::type collect_points(std::vector<IntVec>&) {}

  CoefCollection coefs_;
};

}  // namespace SpatialOps
#endif
