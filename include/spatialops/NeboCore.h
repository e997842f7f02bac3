// Nebo expression engine for sm_103a (drop-in for the expression templates of
// spatialops/NeboRhs.h, NeboOperators.h, NeboCond.h, NeboMask.h, NeboStencils.h,
// NeboLhs.h and NeboAssignment.h).
//
// Every `lhs <<= expr` builds a tree of host nodes at compile time.  The host nodes answer the
// reference's ghost questions (ghosts_with_bc, ghosts_without_bc, extents, has_bc) with the same
// rules, so the write region is the reference's (calculate_actual_ghost, computed by
// nebo_write_limits in the C ABI).  Each host node then yields a small POD device functor, and
// the whole tree becomes ONE kernel instantiation: nebo_assign_kernel<T, Functor>.  x runs over
// the 32 lanes of a warp (coalesced), y over the 8 warps of a block, and each thread marches a
// chunk of z planes; stencil neighbours are re-read through L1 rather than recomputed from HBM.
//
// Arithmetic.  By default the compiler may contract a*b+c into an FMA (results agree with the
// reference's serial walk to rounding).  With NEBO_EXACT_ARITHMETIC defined, + - * / on
// doubles use round-to-nearest intrinsics, never contracted, so expressions made of them and of
// stencils match the reference's serial walk bit for bit.
#ifndef SpatialOps_NeboCore_h
#define SpatialOps_NeboCore_h

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <limits>
#include <sstream>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include <nebo_gb300.h>
#include <spatialops/NeboFixMath.h>
#include <spatialops/structured/FVStaggeredFieldTypes.h>
#include <spatialops/structured/GhostData.h>
#include <spatialops/structured/IndexTriplet.h>
#include <spatialops/structured/SpatialMask.h>

namespace SpatialOps {

// ============================================================================ wrappers
// Type carriers of the reference's API: an expression together with the field type it produces.
template <typename Operand, typename FieldType>
struct NeboExpression {
  typedef FieldType field_type;
  typedef Operand Expression;
  explicit NeboExpression(const Operand& e) : expr_(e) {}
  const Operand& expr() const { return expr_; }

 private:
  Operand expr_;
};

template <typename Operand, typename FieldType>
struct NeboBooleanExpression {
  typedef FieldType field_type;
  typedef Operand Expression;
  explicit NeboBooleanExpression(const Operand& e) : expr_(e) {}
  const Operand& expr() const { return expr_; }

 private:
  Operand expr_;
};

// Expressions whose value is one number held on the device (SingleValue fields combined with
// each other and with scalars; spatialops/NeboBasic.h:211-275).  Where they meet a field they
// broadcast, like a scalar.
template <typename Operand, typename T>
struct NeboSingleValueExpression {
  typedef SpatialField<SingleValue, T> field_type;
  typedef Operand Expression;
  explicit NeboSingleValueExpression(const Operand& e) : expr_(e) {}
  const Operand& expr() const { return expr_; }

 private:
  Operand expr_;
};

template <typename Operand, typename T>
struct NeboBooleanSingleValueExpression {
  typedef SpatialField<SingleValue, T> field_type;
  typedef Operand Expression;
  explicit NeboBooleanSingleValueExpression(const Operand& e) : expr_(e) {}
  const Operand& expr() const { return expr_; }

 private:
  Operand expr_;
};

struct NeboNil {
  enum { length = 0 };
};

namespace nebo_detail {

// ============================================================================ arithmetic
template <typename T>
struct Arith {
  static __device__ __forceinline__ T add(T a, T b) { return a + b; }
  static __device__ __forceinline__ T sub(T a, T b) { return a - b; }
  static __device__ __forceinline__ T mul(T a, T b) { return a * b; }
  static __device__ __forceinline__ T div(T a, T b) { return a / b; }
};
#ifdef NEBO_EXACT_ARITHMETIC
template <>
struct Arith<double> {
  static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
  static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
  static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
  static __device__ __forceinline__ double div(double a, double b) { return __ddiv_rn(a, b); }
};
template <>
struct Arith<float> {
  static __device__ __forceinline__ float add(float a, float b) { return __fadd_rn(a, b); }
  static __device__ __forceinline__ float sub(float a, float b) { return __fsub_rn(a, b); }
  static __device__ __forceinline__ float mul(float a, float b) { return __fmul_rn(a, b); }
  static __device__ __forceinline__ float div(float a, float b) { return __fdiv_rn(a, b); }
};
#endif

// binary value operators (NeboOperators.h: SumOp :32, DiffOp :774, ProdOp :1516, DivOp :2258,
// PowFcn :4397, MaxFcn :13088, MinFcn :13843)
struct OpAdd { template <class T> static __device__ __forceinline__ T apply(T a, T b) { return Arith<T>::add(a, b); } };
struct OpSub { template <class T> static __device__ __forceinline__ T apply(T a, T b) { return Arith<T>::sub(a, b); } };
struct OpMul { template <class T> static __device__ __forceinline__ T apply(T a, T b) { return Arith<T>::mul(a, b); } };
struct OpDiv { template <class T> static __device__ __forceinline__ T apply(T a, T b) { return Arith<T>::div(a, b); } };
struct OpPow { template <class T> static __device__ __forceinline__ T apply(T a, T b) { return pow(a, b); } };
struct OpMax { template <class T> static __device__ __forceinline__ T apply(T a, T b) { return (a > b) ? a : b; } };
struct OpMin { template <class T> static __device__ __forceinline__ T apply(T a, T b) { return (a < b) ? a : b; } };

// unary functions (NeboOperators.h: Sin :3000 ... Cube :6764)
#define NEBO_UNARY_FN(NAME, EXPR) \
  struct NAME { template <class T> static __device__ __forceinline__ T apply(T a) { return EXPR; } };
NEBO_UNARY_FN(FnNeg, -a)
NEBO_UNARY_FN(FnCos, cos(a))
NEBO_UNARY_FN(FnTan, tan(a))
// exp and sin of doubles: the fixed-point forms of NeboFixMath.h (within 0.52 and 1.1 ulp, off
// the FP64 pipe); NEBO_CUDA_LIBM selects CUDA's functions instead.
struct FnExp {
  template <class T> static __device__ __forceinline__ T apply(T a) { return exp(a); }
#ifndef NEBO_CUDA_LIBM
  static __device__ __forceinline__ double apply(double a) { return nebo::fixmath::exp_i(a); }
#endif
};
struct FnSin {
  template <class T> static __device__ __forceinline__ T apply(T a) { return sin(a); }
#ifndef NEBO_CUDA_LIBM
  static __device__ __forceinline__ double apply(double a) { return nebo::fixmath::sin_i(a); }
#endif
};
NEBO_UNARY_FN(FnTanh, tanh(a))
NEBO_UNARY_FN(FnAbs, fabs(a))
NEBO_UNARY_FN(FnSqrt, sqrt(a))
NEBO_UNARY_FN(FnLog, log(a))
NEBO_UNARY_FN(FnLog10, log10(a))
NEBO_UNARY_FN(FnErf, erf(a))
NEBO_UNARY_FN(FnErfc, erfc(a))
NEBO_UNARY_FN(FnInvErf, erfinv(a))
NEBO_UNARY_FN(FnInvErfc, erfcinv(a))
NEBO_UNARY_FN(FnSquare, Arith<T>::mul(a, a))
NEBO_UNARY_FN(FnCube, Arith<T>::mul(Arith<T>::mul(a, a), a))
#undef NEBO_UNARY_FN

// comparisons and logic (NeboOperators.h: == :6969 ... Not :12923)
struct CmpEq { template <class T> static __device__ __forceinline__ bool apply(T a, T b) { return a == b; } };
struct CmpNe { template <class T> static __device__ __forceinline__ bool apply(T a, T b) { return a != b; } };
struct CmpLt { template <class T> static __device__ __forceinline__ bool apply(T a, T b) { return a < b; } };
struct CmpLe { template <class T> static __device__ __forceinline__ bool apply(T a, T b) { return a <= b; } };
struct CmpGt { template <class T> static __device__ __forceinline__ bool apply(T a, T b) { return a > b; } };
struct CmpGe { template <class T> static __device__ __forceinline__ bool apply(T a, T b) { return a >= b; } };
struct LogAnd { static __device__ __forceinline__ bool apply(bool a, bool b) { return a && b; } };
struct LogOr { static __device__ __forceinline__ bool apply(bool a, bool b) { return a || b; } };

// ============================================================================ device functors
// Every device functor evaluates at interior-relative (x,y,z) (eval for values, check for
// booleans) and has two hooks for the tiled lowering (NeboTiled.h):
//   rebase(x0,y0,z0)   moves its leaves' origin to (x0,y0,z0), so that later coordinates are
//                      relative to a tile;
//   fill<H>(tx,ty,tz)  fills the shared-memory buffers of round H below it (tx,ty,tz: how much
//                      a partial tile is short of the full tile on each axis).
#define NEBO_ONE_CHILD(A)                                                                       \
  __device__ __forceinline__ void rebase(int x0, int y0, int z0) { A.rebase(x0, y0, z0); }      \
  template <int Round_>                                                                         \
  __device__ __forceinline__ void fill(int tx, int ty, int tz) const {                          \
    A.template fill<Round_>(tx, ty, tz);                                                        \
  }
#define NEBO_TWO_CHILDREN(A, B)                                                                 \
  __device__ __forceinline__ void rebase(int x0, int y0, int z0) {                              \
    A.rebase(x0, y0, z0);                                                                       \
    B.rebase(x0, y0, z0);                                                                       \
  }                                                                                             \
  template <int Round_>                                                                         \
  __device__ __forceinline__ void fill(int tx, int ty, int tz) const {                          \
    A.template fill<Round_>(tx, ty, tz);                                                        \
    B.template fill<Round_>(tx, ty, tz);                                                        \
  }

template <typename T>
struct DScalar {
  T v;
  __device__ __forceinline__ T eval(int, int, int) const { return v; }
  __device__ __forceinline__ void rebase(int, int, int) {}
  template <int H> __device__ __forceinline__ void fill(int, int, int) const {}
};

// a SingleValue field: the one value, wherever it is read (NeboRhs.h:330-482)
template <typename T>
struct DSingleValue {
  const T* p;
  __device__ __forceinline__ T eval(int, int, int) const { return __ldg(p); }
  __device__ __forceinline__ void rebase(int, int, int) {}
  template <int H> __device__ __forceinline__ void fill(int, int, int) const {}
};

// a boolean scalar (a cond clause tested with true or false)
struct DBoolScalar {
  bool b;
  __device__ __forceinline__ bool check(int, int, int) const { return b; }
  __device__ __forceinline__ void rebase(int, int, int) {}
  template <int H> __device__ __forceinline__ void fill(int, int, int) const {}
};

template <typename T>
struct DField {
  const T* p;  // interior-relative (0,0,0)
  int sy;
  long sz;
  __device__ __forceinline__ T eval(int x, int y, int z) const { return __ldg(p + ((long)x + (long)sy * y + sz * z)); }
  __device__ __forceinline__ void rebase(int x0, int y0, int z0) { p += (long)x0 + (long)sy * y0 + sz * z0; }
  template <int H> __device__ __forceinline__ void fill(int, int, int) const {}
};

struct DMask {
  const uint32_t* w;
  long origin;  // flat index of interior (0,0,0) in the window
  int sy;
  long sz;
  __device__ __forceinline__ bool check(int x, int y, int z) const {
    const long f = origin + (long)x + (long)sy * y + sz * z;
    return (__ldg(w + (f >> 5)) >> (f & 31)) & 1u;
  }
  __device__ __forceinline__ void rebase(int x0, int y0, int z0) { origin += (long)x0 + (long)sy * y0 + sz * z0; }
  template <int H> __device__ __forceinline__ void fill(int, int, int) const {}
};

template <class Op, typename T, class A, class B>
struct DBin {
  A a;
  B b;
  __device__ __forceinline__ T eval(int x, int y, int z) const { return Op::apply(a.eval(x, y, z), b.eval(x, y, z)); }
  NEBO_TWO_CHILDREN(a, b)
};

template <class Fn, typename T, class A>
struct DUn {
  A a;
  __device__ __forceinline__ T eval(int x, int y, int z) const { return Fn::apply(a.eval(x, y, z)); }
  NEBO_ONE_CHILD(a)
};

template <typename T, class A>
struct DPowInt {
  A a;
  int e;
  __device__ __forceinline__ T eval(int x, int y, int z) const { return pow(a.eval(x, y, z), (T)e); }
  NEBO_ONE_CHILD(a)
};

template <class Op, class A, class B>
struct DCmp {
  A a;
  B b;
  __device__ __forceinline__ bool check(int x, int y, int z) const { return Op::apply(a.eval(x, y, z), b.eval(x, y, z)); }
  NEBO_TWO_CHILDREN(a, b)
};

template <class Op, class A, class B>
struct DLogic {
  A a;
  B b;
  __device__ __forceinline__ bool check(int x, int y, int z) const { return Op::apply(a.check(x, y, z), b.check(x, y, z)); }
  NEBO_TWO_CHILDREN(a, b)
};

template <class A>
struct DNot {
  A a;
  __device__ __forceinline__ bool check(int x, int y, int z) const { return !a.check(x, y, z); }
  NEBO_ONE_CHILD(a)
};

// cond: first true clause wins (NeboCond.h:408-413)
template <typename T, class Test, class Val, class Rest>
struct DCond {
  Test t;
  Val v;
  Rest r;
  __device__ __forceinline__ T eval(int x, int y, int z) const { return t.check(x, y, z) ? v.eval(x, y, z) : r.eval(x, y, z); }
  __device__ __forceinline__ void rebase(int x0, int y0, int z0) {
    t.rebase(x0, y0, z0);
    v.rebase(x0, y0, z0);
    r.rebase(x0, y0, z0);
  }
  template <int H> __device__ __forceinline__ void fill(int tx, int ty, int tz) const {
    t.template fill<H>(tx, ty, tz);
    v.template fill<H>(tx, ty, tz);
    r.template fill<H>(tx, ty, tz);
  }
};

}  // namespace nebo_detail

// ============================================================================ stencil points
// NeboStencilPointCollection<Point, Collection>: the first listed point is the innermost type
// (NEBO_FIRST_* creates it, NEBO_ADD_* wraps), and the stencil sum runs in listed order
// (NeboStencils.h:407-448).  Ghost rule: arg ghosts + min over points of
// additive_reductive_point_to_ghost (NeboStencils.h:222-239).
template <typename PointType, typename CollectionType>
struct NeboStencilPointCollection;
namespace nebo_detail {
// Last (the innermost, first-listed point) and AllButLast of a point collection
// (NeboStencils.h:197-278).
template <class P, class C>
struct PtsTail {
  typedef typename C::Last Last;
  typedef NeboStencilPointCollection<P, typename C::AllButLast> AllButLast;
};
template <class P>
struct PtsTail<P, NeboNil> {
  typedef P Last;
  typedef NeboNil AllButLast;
};
}  // namespace nebo_detail

template <typename PointType, typename CollectionType>
struct NeboStencilPointCollection {
  typedef PointType Point;
  typedef CollectionType Collection;
  typedef NeboStencilPointCollection<Point, Collection> MyType;
  typedef Point First;
  typedef Collection AllButFirst;
  typedef typename nebo_detail::PtsTail<Point, Collection>::Last Last;
  typedef typename nebo_detail::PtsTail<Point, Collection>::AllButLast AllButLast;
  enum { length = 1 + Collection::length };
  // the edgeless stencil's ghost rule: this point additive only, the rest as in possible_ghosts
  static GhostData possible_additive_ghosts() {
    return Collection::length == 0 ? additive_point_to_ghost(Point::int_vec())
                                   : min(additive_point_to_ghost(Point::int_vec()), rest_ghosts());
  }
  static GhostData possible_additive_ghosts(const GhostData& g) { return g + possible_additive_ghosts(); }
  template <typename NewPoint>
  struct AddPoint {
    typedef NeboStencilPointCollection<NewPoint, MyType> Result;
  };
  static GhostData possible_ghosts() {
    return Collection::length == 0 ? additive_reductive_point_to_ghost(Point::int_vec())
                                   : min(additive_reductive_point_to_ghost(Point::int_vec()), rest_ghosts());
  }
  static GhostData possible_ghosts(const GhostData& g) { return g + possible_ghosts(); }

 private:
  template <class C = Collection>
  static typename std::enable_if<(C::length > 0), GhostData>::type rest_ghosts() { return C::possible_ghosts(); }
  template <class C = Collection>
  static typename std::enable_if<(C::length == 0), GhostData>::type rest_ghosts() { return GhostData(GHOST_MAX); }
};

#define NEBO_FIRST_POINT_WO_TN(POINT) NeboStencilPointCollection<POINT, NeboNil>
#define NEBO_FIRST_POINT(POINT) typename NEBO_FIRST_POINT_WO_TN(POINT)
#define NEBO_ADD_POINT(POINT) template AddPoint<POINT>::Result
#define NEBO_FIRST_IJK(X, Y, Z) NeboStencilPointCollection<IndexTriplet<X, Y, Z>, NeboNil>
#define NEBO_ADD_IJK(X, Y, Z) AddPoint<IndexTriplet<X, Y, Z> >::Result

// Stencil coefficients in listed order (NeboStencils.h:29-195).
template <int Length>
struct NeboStencilCoefCollection {
  double c[Length];
  NeboStencilCoefCollection() {
    for (int i = 0; i < Length; ++i) c[i] = 0.0;
  }
  NeboStencilCoefCollection(const NeboStencilCoefCollection<Length - 1>& o, double last) {
    for (int i = 0; i < Length - 1; ++i) c[i] = o.c[i];
    c[Length - 1] = last;
  }
  NeboStencilCoefCollection<Length + 1> operator()(double next) const { return NeboStencilCoefCollection<Length + 1>(*this, next); }
  double coef() const { return c[Length - 1]; }
  NeboStencilCoefCollection<Length - 1> others() const {
    NeboStencilCoefCollection<Length - 1> o;
    for (int i = 0; i < Length - 1; ++i) o.c[i] = c[i];
    return o;
  }
  double get_coef(int index) const {
    if (index < 0) throw std::runtime_error("Nebo error in Nebo Stencil Coefficient Collection:\ngiven negative value for coefficient index");
    if (index >= Length) throw std::runtime_error("Nebo error in Nebo Stencil Coefficient Collection:\ntrying to access a coefficient that does not exist");
    return c[index];
  }
  double last() const { return c[0]; }
  // every coefficient but the first listed one
  NeboStencilCoefCollection<Length - 1> all_but_last() const {
    NeboStencilCoefCollection<Length - 1> o;
    for (int i = 0; i < Length - 1; ++i) o.c[i] = c[i + 1];
    return o;
  }
};

template <>
struct NeboStencilCoefCollection<1> {
  double c[1];
  NeboStencilCoefCollection() { c[0] = 0.0; }
  explicit NeboStencilCoefCollection(double v) { c[0] = v; }
  NeboStencilCoefCollection(NeboNil, double v) { c[0] = v; }
  NeboStencilCoefCollection<2> operator()(double next) const;
  double coef() const { return c[0]; }
  double get_coef(int index) const {
    if (index < 0) throw std::runtime_error("Nebo error in Nebo Stencil Coefficient Collection:\ngiven negative value for coefficient index");
    if (index > 1) throw std::runtime_error("Nebo error in Nebo Stencil Coefficient Collection:\ntrying to access a coefficient that does not exist");
    return c[0];
  }
  double last() const { return c[0]; }
};
inline NeboStencilCoefCollection<2> NeboStencilCoefCollection<1>::operator()(double next) const {
  return NeboStencilCoefCollection<2>(*this, next);
}

inline NeboStencilCoefCollection<1> build_coef_collection(double c) { return NeboStencilCoefCollection<1>(c); }
inline NeboStencilCoefCollection<2> build_two_point_coef_collection(double c1, double c2) {
  return NeboStencilCoefCollection<1>(c1)(c2);
}
inline NeboStencilCoefCollection<3> build_three_point_coef_collection(double c1, double c2, double c3) {
  return NeboStencilCoefCollection<1>(c1)(c2)(c3);
}
inline NeboStencilCoefCollection<4> build_four_point_coef_collection(double c1, double c2, double c3, double c4) {
  return NeboStencilCoefCollection<1>(c1)(c2)(c3)(c4);
}
inline NeboStencilCoefCollection<5> build_five_point_coef_collection(double c1, double c2, double c3, double c4,
                                                                     double c5) {
  return NeboStencilCoefCollection<1>(c1)(c2)(c3)(c4)(c5);
}

namespace nebo_detail {

// Device stencil fold in listed order: ((a(p0)*c0 + a(p1)*c1) + a(p2)*c2) + ...
template <class Coll>
struct StencilFold;
// v with the sign bit of s (a point of a signed sum: s = +-1)
__device__ __forceinline__ double sign_of(double v, double s) {
  return __longlong_as_double(__double_as_longlong(v) ^ (__double_as_longlong(s) & (long long)0x8000000000000000ULL));
}
__device__ __forceinline__ float sign_of(float v, double s) {
  return __int_as_float(__float_as_int(v) ^ (int)((unsigned)((unsigned long long)__double_as_longlong(s) >> 32) & 0x80000000u));
}
template <class P>
struct StencilFold<NeboStencilPointCollection<P, NeboNil>> {
  template <typename T, class A>
  static __device__ __forceinline__ T weighted(const A& a, const double* c, int x, int y, int z) {
    return Arith<T>::mul(a.eval(x + P::X, y + P::Y, z + P::Z), (T)c[0]);
  }
  template <typename T, class A>
  static __device__ __forceinline__ T signed_sum(const A& a, const double* c, int x, int y, int z) {
    return sign_of(a.eval(x + P::X, y + P::Y, z + P::Z), c[0]);
  }
  template <typename T, class A>
  static __device__ __forceinline__ T sum(const A& a, int x, int y, int z) {
    return a.eval(x + P::X, y + P::Y, z + P::Z);
  }
};
template <class P, class R>
struct StencilFold<NeboStencilPointCollection<P, R>> {
  template <typename T, class A>
  static __device__ __forceinline__ T weighted(const A& a, const double* c, int x, int y, int z) {
    return Arith<T>::add(StencilFold<R>::template weighted<T>(a, c, x, y, z),
                         Arith<T>::mul(a.eval(x + P::X, y + P::Y, z + P::Z), (T)c[R::length]));
  }
  template <typename T, class A>
  static __device__ __forceinline__ T sum(const A& a, int x, int y, int z) {
    return Arith<T>::add(StencilFold<R>::template sum<T>(a, x, y, z), a.eval(x + P::X, y + P::Y, z + P::Z));
  }
  template <typename T, class A>
  static __device__ __forceinline__ T signed_sum(const A& a, const double* c, int x, int y, int z) {
    return Arith<T>::add(StencilFold<R>::template signed_sum<T>(a, c, x, y, z),
                         sign_of(a.eval(x + P::X, y + P::Y, z + P::Z), c[R::length]));
  }
};

template <typename T, class Pts, class A>
struct DStencil {
  A a;
  double c[Pts::length];
  __device__ __forceinline__ T eval(int x, int y, int z) const { return StencilFold<Pts>::template weighted<T>(a, c, x, y, z); }
  NEBO_ONE_CHILD(a)
};

template <typename T, class Pts, class A>
struct DSumStencil {
  A a;
  __device__ __forceinline__ T eval(int x, int y, int z) const { return StencilFold<Pts>::template sum<T>(a, x, y, z); }
  NEBO_ONE_CHILD(a)
};

// ============================================================================ stream order
// The stream of the kernel being lowered.  A launching call (assign, masked, a reduction, a BC
// builder) names it for the duration of its lowering; every field leaf read on another stream
// then makes it wait for that stream's work, so a kernel never reads a field that an earlier
// call on another stream is still writing.
inline nebo_stream_t& launch_stream() {
  static thread_local nebo_stream_t s = nullptr;
  return s;
}
struct LaunchStreamScope {
  nebo_stream_t saved;
  explicit LaunchStreamScope(nebo_stream_t s) : saved(launch_stream()) { launch_stream() = s; }
  ~LaunchStreamScope() { launch_stream() = saved; }
};
inline void order_read(nebo_stream_t field_stream) {
  const nebo_stream_t s = launch_stream();
  if (field_stream == s) return;
  cudaEvent_t e;
  cudaError_t rc = cudaEventCreateWithFlags(&e, cudaEventDisableTiming);
  if (rc == cudaSuccess) {
    rc = cudaEventRecord(e, (cudaStream_t)field_stream);
    if (rc == cudaSuccess) rc = cudaStreamWaitEvent((cudaStream_t)s, e, 0);
    cudaEventDestroy(e);
  }
  if (rc != cudaSuccess) {
    cudaGetLastError();
    throw std::runtime_error(std::string("Nebo error in Nebo Assignment (stream order):\n") + cudaGetErrorString(rc));
  }
}

// ============================================================================ host nodes
// Ghost-analysis interface of every node (NeboRhs.h / NeboOperators.h "Initial" mode).
template <typename T>
struct ScalarNode {
  typedef T value_type;
  T v;
  explicit ScalarNode(T v_) : v(v_) {}
  GhostData ghosts_with_bc() const { return GhostData(GHOST_MAX); }
  GhostData ghosts_without_bc() const { return GhostData(GHOST_MAX); }
  bool has_extents() const { return false; }
  IntVec extents() const { return IntVec(0, 0, 0); }
  IntVec has_bc() const { return IntVec(0, 0, 0); }
  void prepare() const {}
  DScalar<T> device() const { return DScalar<T>{v}; }
};

// A SingleValue field leaf: no ghost limit (like a scalar), its value read on the device.
template <typename F>
struct SingleValueNode {
  typedef typename F::value_type value_type;
  F f;
  explicit SingleValueNode(const F& f_) : f(f_) {}
  GhostData ghosts_with_bc() const { return GhostData(GHOST_MAX); }
  GhostData ghosts_without_bc() const { return GhostData(GHOST_MAX); }
  bool has_extents() const { return false; }
  IntVec extents() const { return IntVec(0, 0, 0); }
  IntVec has_bc() const { return IntVec(0, 0, 0); }
  void prepare() const { f.device_values_for_read(); }
  DSingleValue<value_type> device() const {
    const value_type* base = f.device_values_for_read();
    order_read(f.get_stream());
    return DSingleValue<value_type>{base + f.interior_origin()};
  }
};

struct BoolScalarNode {
  typedef bool value_type;
  bool b;
  explicit BoolScalarNode(bool b_) : b(b_) {}
  GhostData ghosts_with_bc() const { return GhostData(GHOST_MAX); }
  GhostData ghosts_without_bc() const { return GhostData(GHOST_MAX); }
  bool has_extents() const { return false; }
  IntVec extents() const { return IntVec(0, 0, 0); }
  IntVec has_bc() const { return IntVec(0, 0, 0); }
  void prepare() const {}
  DBoolScalar device() const { return DBoolScalar{b}; }
};

template <typename F>
struct FieldNode {
  typedef typename F::value_type value_type;
  F f;
  explicit FieldNode(const F& f_) : f(f_) {}
  GhostData ghosts_with_bc() const { return f.get_valid_ghost_data() + point_to_ghost(f.boundary_info().has_extra()); }
  GhostData ghosts_without_bc() const { return f.get_valid_ghost_data(); }
  bool has_extents() const { return true; }
  IntVec extents() const { return f.interior_extent(); }
  IntVec has_bc() const { return f.boundary_info().has_bc(); }
  void prepare() const { f.device_values_for_read(); }
  DField<value_type> device() const {
    const value_type* base = f.device_values_for_read();
    order_read(f.get_stream());
    return DField<value_type>{base + f.interior_origin(), (int)f.window_with_ghost().glob_dim(0),
                              (long)f.window_with_ghost().glob_dim(0) * (long)f.window_with_ghost().glob_dim(1)};
  }
};

template <typename F>
struct MaskNode {
  typedef bool value_type;
  SpatialMask<F> m;
  explicit MaskNode(const SpatialMask<F>& m_) : m(m_) {}
  GhostData ghosts_with_bc() const { return m.get_valid_ghost_data() + point_to_ghost(m.boundary_info().has_extra()); }
  GhostData ghosts_without_bc() const { return m.get_valid_ghost_data(); }
  bool has_extents() const { return true; }
  IntVec extents() const { return m.interior_extent(); }
  IntVec has_bc() const { return m.boundary_info().has_bc(); }
  void prepare() const {}
  DMask device() const {
    return DMask{m.mask_values(GPU_INDEX), m.interior_origin(), (int)m.window_with_ghost().glob_dim(0),
                 (long)m.window_with_ghost().glob_dim(0) * (long)m.window_with_ghost().glob_dim(1)};
  }
};

// A mask read at a shifted point (NeboMaskShift, NeboStencils.h:1048-1213): true at (x,y,z) when
// the mask holds (x,y,z) + P.  Ghosts: the mask's plus additive_reductive_point_to_ghost(P).
template <class P>
struct DMaskShift {
  DMask m;
  __device__ __forceinline__ bool check(int x, int y, int z) const { return m.check(x + P::X, y + P::Y, z + P::Z); }
  NEBO_ONE_CHILD(m)
};
template <class P, class F>
struct MaskShiftNode {
  typedef bool value_type;
  MaskNode<F> m;
  explicit MaskShiftNode(const SpatialMask<F>& mk) : m(mk) {}
  GhostData ghosts_with_bc() const { return m.ghosts_with_bc() + additive_reductive_point_to_ghost(P::int_vec()); }
  GhostData ghosts_without_bc() const {
    return m.ghosts_without_bc() + additive_reductive_point_to_ghost(P::int_vec());
  }
  bool has_extents() const { return m.has_extents(); }
  IntVec extents() const { return m.extents(); }
  IntVec has_bc() const { return m.has_bc(); }
  void prepare() const { m.prepare(); }
  DMaskShift<P> device() const { return DMaskShift<P>{m.device()}; }
};

// Nodes with children: ghosts are the min over children; extents and BC flags come from the
// first child that has extents (NeboOperators.h:56-100).
template <class A, class B>
struct PairBase {
  A a;
  B b;
  PairBase(const A& a_, const B& b_) : a(a_), b(b_) {}
  GhostData ghosts_with_bc() const { return min(a.ghosts_with_bc(), b.ghosts_with_bc()); }
  GhostData ghosts_without_bc() const { return min(a.ghosts_without_bc(), b.ghosts_without_bc()); }
  bool has_extents() const { return a.has_extents() || b.has_extents(); }
  IntVec extents() const { return a.has_extents() ? a.extents() : b.extents(); }
  IntVec has_bc() const { return a.has_extents() ? a.has_bc() : b.has_bc(); }
  void prepare() const { a.prepare(); b.prepare(); }
};

template <class Op, class A, class B>
struct BinNode : PairBase<A, B> {
  typedef typename A::value_type value_type;
  BinNode(const A& a_, const B& b_) : PairBase<A, B>(a_, b_) {}
  auto device() const -> DBin<Op, value_type, decltype(this->a.device()), decltype(this->b.device())> {
    return {this->a.device(), this->b.device()};
  }
};

template <class Op, class A, class B>
struct CmpNode : PairBase<A, B> {
  typedef bool value_type;
  CmpNode(const A& a_, const B& b_) : PairBase<A, B>(a_, b_) {}
  auto device() const -> DCmp<Op, decltype(this->a.device()), decltype(this->b.device())> {
    return {this->a.device(), this->b.device()};
  }
};

template <class Op, class A, class B>
struct LogicNode : PairBase<A, B> {
  typedef bool value_type;
  LogicNode(const A& a_, const B& b_) : PairBase<A, B>(a_, b_) {}
  auto device() const -> DLogic<Op, decltype(this->a.device()), decltype(this->b.device())> {
    return {this->a.device(), this->b.device()};
  }
};

template <class A>
struct UnaryBase {
  A a;
  explicit UnaryBase(const A& a_) : a(a_) {}
  GhostData ghosts_with_bc() const { return a.ghosts_with_bc(); }
  GhostData ghosts_without_bc() const { return a.ghosts_without_bc(); }
  bool has_extents() const { return a.has_extents(); }
  IntVec extents() const { return a.extents(); }
  IntVec has_bc() const { return a.has_bc(); }
  void prepare() const { a.prepare(); }
};

template <class Fn, class A>
struct UnNode : UnaryBase<A> {
  typedef typename A::value_type value_type;
  explicit UnNode(const A& a_) : UnaryBase<A>(a_) {}
  auto device() const -> DUn<Fn, value_type, decltype(this->a.device())> { return {this->a.device()}; }
};

template <class A>
struct PowIntNode : UnaryBase<A> {
  typedef typename A::value_type value_type;
  int e;
  PowIntNode(const A& a_, int e_) : UnaryBase<A>(a_), e(e_) {}
  auto device() const -> DPowInt<value_type, decltype(this->a.device())> { return {this->a.device(), e}; }
};

template <class A>
struct NotNode : UnaryBase<A> {
  typedef bool value_type;
  explicit NotNode(const A& a_) : UnaryBase<A>(a_) {}
  auto device() const -> DNot<decltype(this->a.device())> { return {this->a.device()}; }
};

// cond clause chain: ghosts min over test, value and the rest (NeboCond.h:86-92, 284-290)
template <typename T, class Test, class Val, class Rest>
struct CondNode {
  typedef T value_type;
  Test t;
  Val v;
  Rest r;
  CondNode(const Test& t_, const Val& v_, const Rest& r_) : t(t_), v(v_), r(r_) {}
  GhostData ghosts_with_bc() const { return min(min(t.ghosts_with_bc(), v.ghosts_with_bc()), r.ghosts_with_bc()); }
  GhostData ghosts_without_bc() const {
    return min(min(t.ghosts_without_bc(), v.ghosts_without_bc()), r.ghosts_without_bc());
  }
  bool has_extents() const { return t.has_extents() || v.has_extents() || r.has_extents(); }
  IntVec extents() const { return t.has_extents() ? t.extents() : (v.has_extents() ? v.extents() : r.extents()); }
  IntVec has_bc() const { return t.has_extents() ? t.has_bc() : (v.has_extents() ? v.has_bc() : r.has_bc()); }
  void prepare() const { t.prepare(); v.prepare(); r.prepare(); }
  auto device() const -> DCond<T, decltype(t.device()), decltype(v.device()), decltype(r.device())> {
    return {t.device(), v.device(), r.device()};
  }
};

template <typename T, class Pts, class A>
struct StencilNode {
  typedef T value_type;
  A a;
  NeboStencilCoefCollection<Pts::length> coefs;
  StencilNode(const A& a_, const NeboStencilCoefCollection<Pts::length>& c) : a(a_), coefs(c) {}
  GhostData ghosts_with_bc() const { return Pts::possible_ghosts(a.ghosts_with_bc()); }
  GhostData ghosts_without_bc() const { return Pts::possible_ghosts(a.ghosts_without_bc()); }
  bool has_extents() const { return a.has_extents(); }
  IntVec extents() const { return a.extents(); }
  IntVec has_bc() const { return a.has_bc(); }
  void prepare() const { a.prepare(); }
  auto device() const -> DStencil<T, Pts, decltype(a.device())> {
    DStencil<T, Pts, decltype(a.device())> d;
    d.a = a.device();
    for (int i = 0; i < Pts::length; ++i) d.c[i] = coefs.c[i];
    return d;
  }
};

// A stencil without the edge (reductive) part of the ghost rule (NeboEdgelessStencil,
// NeboStencils.h:526-824): the same weighted sum, ghosts from possible_additive_ghosts.
template <typename T, class Pts, class A>
struct EdgelessStencilNode : StencilNode<T, Pts, A> {
  EdgelessStencilNode(const A& a_, const NeboStencilCoefCollection<Pts::length>& c) : StencilNode<T, Pts, A>(a_, c) {}
  GhostData ghosts_with_bc() const { return Pts::possible_additive_ghosts(this->a.ghosts_with_bc()); }
  GhostData ghosts_without_bc() const { return Pts::possible_additive_ghosts(this->a.ghosts_without_bc()); }
};

template <typename T, class Pts, class A>
struct SumStencilNode {
  typedef T value_type;
  A a;
  explicit SumStencilNode(const A& a_) : a(a_) {}
  GhostData ghosts_with_bc() const { return Pts::possible_ghosts(a.ghosts_with_bc()); }
  GhostData ghosts_without_bc() const { return Pts::possible_ghosts(a.ghosts_without_bc()); }
  bool has_extents() const { return a.has_extents(); }
  IntVec extents() const { return a.extents(); }
  IntVec has_bc() const { return a.has_bc(); }
  void prepare() const { a.prepare(); }
  auto device() const -> DSumStencil<T, Pts, decltype(a.device())> { return {a.device()}; }
};

}  // namespace nebo_detail
}  // namespace SpatialOps

#endif
