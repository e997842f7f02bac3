// Constant factors of a `<<=` expression carried on the host (builds that allow reassociation:
// not NEBO_EXACT_ARITHMETIC, not NEBO_UNTILED).
//
// The operators' 2-point stencils have coefficients equal up to sign: Interp {1/2, 1/2},
// Gradient and Divergence {-1/dx, 1/dx}, the 2nd-order FD {-1/2dx, 1/2dx}
// (spatialops/structured/stencil/StencilBuilder.cpp:52-220).  Evaluated as written each costs a
// multiply and a fused multiply-add; as s * (a[p0] +- a[p1]) it costs one add, with the factor s
// carried upward: a product's factor is the product of its operands' factors, a quotient's their
// quotient, a product with a scalar takes the scalar into the factor; a sum of operands without
// factors stays a plain sum, one with a factor s enters as s * x in one FMA, and two with factors
// become fma(s_b / s_a, b', a') with the factor s_a.  Factors are applied where a value is needed (a
// function's argument, a comparison, a cond branch, a stencil of 3 or more points, which takes
// its argument's factor into its weights) and at the root.  The heat expression
//   T + dt * (DivX(InterpX(lambda) * GradX(T)) + DivY(...) + DivZ(...))
// then costs 15 FP64 operations per cell instead of 24: per face an add for the interpolant,
// one for the gradient and the product, per divergence an add, two adds across the axes and one
// FMA with dt / (2 dx^2) folded in.  The values differ from the expression as written by
// rounding only (distributivity, reassociation).
//
// The shape of the factored functor is fixed at compile time: every 2-point weighted stencil is
// taken to be a signed pair.  The launch checks that assumption on the host (equal magnitudes,
// and every factor and ratio finite and nonzero) and otherwise runs the expression as written;
// both kernels are compiled only for expressions the factoring changes.  Integer value types are
// never factored.
#ifndef SpatialOps_NeboFactor_h
#define SpatialOps_NeboFactor_h

#include <cmath>
#include <type_traits>

#include <spatialops/NeboTiled.h>

namespace SpatialOps {
namespace nebo_detail {

#if defined(NEBO_EXACT_ARITHMETIC) || defined(NEBO_UNTILED)
constexpr bool kFactor = false;
#else
constexpr bool kFactor = true;
#endif

inline bool clean_factor(double s) { return std::isfinite(s) && s != 0.0; }

#ifdef __CUDACC__
__device__ __forceinline__ double nebo_fma(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float nebo_fma(float a, float b, float c) { return fmaf(a, b, c); }
#endif

// a child's value times a host-side factor
template <typename T, class A>
struct DScaled {
  A a;
  double r;
#ifdef __CUDACC__
  __device__ __forceinline__ T eval(int x, int y, int z) const { return Arith<T>::mul(a.eval(x, y, z), (T)r); }
#endif
  NEBO_ONE_CHILD(a)
};

// a + r * b (OpAdd) or a - r * b (OpSub): one FMA
template <class Op, typename T, class A, class B>
struct DFmaSum {
  A a;
  B b;
  double r;
#ifdef __CUDACC__
  __device__ __forceinline__ T eval(int x, int y, int z) const {
    const T rr = std::is_same<Op, OpSub>::value ? -(T)r : (T)r;
    return nebo_fma(rr, b.eval(x, y, z), a.eval(x, y, z));
  }
#endif
  NEBO_TWO_CHILDREN(a, b)
};

// r * a + b (OpAdd) or r * a - b (OpSub): one FMA
template <class Op, typename T, class A, class B>
struct DFmaSumL {
  A a;
  B b;
  double r;
#ifdef __CUDACC__
  __device__ __forceinline__ T eval(int x, int y, int z) const {
    const T bb = b.eval(x, y, z);
    return nebo_fma((T)r, a.eval(x, y, z), std::is_same<Op, OpSub>::value ? -bb : bb);
  }
#endif
  NEBO_TWO_CHILDREN(a, b)
};

// a 2-point stencil as a signed sum: a(p0) * sign(c0) + a(p1) * sign(c1) (c holds +-1)
template <typename T, class Pts, class A>
struct DSignedStencil {
  A a;
  double c[Pts::length];
#ifdef __CUDACC__
  __device__ __forceinline__ T eval(int x, int y, int z) const {
    return StencilFold<Pts>::template signed_sum<T>(a, c, x, y, z);
  }
#endif
  NEBO_ONE_CHILD(a)
};

// ---------------------------------------------------------------------------- the transform
// Factor<D>: type    the factored functor F (D = s * F)
//            unit    F's factor is 1 whatever the values (no wrapper needed where values are used)
//            make(d, s, ok)  builds F, sets its factor s; ok turns false when a check fails
template <class D, class Enable = void>
struct Factor {  // leaves and anything left as it is: its value is its own
  typedef D type;
  static constexpr bool unit = true;
  static type make(const D& d, double& s, bool&) {
    s = 1.0;
    return d;
  }
};

// F as a value: itself when its factor is always 1, else DScaled by the factor
template <typename T, class FD, bool Unit>
struct AsValue;
template <typename T, class FD>
struct AsValue<T, FD, true> {
  typedef FD type;
  static type make(const FD& f, double) { return f; }
};
template <typename T, class FD>
struct AsValue<T, FD, false> {
  typedef DScaled<T, FD> type;
  static type make(const FD& f, double s) { return type{f, s}; }
};
template <typename T, class D>
struct ValueOf {
  typedef Factor<D> FD;
  typedef AsValue<T, typename FD::type, FD::unit> V;
  typedef typename V::type type;
  static type make(const D& d, bool& ok) {
    double s;
    const typename FD::type f = FD::make(d, s, ok);
    return V::make(f, s);
  }
};

template <typename T>
struct Floating : std::integral_constant<bool, kFactor && std::is_floating_point<T>::value> {};

template <class D>
struct IsScalar : std::false_type {};
template <typename T>
struct IsScalar<DScalar<T>> : std::true_type {};

// a * b: the factors multiply; a scalar operand goes into the factor
template <typename T, class A, class B>
struct Factor<DBin<OpMul, T, A, B>, typename std::enable_if<Floating<T>::value>::type> {
  typedef Factor<A> FA;
  typedef Factor<B> FB;
  static constexpr int kind = IsScalar<A>::value ? 1 : IsScalar<B>::value ? 2 : 0;
  typedef typename std::conditional<
      kind == 1, typename FB::type,
      typename std::conditional<kind == 2, typename FA::type,
                                DBin<OpMul, T, typename FA::type, typename FB::type>>::type>::type type;
  static constexpr bool unit = kind == 0 && FA::unit && FB::unit;
  static type make(const DBin<OpMul, T, A, B>& d, double& s, bool& ok) { return build(d, s, ok, std::integral_constant<int, kind>()); }

 private:
  static type build(const DBin<OpMul, T, A, B>& d, double& s, bool& ok, std::integral_constant<int, 1>) {
    double sb;
    const type f = FB::make(d.b, sb, ok);
    s = (double)d.a.v * sb;
    ok = ok && clean_factor(s);
    return f;
  }
  static type build(const DBin<OpMul, T, A, B>& d, double& s, bool& ok, std::integral_constant<int, 2>) {
    double sa;
    const type f = FA::make(d.a, sa, ok);
    s = sa * (double)d.b.v;
    ok = ok && clean_factor(s);
    return f;
  }
  static type build(const DBin<OpMul, T, A, B>& d, double& s, bool& ok, std::integral_constant<int, 0>) {
    double sa, sb;
    type f{FA::make(d.a, sa, ok), FB::make(d.b, sb, ok)};
    s = sa * sb;
    ok = ok && clean_factor(s);
    return f;
  }
};

// a / b: the factors divide; a scalar divisor goes into the factor
template <typename T, class A, class B>
struct Factor<DBin<OpDiv, T, A, B>, typename std::enable_if<Floating<T>::value>::type> {
  typedef Factor<A> FA;
  typedef Factor<B> FB;
  static constexpr bool by_scalar = IsScalar<B>::value;
  typedef typename std::conditional<by_scalar, typename FA::type,
                                    DBin<OpDiv, T, typename FA::type, typename FB::type>>::type type;
  static constexpr bool unit = !by_scalar && FA::unit && FB::unit;
  static type make(const DBin<OpDiv, T, A, B>& d, double& s, bool& ok) {
    return build(d, s, ok, std::integral_constant<bool, by_scalar>());
  }

 private:
  static type build(const DBin<OpDiv, T, A, B>& d, double& s, bool& ok, std::true_type) {
    double sa;
    const type f = FA::make(d.a, sa, ok);
    s = sa / (double)d.b.v;
    ok = ok && clean_factor(s);
    return f;
  }
  static type build(const DBin<OpDiv, T, A, B>& d, double& s, bool& ok, std::false_type) {
    double sa, sb;
    type f{FA::make(d.a, sa, ok), FB::make(d.b, sb, ok)};
    s = sa / sb;
    ok = ok && clean_factor(s);
    return f;
  }
};

// a +- b.  Operands without factors stay a plain sum (so the compiler still fuses a product
// operand into an FMA); one operand with a factor r enters as r * x in one FMA and the sum keeps
// factor 1; two operands with factors keep the left one's and scale the right one by their ratio.
template <class Op, typename T, class A, class B>
struct Factor<DBin<Op, T, A, B>, typename std::enable_if<Floating<T>::value && (std::is_same<Op, OpAdd>::value ||
                                                                             std::is_same<Op, OpSub>::value)>::type> {
  typedef Factor<A> FA;
  typedef Factor<B> FB;
  typedef typename FA::type TA;
  typedef typename FB::type TB;
  static constexpr int kind = FA::unit && FB::unit ? 0 : FA::unit ? 1 : FB::unit ? 2 : 3;
  typedef typename std::conditional<
      kind == 0, DBin<Op, T, TA, TB>,
      typename std::conditional<kind == 2, DFmaSumL<Op, T, TA, TB>, DFmaSum<Op, T, TA, TB>>::type>::type type;
  static constexpr bool unit = kind != 3;
  static type make(const DBin<Op, T, A, B>& d, double& s, bool& ok) {
    double sa, sb;
    const TA fa = FA::make(d.a, sa, ok);
    const TB fb = FB::make(d.b, sb, ok);
    return build(fa, fb, sa, sb, s, ok, std::integral_constant<int, kind>());
  }

 private:
  static type build(const TA& fa, const TB& fb, double, double, double& s, bool&, std::integral_constant<int, 0>) {
    s = 1.0;
    return type{fa, fb};
  }
  static type build(const TA& fa, const TB& fb, double, double sb, double& s, bool& ok, std::integral_constant<int, 1>) {
    s = 1.0;
    ok = ok && clean_factor(sb);
    return type{fa, fb, sb};
  }
  static type build(const TA& fa, const TB& fb, double sa, double, double& s, bool& ok, std::integral_constant<int, 2>) {
    s = 1.0;
    ok = ok && clean_factor(sa);
    return type{fa, fb, sa};
  }
  static type build(const TA& fa, const TB& fb, double sa, double sb, double& s, bool& ok,
                    std::integral_constant<int, 3>) {
    s = sa;
    const double r = sb / sa;
    ok = ok && clean_factor(sa) && clean_factor(r);
    return type{fa, fb, r};
  }
};

// other binary value operators (pow, max, min): operands as values
template <class Op, typename T, class A, class B>
struct Factor<DBin<Op, T, A, B>,
              typename std::enable_if<Floating<T>::value && !std::is_same<Op, OpAdd>::value &&
                                      !std::is_same<Op, OpSub>::value && !std::is_same<Op, OpMul>::value &&
                                      !std::is_same<Op, OpDiv>::value>::type> {
  typedef ValueOf<T, A> VA;
  typedef ValueOf<T, B> VB;
  typedef DBin<Op, T, typename VA::type, typename VB::type> type;
  static constexpr bool unit = true;
  static type make(const DBin<Op, T, A, B>& d, double& s, bool& ok) {
    s = 1.0;
    return type{VA::make(d.a, ok), VB::make(d.b, ok)};
  }
};

template <class Fn, typename T, class A>
struct Factor<DUn<Fn, T, A>, typename std::enable_if<Floating<T>::value>::type> {
  typedef ValueOf<T, A> VA;
  typedef DUn<Fn, T, typename VA::type> type;
  static constexpr bool unit = true;
  static type make(const DUn<Fn, T, A>& d, double& s, bool& ok) {
    s = 1.0;
    return type{VA::make(d.a, ok)};
  }
};

template <typename T, class A>
struct Factor<DPowInt<T, A>, typename std::enable_if<Floating<T>::value>::type> {
  typedef ValueOf<T, A> VA;
  typedef DPowInt<T, typename VA::type> type;
  static constexpr bool unit = true;
  static type make(const DPowInt<T, A>& d, double& s, bool& ok) {
    s = 1.0;
    return type{VA::make(d.a, ok), d.e};
  }
};

// cond: the tests as written, the branches as values
template <typename T, class Test, class Val, class Rest>
struct Factor<DCond<T, Test, Val, Rest>, typename std::enable_if<Floating<T>::value>::type> {
  typedef ValueOf<T, Val> VV;
  typedef ValueOf<T, Rest> VR;
  typedef DCond<T, Test, typename VV::type, typename VR::type> type;
  static constexpr bool unit = true;
  static type make(const DCond<T, Test, Val, Rest>& d, double& s, bool& ok) {
    s = 1.0;
    return type{d.t, VV::make(d.v, ok), VR::make(d.r, ok)};
  }
};

// a sum stencil: its argument's factor
template <typename T, class Pts, class A>
struct Factor<DSumStencil<T, Pts, A>, typename std::enable_if<Floating<T>::value>::type> {
  typedef Factor<A> FA;
  typedef DSumStencil<T, Pts, typename FA::type> type;
  static constexpr bool unit = FA::unit;
  static type make(const DSumStencil<T, Pts, A>& d, double& s, bool& ok) { return type{FA::make(d.a, s, ok)}; }
};

// a weighted stencil: 2 points as a signed pair with the common magnitude in the factor, more
// points with the argument's factor in the weights
template <typename T, class Pts, class A>
struct Factor<DStencil<T, Pts, A>, typename std::enable_if<Floating<T>::value>::type> {
  typedef Factor<A> FA;
  static constexpr bool pair = Pts::length == 2;
  typedef typename std::conditional<pair, DSignedStencil<T, Pts, typename FA::type>,
                                    DStencil<T, Pts, typename FA::type>>::type type;
  static constexpr bool unit = !pair;
  static type make(const DStencil<T, Pts, A>& d, double& s, bool& ok) {
    double sa;
    type f;
    f.a = FA::make(d.a, sa, ok);
    if (pair) {
      const double m = std::fabs(d.c[0]);
      ok = ok && m == std::fabs(d.c[1]);
      for (int i = 0; i < Pts::length; ++i) f.c[i] = std::signbit(d.c[i]) ? -1.0 : 1.0;
      s = m * sa;
      ok = ok && clean_factor(s);
    } else {
      for (int i = 0; i < Pts::length; ++i) {
        f.c[i] = d.c[i] * sa;
        ok = ok && std::isfinite(f.c[i]);
      }
      s = 1.0;
    }
    return f;
  }
};

// The root: the factored functor as the value the expression assigns.
template <typename T, class D>
struct FactorRoot {
  typedef ValueOf<T, D> V;
  typedef typename V::type type;
  static constexpr bool changes = !std::is_same<type, D>::value;
  static type make(const D& d, bool& ok) { return V::make(d, ok); }
};

// ---------------------------------------------------------------------------- tiled lowering
#ifdef __CUDACC__
// a factor applied to a z pair (the box filter's 1/27 at the root)
template <typename T, class A>
struct PairZ<T, DScaled<T, A>> {
  static __device__ __forceinline__ void eval(const DScaled<T, A>& f, int x, int y, int z, T& v0, T& v1) {
    PairZ<T, A>::eval(f.a, x, y, z, v0, v1);
    v0 = Arith<T>::mul(v0, (T)f.r);
    v1 = Arith<T>::mul(v1, (T)f.r);
  }
};
#endif

template <typename T, class A, class R, int Off>
struct Tile<DScaled<T, A>, R, Off> {
  typedef Tile<A, R, Off> TA;
  typedef DScaled<T, typename TA::type> type;
  enum { end = TA::end, rounds = TA::rounds };
  static type make(const DScaled<T, A>& d) { return type{TA::make(d.a), d.r}; }
};
template <class Op, typename T, class A, class B, class R, int Off>
struct Tile<DFmaSum<Op, T, A, B>, R, Off> {
  typedef Tile<A, R, Off> TA;
  typedef Tile<B, R, TA::end> TB;
  typedef DFmaSum<Op, T, typename TA::type, typename TB::type> type;
  enum { end = TB::end, rounds = cmax(TA::rounds, TB::rounds) };
  static type make(const DFmaSum<Op, T, A, B>& d) { return type{TA::make(d.a), TB::make(d.b), d.r}; }
};
template <class Op, typename T, class A, class B, class R, int Off>
struct Tile<DFmaSumL<Op, T, A, B>, R, Off> {
  typedef Tile<A, R, Off> TA;
  typedef Tile<B, R, TA::end> TB;
  typedef DFmaSumL<Op, T, typename TA::type, typename TB::type> type;
  enum { end = TB::end, rounds = cmax(TA::rounds, TB::rounds) };
  static type make(const DFmaSumL<Op, T, A, B>& d) { return type{TA::make(d.a), TB::make(d.b), d.r}; }
};
// a signed pair of a leaf reads its neighbours directly; of an expression, from shared memory
template <typename T, class Pts, class A, class R, int Off>
struct Tile<DSignedStencil<T, Pts, A>, R, Off, typename std::enable_if<IsLeaf<A>::value>::type> {
  typedef DSignedStencil<T, Pts, A> type;
  enum { end = Off, rounds = 0 };
  static type make(const type& d) { return d; }
};
template <typename T, class Pts, class A, class R, int Off>
struct Tile<DSignedStencil<T, Pts, A>, R, Off, typename std::enable_if<!IsLeaf<A>::value>::type>
    : TileSmemStencil<T, Pts, A, R, Off, kSigned> {
  typedef TileSmemStencil<T, Pts, A, R, Off, kSigned> B;
  static typename B::type make(const DSignedStencil<T, Pts, A>& d) {
    typename B::type t;
    t.a = B::TA::make(d.a);
    for (int i = 0; i < Pts::length; ++i) t.c[i] = d.c[i];
    return t;
  }
};

}  // namespace nebo_detail
}  // namespace SpatialOps

#endif
