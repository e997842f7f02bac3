// Pointwise operators, functions, comparisons, logic and cond of the Nebo language
// (drop-in for spatialops/NeboOperators.h and spatialops/NeboCond.h; the list of operators is
// the reference's, NeboOperators.txt and NeboCond.txt).
//
// Operands are scalars, SpatialFields and NeboExpressions; boolean operands are
// NeboBooleanExpressions and SpatialMasks.  Two non-scalar operands must produce the same field
// type (the reference's NeboFieldCheck, spatialops/NeboBasic.h:102-110); scalars take the value
// type of the field they meet.
#ifndef SpatialOps_NeboOperators_h
#define SpatialOps_NeboOperators_h

#include <type_traits>

#include <spatialops/NeboCore.h>

namespace SpatialOps {
namespace nebo_detail {

// ------------------------------------------------------------------ operand classification
template <class X, class Enable = void>
struct Operand {
  static constexpr bool ok = false;
  static constexpr bool scalar = false;
};
template <class X>
struct Operand<X, typename std::enable_if<std::is_arithmetic<X>::value>::type> {
  static constexpr bool ok = true;
  static constexpr bool scalar = true;
  typedef void field_type;
  template <class T> static ScalarNode<T> node(const X& x) { return ScalarNode<T>((T)x); }
};
template <class L, class V>
struct Operand<SpatialField<L, V>, void> {
  static constexpr bool ok = true;
  static constexpr bool scalar = false;
  typedef SpatialField<L, V> field_type;
  template <class T> static FieldNode<field_type> node(const field_type& f) { return FieldNode<field_type>(f); }
};
template <class E, class F>
struct Operand<NeboExpression<E, F>, void> {
  static constexpr bool ok = true;
  static constexpr bool scalar = false;
  typedef F field_type;
  template <class T> static E node(const NeboExpression<E, F>& e) { return e.expr(); }
};
// SingleValue fields and expressions: field type SpatialField<SingleValue, V>, which gives way
// to any other field type they meet (MergeField)
template <class V>
struct Operand<SpatialField<SingleValue, V>, void> {
  static constexpr bool ok = true;
  static constexpr bool scalar = false;
  typedef SpatialField<SingleValue, V> field_type;
  template <class T> static SingleValueNode<field_type> node(const field_type& f) { return SingleValueNode<field_type>(f); }
};
template <class E, class V>
struct Operand<NeboSingleValueExpression<E, V>, void> {
  static constexpr bool ok = true;
  static constexpr bool scalar = false;
  typedef SpatialField<SingleValue, V> field_type;
  template <class T> static E node(const NeboSingleValueExpression<E, V>& e) { return e.expr(); }
};

template <class X>
struct BoolOperand {
  static constexpr bool ok = false;
};
template <>
struct BoolOperand<bool> {
  static constexpr bool ok = true;
  typedef void field_type;
  static BoolScalarNode node(bool b) { return BoolScalarNode(b); }
};
template <class E, class V>
struct BoolOperand<NeboBooleanSingleValueExpression<E, V>> {
  static constexpr bool ok = true;
  typedef SpatialField<SingleValue, V> field_type;
  static E node(const NeboBooleanSingleValueExpression<E, V>& e) { return e.expr(); }
};
template <class E, class F>
struct BoolOperand<NeboBooleanExpression<E, F>> {
  static constexpr bool ok = true;
  typedef F field_type;
  static E node(const NeboBooleanExpression<E, F>& e) { return e.expr(); }
};
template <class F>
struct BoolOperand<SpatialMask<F>> {
  static constexpr bool ok = true;
  typedef F field_type;
  static MaskNode<F> node(const SpatialMask<F>& m) { return MaskNode<F>(m); }
};

// field type of a combination (void for two scalars; a SingleValue field gives way to any other
// field type, as the reference's Field x SingleValue overloads do)
template <class F>
struct IsSingleValue : std::false_type {};
template <class V>
struct IsSingleValue<SpatialField<SingleValue, V>> : std::true_type {};

template <class FA, class FB,
          int K = (std::is_void<FA>::value || std::is_void<FB>::value) ? 0
                  : (IsSingleValue<FA>::value && !IsSingleValue<FB>::value) ? 1
                  : (IsSingleValue<FB>::value && !IsSingleValue<FA>::value) ? 2 : 0>
struct MergeField {
  static_assert(std::is_same<FA, FB>::value, "Nebo: operands of one expression must have the same field type");
  typedef FA type;
};
template <class FA, class FB> struct MergeField<FA, FB, 1> {
  static_assert(std::is_same<typename FA::value_type, typename FB::value_type>::value,
                "Nebo: a SingleValue field must have the value type of the field it meets");
  typedef FB type;
};
template <class FA, class FB> struct MergeField<FA, FB, 2> {
  static_assert(std::is_same<typename FA::value_type, typename FB::value_type>::value,
                "Nebo: a SingleValue field must have the value type of the field it meets");
  typedef FA type;
};
template <class FB> struct MergeField<void, FB, 0> { typedef FB type; };
template <class FA> struct MergeField<FA, void, 0> { typedef FA type; };
template <> struct MergeField<void, void, 0> { typedef void type; };

// the wrapper of a value / boolean expression of field type F
template <class N, class F>
struct Wrap {
  typedef NeboExpression<N, F> type;
};
template <class N, class V>
struct Wrap<N, SpatialField<SingleValue, V>> {
  typedef NeboSingleValueExpression<N, V> type;
};
template <class N, class F>
struct WrapBool {
  typedef NeboBooleanExpression<N, F> type;
};
template <class N, class V>
struct WrapBool<N, SpatialField<SingleValue, V>> {
  typedef NeboBooleanSingleValueExpression<N, V> type;
};

template <class A, class B>
struct BinaryTraits {
  static constexpr bool ok = Operand<A>::ok && Operand<B>::ok && !(Operand<A>::scalar && Operand<B>::scalar);
};
template <class A, class B, bool OK = BinaryTraits<A, B>::ok>
struct Binary {};
template <class A, class B>
struct Binary<A, B, true> {
  typedef typename MergeField<typename Operand<A>::field_type, typename Operand<B>::field_type>::type field_type;
  typedef typename field_type::value_type T;
  typedef decltype(Operand<A>::template node<T>(std::declval<A>())) NA;
  typedef decltype(Operand<B>::template node<T>(std::declval<B>())) NB;
  static NA na(const A& a) { return Operand<A>::template node<T>(a); }
  static NB nb(const B& b) { return Operand<B>::template node<T>(b); }
};

template <class A, bool OK = Operand<A>::ok && !Operand<A>::scalar>
struct Unary {};
template <class A>
struct Unary<A, true> {
  typedef typename Operand<A>::field_type field_type;
  typedef typename field_type::value_type T;
  typedef decltype(Operand<A>::template node<T>(std::declval<A>())) NA;
  static NA na(const A& a) { return Operand<A>::template node<T>(a); }
};

template <class A, class B, bool OK = BoolOperand<A>::ok && BoolOperand<B>::ok>
struct BoolBinary {};
template <class A, class B>
struct BoolBinary<A, B, true> {
  typedef typename MergeField<typename BoolOperand<A>::field_type, typename BoolOperand<B>::field_type>::type field_type;
  typedef decltype(BoolOperand<A>::node(std::declval<A>())) NA;
  typedef decltype(BoolOperand<B>::node(std::declval<B>())) NB;
};

}  // namespace nebo_detail

// ------------------------------------------------------------------ arithmetic
#define NEBO_BINARY_OPERATOR(SYM, OP)                                                                          \
  template <class A, class B, class Bn = nebo_detail::Binary<A, B>>                                            \
  typename nebo_detail::Wrap<nebo_detail::BinNode<nebo_detail::OP, typename Bn::NA, typename Bn::NB>,          \
                             typename Bn::field_type>::type                                                    \
  operator SYM(const A& a, const B& b) {                                                                       \
    typedef nebo_detail::BinNode<nebo_detail::OP, typename Bn::NA, typename Bn::NB> N;                         \
    return typename nebo_detail::Wrap<N, typename Bn::field_type>::type(N(Bn::na(a), Bn::nb(b)));              \
  }
NEBO_BINARY_OPERATOR(+, OpAdd)
NEBO_BINARY_OPERATOR(-, OpSub)
NEBO_BINARY_OPERATOR(*, OpMul)
NEBO_BINARY_OPERATOR(/, OpDiv)
#undef NEBO_BINARY_OPERATOR

#define NEBO_BINARY_FUNCTION(NAME, OP)                                                                         \
  template <class A, class B, class Bn = nebo_detail::Binary<A, B>>                                            \
  typename nebo_detail::Wrap<nebo_detail::BinNode<nebo_detail::OP, typename Bn::NA, typename Bn::NB>,          \
                             typename Bn::field_type>::type                                                    \
  NAME(const A& a, const B& b) {                                                                               \
    typedef nebo_detail::BinNode<nebo_detail::OP, typename Bn::NA, typename Bn::NB> N;                         \
    return typename nebo_detail::Wrap<N, typename Bn::field_type>::type(N(Bn::na(a), Bn::nb(b)));              \
  }
NEBO_BINARY_FUNCTION(max, OpMax)
NEBO_BINARY_FUNCTION(min, OpMin)
#undef NEBO_BINARY_FUNCTION

// pow(x, y): an int exponent selects PowIntFcn (NeboOperators.h:14598), anything else PowFcn.
template <class A, class B, class Bn = nebo_detail::Binary<A, B>,
          class = typename std::enable_if<!std::is_integral<B>::value>::type>
typename nebo_detail::Wrap<nebo_detail::BinNode<nebo_detail::OpPow, typename Bn::NA, typename Bn::NB>,
                           typename Bn::field_type>::type
pow(const A& a, const B& b) {
  typedef nebo_detail::BinNode<nebo_detail::OpPow, typename Bn::NA, typename Bn::NB> N;
  return typename nebo_detail::Wrap<N, typename Bn::field_type>::type(N(Bn::na(a), Bn::nb(b)));
}
template <class A, class U = nebo_detail::Unary<A>>
typename nebo_detail::Wrap<nebo_detail::PowIntNode<typename U::NA>, typename U::field_type>::type pow(const A& a,
                                                                                                     int e) {
  typedef nebo_detail::PowIntNode<typename U::NA> N;
  return typename nebo_detail::Wrap<N, typename U::field_type>::type(N(U::na(a), e));
}

#define NEBO_UNARY_FUNCTION(NAME, FN)                                                                          \
  template <class A, class U = nebo_detail::Unary<A>>                                                          \
  typename nebo_detail::Wrap<nebo_detail::UnNode<nebo_detail::FN, typename U::NA>, typename U::field_type>::type \
  NAME(const A& a) {                                                                                           \
    typedef nebo_detail::UnNode<nebo_detail::FN, typename U::NA> N;                                            \
    return typename nebo_detail::Wrap<N, typename U::field_type>::type(N(U::na(a)));                           \
  }
NEBO_UNARY_FUNCTION(operator-, FnNeg)
NEBO_UNARY_FUNCTION(sin, FnSin)
NEBO_UNARY_FUNCTION(cos, FnCos)
NEBO_UNARY_FUNCTION(tan, FnTan)
NEBO_UNARY_FUNCTION(exp, FnExp)
NEBO_UNARY_FUNCTION(tanh, FnTanh)
NEBO_UNARY_FUNCTION(abs, FnAbs)
NEBO_UNARY_FUNCTION(sqrt, FnSqrt)
NEBO_UNARY_FUNCTION(log, FnLog)
NEBO_UNARY_FUNCTION(log10, FnLog10)
NEBO_UNARY_FUNCTION(erf, FnErf)
NEBO_UNARY_FUNCTION(erfc, FnErfc)
NEBO_UNARY_FUNCTION(inv_erf, FnInvErf)
NEBO_UNARY_FUNCTION(inv_erfc, FnInvErfc)
NEBO_UNARY_FUNCTION(square, FnSquare)
NEBO_UNARY_FUNCTION(cube, FnCube)
#undef NEBO_UNARY_FUNCTION

// ------------------------------------------------------------------ comparisons -> booleans
#define NEBO_COMPARISON(SYM, OP)                                                                                \
  template <class A, class B, class Bn = nebo_detail::Binary<A, B>>                                             \
  typename nebo_detail::WrapBool<nebo_detail::CmpNode<nebo_detail::OP, typename Bn::NA, typename Bn::NB>,       \
                                 typename Bn::field_type>::type                                                 \
  operator SYM(const A& a, const B& b) {                                                                        \
    typedef nebo_detail::CmpNode<nebo_detail::OP, typename Bn::NA, typename Bn::NB> N;                          \
    return typename nebo_detail::WrapBool<N, typename Bn::field_type>::type(N(Bn::na(a), Bn::nb(b)));           \
  }
NEBO_COMPARISON(==, CmpEq)
NEBO_COMPARISON(!=, CmpNe)
NEBO_COMPARISON(<, CmpLt)
NEBO_COMPARISON(<=, CmpLe)
NEBO_COMPARISON(>, CmpGt)
NEBO_COMPARISON(>=, CmpGe)
#undef NEBO_COMPARISON

#define NEBO_LOGIC(SYM, OP)                                                                                     \
  template <class A, class B, class Bb = nebo_detail::BoolBinary<A, B>>                                         \
  typename nebo_detail::WrapBool<nebo_detail::LogicNode<nebo_detail::OP, typename Bb::NA, typename Bb::NB>,     \
                                 typename Bb::field_type>::type                                                 \
  operator SYM(const A& a, const B& b) {                                                                        \
    typedef nebo_detail::LogicNode<nebo_detail::OP, typename Bb::NA, typename Bb::NB> N;                        \
    return typename nebo_detail::WrapBool<N, typename Bb::field_type>::type(                                    \
        N(nebo_detail::BoolOperand<A>::node(a), nebo_detail::BoolOperand<B>::node(b)));                         \
  }
NEBO_LOGIC(&&, LogAnd)
NEBO_LOGIC(||, LogOr)
#undef NEBO_LOGIC

template <class A, class = typename std::enable_if<nebo_detail::BoolOperand<A>::ok && !std::is_same<A, bool>::value>::type>
typename nebo_detail::WrapBool<nebo_detail::NotNode<decltype(nebo_detail::BoolOperand<A>::node(std::declval<A>()))>,
                               typename nebo_detail::BoolOperand<A>::field_type>::type
operator!(const A& a) {
  typedef nebo_detail::NotNode<decltype(nebo_detail::BoolOperand<A>::node(std::declval<A>()))> N;
  return typename nebo_detail::WrapBool<N, typename nebo_detail::BoolOperand<A>::field_type>::type(
      N(nebo_detail::BoolOperand<A>::node(a)));
}

// ------------------------------------------------------------------ cond(...)(...)...(default)
// cond(test, value)(test, value)...(default): the first clause whose test holds gives the value
// (NeboCond.h:408-413).  Tests are boolean expressions, masks or plain bools; values are scalars,
// fields, SingleValue fields or expressions.  cond(value) alone is the value.  A cond made of
// scalars and bools only is evaluated on the host and is a plain number (NeboCond.h's simple
// conds: `double d = cond(false, 1.0)(2.0);`).
namespace nebo_detail {
struct ClauseEnd {};
template <class Prev, class TN, class VN>
struct ClauseLink {
  Prev prev;
  TN t;
  VN v;
};

template <class F>
struct ValueTypeOf {
  typedef typename F::value_type type;
};
template <>
struct ValueTypeOf<void> {
  typedef double type;
};

template <typename T, class Tail>
Tail fold_cond(const ClauseEnd&, const Tail& tail) {
  return tail;
}
template <typename T, class Prev, class TN, class VN, class Tail>
auto fold_cond(const ClauseLink<Prev, TN, VN>& c, const Tail& tail) {
  return fold_cond<T>(c.prev, CondNode<T, TN, VN, Tail>(c.t, c.v, tail));
}

// all-scalar chains: evaluated here, first clause first
template <typename T>
T host_cond(const ClauseEnd&, T tail) {
  return tail;
}
template <typename T, class Prev, class TN, class VN>
T host_cond(const ClauseLink<Prev, TN, VN>& c, T tail) {
  return host_cond<T>(c.prev, c.t.b ? (T)c.v.v : tail);
}

template <class F, class Chain>
struct CondBuilder {
  typedef typename ValueTypeOf<F>::type T;
  Chain chain;

  template <class Tst, class V>
  auto operator()(const Tst& t, const V& v) const {
    static_assert(BoolOperand<Tst>::ok, "Nebo cond: a clause test must be a boolean expression, a mask or a bool");
    typedef typename MergeField<typename MergeField<F, typename BoolOperand<Tst>::field_type>::type,
                                typename Operand<V>::field_type>::type F2;
    auto tn = BoolOperand<Tst>::node(t);
    auto vn = Operand<V>::template node<T>(v);
    typedef ClauseLink<Chain, decltype(tn), decltype(vn)> Link;
    return CondBuilder<F2, Link>{Link{chain, tn, vn}};
  }
  template <class V>
  auto operator()(const V& v) const {
    typedef typename MergeField<F, typename Operand<V>::field_type>::type F2;
    return finish<F2>(v);
  }

 private:
  template <class F2, class V>
  typename std::enable_if<std::is_void<F2>::value, T>::type finish(const V& v) const {
    return host_cond<T>(chain, (T)v);
  }
  template <class F2, class V>
  auto finish(const V& v, typename std::enable_if<!std::is_void<F2>::value, int>::type = 0) const {
    auto tail = Operand<V>::template node<T>(v);
    auto node = fold_cond<T>(chain, tail);
    return typename Wrap<decltype(node), F2>::type(node);
  }
};
}  // namespace nebo_detail

template <class Tst, class V>
auto cond(const Tst& t, const V& v) {
  static_assert(nebo_detail::BoolOperand<Tst>::ok, "Nebo cond: a clause test must be a boolean expression, a mask or a bool");
  typedef typename nebo_detail::MergeField<typename nebo_detail::BoolOperand<Tst>::field_type,
                                           typename nebo_detail::Operand<V>::field_type>::type F;
  typedef typename nebo_detail::ValueTypeOf<F>::type T;
  auto tn = nebo_detail::BoolOperand<Tst>::node(t);
  auto vn = nebo_detail::Operand<V>::template node<T>(v);
  typedef nebo_detail::ClauseLink<nebo_detail::ClauseEnd, decltype(tn), decltype(vn)> Link;
  return nebo_detail::CondBuilder<F, Link>{Link{nebo_detail::ClauseEnd(), tn, vn}};
}

// cond(value): the value itself (a number for a scalar, else the same expression)
template <class V, class = typename std::enable_if<std::is_arithmetic<V>::value>::type>
double cond(const V& v) {
  return (double)v;
}
template <class V, class = typename std::enable_if<nebo_detail::Operand<V>::ok && !nebo_detail::Operand<V>::scalar>::type,
          class = void>
auto cond(const V& v) {
  typedef typename nebo_detail::Operand<V>::field_type F;
  typedef typename F::value_type T;
  auto node = nebo_detail::Operand<V>::template node<T>(v);
  return typename nebo_detail::Wrap<decltype(node), F>::type(node);
}

}  // namespace SpatialOps
#endif
