// apply_pointwise<Functor>(op1, ..., opN), N = 1..10 (drop-in for spatialops/NeboApplyPointwise.h:
// ApplyPointwise1..10 and the apply_pointwise entry points, e.g. :2047-2116).
//
// The value at each cell is Functor()(op1.eval(x,y,z), ..., opN.eval(x,y,z)); operands are fields,
// scalars or Nebo expressions of one field type; ghosts are the minimum over the operands and
// extents / BC flags come from the first operand that has them, as for any other Nebo node.
// The reference's GPU walk of this node is a stub that returns 0; here the functor is called
// inside the fused kernel of the enclosing `<<=`, so it must be callable on the device: declare
// its operator() (and nothing it calls that is host-only) __host__ __device__ (NEBO_HD).
#ifndef SpatialOps_NeboApplyPointwise_h
#define SpatialOps_NeboApplyPointwise_h

#include <tuple>
#include <type_traits>

#include <spatialops/NeboCore.h>
#include <spatialops/NeboOperators.h>

namespace SpatialOps {
namespace nebo_detail {

// device-side operand list (a plain aggregate: device functors are aggregates too)
template <class... D>
struct DTuple;
template <>
struct DTuple<> {
  __device__ __forceinline__ void rebase(int, int, int) {}
  template <int K> __device__ __forceinline__ void fill(int, int, int) const {}
};
template <class H, class... R>
struct DTuple<H, R...> {
  H h;
  DTuple<R...> r;
  NEBO_TWO_CHILDREN(h, r)
};

inline DTuple<> make_dtuple() { return DTuple<>(); }
template <class H, class... R>
DTuple<H, R...> make_dtuple(const H& h, const R&... r) {
  DTuple<H, R...> t;
  t.h = h;
  t.r = make_dtuple(r...);
  return t;
}

// evaluates the operands in order, then calls the functor with all of them
template <typename T, class Fn>
struct ApplyCall {
  template <class... V>
  static __device__ __forceinline__ T go(const DTuple<>&, int, int, int, V... v) {
    return (T)Fn()(v...);
  }
  template <class H, class... R, class... V>
  static __device__ __forceinline__ T go(const DTuple<H, R...>& t, int x, int y, int z, V... v) {
    return go(t.r, x, y, z, v..., t.h.eval(x, y, z));
  }
};

template <typename T, class Fn, class... D>
struct DApply {
  DTuple<D...> ops;
  __device__ __forceinline__ T eval(int x, int y, int z) const { return ApplyCall<T, Fn>::go(ops, x, y, z); }
  NEBO_ONE_CHILD(ops)
};

template <class... F>
struct MergeAll;
template <>
struct MergeAll<> {
  typedef void type;
};
template <class F, class... R>
struct MergeAll<F, R...> {
  typedef typename MergeField<F, typename MergeAll<R...>::type>::type type;
};

template <typename T, class Fn, class... N>
struct ApplyNode {
  typedef T value_type;
  std::tuple<N...> n;
  explicit ApplyNode(const N&... ns) : n(ns...) {}

  GhostData ghosts_with_bc() const {
    return std::apply([](const N&... a) { return fold_min(a.ghosts_with_bc()...); }, n);
  }
  GhostData ghosts_without_bc() const {
    return std::apply([](const N&... a) { return fold_min(a.ghosts_without_bc()...); }, n);
  }
  bool has_extents() const {
    return std::apply([](const N&... a) { return (a.has_extents() || ...); }, n);
  }
  IntVec extents() const {
    IntVec r(0, 0, 0);
    bool found = false;
    std::apply([&](const N&... a) { ((found ? void() : (a.has_extents() ? (r = a.extents(), found = true, void()) : void())), ...); }, n);
    return r;
  }
  IntVec has_bc() const {
    IntVec r(0, 0, 0);
    bool found = false;
    std::apply([&](const N&... a) { ((found ? void() : (a.has_extents() ? (r = a.has_bc(), found = true, void()) : void())), ...); }, n);
    return r;
  }
  void prepare() const {
    std::apply([](const N&... a) { (a.prepare(), ...); }, n);
  }
  auto device() const -> DApply<T, Fn, decltype(std::declval<const N&>().device())...> {
    DApply<T, Fn, decltype(std::declval<const N&>().device())...> d;
    d.ops = std::apply([](const N&... a) { return make_dtuple(a.device()...); }, n);
    return d;
  }

 private:
  static GhostData fold_min(const GhostData& g) { return g; }
  template <class... G>
  static GhostData fold_min(const GhostData& g, const G&... rest) {
    return min(g, fold_min(rest...));
  }
};

}  // namespace nebo_detail

template <typename Functor, typename... Ops>
NeboExpression<nebo_detail::ApplyNode<typename nebo_detail::MergeAll<typename nebo_detail::Operand<Ops>::field_type...>::type::value_type,
                                      Functor,
                                      decltype(nebo_detail::Operand<Ops>::template node<
                                               typename nebo_detail::MergeAll<typename nebo_detail::Operand<Ops>::field_type...>::type::value_type>(
                                          std::declval<const Ops&>()))...>,
               typename nebo_detail::MergeAll<typename nebo_detail::Operand<Ops>::field_type...>::type>
apply_pointwise(const Ops&... ops) {
  static_assert(sizeof...(Ops) >= 1 && sizeof...(Ops) <= 10, "apply_pointwise takes 1 to 10 operands");
  typedef typename nebo_detail::MergeAll<typename nebo_detail::Operand<Ops>::field_type...>::type F;
  static_assert(!std::is_void<F>::value, "apply_pointwise needs at least one field or expression operand");
  typedef typename F::value_type T;
  typedef nebo_detail::ApplyNode<T, Functor, decltype(nebo_detail::Operand<Ops>::template node<T>(ops))...> N;
  return NeboExpression<N, F>(N(nebo_detail::Operand<Ops>::template node<T>(ops)...));
}

}  // namespace SpatialOps
#endif
