// Tiled lowering of `<<=` (the evaluation that replaces spatialops/NeboLhs.h:29-41 and 592-699,
// the reference's one-thread-per-column walks).
//
// The reference evaluates a nested stencil by recomputing its argument at every point of every
// enclosing stencil: Interp(Grad(Interp(a))) reads `a` eight times per output and computes the
// inner interpolant four times (spatialops/NeboStencils.h:407-448).  Here a block of 32 x 8
// threads owns a tile of 32 x 8 x TZ output cells.  Before the output pass, the argument of every
// stencil whose argument is itself an expression (not a field leaf or a scalar) is materialised
// ONCE per tile in shared memory, over the tile grown by the reach of that stencil and of every
// stencil above it; the stencil then reads its neighbours from shared memory.  Inner levels are
// filled first (fill rounds 1..H, one barrier per round), so each level of a deep chain is
// computed once per point.  Field leaves are read with coalesced read-only loads (a tile's
// neighbours hit L1 and L2, so each input is read from HBM about once).
//
// In builds that allow reassociation, a 27-point box sum is first split into three 3-point line
// sums (x, then y, then z), so the box filter's partial sums are shared too.
//
// Everything is decided at compile time from the expression's type: which nodes are
// materialised, each buffer's box (per-axis reach of the point collections, summed through
// nested stencils), its shared-memory offset, the fill round, and the tile depth TZ (8, 4, 2
// or 1: the deepest whose buffers fit the budget).  An expression without such a stencil keeps
// the plain one-pass kernel.
//
// Values: each materialised point is the same functor evaluated at the same point with the same
// operations in the same order, and the stencil folds its points in the reference's order, so
// the results are bit for bit those of the plain kernel (and, with NEBO_EXACT_ARITHMETIC, of the
// reference's serial walk).
//
// Bounds: a buffer point is computed only when some output cell of the (possibly partial) tile
// reads it; the write region (calculate_actual_ghost) guarantees that every such point's reads
// lie inside the fields' valid windows, because the windows are boxes and each buffer covers the
// box hull of the reads.
#ifndef SpatialOps_NeboTiled_h
#define SpatialOps_NeboTiled_h

#include <cuda_runtime.h>

#include <spatialops/NeboCore.h>

#ifdef __CUDACC__
#include <spatialops/NeboApplyPointwise.h>
#endif

namespace SpatialOps {
namespace nebo_detail {

constexpr int kTileX = 32;
constexpr int kTileY = 8;
constexpr int kTileThreads = kTileX * kTileY;
#ifndef NEBO_TILE_SMEM_BUDGET
#define NEBO_TILE_SMEM_BUDGET (64 * 1024)
#endif
constexpr int kTileSmemBudget = NEBO_TILE_SMEM_BUDGET;

constexpr int cmin(int a, int b) { return a < b ? a : b; }
constexpr int cmax(int a, int b) { return a > b ? a : b; }

// A box of local (tile-relative) coordinates, bounds inclusive.
template <int XL, int XH, int YL, int YH, int ZL, int ZH>
struct TBox {
  enum { xl = XL, xh = XH, yl = YL, yh = YH, zl = ZL, zh = ZH };
  enum { nx = XH - XL + 1, ny = YH - YL + 1, nz = ZH - ZL + 1 };
  enum { n = nx * ny * nz };
};

// Per-axis hull of a point collection.
template <class Pts>
struct PtsHull;
template <class P>
struct PtsHull<NeboStencilPointCollection<P, NeboNil>> {
  enum { xl = P::X, xh = P::X, yl = P::Y, yh = P::Y, zl = P::Z, zh = P::Z };
};
template <class P, class R>
struct PtsHull<NeboStencilPointCollection<P, R>> {
  typedef PtsHull<R> H;
  enum {
    xl = cmin(P::X, H::xl), xh = cmax(P::X, H::xh),
    yl = cmin(P::Y, H::yl), yh = cmax(P::Y, H::yh),
    zl = cmin(P::Z, H::zl), zh = cmax(P::Z, H::zh)
  };
};

// The box an argument is needed on: the stencil's box grown by its points.
template <class B, class Pts>
struct GrowBox {
  typedef PtsHull<Pts> H;
  typedef TBox<B::xl + H::xl, B::xh + H::xh, B::yl + H::yl, B::yh + H::yh, B::zl + H::zl, B::zh + H::zh> type;
};

#ifdef __CUDACC__
__device__ __forceinline__ unsigned char* tile_smem() {
  extern __shared__ __align__(16) unsigned char nebo_tile_dyn_smem[];
  return nebo_tile_dyn_smem;
}
#endif

// Read access to a buffer over box R at byte offset Off.
template <typename T, class R, int Off>
struct SmemView {
#ifdef __CUDACC__
  __device__ __forceinline__ T eval(int x, int y, int z) const {
    const T* buf = reinterpret_cast<const T*>(tile_smem() + Off);
    return buf[(x - R::xl) + R::nx * ((y - R::yl) + R::ny * (z - R::zl))];
  }
#endif
};

// The folds of a materialised stencil: weighted (c in listed order), plain sum, signed sum (the
// points' values with the sign bits of c, added in listed order; NeboFactor.h).
enum StencilKind { kWeighted = 0, kSum = 1, kSigned = 2 };

// How the fill of a buffer whose points are the values of A may share work between two
// neighbouring points: 0 none, 1 x pairs, 2 y pairs (specialised below for the line sums of a
// split box filter, whose neighbouring sums share their middle pair).
template <typename T, class A>
struct PairFill {
  static constexpr int axis = 0;
};

// A stencil whose argument is materialised over box R at byte offset Off in fill round Round.
template <typename T, class Pts, class A, class R, int Off, int Round, int Kind>
struct DStencilSmem {
  A a;
  double c[Pts::length];
#ifdef __CUDACC__
  __device__ __forceinline__ T eval(int x, int y, int z) const {
    if (Kind == kSum) return StencilFold<Pts>::template sum<T>(SmemView<T, R, Off>(), x, y, z);
    if (Kind == kSigned) return StencilFold<Pts>::template signed_sum<T>(SmemView<T, R, Off>(), c, x, y, z);
    return StencilFold<Pts>::template weighted<T>(SmemView<T, R, Off>(), c, x, y, z);
  }
  __device__ __forceinline__ void rebase(int x0, int y0, int z0) { a.rebase(x0, y0, z0); }
  template <int H>
  __device__ __forceinline__ void fill(int tx, int ty, int tz) const {
    a.template fill<H>(tx, ty, tz);
    if (H != Round) return;
    T* buf = reinterpret_cast<T*>(tile_smem() + Off);
    // points read by the tile's output cells: the box, its upper ends cut by the partial tile
    const int hx = R::xh - tx, hy = R::yh - ty, hz = R::zh - tz;
    const int tid = (int)(threadIdx.x + blockDim.x * threadIdx.y);
    constexpr int ax = PairFill<T, A>::axis;
    if constexpr (ax == 1 && R::nx % 2 == 0) {
      // x pairs (lx, lx+1): the second point (and its extra read) only when a cell needs it
      constexpr int hn = R::nx / 2;
#pragma unroll 2
      for (int i = tid; i < R::n / 2; i += kTileThreads) {
        const int px = i % hn, r = i / hn;
        const int lx = R::xl + 2 * px, ly = R::yl + r % R::ny, lz = R::zl + r / R::ny;
        if (lx <= hx && ly <= hy && lz <= hz) {
          const bool second = lx + 1 <= hx;
          T v0, v1;
          PairFill<T, A>::pair(a, lx, ly, lz, second, v0, v1);
          const int bi = 2 * px + R::nx * r;
          buf[bi] = v0;
          if (second) buf[bi + 1] = v1;
        }
      }
    } else if constexpr (ax == 2 && R::ny % 2 == 0) {
      // y pairs (ly, ly+1)
      constexpr int hn = R::ny / 2;
#pragma unroll 2
      for (int i = tid; i < R::n / 2; i += kTileThreads) {
        const int ox = i % R::nx, r = i / R::nx, py = r % hn, oz = r / hn;
        const int lx = R::xl + ox, ly = R::yl + 2 * py, lz = R::zl + oz;
        if (lx <= hx && ly <= hy && lz <= hz) {
          const bool second = ly + 1 <= hy;
          T v0, v1;
          PairFill<T, A>::pair(a, lx, ly, lz, second, v0, v1);
          const int bi = ox + R::nx * (2 * py + R::ny * oz);
          buf[bi] = v0;
          if (second) buf[bi + R::nx] = v1;
        }
      }
    } else {
#pragma unroll 2
      for (int i = tid; i < R::n; i += kTileThreads) {
        const int lx = R::xl + i % R::nx;
        const int r = i / R::nx;
        const int ly = R::yl + r % R::ny;
        const int lz = R::zl + r / R::ny;
        if (lx <= hx && ly <= hy && lz <= hz) buf[i] = a.eval(lx, ly, lz);
      }
    }
  }
#endif
};

// ---------------------------------------------------------------------------- the transform
// Tile<D, R, Off>: D evaluated over box R with its buffers from byte offset Off.
//   type   the functor with every materialised stencil replaced by DStencilSmem
//   end    byte offset after the subtree's buffers
//   rounds fill rounds the subtree needs (0: no buffer)
//   make   copies the run-time values (pointers, strides, coefficients, scalars)
template <class D>
struct IsLeaf : std::false_type {};
template <typename T>
struct IsLeaf<DField<T>> : std::true_type {};
template <typename T>
struct IsLeaf<DScalar<T>> : std::true_type {};
template <typename T>
struct IsLeaf<DSingleValue<T>> : std::true_type {};

template <class D, class R, int Off, class Enable = void>
struct Tile {  // leaves, masks and anything without children that matter
  typedef D type;
  enum { end = Off, rounds = 0 };
  static type make(const D& d) { return d; }
};

template <class Op, typename T, class A, class B, class R, int Off>
struct Tile<DBin<Op, T, A, B>, R, Off> {
  typedef Tile<A, R, Off> TA;
  typedef Tile<B, R, TA::end> TB;
  typedef DBin<Op, T, typename TA::type, typename TB::type> type;
  enum { end = TB::end, rounds = cmax(TA::rounds, TB::rounds) };
  static type make(const DBin<Op, T, A, B>& d) { return type{TA::make(d.a), TB::make(d.b)}; }
};

template <class Fn, typename T, class A, class R, int Off>
struct Tile<DUn<Fn, T, A>, R, Off> {
  typedef Tile<A, R, Off> TA;
  typedef DUn<Fn, T, typename TA::type> type;
  enum { end = TA::end, rounds = TA::rounds };
  static type make(const DUn<Fn, T, A>& d) { return type{TA::make(d.a)}; }
};

template <typename T, class A, class R, int Off>
struct Tile<DPowInt<T, A>, R, Off> {
  typedef Tile<A, R, Off> TA;
  typedef DPowInt<T, typename TA::type> type;
  enum { end = TA::end, rounds = TA::rounds };
  static type make(const DPowInt<T, A>& d) { return type{TA::make(d.a), d.e}; }
};

template <class Op, class A, class B, class R, int Off>
struct Tile<DCmp<Op, A, B>, R, Off> {
  typedef Tile<A, R, Off> TA;
  typedef Tile<B, R, TA::end> TB;
  typedef DCmp<Op, typename TA::type, typename TB::type> type;
  enum { end = TB::end, rounds = cmax(TA::rounds, TB::rounds) };
  static type make(const DCmp<Op, A, B>& d) { return type{TA::make(d.a), TB::make(d.b)}; }
};

template <class Op, class A, class B, class R, int Off>
struct Tile<DLogic<Op, A, B>, R, Off> {
  typedef Tile<A, R, Off> TA;
  typedef Tile<B, R, TA::end> TB;
  typedef DLogic<Op, typename TA::type, typename TB::type> type;
  enum { end = TB::end, rounds = cmax(TA::rounds, TB::rounds) };
  static type make(const DLogic<Op, A, B>& d) { return type{TA::make(d.a), TB::make(d.b)}; }
};

template <class A, class R, int Off>
struct Tile<DNot<A>, R, Off> {
  typedef Tile<A, R, Off> TA;
  typedef DNot<typename TA::type> type;
  enum { end = TA::end, rounds = TA::rounds };
  static type make(const DNot<A>& d) { return type{TA::make(d.a)}; }
};

template <typename T, class Test, class Val, class Rest, class R, int Off>
struct Tile<DCond<T, Test, Val, Rest>, R, Off> {
  typedef Tile<Test, R, Off> TT;
  typedef Tile<Val, R, TT::end> TV;
  typedef Tile<Rest, R, TV::end> TR;
  typedef DCond<T, typename TT::type, typename TV::type, typename TR::type> type;
  enum { end = TR::end, rounds = cmax(TT::rounds, cmax(TV::rounds, TR::rounds)) };
  static type make(const DCond<T, Test, Val, Rest>& d) { return type{TT::make(d.t), TV::make(d.v), TR::make(d.r)}; }
};

// The 27-point box sum (the box filters, NeboStencilBuilder.h:454-465) as three 3-point sums,
// one axis each, when the build allows reassociation (not NEBO_EXACT_ARITHMETIC): about 7 FP64
// additions per cell instead of 26, the x and y partial sums shared through shared memory.  The
// result differs from the reference's point-by-point order by rounding only.
template <class Pts>
struct BoxMask;
template <class P>
struct BoxMask<NeboStencilPointCollection<P, NeboNil>> {
  static constexpr bool inside = P::X >= -1 && P::X <= 1 && P::Y >= -1 && P::Y <= 1 && P::Z >= -1 && P::Z <= 1;
  static constexpr long long bits = inside ? (1LL << ((P::X + 1) + 3 * (P::Y + 1) + 9 * (P::Z + 1))) : 0;
  static constexpr bool ok = inside;
};
template <class P, class R>
struct BoxMask<NeboStencilPointCollection<P, R>> {
  typedef BoxMask<NeboStencilPointCollection<P, NeboNil>> H;
  static constexpr long long bits = H::bits | BoxMask<R>::bits;
  static constexpr bool ok = H::ok && BoxMask<R>::ok;
};
template <class Pts>
struct IsBox27 {
  static constexpr bool value = Pts::length == 27 && BoxMask<Pts>::ok && BoxMask<Pts>::bits == (1LL << 27) - 1;
};
#ifdef NEBO_EXACT_ARITHMETIC
constexpr bool kReassociate = false;
#else
constexpr bool kReassociate = true;
#endif
template <class Pts>
struct SplitBox {
  static constexpr bool value = kReassociate && IsBox27<Pts>::value;
};
typedef NEBO_FIRST_IJK(-1, 0, 0)::NEBO_ADD_IJK(0, 0, 0)::NEBO_ADD_IJK(1, 0, 0) Line3X;
typedef NEBO_FIRST_IJK(0, -1, 0)::NEBO_ADD_IJK(0, 0, 0)::NEBO_ADD_IJK(0, 1, 0) Line3Y;
typedef NEBO_FIRST_IJK(0, 0, -1)::NEBO_ADD_IJK(0, 0, 0)::NEBO_ADD_IJK(0, 0, 1) Line3Z;

#ifdef __CUDACC__
// The line sums' shared pairs: s(p) = v(p-1) + m and s(p+1) = m + v(p+2) with m = v(p) + v(p+1),
// 3 additions for two sums instead of 4 (reassociating builds only: the split box is theirs).
template <typename T, class F>
struct PairFill<T, DSumStencil<T, Line3X, F>> {  // x sums of any functor, read point by point
  static constexpr int axis = 1;
  static __device__ __forceinline__ void pair(const DSumStencil<T, Line3X, F>& s, int x, int y, int z, bool second,
                                              T& v0, T& v1) {
    const T m = Arith<T>::add(s.a.eval(x, y, z), s.a.eval(x + 1, y, z));
    v0 = Arith<T>::add(s.a.eval(x - 1, y, z), m);
    v1 = second ? Arith<T>::add(m, s.a.eval(x + 2, y, z)) : m;
  }
};
template <typename T, class X, class RB, int OffB, int RoundB>
struct PairFill<T, DStencilSmem<T, Line3Y, X, RB, OffB, RoundB, kSum>> {  // y sums of a buffer
  static constexpr int axis = 2;
  static __device__ __forceinline__ void pair(const DStencilSmem<T, Line3Y, X, RB, OffB, RoundB, kSum>&, int x, int y,
                                              int z, bool second, T& v0, T& v1) {
    const SmemView<T, RB, OffB> b;
    const T m = Arith<T>::add(b.eval(x, y, z), b.eval(x, y + 1, z));
    v0 = Arith<T>::add(b.eval(x, y - 1, z), m);
    v1 = second ? Arith<T>::add(m, b.eval(x, y + 2, z)) : m;
  }
};

// The output pass evaluates two z-neighbouring cells at once: two evaluations, except for the z
// sums of a split box filter (the same shared middle pair) and a factor applied to them.
template <typename T, class D>
struct PairZ {
  static __device__ __forceinline__ void eval(const D& f, int x, int y, int z, T& v0, T& v1) {
    v0 = f.eval(x, y, z);
    v1 = f.eval(x, y, z + 1);
  }
};
template <typename T, class X, class RB, int OffB, int RoundB>
struct PairZ<T, DStencilSmem<T, Line3Z, X, RB, OffB, RoundB, kSum>> {
  static __device__ __forceinline__ void eval(const DStencilSmem<T, Line3Z, X, RB, OffB, RoundB, kSum>&, int x, int y,
                                              int z, T& v0, T& v1) {
    const SmemView<T, RB, OffB> b;
    const T m = Arith<T>::add(b.eval(x, y, z), b.eval(x, y, z + 1));
    v0 = Arith<T>::add(b.eval(x, y, z - 1), m);
    v1 = Arith<T>::add(m, b.eval(x, y, z + 2));
  }
};
#endif

template <typename T, class Pts, class A, class R, int Off>
struct Tile<DSumStencil<T, Pts, A>, R, Off, typename std::enable_if<SplitBox<Pts>::value>::type> {
  typedef DSumStencil<T, Line3Z, DSumStencil<T, Line3Y, DSumStencil<T, Line3X, A>>> Split;
  typedef Tile<Split, R, Off> TS;
  typedef typename TS::type type;
  enum { end = TS::end, rounds = TS::rounds };
  static type make(const DSumStencil<T, Pts, A>& d) {
    Split s;
    s.a.a.a = d.a;
    return TS::make(s);
  }
};

// a stencil of a leaf: reads its neighbours directly
template <typename T, class Pts, class A, class R, int Off>
struct Tile<DStencil<T, Pts, A>, R, Off, typename std::enable_if<IsLeaf<A>::value>::type> {
  typedef DStencil<T, Pts, A> type;
  enum { end = Off, rounds = 0 };
  static type make(const type& d) { return d; }
};
template <typename T, class Pts, class A, class R, int Off>
struct Tile<DSumStencil<T, Pts, A>, R, Off,
            typename std::enable_if<IsLeaf<A>::value && !SplitBox<Pts>::value>::type> {
  typedef DSumStencil<T, Pts, A> type;
  enum { end = Off, rounds = 0 };
  static type make(const type& d) { return d; }
};

constexpr int round16(int b) { return (b + 15) / 16 * 16; }

// a stencil of an expression: the argument is materialised over the grown box
template <typename T, class Pts, class A, class R, int Off, int Kind>
struct TileSmemStencil {
  typedef typename GrowBox<R, Pts>::type RA;
  typedef Tile<A, RA, Off> TA;
  enum { my_off = TA::end, end = TA::end + round16(RA::n * (int)sizeof(T)), rounds = TA::rounds + 1 };
  typedef DStencilSmem<T, Pts, typename TA::type, RA, my_off, rounds, Kind> type;
};
template <typename T, class Pts, class A, class R, int Off>
struct Tile<DStencil<T, Pts, A>, R, Off, typename std::enable_if<!IsLeaf<A>::value>::type>
    : TileSmemStencil<T, Pts, A, R, Off, kWeighted> {
  typedef TileSmemStencil<T, Pts, A, R, Off, kWeighted> B;
  static typename B::type make(const DStencil<T, Pts, A>& d) {
    typename B::type t;
    t.a = B::TA::make(d.a);
    for (int i = 0; i < Pts::length; ++i) t.c[i] = d.c[i];
    return t;
  }
};
template <typename T, class Pts, class A, class R, int Off>
struct Tile<DSumStencil<T, Pts, A>, R, Off,
            typename std::enable_if<!IsLeaf<A>::value && !SplitBox<Pts>::value>::type>
    : TileSmemStencil<T, Pts, A, R, Off, kSum> {
  typedef TileSmemStencil<T, Pts, A, R, Off, kSum> B;
  static typename B::type make(const DSumStencil<T, Pts, A>& d) {
    typename B::type t;
    t.a = B::TA::make(d.a);
    for (int i = 0; i < Pts::length; ++i) t.c[i] = 0.0;
    return t;
  }
};

#ifdef __CUDACC__
// apply_pointwise operands
template <class Tup, class R, int Off>
struct TileTuple;
template <class R, int Off>
struct TileTuple<DTuple<>, R, Off> {
  typedef DTuple<> type;
  enum { end = Off, rounds = 0 };
  static type make(const DTuple<>&) { return type(); }
};
template <class H, class... Rest, class R, int Off>
struct TileTuple<DTuple<H, Rest...>, R, Off> {
  typedef Tile<H, R, Off> TH;
  typedef TileTuple<DTuple<Rest...>, R, TH::end> TR;
  typedef DTuple<typename TH::type, typename TR::type> Dummy;
  enum { end = TR::end, rounds = cmax(TH::rounds, TR::rounds) };
  template <class TRT>
  struct Cons;
  template <class... X>
  struct Cons<DTuple<X...>> {
    typedef DTuple<typename TH::type, X...> type;
  };
  typedef typename Cons<typename TR::type>::type type;
  static type make(const DTuple<H, Rest...>& t) {
    type o;
    o.h = TH::make(t.h);
    o.r = TR::make(t.r);
    return o;
  }
};
template <typename T, class Fn, class... D, class R, int Off>
struct Tile<DApply<T, Fn, D...>, R, Off> {
  typedef TileTuple<DTuple<D...>, R, Off> TT;
  template <class TupT>
  struct Of;
  template <class... X>
  struct Of<DTuple<X...>> {
    typedef DApply<T, Fn, X...> type;
  };
  typedef typename Of<typename TT::type>::type type;
  enum { end = TT::end, rounds = TT::rounds };
  static type make(const DApply<T, Fn, D...>& d) {
    type o;
    o.ops = TT::make(d.ops);
    return o;
  }
};
#endif

// ---------------------------------------------------------------------------- stencil composition
// In builds that allow reassociation (and not NEBO_UNTILED), a weighted stencil whose argument
// is a weighted stencil becomes ONE weighted stencil of the inner argument: its points are the
// sums p + q of the outer and inner points (the Minkowski sum, each sum listed once), and a
// point's coefficient is the sum of the products c_outer[i] * c_inner[j] of the pairs landing
// on it, computed on the host once per launch.  Interp(Grad(Interp(a))) thus becomes the
// 4-point stencil (g/4) * (-a[i-2] - a[i-1] + a[i] + a[i+1]) of the field a, read directly
// instead of materialised level by level.  The composed stencil reads exactly the points the
// nested sums read (the write region's guarantee holds); its values differ from the nested
// evaluation by rounding only.  Compositions of more than kComposeMaxPoints points, box sums
// and stencils of different value types are left as they are.
constexpr int kComposeMaxPoints = 27;
#if defined(NEBO_EXACT_ARITHMETIC) || defined(NEBO_UNTILED)
constexpr bool kCompose = false;
#else
constexpr bool kCompose = true;
#endif

template <class L, class P>
struct HasPt;
template <class P>
struct HasPt<NeboNil, P> : std::false_type {};
template <class Q, class R, class P>
struct HasPt<NeboStencilPointCollection<Q, R>, P>
    : std::integral_constant<bool, (Q::X == P::X && Q::Y == P::Y && Q::Z == P::Z) || HasPt<R, P>::value> {};

// L with P appended as its last-listed point, unless L holds P already (L may be NeboNil)
template <class L, class P>
struct PushPt {
  typedef typename std::conditional<HasPt<L, P>::value, L, NeboStencilPointCollection<P, L>>::type type;
};

// Acc with every point of L (in listed order) shifted by Q appended
template <class Acc, class L, class Q>
struct AddShifted;
template <class Acc, class Q>
struct AddShifted<Acc, NeboNil, Q> {
  typedef Acc type;
};
template <class Acc, class P, class R, class Q>
struct AddShifted<Acc, NeboStencilPointCollection<P, R>, Q> {
  typedef typename AddShifted<Acc, R, Q>::type A1;  // R holds the points listed before P
  typedef typename PushPt<A1, IndexTriplet<P::X + Q::X, P::Y + Q::Y, P::Z + Q::Z>>::type type;
};

// Minkowski sum of two point collections: for each q of L2 in listed order, L1 shifted by q
template <class Acc, class L1, class L2>
struct MinkAcc;
template <class Acc, class L1>
struct MinkAcc<Acc, L1, NeboNil> {
  typedef Acc type;
};
template <class Acc, class L1, class Q, class R>
struct MinkAcc<Acc, L1, NeboStencilPointCollection<Q, R>> {
  typedef typename MinkAcc<Acc, L1, R>::type A1;
  typedef typename AddShifted<A1, L1, Q>::type type;
};
template <class L1, class L2>
struct MinkSum {
  typedef typename MinkAcc<NeboNil, L1, L2>::type type;
};

// The points of a collection by listed index (the index of a point's coefficient), host side.
template <class L>
struct PtsAt;
template <>
struct PtsAt<NeboNil> {
  static int x(int) { return 0; }
  static int y(int) { return 0; }
  static int z(int) { return 0; }
  static int index_of(int, int, int) { return -1; }
};
template <class P, class R>
struct PtsAt<NeboStencilPointCollection<P, R>> {
  static int x(int i) { return i == R::length ? P::X : PtsAt<R>::x(i); }
  static int y(int i) { return i == R::length ? P::Y : PtsAt<R>::y(i); }
  static int z(int i) { return i == R::length ? P::Z : PtsAt<R>::z(i); }
  static int index_of(int px, int py, int pz) {
    return (P::X == px && P::Y == py && P::Z == pz) ? R::length : PtsAt<R>::index_of(px, py, pz);
  }
};

// An outer stencil (points P1, coefficients c1) over an already composed argument AC.
template <typename T, class P1, class AC, class Enable = void>
struct StencilMerge {  // kept nested
  typedef DStencil<T, P1, AC> type;
  static type make(const double* c1, const AC& a) {
    type o;
    o.a = a;
    for (int i = 0; i < P1::length; ++i) o.c[i] = c1[i];
    return o;
  }
};
template <typename T, class P1, class P2, class A2>
struct StencilMerge<T, P1, DStencil<T, P2, A2>,
                    typename std::enable_if<kCompose && (MinkSum<P1, P2>::type::length <= kComposeMaxPoints)>::type> {
  typedef typename MinkSum<P1, P2>::type PM;
  typedef DStencil<T, PM, A2> type;
  static type make(const double* c1, const DStencil<T, P2, A2>& in) {
    type o;
    o.a = in.a;
    for (int k = 0; k < PM::length; ++k) o.c[k] = 0.0;
    for (int i = 0; i < P1::length; ++i)
      for (int j = 0; j < P2::length; ++j) {
        const int k = PtsAt<PM>::index_of(PtsAt<P1>::x(i) + PtsAt<P2>::x(j), PtsAt<P1>::y(i) + PtsAt<P2>::y(j),
                                          PtsAt<P1>::z(i) + PtsAt<P2>::z(j));
        o.c[k] += c1[i] * in.c[j];
      }
    return o;
  }
};

// Compose<D>: D with every composable stencil pair merged (identity for anything else).
template <class D>
struct Compose {
  typedef D type;
  static type make(const D& d) { return d; }
};
template <class Op, typename T, class A, class B>
struct Compose<DBin<Op, T, A, B>> {
  typedef Compose<A> CA;
  typedef Compose<B> CB;
  typedef DBin<Op, T, typename CA::type, typename CB::type> type;
  static type make(const DBin<Op, T, A, B>& d) { return type{CA::make(d.a), CB::make(d.b)}; }
};
template <class Fn, typename T, class A>
struct Compose<DUn<Fn, T, A>> {
  typedef Compose<A> CA;
  typedef DUn<Fn, T, typename CA::type> type;
  static type make(const DUn<Fn, T, A>& d) { return type{CA::make(d.a)}; }
};
template <typename T, class A>
struct Compose<DPowInt<T, A>> {
  typedef Compose<A> CA;
  typedef DPowInt<T, typename CA::type> type;
  static type make(const DPowInt<T, A>& d) { return type{CA::make(d.a), d.e}; }
};
template <class Op, class A, class B>
struct Compose<DCmp<Op, A, B>> {
  typedef Compose<A> CA;
  typedef Compose<B> CB;
  typedef DCmp<Op, typename CA::type, typename CB::type> type;
  static type make(const DCmp<Op, A, B>& d) { return type{CA::make(d.a), CB::make(d.b)}; }
};
template <class Op, class A, class B>
struct Compose<DLogic<Op, A, B>> {
  typedef Compose<A> CA;
  typedef Compose<B> CB;
  typedef DLogic<Op, typename CA::type, typename CB::type> type;
  static type make(const DLogic<Op, A, B>& d) { return type{CA::make(d.a), CB::make(d.b)}; }
};
template <class A>
struct Compose<DNot<A>> {
  typedef Compose<A> CA;
  typedef DNot<typename CA::type> type;
  static type make(const DNot<A>& d) { return type{CA::make(d.a)}; }
};
template <typename T, class Test, class Val, class Rest>
struct Compose<DCond<T, Test, Val, Rest>> {
  typedef Compose<Test> CT;
  typedef Compose<Val> CV;
  typedef Compose<Rest> CR;
  typedef DCond<T, typename CT::type, typename CV::type, typename CR::type> type;
  static type make(const DCond<T, Test, Val, Rest>& d) { return type{CT::make(d.t), CV::make(d.v), CR::make(d.r)}; }
};
template <typename T, class Pts, class A>
struct Compose<DSumStencil<T, Pts, A>> {
  typedef Compose<A> CA;
  typedef DSumStencil<T, Pts, typename CA::type> type;
  static type make(const DSumStencil<T, Pts, A>& d) { return type{CA::make(d.a)}; }
};
template <typename T, class P1, class A>
struct Compose<DStencil<T, P1, A>> {
  typedef Compose<A> CA;
  typedef StencilMerge<T, P1, typename CA::type> M;
  typedef typename M::type type;
  static type make(const DStencil<T, P1, A>& d) { return M::make(d.c, CA::make(d.a)); }
};

// The plan for a functor: the tile depth TZ whose buffers fit the budget, or 0 when no stencil
// needs a buffer (or none fits): the plain kernel then runs.
template <class D, int TZ>
struct TileAt {
  typedef Tile<D, TBox<0, kTileX - 1, 0, kTileY - 1, 0, TZ - 1>, 0> type;
};
template <class D>
struct TilePlan {
  enum {
    rounds = TileAt<D, 8>::type::rounds,
    tz = rounds == 0 ? 0
         : (int)TileAt<D, 8>::type::end <= kTileSmemBudget ? 8
         : (int)TileAt<D, 4>::type::end <= kTileSmemBudget ? 4
         : (int)TileAt<D, 2>::type::end <= kTileSmemBudget ? 2
         : (int)TileAt<D, 1>::type::end <= kTileSmemBudget ? 1 : 0
  };
};

#ifdef __CUDACC__
template <int H>
struct FillRounds {
  template <class F>
  static __device__ __forceinline__ void run(const F& f, int tx, int ty, int tz) {
    FillRounds<H - 1>::run(f, tx, ty, tz);
    f.template fill<H>(tx, ty, tz);
    __syncthreads();
  }
};
template <>
struct FillRounds<0> {
  template <class F>
  static __device__ __forceinline__ void run(const F&, int, int, int) {}
};

// One block per 32 x 8 x TZ tile of the write region (interior-relative limits).
template <typename T, class DT, int TZ, int ROUNDS>
__global__ void __launch_bounds__(kTileThreads) nebo_tiled_assign_kernel(T* __restrict__ out, int sy, long sz, int xlo,
                                                                        int xhi, int ylo, int yhi, int zlo, int zhi,
                                                                        DT rhs) {
  const int x0 = xlo + (int)blockIdx.x * kTileX;
  const int y0 = ylo + (int)blockIdx.y * kTileY;
  const int z0 = zlo + (int)blockIdx.z * TZ;
  const int nx = cmin(kTileX, xhi - x0), ny = cmin(kTileY, yhi - y0), nz = cmin(TZ, zhi - z0);
  DT f = rhs;
  f.rebase(x0, y0, z0);
  FillRounds<ROUNDS>::run(f, kTileX - nx, kTileY - ny, TZ - nz);
  const int lx = (int)threadIdx.x, ly = (int)threadIdx.y;
  if (lx >= nx || ly >= ny) return;
  T* o = out + ((long)x0 + lx) + (long)sy * (y0 + ly) + sz * z0;
  int lz = 0;
#pragma unroll 1
  for (; lz + 1 < nz; lz += 2) {
    T v0, v1;
    PairZ<T, DT>::eval(f, lx, ly, lz, v0, v1);
    o[sz * lz] = v0;
    o[sz * (lz + 1)] = v1;
  }
  if (lz < nz) o[sz * lz] = f.eval(lx, ly, lz);
}
#endif

}  // namespace nebo_detail
}  // namespace SpatialOps
#endif
