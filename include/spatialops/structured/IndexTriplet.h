// Compile-time index triplets used for staggering offsets and stencil points
// (drop-in for spatialops/structured/IndexTriplet.h: Add, Subtract, Multiply, LessThan,
// GreaterThan, Negate, UnitTriplet, int_vec()).
#ifndef SpatialOps_IndexTriplet_h
#define SpatialOps_IndexTriplet_h

#include <spatialops/structured/IntVec.h>

namespace SpatialOps {

struct XDIR { enum { value = 0 }; };
struct YDIR { enum { value = 1 }; };
struct ZDIR { enum { value = 2 }; };
struct NODIR { enum { value = -10 }; };

template <int i1, int i2, int i3>
struct IndexTriplet {
  enum { X = i1, Y = i2, Z = i3 };
  typedef IndexTriplet<-i1, -i2, -i3> Negate;
  static IntVec int_vec() { return IntVec(i1, i2, i3); }
  NEBO_HD static constexpr int value(int d) { return d == 0 ? i1 : (d == 1 ? i2 : i3); }
  NEBO_HD static constexpr int value_gpu(int d) { return value(d); }
};

template <typename A, typename B> struct Add { typedef IndexTriplet<A::X + B::X, A::Y + B::Y, A::Z + B::Z> result; };
template <typename A, typename B> struct Subtract { typedef IndexTriplet<A::X - B::X, A::Y - B::Y, A::Z - B::Z> result; };
template <typename A, typename B> struct Multiply { typedef IndexTriplet<A::X * B::X, A::Y * B::Y, A::Z * B::Z> result; };
template <typename A, typename B>
struct LessThan {
  typedef IndexTriplet<((int)A::X < (int)B::X), ((int)A::Y < (int)B::Y), ((int)A::Z < (int)B::Z)> result;
};
template <typename A, typename B>
struct GreaterThan {
  typedef IndexTriplet<((int)A::X > (int)B::X), ((int)A::Y > (int)B::Y), ((int)A::Z > (int)B::Z)> result;
};

template <typename Dir> struct UnitTriplet;
template <> struct UnitTriplet<XDIR> { typedef IndexTriplet<1, 0, 0> type; };
template <> struct UnitTriplet<YDIR> { typedef IndexTriplet<0, 1, 0> type; };
template <> struct UnitTriplet<ZDIR> { typedef IndexTriplet<0, 0, 1> type; };
template <> struct UnitTriplet<NODIR> { typedef IndexTriplet<0, 0, 0> type; };

}  // namespace SpatialOps
#endif
