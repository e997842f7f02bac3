// Grid: a uniform mesh of npts cells over a box of the given length, and the coordinates of a
// field's points (drop-in for spatialops/structured/Grid.h and Grid.cpp:36-102).
//
// set_coord<Dir>(f) writes, at every point of f's window (ghosts included), the coordinate
//     spacing[dir] * (i[dir] - interior offset[dir]) + shift * spacing[dir],
// shift = (1 + the location's staggering offset along dir) / 2: 0.5 for cell centres, 0 for
// faces.  The values are written through the host mirror, as the reference does on a GPU field.
#ifndef SpatialOps_structured_Grid_h
#define SpatialOps_structured_Grid_h

#include <cassert>

#include <spatialops/structured/DoubleVec.h>
#include <spatialops/structured/IndexTriplet.h>
#include <spatialops/structured/IntVec.h>
#include <spatialops/structured/MemoryWindow.h>

namespace SpatialOps {

class Grid {
  const IntVec npts_;
  const DoubleVec length_, spacing_;

 public:
  Grid(const IntVec npts, const DoubleVec length) : npts_(npts), length_(length), spacing_(length / npts) {}

  template <typename CoordT>
  double spacing() const {
    return spacing_[CoordT::value];
  }
  const DoubleVec& spacing() const { return spacing_; }
  const IntVec& extent() const { return npts_; }
  int extent(const size_t i) const {
    assert(i < 3);
    return npts_[(int)i];
  }
  const DoubleVec& length() const { return length_; }
  double length(const size_t i) const {
    assert(i < 3);
    return length_[(int)i];
  }

  template <typename CoordT, typename FieldT>
  void set_coord(FieldT& f) const {
    const int dir = CoordT::value;
    const double offset = 0.5 * double(1 + FieldT::Location::Offset::value(dir)) * spacing_[dir];
    const MemoryWindow mwInterior = f.window_without_ghost();
    const MemoryWindow& mw = f.window_with_ghost();
    const IntVec hi = mw.extent();
    const int ixOffset = (int)mwInterior.offset(dir);
    IntVec ix;
    for (ix[2] = 0; ix[2] < hi[2]; ++ix[2])
      for (ix[1] = 0; ix[1] < hi[1]; ++ix[1])
        for (ix[0] = 0; ix[0] < hi[0]; ++ix[0]) {
          // product and sum rounded separately (no fused multiply-add), as on the reference's host
          volatile double t = spacing_[dir] * double(ix[dir] - ixOffset);
          f(ix) = t + offset;
        }
  }
};

}  // namespace SpatialOps
#endif
