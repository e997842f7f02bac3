// MemoryWindow: a window (offset, extent) into a global x-fastest allocation
// (drop-in for spatialops/structured/MemoryWindow.h, including get_window_with_ghost).
#ifndef SpatialOps_MemoryWindow_h
#define SpatialOps_MemoryWindow_h

#include <cstddef>

#include <spatialops/structured/BoundaryCellInfo.h>
#include <spatialops/structured/GhostData.h>
#include <spatialops/structured/IntVec.h>

namespace SpatialOps {

class MemoryWindow {
  IntVec nptsGlob_, offset_, extent_;

 public:
  explicit MemoryWindow(const IntVec& npts) : nptsGlob_(npts), offset_(0, 0, 0), extent_(npts) {}
  MemoryWindow(const IntVec& glob, const IntVec& offset, const IntVec& extent)
      : nptsGlob_(glob), offset_(offset), extent_(extent) {}
  MemoryWindow(const int npts[3]) : nptsGlob_(npts), offset_(0, 0, 0), extent_(npts) {}

  size_t glob_dim(int i) const { return (size_t)nptsGlob_[i]; }
  IntVec glob_dim() const { return nptsGlob_; }
  size_t offset(int i) const { return (size_t)offset_[i]; }
  IntVec offset() const { return offset_; }
  size_t extent(int i) const { return (size_t)extent_[i]; }
  IntVec extent() const { return extent_; }
  IntVec extents() const { return extent_; }
  size_t glob_npts() const { return (size_t)nptsGlob_[0] * nptsGlob_[1] * nptsGlob_[2]; }
  size_t local_npts() const { return (size_t)extent_[0] * extent_[1] * extent_[2]; }
  // Window-relative (i,j,k) -> allocation index; an axis of allocation extent 1 is always index 0
  // (MemoryWindow.h:121-131 of the reference).
  size_t flat_index(IntVec loc) const {
    for (int d = 0; d < 3; ++d) loc[d] = nptsGlob_[d] > 1 ? loc[d] + offset_[d] : 0;
    return (size_t)loc[0] + (size_t)nptsGlob_[0] * ((size_t)loc[1] + (size_t)nptsGlob_[1] * (size_t)loc[2]);
  }
  bool fits_between(const MemoryWindow& inner, const MemoryWindow& outer) const {
    for (int i = 0; i < 3; ++i) {
      if (offset_[i] > inner.offset_[i] || offset_[i] < outer.offset_[i]) return false;
      if (offset_[i] + extent_[i] < inner.offset_[i] + inner.extent_[i]) return false;
      if (offset_[i] + extent_[i] > outer.offset_[i] + outer.extent_[i]) return false;
    }
    return true;
  }
  MemoryWindow remove_ghosts(const GhostData& g) const {
    return MemoryWindow(nptsGlob_, offset_ + g.get_minus(), extent_ - g.get_minus() - g.get_plus());
  }
  MemoryWindow reset_ghosts(const GhostData& oldg, const GhostData& newg) const {
    return MemoryWindow(nptsGlob_, offset_ + oldg.get_minus() - newg.get_minus(),
                        extent_ - oldg.get_minus() - oldg.get_plus() + newg.get_minus() + newg.get_plus());
  }
  bool operator==(const MemoryWindow& o) const {
    return nptsGlob_ == o.nptsGlob_ && offset_ == o.offset_ && extent_ == o.extent_;
  }
  bool operator!=(const MemoryWindow& o) const { return !(*this == o); }
  bool sanity_check() const {
    for (int i = 0; i < 3; ++i)
      if (extent_[i] < 1 || offset_[i] < 0 || offset_[i] + extent_[i] > nptsGlob_[i]) return false;
    return true;
  }
};

inline int get_dim_with_ghost(int nNoGhost, int minusGhost, int plusGhost, int bc) {
  return nNoGhost > 1 ? nNoGhost + minusGhost + plusGhost + bc : 1;
}

inline MemoryWindow get_window_with_ghost(const IntVec& localDim, const GhostData& ghost, const BoundaryCellInfo& bc) {
  return MemoryWindow(IntVec(get_dim_with_ghost(localDim[0], ghost.get_minus(0), ghost.get_plus(0), bc.has_extra(0)),
                             get_dim_with_ghost(localDim[1], ghost.get_minus(1), ghost.get_plus(1), bc.has_extra(1)),
                             get_dim_with_ghost(localDim[2], ghost.get_minus(2), ghost.get_plus(2), bc.has_extra(2))));
}

}  // namespace SpatialOps
#endif
