// SpatialMask: a set of points of a field's window, bit-packed on the GPU
// (drop-in for spatialops/structured/SpatialMask.h:67-276 with the word layout of
// spatialops/structured/BitField.h:291-333: bit flat%32 of word flat/32, x fastest over the
// ghosted window; points are interior-relative, ghost cells at -1 ...).
#ifndef SpatialOps_SpatialMask_h
#define SpatialOps_SpatialMask_h

#include <memory>
#include <vector>

#include <nebo_gb300.h>
#include <spatialops/structured/SpatialField.h>

namespace SpatialOps {

namespace nebo_detail {
struct MaskStore {
  uint32_t* words = nullptr;   // device bit words
  int32_t* points = nullptr;   // device point list (x,y,z) for masked_assign
  size_t nwords = 0;
  int npoints = 0;
  ~MaskStore() {
    if (words) nebo_free(words, nullptr);
    if (points) nebo_free(points, nullptr);
  }
};
}  // namespace nebo_detail

template <typename FieldType>
class SpatialMask {
 public:
  typedef FieldType field_type;
  typedef typename FieldType::Location Location;

 private:
  MemoryWindow maskWindow_;
  BoundaryCellInfo bcInfo_;
  GhostData ghosts_, validGhosts_;
  std::shared_ptr<std::vector<IntVec>> points_;
  std::shared_ptr<nebo_detail::MaskStore> store_;
  IntVec pmin_, pmax_;  // per-axis bounds of the points (when there are any)

  void build() {
    store_ = std::make_shared<nebo_detail::MaskStore>();
    const size_t npts = maskWindow_.glob_npts();
    store_->nwords = (npts + 31) / 32;
    void* w = nullptr;
    nebo_detail::throw_status(nebo_alloc(store_->nwords * 4, &w, nullptr), "SpatialMask allocation");
    store_->words = static_cast<uint32_t*>(w);
    nebo_detail::throw_status(nebo_memset(w, 0, store_->nwords * 4, nullptr), "SpatialMask allocation");
    std::vector<int32_t> host;
    host.reserve(points_->size() * 3);
    if (!points_->empty()) pmin_ = pmax_ = points_->front();
    for (const IntVec& p : *points_) {
      host.push_back(p[0]);
      host.push_back(p[1]);
      host.push_back(p[2]);
      for (int i = 0; i < 3; ++i) {
        pmin_[i] = p[i] < pmin_[i] ? p[i] : pmin_[i];
        pmax_[i] = p[i] > pmax_[i] ? p[i] : pmax_[i];
      }
    }
    store_->npoints = (int)points_->size();
    if (!host.empty()) {
      void* d = nullptr;
      nebo_detail::throw_status(nebo_alloc(host.size() * 4, &d, nullptr), "SpatialMask allocation");
      store_->points = static_cast<int32_t*>(d);
      nebo_detail::throw_status(nebo_memcpy_h2d(d, host.data(), host.size() * 4, nullptr), "SpatialMask upload");
      int32_t glob[3], off[3];
      for (int i = 0; i < 3; ++i) {
        glob[i] = (int32_t)maskWindow_.glob_dim(i);
        off[i] = (int32_t)maskWindow_.offset(i) + validGhosts_.get_minus(i);
      }
      nebo_detail::throw_status(
          nebo_mask_from_points(store_->words, glob, off, store_->points, store_->npoints, nullptr), "SpatialMask");
    }
  }

 public:
  SpatialMask(const MemoryWindow& window, const BoundaryCellInfo& bc, const GhostData& ghosts,
              const std::vector<IntVec>& points)
      : maskWindow_(window), bcInfo_(bc), ghosts_(ghosts), validGhosts_(ghosts),
        points_(std::make_shared<std::vector<IntVec>>(points)) {
    build();
  }
  SpatialMask(const FieldType& prototype, const std::vector<IntVec>& points)
      : maskWindow_(prototype.window_with_ghost()),
        bcInfo_(prototype.boundary_info()),
        ghosts_(prototype.get_ghost_data()),
        validGhosts_(prototype.get_valid_ghost_data()),
        points_(std::make_shared<std::vector<IntVec>>(points)) {
    build();
  }
  template <typename PrototypeType>
  static SpatialMask build(const PrototypeType& prototype, const std::vector<IntVec>& points) {
    return SpatialMask(prototype, points);
  }

  const std::vector<IntVec>& points() const { return *points_; }
  const MemoryWindow& window_with_ghost() const { return maskWindow_; }
  MemoryWindow window_without_ghost() const { return maskWindow_.remove_ghosts(validGhosts_); }
  const BoundaryCellInfo& boundary_info() const { return bcInfo_; }
  const GhostData& get_ghost_data() const { return ghosts_; }
  const GhostData& get_valid_ghost_data() const { return validGhosts_; }
  // masks are built on the GPU; these keep the reference's calls valid
  void add_consumer(short int) {}
  bool find_consumer(short int) const { return true; }
  const uint32_t* mask_values(short int = GPU_INDEX) const { return store_->words; }
  const int32_t* device_points() const { return store_->points; }
  int num_points() const { return store_->npoints; }
  // the smallest and largest coordinate of the points along each axis (num_points() > 0)
  const IntVec& point_min() const { return pmin_; }
  const IntVec& point_max() const { return pmax_; }
  long interior_origin() const {
    return (long)(maskWindow_.offset(0) + validGhosts_.get_minus(0)) +
           (long)maskWindow_.glob_dim(0) *
               ((long)(maskWindow_.offset(1) + validGhosts_.get_minus(1)) +
                (long)maskWindow_.glob_dim(1) * (long)(maskWindow_.offset(2) + validGhosts_.get_minus(2)));
  }
  IntVec interior_extent() const {
    return maskWindow_.extent() - validGhosts_.get_minus() - validGhosts_.get_plus();
  }
};

}  // namespace SpatialOps
#endif
