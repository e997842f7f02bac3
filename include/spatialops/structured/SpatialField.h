// SpatialField: a handle to one field on a structured, ghosted window
// (drop-in for spatialops/structured/SpatialField.h:128-603 and the FieldInfo state of
// spatialops/structured/FieldInfo.h:92-415).
//
// GB300 design: the values always live in one device allocation (from the library's
// stream-ordered pool, nebo_alloc); a host mirror exists only while host code touches the field
// (field_values(CPU_INDEX), operator[], iterators).  Validity flags decide when to copy:
//   * a const host access downloads the device copy if the mirror is stale;
//   * a non-const host access also marks the device copy stale, so the next `<<=` that reads the
//     field uploads it first;
//   * every `<<=` into the field leaves the device copy valid and the mirror stale.
// Copies of a SpatialField are shallow (they share the storage), as in the reference.
#ifndef SpatialOps_SpatialField_h
#define SpatialOps_SpatialField_h

#include <cstring>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <vector>

#include <nebo_gb300.h>
#include <spatialops/structured/BoundaryCellInfo.h>
#include <spatialops/structured/FVStaggeredLocationTypes.h>
#include <spatialops/structured/GhostData.h>
#include <spatialops/structured/MemoryTypes.h>
#include <spatialops/structured/MemoryWindow.h>

namespace SpatialOps {

namespace nebo_detail {

inline void throw_status(int rc, const char* where) {
  if (rc == NEBO_OK) return;
  std::ostringstream msg;
  const char* last = nebo_last_error();
  if (last && *last)
    msg << last;
  else
    msg << "Nebo error in " << where << ": " << nebo_status_string(rc);
  throw std::runtime_error(msg.str());
}

template <typename T> struct DType;
template <> struct DType<double> { enum { value = NEBO_F64 }; };
template <> struct DType<float> { enum { value = NEBO_F32 }; };

// Shared state of all copies of one field (the role of FieldInfo).
template <typename T>
struct FieldStore {
  size_t npts = 0;
  T* dev = nullptr;
  bool ownsDev = false;
  T* hostExt = nullptr;        // caller-owned host storage (ExternalStorage on CPU_INDEX)
  std::vector<T> hostOwn;      // mirror allocated on demand
  bool devValid = true;
  bool hostValid = false;
  nebo_stream_t stream = nullptr;

  ~FieldStore() {
    if (ownsDev && dev) nebo_free(dev, stream);
  }
  T* host_base() {
    if (hostExt) return hostExt;
    if (hostOwn.size() != npts) hostOwn.resize(npts);
    return hostOwn.data();
  }
  void download() {
    if (hostValid) return;
    T* h = host_base();
    if (devValid) {
      throw_status(nebo_memcpy_d2h(h, dev, npts * sizeof(T), stream), "SpatialField host copy");
      throw_status(nebo_stream_sync(stream), "SpatialField host copy");
    }
    hostValid = true;
  }
  void upload() {
    if (devValid) return;
    throw_status(nebo_memcpy_h2d(dev, host_base(), npts * sizeof(T), stream), "SpatialField device copy");
    throw_status(nebo_stream_sync(stream), "SpatialField device copy");
    devValid = true;
  }
};

}  // namespace nebo_detail

template <typename FieldLocation, typename T = double>
class SpatialField {
 public:
  typedef SpatialField<FieldLocation, T> field_type;
  typedef FieldLocation Location;
  typedef T value_type;
  typedef MemoryWindow memory_window;
  typedef T* iterator;
  typedef const T* const_iterator;

 private:
  MemoryWindow localWindow_;
  BoundaryCellInfo bcInfo_;
  GhostData totalGhosts_;
  GhostData localValidGhosts_;
  std::shared_ptr<nebo_detail::FieldStore<T>> info_;

 public:
  SpatialField(const MemoryWindow window, const BoundaryCellInfo bc, const GhostData ghosts, T* const fieldValues = NULL,
               const StorageMode mode = InternalStorage, const short int devIdx = CPU_INDEX)
      : localWindow_(window),
        bcInfo_(bc.limit_by_extent(window.extent())),
        totalGhosts_(ghosts.limit_by_extent(window.extent())),
        localValidGhosts_(ghosts.limit_by_extent(window.extent())),
        info_(std::make_shared<nebo_detail::FieldStore<T>>()) {
    auto& s = *info_;
    s.npts = window.glob_npts();
    if (mode == ExternalStorage && fieldValues && IS_GPU_INDEX(devIdx)) {
      s.dev = fieldValues;  // caller's device memory, used in place
      s.ownsDev = false;
      s.devValid = true;
      return;
    }
    void* p = nullptr;
    nebo_detail::throw_status(nebo_alloc(s.npts * sizeof(T), &p, s.stream), "SpatialField allocation");
    s.dev = static_cast<T*>(p);
    s.ownsDev = true;
    if (fieldValues && mode == ExternalStorage) {
      s.hostExt = fieldValues;  // host storage shared with the caller: current contents are the values
      s.hostValid = true;
      s.devValid = false;
    } else if (fieldValues) {
      std::memcpy(s.host_base(), fieldValues, s.npts * sizeof(T));  // internal copy of the initial values
      s.hostValid = true;
      s.devValid = false;
    } else {
      nebo_detail::throw_status(nebo_memset(s.dev, 0, s.npts * sizeof(T), s.stream), "SpatialField allocation");
      s.devValid = true;
    }
  }

  SpatialField(const SpatialField& o) = default;
  SpatialField(const MemoryWindow window, const SpatialField& o)
      : localWindow_(window),
        bcInfo_(o.bcInfo_),
        totalGhosts_(o.totalGhosts_),
        localValidGhosts_(o.localValidGhosts_.limit_by_extent(window.extent())),
        info_(o.info_) {}

  // Deep copy of values (the reference's SpatialField::operator=).
  SpatialField& operator=(const SpatialField& o) {
    if (info_ == o.info_) return *this;
    if (localWindow_.glob_npts() != o.localWindow_.glob_npts())
      throw std::runtime_error("Nebo error in SpatialField::operator=: fields differ in size");
    o.info_->upload();
    nebo_detail::throw_status(
        nebo_memcpy_d2d(info_->dev, o.info_->dev, info_->npts * sizeof(T), info_->stream), "SpatialField copy");
    info_->devValid = true;
    info_->hostValid = false;
    return *this;
  }

  const MemoryWindow& window_with_ghost() const { return localWindow_; }
  MemoryWindow window_without_ghost() const { return localWindow_.remove_ghosts(localValidGhosts_); }
  const BoundaryCellInfo& boundary_info() const { return bcInfo_; }
  const GhostData& get_ghost_data() const { return totalGhosts_; }
  const GhostData& get_valid_ghost_data() const { return localValidGhosts_; }
  void reset_valid_ghosts(const GhostData& input) {
    const GhostData g = input.limit_by_extent(localWindow_.extent());
    localWindow_ = localWindow_.reset_ghosts(localValidGhosts_, g);
    localValidGhosts_ = g;
  }
  unsigned int allocated_bytes() const { return (unsigned int)(info_->npts * sizeof(T)); }

  // Stream on which this field's copies and the kernels that write it run.
  void set_stream(const nebo_stream_t& s) { info_->stream = s; }
  const nebo_stream_t& get_stream() const { return info_->stream; }
  void wait_for_synchronization() { nebo_detail::throw_status(nebo_stream_sync(info_->stream), "SpatialField sync"); }

  short int active_device_index() const { return GPU_INDEX; }
  bool is_valid(short int idx) const { return IS_CPU_INDEX(idx) ? info_->hostValid : info_->devValid; }
  void add_device(short int idx) {
    if (IS_CPU_INDEX(idx))
      info_->download();
    else
      info_->upload();
  }
  void set_device_as_active(short int idx) { add_device(idx); }
  void validate_device(short int idx) { add_device(idx); }

  // Raw values on a device (CPU_INDEX: the host mirror).  The non-const host form marks the
  // device copy stale.
  T* field_values(short int idx = CPU_INDEX) {
    if (IS_CPU_INDEX(idx)) {
      info_->download();
      info_->devValid = false;
      return info_->host_base();
    }
    info_->upload();
    info_->hostValid = false;
    return info_->dev;
  }
  const T* field_values(short int idx = CPU_INDEX) const {
    if (IS_CPU_INDEX(idx)) {
      info_->download();
      return info_->host_base();
    }
    info_->upload();
    return info_->dev;
  }

  // Host element access in the window's flat (glob) index space.
  T& operator[](size_t i) { return field_values(CPU_INDEX)[i]; }
  const T& operator[](size_t i) const { return field_values(CPU_INDEX)[i]; }
  T& operator()(int i, int j, int k) { return field_values(CPU_INDEX)[localWindow_.flat_index(IntVec(i, j, k))]; }
  const T& operator()(int i, int j, int k) const {
    return field_values(CPU_INDEX)[localWindow_.flat_index(IntVec(i, j, k))];
  }
  T& operator()(const IntVec& ijk) { return (*this)(ijk[0], ijk[1], ijk[2]); }

  iterator begin() { return field_values(CPU_INDEX); }
  iterator end() { return field_values(CPU_INDEX) + info_->npts; }
  const_iterator begin() const { return field_values(CPU_INDEX); }
  const_iterator end() const { return field_values(CPU_INDEX) + info_->npts; }

  // ---- used by the expression engine (not part of the reference API)
  // Device pointer after making the device copy current (uploading host edits).
  T* device_values_for_read() const {
    info_->upload();
    return info_->dev;
  }
  // Device pointer for a kernel that writes part of the field: the device copy must be current
  // (cells outside the write region keep their values); afterwards the mirror is stale.
  T* device_values_for_write() {
    info_->upload();
    info_->hostValid = false;
    return info_->dev;
  }
  nebo_field descriptor() const {
    nebo_field d;
    d.data = info_->dev;
    for (int i = 0; i < 3; ++i) {
      d.glob[i] = (int32_t)localWindow_.glob_dim(i);
      d.offset[i] = (int32_t)localWindow_.offset(i);
      d.extent[i] = (int32_t)localWindow_.extent(i);
      d.ghost_minus[i] = localValidGhosts_.get_minus(i);
      d.ghost_plus[i] = localValidGhosts_.get_plus(i);
      d.has_bc[i] = bcInfo_.has_bc(i) ? 1 : 0;
      d.bc_extra[i] = bcInfo_.has_extra(i);
    }
    d.dtype = nebo_detail::DType<T>::value;
    return d;
  }
  // Interior extents (window minus valid ghosts; BC cells included), as NeboConstField::extents.
  IntVec interior_extent() const {
    return localWindow_.extent() - localValidGhosts_.get_minus() - localValidGhosts_.get_plus();
  }
  // Flat offset of interior-relative (0,0,0) within the allocation.
  long interior_origin() const {
    return (long)(localWindow_.offset(0) + localValidGhosts_.get_minus(0)) +
           (long)localWindow_.glob_dim(0) *
               ((long)(localWindow_.offset(1) + localValidGhosts_.get_minus(1)) +
                (long)localWindow_.glob_dim(1) * (long)(localWindow_.offset(2) + localValidGhosts_.get_minus(2)));
  }
};

}  // namespace SpatialOps
#endif
