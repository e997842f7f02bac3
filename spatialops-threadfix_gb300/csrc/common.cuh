// Shared helpers of the sm_103a Nebo library: status/error plumbing, descriptor checks and the
// device-side view of a field (the reference's NeboField/NeboConstField GPUWalk indexing,
// spatialops/NeboLhs.h:632-699 and spatialops/NeboRhs.h:294-327).
#pragma once

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>

#include "nebo_gb300.h"

namespace nebo {

// Record a message for nebo_last_error() and return the status.
int fail(int status, const char* fmt, ...);
// Map a CUDA error to NEBO_ERR_LAUNCH (or NEBO_OK) with context.
int cuda_fail(cudaError_t e, const char* where);

#define NEBO_CUDA_TRY(call)                                   \
  do {                                                        \
    cudaError_t e_ = (call);                                  \
    if (e_ != cudaSuccess) return ::nebo::cuda_fail(e_, #call); \
  } while (0)

#define NEBO_LAUNCH_CHECK(where)                              \
  do {                                                        \
    cudaError_t e_ = cudaGetLastError();                      \
    if (e_ != cudaSuccess) return ::nebo::cuda_fail(e_, where); \
  } while (0)

inline size_t elem_size(int dtype) { return dtype == NEBO_F32 ? 4 : 8; }

// Interior extents of a field: window extent minus valid ghosts (includes BC cells).
inline void interior_extent(const nebo_field& f, int n[3]) {
  for (int i = 0; i < 3; ++i) n[i] = f.extent[i] - f.ghost_minus[i] - f.ghost_plus[i];
}

// Structural checks every entry point applies to a descriptor.
int check_field(const nebo_field* f, const char* what);
// Bounded device-side waits that gave up since the last call (heat.cu; cleared by the read).
int bulk_wait_timeouts(unsigned int* count);
// The same for the patch kernels (patches.cu).
int patch_wait_timeouts(unsigned int* count);
// The same for the tensor-staged transport stage kernel (transport.cu).
int transport_wait_timeouts(unsigned int* count);
// Same shape, ghosts and dtype.
int check_same_layout(const nebo_field* a, const nebo_field* b, const char* what);
// Uniform periodic patch: equal ghosts g on all six faces, no BC cells, window == allocation.
int check_periodic_patch(const nebo_field* f, int g, const char* what);

// Device view: interior-relative (x,y,z) -> element.
template <typename T>
struct View {
  T* base;  // element (0,0,0) of the interior
  int sy;   // glob[0]
  long sz;  // glob[0]*glob[1]
  __host__ __device__ long idx(int x, int y, int z) const { return (long)x + (long)sy * y + sz * z; }
};

template <typename T>
inline View<T> make_view(const nebo_field& f) {
  View<T> v;
  v.sy = f.glob[0];
  v.sz = (long)f.glob[0] * f.glob[1];
  v.base = static_cast<T*>(f.data) + (long)(f.offset[0] + f.ghost_minus[0]) +
           (long)v.sy * (f.offset[1] + f.ghost_minus[1]) + v.sz * (f.offset[2] + f.ghost_minus[2]);
  return v;
}

// Counts one kernel launch and, while profiling is on, times it with events on its stream.
// Construct immediately before the launch; the destructor records the end event.
class LaunchScope {
 public:
  LaunchScope(const char* name, cudaStream_t s);
  ~LaunchScope();
  LaunchScope(const LaunchScope&) = delete;
  LaunchScope& operator=(const LaunchScope&) = delete;

 private:
  const char* name_;
  cudaStream_t s_;
  void* a_;
  void* b_;
};

// Make the current device's default memory pool keep freed blocks (release threshold = max) so
// that stream-ordered allocations that recur every step (work lists, entry lists) are served
// from the pool instead of new CUDA driver allocations.  Once per device; a process-local pool
// setting.
void pool_retain();

// Periodic ghost fill of one uniform-ghost patch (ghost.cu).
int fill_periodic_any(const nebo_field* f, cudaStream_t s);

// SM count of the current device, queried once (callers on several threads may race to the
// first query; they store the same value).
inline int num_sms() {
  static std::atomic<int> cached{0};
  int n = cached.load(std::memory_order_relaxed);
  if (!n) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 152;
    cached.store(n, std::memory_order_relaxed);
  }
  return n;
}

// Resident blocks per SM of `kernel` at `threads` threads and no dynamic shared memory, kept in
// the caller's `cache` after the first query (same race rule as num_sms).
template <class K>
inline int blocks_per_sm(K kernel, int threads, std::atomic<int>& cache) {
  int v = cache.load(std::memory_order_relaxed);
  if (!v) {
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, kernel, threads, 0) != cudaSuccess || v <= 0) {
      cudaGetLastError();
      v = 1;
    }
    cache.store(v, std::memory_order_relaxed);
  }
  return v;
}

// Planes per z chunk for a kernel whose blocks each walk zc planes of one (x, y) tile: the zc
// (a multiple of `align`, at least min_planes unless nz is smaller) that minimises
// rounds * (zc + overhead), where rounds = ceil(blocks / slots) is the number of waves of
// `slots` resident blocks and `overhead` the planes a chunk reads beyond its own (halo, ring
// fill).  Splits of at least six waves are preferred when the field allows them: blocks that
// start at staggered times keep every SM busy to the end (a sweep of zc on the FP64 heat step
// at 192^3 and 256^3 and the FP32 transport stage at 256^3 found the fastest split there).
inline int wave_zchunk(long tiles, long slots, int nz, int overhead, int min_planes, int align) {
  if (tiles < 1) tiles = 1;
  if (slots < 1) slots = 1;
  const int lo = min_planes < nz ? min_planes : nz;
  const int top = (nz + align - 1) / align * align;
  int best_zc = top;
  for (int min_rounds = 6; min_rounds >= 1; min_rounds -= 5) {
    long best = -1;
    for (int zc = top; zc >= lo && zc >= 1; zc -= align) {
      const long chunks = (nz + zc - 1) / zc;
      const long rounds = (tiles * chunks + slots - 1) / slots;
      if (rounds < min_rounds) continue;
      const long cost = rounds * (zc + overhead);
      if (best < 0 || cost < best) {
        best = cost;
        best_zc = zc;
      }
    }
    if (best >= 0) break;
  }
  return best_zc;
}

}  // namespace nebo
