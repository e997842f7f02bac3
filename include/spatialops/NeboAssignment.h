// `<<=`, interior_assign and masked_assign (drop-in for spatialops/NeboAssignment.h:29-313 and
// the execution of spatialops/NeboLhs.h:67-283).
//
// lhs <<= expr:
//   1. the write region: calculate_actual_ghost(lhs ghosts, lhs BC, expr.ghosts_with_bc())
//      (nebo_write_limits in the C ABI, the reference's rule, spatialops/NeboBasic.h:61-100);
//   2. every field the expression reads is made current on the GPU;
//   3. ONE kernel evaluates the fused tree over the region:
//      * an expression with a stencil of an expression (a nested chain, a divergence of face
//        fluxes) runs as nebo_tiled_assign_kernel (NeboTiled.h): 32 x 8 x TZ tiles, each inner
//        level materialised once per tile in shared memory;
//      * any other runs as nebo_assign_kernel<T, Functor>: 32 lanes along x (coalesced), 8 warps
//        along y, and enough z-chunks for about 8 resident blocks per SM; each thread marches its
//        chunk of z planes.
//   NEBO_UNTILED keeps every expression on the second form (for comparisons).
#ifndef SpatialOps_NeboAssignment_h
#define SpatialOps_NeboAssignment_h

#include <cuda_runtime.h>

#include <atomic>
#include <cmath>

#include <spatialops/NeboCore.h>
#include <spatialops/NeboFactor.h>
#include <spatialops/NeboOperators.h>
#include <spatialops/NeboTiled.h>

namespace SpatialOps {
namespace nebo_detail {

template <typename T, class D>
__global__ void __launch_bounds__(256) nebo_assign_kernel(T* __restrict__ out, int sy, long sz, int xlo, int xhi, int ylo,
                                                          int yhi, int zlo, int zhi, int zchunk, D rhs) {
  const int x = xlo + (int)(blockIdx.x * 32 + threadIdx.x);
  const int y = ylo + (int)(blockIdx.y * 8 + threadIdx.y);
  if (x >= xhi || y >= yhi) return;
  const int z0 = zlo + (int)blockIdx.z * zchunk;
  const int z1 = z0 + zchunk < zhi ? z0 + zchunk : zhi;
  for (int z = z0; z < z1; ++z) out[(long)x + (long)sy * y + sz * z] = rhs.eval(x, y, z);
}

template <typename T, class D>
__global__ void __launch_bounds__(256) nebo_masked_assign_kernel(T* __restrict__ out, int sy, long sz,
                                                                 const int32_t* __restrict__ pts, int npts, D rhs) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < npts; i += gridDim.x * blockDim.x) {
    const int x = pts[3 * i], y = pts[3 * i + 1], z = pts[3 * i + 2];
    out[(long)x + (long)sy * y + sz * z] = rhs.eval(x, y, z);
  }
}

// SM count of the current device, cached per device.  Relaxed atomics: several host threads may
// launch at once; each either reads 0 (and queries) or a value some thread stored.
inline int device_sm_count() {
  constexpr int kMaxDevices = 64;
  static std::atomic<int> cache[kMaxDevices];
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    dev = 0;
  }
  const bool cached = dev >= 0 && dev < kMaxDevices;
  int n = cached ? cache[dev].load(std::memory_order_relaxed) : 0;
  if (n > 0) return n;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) {
    cudaGetLastError();
    n = 152;
  }
  if (cached) cache[dev].store(n, std::memory_order_relaxed);
  return n;
}

inline void throw_cuda(cudaError_t e, const char* where) {
  if (e == cudaSuccess) return;
  std::ostringstream msg;
  msg << "Nebo error in " << where << ":\n" << cudaGetErrorString(e);
  throw std::runtime_error(msg.str());
}

// Write region of lhs <<= rhs (interior-relative, [lo, hi) per axis); false if empty.
template <class F, class Node>
bool write_region(const F& lhs, const Node& rhs, bool useGhost, int32_t lim[6]) {
  const GhostData g = rhs.ghosts_with_bc();
  const nebo_field d = lhs.descriptor();
  int32_t m[3], p[3];
  for (int i = 0; i < 3; ++i) {
    m[i] = g.get_minus(i);
    p[i] = g.get_plus(i);
  }
  throw_status(nebo_write_limits(&d, useGhost ? 1 : 0, m, p, lim), "Nebo Assignment");
  return lim[1] > lim[0] && lim[3] > lim[2] && lim[5] > lim[4];
}

template <typename T, class D>
void assign_plain(T* out, int sy, long sz, const int32_t lim[6], const D& dev, cudaStream_t s);

// One kernel for functor D over the write region: tiled when D has a stencil of an expression.
template <typename T, class D>
void assign_launch(T* out, int sy, long sz, const int32_t lim[6], const D& dev, cudaStream_t s) {
#ifndef NEBO_UNTILED
  if constexpr (TilePlan<D>::tz > 0) {
    // nested stencils: one block per 32 x 8 x TZ tile, inner levels materialised in shared memory
    const int nx = lim[1] - lim[0], ny = lim[3] - lim[2], nz = lim[5] - lim[4];
    constexpr int TZ = TilePlan<D>::tz;
    typedef typename TileAt<D, TZ>::type Plan;
    typedef typename Plan::type DT;
    const DT dt = Plan::make(dev);
    constexpr int smem = Plan::end;
    auto kern = nebo_tiled_assign_kernel<T, DT, TZ, Plan::rounds>;
    if (smem > 48 * 1024)
      throw_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem),
                 "Nebo Assignment (shared memory)");
    const dim3 grid((nx + kTileX - 1) / kTileX, (ny + kTileY - 1) / kTileY, (nz + TZ - 1) / TZ);
    kern<<<grid, dim3(kTileX, kTileY, 1), smem, s>>>(out, sy, sz, lim[0], lim[1], lim[2], lim[3], lim[4], lim[5], dt);
    throw_cuda(cudaGetLastError(), "Nebo Assignment (kernel launch)");
    return;
  }
#endif
  assign_plain<T>(out, sy, sz, lim, dev, s);
}

template <class F, class Node>
void assign(F& lhs, const Node& rhs, bool useGhost) {
  typedef typename F::value_type T;
  int32_t lim[6];
  if (!write_region(lhs, rhs, useGhost, lim)) return;
  LaunchStreamScope scope(lhs.get_stream());
  const auto dev = rhs.device();  // uploads any input edited on the host; orders other streams' writes
  T* out = lhs.device_values_for_write() + lhs.interior_origin();
  const int sy = (int)lhs.window_with_ghost().glob_dim(0);
  const long sz = (long)lhs.window_with_ghost().glob_dim(0) * (long)lhs.window_with_ghost().glob_dim(1);
  cudaStream_t s = (cudaStream_t)lhs.get_stream();
  // linear stencils of linear stencils merged into one (reassociating builds; NeboTiled.h)
  typedef Compose<typename std::decay<decltype(dev)>::type> CP;
  typedef typename CP::type D;
  const D devc = CP::make(dev);
  // constant factors carried on the host (reassociating builds; NeboFactor.h), when the launch's
  // coefficients allow it
  typedef FactorRoot<T, D> FR;
  if constexpr (FR::changes) {
    bool ok = true;
    const typename FR::type fac = FR::make(devc, ok);
    if (ok) {
      assign_launch<T>(out, sy, sz, lim, fac, s);
      return;
    }
  }
  assign_launch<T>(out, sy, sz, lim, devc, s);
}

// The one-pass form: one thread per (x, y) column of a z-chunk.  The z split: the whole number
// of resident-block waves (at most 8) whose last wave is fullest (a split that leaves most of a
// last wave idle costs a whole wave); NEBO_UNTILED keeps the plain rule of about 8 blocks per SM.
template <typename T, class D>
void assign_plain(T* out, int sy, long sz, const int32_t lim[6], const D& dev, cudaStream_t s) {
  const int nx = lim[1] - lim[0], ny = lim[3] - lim[2], nz = lim[5] - lim[4];
  dim3 block(32, 8, 1);
  dim3 grid((nx + 31) / 32, (ny + 7) / 8, 1);
  const long plane_blocks = (long)grid.x * grid.y;
#ifndef NEBO_UNTILED
  static std::atomic<int> per_sm{0};  // resident blocks of this instantiation (one architecture)
  int bps = per_sm.load(std::memory_order_relaxed);
  if (bps <= 0) {
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, nebo_assign_kernel<T, D>, 256, 0) != cudaSuccess ||
        bps < 1) {
      cudaGetLastError();
      bps = 1;
    }
    per_sm.store(bps, std::memory_order_relaxed);
  }
  const long slots = (long)device_sm_count() * bps;
  long chunks = 1;
  double best = -1.0;
  for (long k = 1; k <= nz && plane_blocks * k <= 8 * slots; ++k) {
    const double waves = (double)(plane_blocks * k) / (double)slots;
    const double fill = waves / std::ceil(waves);
    if (fill > best + 1e-3) {
      best = fill;
      chunks = k;
    }
  }
#else
  long chunks = (8L * device_sm_count() + plane_blocks - 1) / plane_blocks;
  if (chunks < 1) chunks = 1;
  if (chunks > nz) chunks = nz;
#endif
  const int zchunk = (int)((nz + chunks - 1) / chunks);
  grid.z = (unsigned)((nz + zchunk - 1) / zchunk);
  nebo_assign_kernel<T, D><<<grid, block, 0, s>>>(
      out, sy, sz, lim[0], lim[1], lim[2], lim[3], lim[4], lim[5], zchunk, dev);
  throw_cuda(cudaGetLastError(), "Nebo Assignment (kernel launch)");
}

template <class F, class Node>
void masked(const SpatialMask<F>& mask, F& lhs, const Node& rhs) {
  typedef typename F::value_type T;
  const int np = mask.num_points();
  if (np == 0) return;
  LaunchStreamScope scope(lhs.get_stream());
  typedef Compose<typename std::decay<decltype(rhs.device())>::type> CP;
  const auto dev = CP::make(rhs.device());
  T* out = lhs.device_values_for_write() + lhs.interior_origin();
  const int sy = (int)lhs.window_with_ghost().glob_dim(0);
  const long sz = (long)lhs.window_with_ghost().glob_dim(0) * (long)lhs.window_with_ghost().glob_dim(1);
  const int threads = 256;
  int blocks = (np + threads - 1) / threads;
  if (blocks > 8 * device_sm_count()) blocks = 8 * device_sm_count();
  cudaStream_t s = (cudaStream_t)lhs.get_stream();
  nebo_masked_assign_kernel<T, typename std::decay<decltype(dev)>::type><<<blocks, threads, 0, s>>>(
      out, sy, sz, mask.device_points(), np, dev);
  throw_cuda(cudaGetLastError(), "Nebo Masked Assignment (kernel launch)");
}

}  // namespace nebo_detail

// ------------------------------------------------------------------ lhs <<= rhs
template <typename L, typename T>
const SpatialField<L, T>& operator<<=(SpatialField<L, T>& lhs, const typename std::common_type<T>::type& rhs) {
  nebo_detail::assign(lhs, nebo_detail::ScalarNode<T>(rhs), true);
  return lhs;
}
template <typename L, typename T>
const SpatialField<L, T>& operator<<=(SpatialField<L, T>& lhs, const SpatialField<L, T>& rhs) {
  nebo_detail::assign(lhs, nebo_detail::FieldNode<SpatialField<L, T>>(rhs), true);
  return lhs;
}
template <typename E, typename L, typename T>
const SpatialField<L, T>& operator<<=(SpatialField<L, T>& lhs, const NeboExpression<E, SpatialField<L, T>>& rhs) {
  nebo_detail::assign(lhs, rhs.expr(), true);
  return lhs;
}

// SingleValue right-hand sides: the value broadcast over the write region
// (spatialops/NeboAssignment.h:61-133)
template <typename L, typename T, class = typename std::enable_if<!std::is_same<L, SingleValue>::value>::type>
const SpatialField<L, T>& operator<<=(SpatialField<L, T>& lhs, const SpatialField<SingleValue, T>& rhs) {
  nebo_detail::assign(lhs, nebo_detail::SingleValueNode<SpatialField<SingleValue, T>>(rhs), true);
  return lhs;
}
template <typename E, typename L, typename T>
const SpatialField<L, T>& operator<<=(SpatialField<L, T>& lhs, const NeboSingleValueExpression<E, T>& rhs) {
  nebo_detail::assign(lhs, rhs.expr(), true);
  return lhs;
}

// ------------------------------------------------------------------ interior_assign
template <typename L, typename T>
const SpatialField<L, T>& interior_assign(SpatialField<L, T>& lhs, const typename std::common_type<T>::type& rhs) {
  nebo_detail::assign(lhs, nebo_detail::ScalarNode<T>(rhs), false);
  return lhs;
}
template <typename L, typename T>
const SpatialField<L, T>& interior_assign(SpatialField<L, T>& lhs, const SpatialField<L, T>& rhs) {
  nebo_detail::assign(lhs, nebo_detail::FieldNode<SpatialField<L, T>>(rhs), false);
  return lhs;
}
template <typename E, typename L, typename T>
const SpatialField<L, T>& interior_assign(SpatialField<L, T>& lhs, const NeboExpression<E, SpatialField<L, T>>& rhs) {
  nebo_detail::assign(lhs, rhs.expr(), false);
  return lhs;
}

template <typename L, typename T, class = typename std::enable_if<!std::is_same<L, SingleValue>::value>::type>
const SpatialField<L, T>& interior_assign(SpatialField<L, T>& lhs, const SpatialField<SingleValue, T>& rhs) {
  nebo_detail::assign(lhs, nebo_detail::SingleValueNode<SpatialField<SingleValue, T>>(rhs), false);
  return lhs;
}
template <typename E, typename L, typename T>
const SpatialField<L, T>& interior_assign(SpatialField<L, T>& lhs, const NeboSingleValueExpression<E, T>& rhs) {
  nebo_detail::assign(lhs, rhs.expr(), false);
  return lhs;
}

// ------------------------------------------------------------------ masked_assign
// Writes rhs at the mask's points only (the reference's point loop, NeboLhs.h:164-283; the
// reference has no GPU path for it).
template <typename L, typename T>
const SpatialField<L, T>& masked_assign(const SpatialMask<SpatialField<L, T>>& mask, SpatialField<L, T>& lhs,
                                        const typename std::common_type<T>::type& rhs) {
  nebo_detail::masked(mask, lhs, nebo_detail::ScalarNode<T>(rhs));
  return lhs;
}
template <typename L, typename T>
const SpatialField<L, T>& masked_assign(const SpatialMask<SpatialField<L, T>>& mask, SpatialField<L, T>& lhs,
                                        const SpatialField<L, T>& rhs) {
  nebo_detail::masked(mask, lhs, nebo_detail::FieldNode<SpatialField<L, T>>(rhs));
  return lhs;
}
template <typename E, typename L, typename T>
const SpatialField<L, T>& masked_assign(const SpatialMask<SpatialField<L, T>>& mask, SpatialField<L, T>& lhs,
                                        const NeboExpression<E, SpatialField<L, T>>& rhs) {
  nebo_detail::masked(mask, lhs, rhs.expr());
  return lhs;
}

}  // namespace SpatialOps
#endif
