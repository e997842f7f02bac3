// nebo_sum / nebo_max / nebo_min / nebo_norm and their _interior forms
// (drop-in for spatialops/NeboReductions.h:45-240; field_* aliases included).
//
// Region: the expression's valid ghosts without BC cells (interior only for _interior) over its
// extents, as nebo_fold.  A plain field goes to the library's reduction (nebo_reduce); an
// expression is evaluated inside a reduction kernel instantiated for it (one partial per block,
// FP64 Neumaier-compensated), and the block partials are combined on the host in a fixed order,
// so results are deterministic.  norm = sqrt(sum(v*v)).
#ifndef SpatialOps_NeboReductions_h
#define SpatialOps_NeboReductions_h

#include <cmath>
#include <limits>
#include <vector>

#include <spatialops/NeboAssignment.h>
#include <spatialops/NeboCore.h>

#define field_max nebo_max
#define field_max_interior nebo_max_interior
#define field_min nebo_min
#define field_min_interior nebo_min_interior
#define field_sum nebo_sum
#define field_sum_interior nebo_sum_interior
#define field_norm nebo_norm
#define field_norm_interior nebo_norm_interior

namespace SpatialOps {
namespace nebo_detail {

struct RedAcc {
  double s, c;
};

__device__ __forceinline__ void red_add(RedAcc& a, double v) {
  const double t = a.s + v;
  a.c += (fabs(a.s) >= fabs(v)) ? ((a.s - t) + v) : ((v - t) + a.s);
  a.s = t;
}

template <class D>
__global__ void __launch_bounds__(256) nebo_reduce_expr_kernel(D e, int x0, int x1, int y0, int ny, int z0, long nrows,
                                                               int op, RedAcc* __restrict__ partials) {
  RedAcc a;
  a.s = op == NEBO_RED_MAX ? -INFINITY : (op == NEBO_RED_MIN ? INFINITY : 0.0);
  a.c = 0.0;
  for (long r = blockIdx.x; r < nrows; r += gridDim.x) {
    const int y = y0 + (int)(r % ny), z = z0 + (int)(r / ny);
    for (int x = x0 + (int)threadIdx.x; x < x1; x += blockDim.x) {
      const double v = (double)e.eval(x, y, z);
      if (op == NEBO_RED_MAX)
        a.s = (a.s < v) ? v : a.s;
      else if (op == NEBO_RED_MIN)
        a.s = (a.s > v) ? v : a.s;
      else if (op == NEBO_RED_NORM)
        red_add(a, v * v);
      else
        red_add(a, v);
    }
  }
  __shared__ RedAcc sh[256];
  sh[threadIdx.x] = a;
  __syncthreads();
  if (threadIdx.x == 0) {
    RedAcc t = sh[0];
    for (int i = 1; i < (int)blockDim.x; ++i) {
      const RedAcc b = sh[i];
      if (op == NEBO_RED_MAX)
        t.s = (t.s < b.s) ? b.s : t.s;
      else if (op == NEBO_RED_MIN)
        t.s = (t.s > b.s) ? b.s : t.s;
      else {
        red_add(t, b.s);
        t.c += b.c;
      }
    }
    partials[blockIdx.x] = t;
  }
}

template <class Node>
double fold_expr(const Node& e, bool useGhost, int op) {
  const GhostData g = useGhost ? e.ghosts_without_bc() : GhostData(0);
  const IntVec ext = e.extents();
  const int lo[3] = {-g.get_minus(0), -g.get_minus(1), -g.get_minus(2)};
  const int hi[3] = {ext[0] + g.get_plus(0), ext[1] + g.get_plus(1), ext[2] + g.get_plus(2)};
  const long nrows = (long)(hi[1] - lo[1]) * (hi[2] - lo[2]);
  double r0 = op == NEBO_RED_MAX ? -std::numeric_limits<double>::infinity()
              : op == NEBO_RED_MIN ? std::numeric_limits<double>::infinity() : 0.0;
  if (nrows <= 0 || hi[0] <= lo[0]) return op == NEBO_RED_NORM ? 0.0 : r0;
  LaunchStreamScope scope(nullptr);  // the fold runs on the default stream
  const auto dev = e.device();
  int blocks = (int)(nrows < 4L * device_sm_count() ? nrows : 4L * device_sm_count());
  void* p = nullptr;
  throw_status(nebo_alloc(sizeof(RedAcc) * blocks, &p, nullptr), "Nebo reduction");
  nebo_reduce_expr_kernel<typename std::decay<decltype(dev)>::type><<<blocks, 256, 0, nullptr>>>(
      dev, lo[0], hi[0], lo[1], hi[1] - lo[1], lo[2], nrows, op, static_cast<RedAcc*>(p));
  cudaError_t le = cudaGetLastError();
  std::vector<RedAcc> host(blocks);
  int rc = le == cudaSuccess ? nebo_memcpy_d2h(host.data(), p, sizeof(RedAcc) * blocks, nullptr) : NEBO_OK;
  if (rc == NEBO_OK) rc = nebo_stream_sync(nullptr);
  nebo_free(p, nullptr);
  throw_cuda(le, "Nebo reduction (kernel launch)");
  throw_status(rc, "Nebo reduction");
  double s = r0, c = 0.0;
  for (const RedAcc& b : host) {
    if (op == NEBO_RED_MAX)
      s = (s < b.s) ? b.s : s;
    else if (op == NEBO_RED_MIN)
      s = (s > b.s) ? b.s : s;
    else {
      const double t = s + b.s;
      c += (std::fabs(s) >= std::fabs(b.s)) ? ((s - t) + b.s) : ((b.s - t) + s);
      s = t;
      c += b.c;
    }
  }
  if (op == NEBO_RED_SUM) return s + c;
  if (op == NEBO_RED_NORM) return std::sqrt(s + c);
  return s;
}

template <typename L, typename T>
T fold_field(const SpatialField<L, T>& f, bool useGhost, int op) {
  f.device_values_for_read();
  const nebo_field d = f.descriptor();
  double r = 0.0;
  throw_status(nebo_reduce(&d, op, useGhost ? 0 : 1, &r, f.get_stream()), "Nebo reduction");
  return (T)r;
}

}  // namespace nebo_detail

#define NEBO_REDUCTION(NAME, OP, GHOST)                                                          \
  template <typename L, typename T>                                                              \
  T NAME(const SpatialField<L, T>& f) {                                                          \
    return nebo_detail::fold_field(f, GHOST, OP);                                                \
  }                                                                                              \
  template <typename E, typename F>                                                              \
  typename F::value_type NAME(const NeboExpression<E, F>& e) {                                   \
    return (typename F::value_type)nebo_detail::fold_expr(e.expr(), GHOST, OP);                  \
  }
NEBO_REDUCTION(nebo_sum, NEBO_RED_SUM, true)
NEBO_REDUCTION(nebo_max, NEBO_RED_MAX, true)
NEBO_REDUCTION(nebo_min, NEBO_RED_MIN, true)
NEBO_REDUCTION(nebo_norm, NEBO_RED_NORM, true)
NEBO_REDUCTION(nebo_sum_interior, NEBO_RED_SUM, false)
NEBO_REDUCTION(nebo_max_interior, NEBO_RED_MAX, false)
NEBO_REDUCTION(nebo_min_interior, NEBO_RED_MIN, false)
NEBO_REDUCTION(nebo_norm_interior, NEBO_RED_NORM, false)
#undef NEBO_REDUCTION

}  // namespace SpatialOps
#endif
