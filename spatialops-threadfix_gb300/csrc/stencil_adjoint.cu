// Transposed (adjoint) stencil operators: the reverse-mode counterpart of a Nebo stencil
// assignment, for differentiating user code written with the reference's operators (no
// counterpart in the reference, which has no differentiation).
//
// A stencil assignment  dst(i) = sum_k c_k src(i + p_k)  over the write region R of dst
// (interior-relative coordinates of each field; p_k and c_k are the operator's point collection
// and coefficients in listed order, spatialops/NeboStencilBuilder.h:154-232 and
// spatialops/structured/stencil/StencilBuilder.cpp:52-220) has the transpose
//   src_bar(j) = sum_k c_k dst_bar(j - p_k)   over the k with j - p_k in R,
// which this file evaluates as a gather: one thread per src cell, the points in listed order, no
// atomics, so the result is deterministic.  Interpolant, Gradient, Divergence, the FD stencils and
// the box filter are all of this form; the caller passes the forward operator's points and
// coefficients and the forward write region (nebo_write_limits).
#include "common.cuh"

namespace nebo {
namespace {

constexpr int SA_MAX_POINTS = 32;

struct StencilPoints {
  int n;
  int p[SA_MAX_POINTS][3];
  double c[SA_MAX_POINTS];
};

// src_bar over its whole window (interior-relative j from -gm to n + gp + bc cells)
__global__ void stencil_transpose_kernel(const double* __restrict__ dbar, int dsy, long dsz,
                                         double* __restrict__ sbar, int ssy, long ssz, int jx0, int jy0, int jz0,
                                         int nx, int ny, int nz, int lx0, int lx1, int ly0, int ly1, int lz0, int lz1,
                                         StencilPoints pts, int accumulate) {
  const long total = (long)nx * ny * nz;
  for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < total; q += (long)gridDim.x * blockDim.x) {
    const int jx = jx0 + (int)(q % nx), jy = jy0 + (int)((q / nx) % ny), jz = jz0 + (int)(q / ((long)nx * ny));
    double acc = 0.0;
    bool any = false;
    for (int k = 0; k < pts.n; ++k) {
      const int ix = jx - pts.p[k][0], iy = jy - pts.p[k][1], iz = jz - pts.p[k][2];
      if (ix < lx0 || ix >= lx1 || iy < ly0 || iy >= ly1 || iz < lz0 || iz >= lz1) continue;
      const double t = pts.c[k] * __ldg(dbar + (long)ix + (long)dsy * iy + dsz * iz);
      acc = any ? acc + t : t;
      any = true;
    }
    double* o = sbar + (long)jx + (long)ssy * jy + ssz * jz;
    if (accumulate)
      *o += acc;
    else
      *o = acc;
  }
}

}  // namespace
}  // namespace nebo

using namespace nebo;

extern "C" int nebo_stencil_transpose(const nebo_field* dst_bar, const int32_t limits[6], const nebo_field* src_bar,
                                      int32_t npoints, const int32_t* points, const double* coefs, int accumulate,
                                      nebo_stream_t stream) {
  const char* what = "nebo_stencil_transpose";
  int rc = check_field(dst_bar, what);
  if (rc) return rc;
  if ((rc = check_field(src_bar, what))) return rc;
  if (dst_bar->dtype != NEBO_F64 || src_bar->dtype != NEBO_F64)
    return fail(NEBO_ERR_UNSUPPORTED, "Nebo error in %s: FP64 only", what);
  if (!limits || !points || !coefs) return fail(NEBO_ERR_INVALID, "Nebo error in %s: null argument", what);
  if (npoints < 1 || npoints > SA_MAX_POINTS)
    return fail(NEBO_ERR_INVALID, "Nebo error in %s: %d points (1 to %d)", what, npoints, SA_MAX_POINTS);
  // the forward write region must lie inside dst_bar's window
  for (int d = 0; d < 3; ++d) {
    const int lo = -(dst_bar->ghost_minus[d]);
    const int hi = dst_bar->extent[d] - dst_bar->ghost_minus[d];
    if (limits[2 * d] < lo || limits[2 * d + 1] > hi || limits[2 * d] > limits[2 * d + 1])
      return fail(NEBO_ERR_INVALID, "Nebo error in %s: write region outside the dst window on axis %d", what, d);
  }
  StencilPoints sp;
  sp.n = npoints;
  for (int k = 0; k < npoints; ++k) {
    for (int d = 0; d < 3; ++d) sp.p[k][d] = points[3 * k + d];
    sp.c[k] = coefs[k];
  }
  const View<double> vd = make_view<double>(*dst_bar), vs = make_view<double>(*src_bar);
  const int j0[3] = {-(src_bar->ghost_minus[0]), -(src_bar->ghost_minus[1]), -(src_bar->ghost_minus[2])};
  const int n[3] = {src_bar->extent[0], src_bar->extent[1], src_bar->extent[2]};
  const long total = (long)n[0] * n[1] * n[2];
  if (total == 0) return NEBO_OK;
  const int threads = 256;
  const long want = (total + threads - 1) / threads;
  const int blocks = (int)(want < (long)num_sms() * 16 ? want : (long)num_sms() * 16);
  cudaStream_t s = (cudaStream_t)stream;
  LaunchScope ls("stencil_transpose", s);
  stencil_transpose_kernel<<<blocks, threads, 0, s>>>(vd.base, vd.sy, vd.sz, vs.base, vs.sy, vs.sz, j0[0], j0[1], j0[2],
                                                      n[0], n[1], n[2], limits[0], limits[1], limits[2], limits[3],
                                                      limits[4], limits[5], sp, accumulate);
  NEBO_LAUNCH_CHECK(what);
  return NEBO_OK;
}
