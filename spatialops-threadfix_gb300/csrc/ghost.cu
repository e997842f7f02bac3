// Periodic ghost exchange inside one GPU's memory: every ghost cell of a uniform-ghost patch
// takes the value of its wrapped interior image.  This is the single-patch stand-in for the
// halo exchange that callers of the reference perform between patches (the reference itself
// has no periodic support; its heat driver fills ghosts by copy before each step).
#include "common.cuh"

namespace nebo {
namespace {

// One thread per ghost cell of one slab.  The ghost shell is split into the two z slabs
// (full x,y extent), the two y slabs (interior z) and the two x slabs (interior y,z), so every
// ghost cell is visited exactly once and no interior cell is touched.
template <typename T>
__global__ void fill_periodic_kernel(T* __restrict__ base, int sy, long sz, int nx, int ny, int nz, int g) {
  const int gx = nx + 2 * g, gy = ny + 2 * g;
  const long zslab = (long)gx * gy * g;        // cells in one z slab
  const long yslab = (long)gx * g * nz;        // cells in one y slab
  const long xslab = (long)g * ny * nz;        // cells in one x slab
  const long total = 2 * (zslab + yslab + xslab);
  for (long t = blockIdx.x * (long)blockDim.x + threadIdx.x; t < total; t += (long)gridDim.x * blockDim.x) {
    long r = t;
    int x, y, z;
    if (r < 2 * zslab) {
      const int side = r >= zslab;
      r -= side * zslab;
      x = (int)(r % gx) - g;
      r /= gx;
      y = (int)(r % gy) - g;
      z = (int)(r / gy) + (side ? nz : -g);
    } else if ((r -= 2 * zslab) < 2 * yslab) {
      const int side = r >= yslab;
      r -= side * yslab;
      x = (int)(r % gx) - g;
      r /= gx;
      y = (int)(r % g) + (side ? ny : -g);
      z = (int)(r / g);
    } else {
      r -= 2 * yslab;
      const int side = r >= xslab;
      r -= side * xslab;
      x = (int)(r % g) + (side ? nx : -g);
      r /= g;
      y = (int)(r % ny);
      z = (int)(r / ny);
    }
    const int sx_ = ((x % nx) + nx) % nx, sy_ = ((y % ny) + ny) % ny, sz_ = ((z % nz) + nz) % nz;
    base[(long)x + (long)sy * y + sz * z] = base[(long)sx_ + (long)sy * sy_ + sz * sz_];
  }
}

}  // namespace

int fill_periodic_any(const nebo_field* f, cudaStream_t s) {
  int rc = check_field(f, "nebo_fill_periodic");
  if (rc) return rc;
  const int g = f->ghost_minus[0];
  if ((rc = check_periodic_patch(f, g, "nebo_fill_periodic"))) return rc;
  if (g == 0) return NEBO_OK;
  int n[3];
  interior_extent(*f, n);
  const long total = 2L * ((long)(n[0] + 2 * g) * (n[1] + 2 * g) * g + (long)(n[0] + 2 * g) * g * n[2] + (long)g * n[1] * n[2]);
  const int threads = 256;
  const long want = (total + threads - 1) / threads;
  const int blocks = (int)(want < (long)num_sms() * 16 ? want : (long)num_sms() * 16);
  LaunchScope ls("fill_periodic", s);
  if (f->dtype == NEBO_F64) {
    View<double> v = make_view<double>(*f);
    fill_periodic_kernel<double><<<blocks, threads, 0, s>>>(v.base, v.sy, v.sz, n[0], n[1], n[2], g);
  } else {
    View<float> v = make_view<float>(*f);
    fill_periodic_kernel<float><<<blocks, threads, 0, s>>>(v.base, v.sy, v.sz, n[0], n[1], n[2], g);
  }
  NEBO_LAUNCH_CHECK("nebo_fill_periodic");
  return NEBO_OK;
}

}  // namespace nebo

extern "C" int nebo_fill_periodic(const nebo_field* f, nebo_stream_t stream) {
  return nebo::fill_periodic_any(f, (cudaStream_t)stream);
}
