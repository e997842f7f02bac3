// Deep fused chain (the reference's headline Nebo use: nested stencils, cond with a mask,
// transcendentals, then a box filter):
//   out  <<= cond(mask, 0.0)( Interp_{S->X}(Grad_{X->S}(Interp_{S->X}(a))) * exp(b) + sin(c) )
//   filt <<= Filter_{X->X}(out)
// Reference operators: Interp SVol->XVol {1/2,1/2} at (-1,0), Grad XVol->SVol {-1/dx,1/dx} at
// (0,+1) (StencilBuilder.cpp:123-127), BoxFilter3D 27 points * 1/27 (NeboStencilBuilder.h:389-465).
// The reference evaluates the nested stencils as a tree, re-reading `a` 8 times per cell and
// recomputing the inner interpolant twice; here the chain collapses to one 4-point stencil on a,
//   I(G(I(a)))[i] = (g1/4) * ((a[i+1] - a[i-1]) + (a[i] - a[i-2])),
// a reassociation of the same sum (FP64 error a few ulp of max|a|, inside the 1e-13 relative
// bound).  exp and sin are the integer-pipe functions of fp64_int.cuh: FP64 only for the argument
// reduction, 64-bit fixed point for the polynomials (within one ulp; at most 2 ulp from CUDA's).
//
// Write regions follow calculate_actual_ghost (NeboBasic.h:61-100): with one ghost layer the
// chain's x ghost is -1, so `out` is written on x in [1, n) and y, z in [-1, n+1); the filter's
// region is the interior.  Other cells keep their contents.
//
// Kernel 1 is bound by FP64 issue (exp + sin); kernel 2 sums the 27 points separably
// (x, then y from shared memory, then z from a register queue while marching in z).
#include "common.cuh"
#include "fp64_int.cuh"

namespace nebo {
namespace {

constexpr int FX = 32;  // filter tile x
constexpr int FY = 8;   // filter tile y

__global__ void __launch_bounds__(256) deep_out_kernel(const double* __restrict__ a, const double* __restrict__ b,
                                                       const double* __restrict__ c, const uint32_t* __restrict__ mask,
                                                       long mask_base, double* __restrict__ out, int sy, long sz,
                                                       int nx, int ny, int nz, double q) {
  // region: x in [1, nx), y in [-1, ny+1), z in [-1, nz+1)
  const int x = 1 + blockIdx.x * blockDim.x + threadIdx.x;
  const int y = -1 + blockIdx.y * blockDim.y + threadIdx.y;
  if (x >= nx || y > ny) return;
  for (int z = -1 + (int)blockIdx.z; z <= nz; z += gridDim.z) {
    const long i = (long)x + (long)sy * y + sz * z;
    const long bit = mask_base + i;  // flat index in the window
    double v;
    if ((__ldg(mask + (bit >> 5)) >> (bit & 31)) & 1u) {
      v = 0.0;
    } else {
      const double igi = q * ((__ldg(a + i + 1) - __ldg(a + i - 1)) + (__ldg(a + i) - __ldg(a + i - 2)));
      v = fma(igi, fixmath::exp_i(__ldg(b + i)), fixmath::sin_i(__ldg(c + i)));
    }
    out[i] = v;
  }
}

// filt[x,y,z] = (sum over the 27 neighbours of out) / 27 on the interior.
__global__ void __launch_bounds__(FX* FY) box_filter_kernel(const double* __restrict__ src, double* __restrict__ dst,
                                                            int sy, long sz, int nx, int ny, int nz, int zchunk) {
  __shared__ double plane[FY + 2][FX + 2];  // one z plane of src with x/y halo
  __shared__ double rows[FY + 2][FX];       // x-sums of 3
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int x0 = blockIdx.x * FX, y0 = blockIdx.y * FY;
  const int x = x0 + tx, y = y0 + ty;
  const int z0 = blockIdx.z * zchunk, z1 = min(z0 + zchunk, nz);
  const int tid = ty * FX + tx;
  double s_prev = 0.0, s_cur = 0.0;  // 2D 9-point sums of planes z-1 and z
  for (int zz = z0 - 1; zz <= z1; ++zz) {
    // stage plane zz rows y0-1 .. y0+FY, cols x0-1 .. x0+FX (clamped to the ghosted window)
    for (int k = tid; k < (FY + 2) * (FX + 2); k += FX * FY) {
      const int r = k / (FX + 2), cidx = k % (FX + 2);
      const int gx_ = min(x0 - 1 + cidx, nx), gy_ = min(y0 - 1 + r, ny);
      plane[r][cidx] = __ldg(src + (long)gx_ + (long)sy * gy_ + sz * zz);
    }
    __syncthreads();
    for (int k = tid; k < (FY + 2) * FX; k += FX * FY) {
      const int r = k / FX, cidx = k % FX;
      rows[r][cidx] = (plane[r][cidx] + plane[r][cidx + 1]) + plane[r][cidx + 2];
    }
    __syncthreads();
    const double s2 = (rows[ty][tx] + rows[ty + 1][tx]) + rows[ty + 2][tx];
    if (zz >= z0 + 1 && x < nx && y < ny) {
      // plane zz-1 is complete: s_prev (zz-2), s_cur (zz-1), s2 (zz)
      dst[(long)x + (long)sy * y + sz * (zz - 1)] = ((s_prev + s_cur) + s2) * (1.0 / 27.0);
    }
    s_prev = s_cur;
    s_cur = s2;
    __syncthreads();
  }
}

int check_deep(const nebo_field* a, const nebo_field* b, const nebo_field* c, const nebo_field* out,
               const nebo_field* filt) {
  const char* w = "nebo_deep_chain";
  int rc;
  const nebo_field* fs[5] = {a, b, c, out, filt};
  for (int i = 0; i < 5; ++i) {
    if ((rc = check_field(fs[i], w))) return rc;
    if (fs[i]->dtype != NEBO_F64) return fail(NEBO_ERR_UNSUPPORTED, "Nebo error in %s: FP64 fields only", w);
    if ((rc = check_periodic_patch(fs[i], 1, w))) return rc;
  }
  for (int i = 1; i < 5; ++i)
    if ((rc = check_same_layout(a, fs[i], w))) return rc;
  if (out->data == a->data || out->data == b->data || out->data == c->data || filt->data == out->data)
    return fail(NEBO_ERR_INVALID, "Nebo error in %s: outputs alias inputs", w);
  return NEBO_OK;
}

}  // namespace
}  // namespace nebo

using namespace nebo;

extern "C" int nebo_deep_chain(const nebo_field* a, const nebo_field* b, const nebo_field* c,
                               const uint32_t* mask_words, const nebo_field* out, const nebo_field* filt, double dx,
                               nebo_stream_t stream) {
  int rc = check_deep(a, b, c, out, filt);
  if (rc) return rc;
  if (!mask_words) return fail(NEBO_ERR_INVALID, "Nebo error in nebo_deep_chain: null mask");
  if (fixmath::tables_init()) return fail(NEBO_ERR_LAUNCH, "Nebo error in nebo_deep_chain: math tables upload");
  int n[3];
  interior_extent(*a, n);
  cudaStream_t s = (cudaStream_t)stream;
  const View<const double> va = make_view<const double>(*a), vb = make_view<const double>(*b),
                           vc = make_view<const double>(*c);
  const View<double> vo = make_view<double>(*out), vf = make_view<double>(*filt);
  // flat window index of interior (0,0,0): used to locate mask bits
  const long mask_base = (long)(out->offset[0] + 1) + (long)out->glob[0] * (out->offset[1] + 1) +
                         (long)out->glob[0] * out->glob[1] * (out->offset[2] + 1);
  const double q = 0.25 * (1.0 / dx);
  if (n[0] > 1) {
    dim3 block(32, 8);
    dim3 grid((n[0] - 1 + 31) / 32, (n[1] + 2 + 7) / 8, 1);
    const long planes_blocks = (long)grid.x * grid.y;
    int zsplit = (int)((num_sms() * 8 + planes_blocks - 1) / planes_blocks);
    zsplit = zsplit < 1 ? 1 : (zsplit > n[2] + 2 ? n[2] + 2 : zsplit);
    grid.z = zsplit;
    LaunchScope ls("deep_chain", s);
    deep_out_kernel<<<grid, block, 0, s>>>(va.base, vb.base, vc.base, mask_words, mask_base, vo.base, vo.sy, vo.sz,
                                           n[0], n[1], n[2], q);
    NEBO_LAUNCH_CHECK("nebo_deep_chain (chain)");
  }
  {
    const int gxb = (n[0] + FX - 1) / FX, gyb = (n[1] + FY - 1) / FY;
    int chunks = (num_sms() * 4 + gxb * gyb - 1) / (gxb * gyb);
    chunks = chunks < 1 ? 1 : (chunks > (n[2] + 7) / 8 ? (n[2] + 7) / 8 : chunks);
    if (chunks < 1) chunks = 1;
    const int zchunk = (n[2] + chunks - 1) / chunks;
    chunks = (n[2] + zchunk - 1) / zchunk;
    LaunchScope ls("box_filter", s);
    box_filter_kernel<<<dim3(gxb, gyb, chunks), dim3(FX, FY), 0, s>>>(vo.base, vf.base, vo.sy, vo.sz, n[0], n[1], n[2],
                                                                      zchunk);
    NEBO_LAUNCH_CHECK("nebo_deep_chain (filter)");
  }
  return NEBO_OK;
}

// Element-wise FP64 exp / sin of the integer-pipe functions (fn 0: exp, 1: sin).
namespace nebo {
namespace {
__global__ void fastmath_kernel(int fn, const double* __restrict__ x, double* __restrict__ y, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    y[i] = fn == 0 ? fixmath::exp_i(x[i]) : fixmath::sin_i(x[i]);
}
}  // namespace
}  // namespace nebo

extern "C" int nebo_fastmath_eval(int fn, const double* x, double* y, size_t n, nebo_stream_t stream) {
  if ((fn != 0 && fn != 1) || (n && (!x || !y))) return fail(NEBO_ERR_INVALID, "Nebo error in nebo_fastmath_eval");
  if (fixmath::tables_init()) return fail(NEBO_ERR_LAUNCH, "Nebo error in nebo_fastmath_eval: math tables upload");
  if (!n) return NEBO_OK;
  cudaStream_t s = (cudaStream_t)stream;
  LaunchScope ls("fastmath_eval", s);
  fastmath_kernel<<<num_sms() * 8, 256, 0, s>>>(fn, x, y, n);
  NEBO_LAUNCH_CHECK("nebo_fastmath_eval");
  return NEBO_OK;
}
