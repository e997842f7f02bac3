// Adjoint of the fused heat step (no counterpart in the reference, which has no differentiation):
// gradients of  J = 1/2 * sum_interior (T_N - T_target)^2  with respect to T_0 and lambda, for
// T_{k+1} = T_k + dt * sum_d Div_d(Interp_d(lambda) * Grad_d(T_k)) on a periodic SVol patch with
// one ghost layer and unit spacing (the forward step is nebo_heat_step's, bit-exact FP64).
//
// Reverse step (abar' = dJ/dT_{k+1}, both with periodic ghost images):
//   abar[c]  = abar'[c] + dt * sum_d ( lf[c+s] (abar'[c+s]-abar'[c]) - lf[c] (abar'[c]-abar'[c-s]) )
//              -- the forward operator applied to abar' (it is self-adjoint on the periodic
//                 grid; the ghost fill's transpose folds ghost contributions onto their
//                 interior images, which the periodic ghost reads express);
//   glam[c] -= (dt/2) * sum_d ( (T[c]-T[c-s])(abar'[c]-abar'[c-s]) + (T[c+s]-T[c])(abar'[c+s]-abar'[c]) )
//              -- lambda[c] enters the face coefficients lf[c] and lf[c+s] with weight 1/2.
// One kernel per reverse step computes both, with every face quantity computed once and shared
// through shared memory (x, y) or carried in a register (z), and writes abar's ghost images.
//
// Memory: sqrt(N) checkpointing.  The forward sweep keeps T at every L-th step (L = ceil(sqrt N))
// and the states of the last segment; the reverse sweep recomputes each earlier segment's states
// from its checkpoint into a segment buffer and walks it backwards, so device memory grows like
// 2*sqrt(N) fields, not N, and the forward work is about 2N - sqrt(N) steps.
#include <cmath>
#include <vector>

#include <type_traits>

#include "common.cuh"
#include "fp64_int.cuh"

namespace nebo {
namespace {

constexpr int BX = 32;
constexpr int BY = 8;

// A forward state as a double (FP32 states widen exactly).
__device__ __forceinline__ double to_f64(double v) { return v; }
__device__ __forceinline__ double to_f64(float v) { return (double)v; }

__device__ __forceinline__ void store_images1(double* base, int sy, long sz, int x, int y, int z, int nx, int ny, int nz,
                                              double v) {
  base[(long)x + (long)sy * y + sz * z] = v;
  if (x != 0 && x != nx - 1 && y != 0 && y != ny - 1 && z != 0 && z != nz - 1) return;
  // a boundary cell: also write its periodic ghost images (up to 7 more cells; n >= 2 per axis)
  const int ax = x == 0 ? nx : -1, ay = y == 0 ? ny : -1, az = z == 0 ? nz : -1;
  const int m = (x == 0 || x == nx - 1) | ((y == 0 || y == ny - 1) << 1) | ((z == 0 || z == nz - 1) << 2);
  for (int b = 1; b < 8; ++b) {
    if (b & ~m) continue;
    const int xx = (b & 1) ? ax : x, yy = (b & 2) ? ay : y, zz = (b & 4) ? az : z;
    base[(long)xx + (long)sy * yy + sz * zz] = v;
  }
}

// One reverse step.  Per face (a, b = a + s) the thread that owns the face computes
//   dA = A[b] - A[a],  dT = T[b] - T[a]                                   (FP64)
// and shares them (x, y through shared memory, z in a register).  Per cell c:
//   Aout[c] = A[c] + (dt/2) * sum_faces +-lf_face * dA_face              (FP64 FMA chain)
//   glam[c] -= (dt/2) * sum_faces dT_face * dA_face
// with lf_face = lambda[a] + lambda[b] either read from precomputed face arrays (LF) or summed
// from lambda.  EXACT: the face products dT*dA in FP64 (an FMA chain).  Otherwise each face
// product is an FP32 product of the FP32-rounded FP64 differences (relative error ~1e-7; the
// differences themselves are exact FP64, so no cancellation is amplified), their sum is FP32 and
// only the fold into glam is FP64: 6 FP64 operations per cell fewer, and the adjoint state A,
// hence dJ/dT0, is unaffected.
template <bool EXACT, bool LF, typename S = double>
__global__ void __launch_bounds__(BX* BY, 4) heat_adjoint_kernel(const S* __restrict__ T, const double* __restrict__ Ain,
                                                              double* __restrict__ Aout, const double* __restrict__ L,
                                                              const double* __restrict__ lfx,
                                                              const double* __restrict__ lfy,
                                                              const double* __restrict__ lfz, double* __restrict__ glam,
                                                              int sy, long sz, int nx, int ny, int nz, int zchunk,
                                                              double hdt) {
  typedef typename std::conditional<EXACT, double, float>::type P;  // face-product operand type
  __shared__ double sax[2][BY][BX + 1];
  __shared__ double say[2][BY + 1][BX];
  __shared__ P stx[2][BY][BX + 1];
  __shared__ P sty[2][BY + 1][BX];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int x0 = blockIdx.x * BX, y0 = blockIdx.y * BY;
  const int x = x0 + tx, y = y0 + ty;
  const int z0 = blockIdx.z * zchunk, z1 = min(z0 + zchunk, nz);
  const bool active = x < nx && y < ny;
  const int xc = min(x, nx), yc = min(y, ny);
  auto at = [&](int i, int j, int k) { return (long)i + (long)sy * j + sz * k; };
  // (dA, dT) of face (a, b); dT as the product operand type
  auto face = [&](long a, long b, double& da, P& dt) {
    da = __ldg(Ain + b) - __ldg(Ain + a);
    const double d = to_f64(__ldg(T + b)) - to_f64(__ldg(T + a));  // exact for FP32 states too
    if constexpr (EXACT) dt = d; else dt = fixmath::f32_trunc(d);
  };
  auto coef = [&](const double* lf, long a, long b) { return LF ? __ldg(lf + b) : __ldg(L + a) + __ldg(L + b); };
  double dazl;
  P dtzl;
  face(at(xc, yc, z0 - 1), at(xc, yc, z0), dazl, dtzl);
  for (int z = z0; z < z1; ++z) {
    const int buf = z & 1;
    const long c = at(xc, yc, z);
    double dazh, dax, day;
    P dtzh, dtx, dty;
    face(c, c + sz, dazh, dtzh);
    face(c - 1, c, dax, dtx);
    face(c - sy, c, day, dty);
    sax[buf][ty][tx] = dax;
    stx[buf][ty][tx] = dtx;
    say[buf][ty][tx] = day;
    sty[buf][ty][tx] = dty;
    if (ty == 0) {
      const int yh = y0 + BY;
      if (yh <= ny && x <= nx) face(at(xc, yh - 1, z), at(xc, yh, z), say[buf][BY][tx], sty[buf][BY][tx]);
    } else if (ty == 1 && tx < BY) {
      const int xh = x0 + BX, yr = y0 + tx;
      if (xh <= nx && yr < ny) face(at(xh - 1, yr, z), at(xh, yr, z), sax[buf][tx][BX], stx[buf][tx][BX]);
    }
    __syncthreads();
    if (active) {
      const double daxh = sax[buf][ty][tx + 1], dayh = say[buf][ty + 1][tx];
      const P dtxh = stx[buf][ty][tx + 1], dtyh = sty[buf][ty + 1][tx];
      double s = dazh * coef(lfz, c, c + sz);
      s = fma(-dazl, coef(lfz, c - sz, c), s);
      s = fma(dayh, coef(lfy, c, c + sy), s);
      s = fma(-day, coef(lfy, c - sy, c), s);
      s = fma(daxh, coef(lfx, c, c + 1), s);
      s = fma(-dax, coef(lfx, c - 1, c), s);
      store_images1(Aout, sy, sz, x, y, z, nx, ny, nz, fma(hdt, s, Ain[c]));
      double ps;
      if constexpr (EXACT) {
        ps = dtzh * dazh;
        ps = fma(dtzl, dazl, ps);
        ps = fma(dtyh, dayh, ps);
        ps = fma(dty, day, ps);
        ps = fma(dtxh, daxh, ps);
        ps = fma(dtx, dax, ps);
      } else {
        using fixmath::f32_trunc;
        float q = dtzh * f32_trunc(dazh);
        q = fmaf(dtzl, f32_trunc(dazl), q);
        q = fmaf(dtyh, f32_trunc(dayh), q);
        q = fmaf(dty, f32_trunc(day), q);
        q = fmaf(dtxh, f32_trunc(daxh), q);
        q = fmaf(dtx, f32_trunc(dax), q);
        ps = fixmath::f32_to_f64(q);
      }
      glam[c] = fma(-hdt, ps, glam[c]);
    }
    dazl = dazh;
    dtzl = dtzh;
  }
}

// Face coefficients lf_d[c] = lambda[c - s_d] + lambda[c] for the faces the reverse step reads:
// along axis d indices 0..n_d (the last one is the high face of the last cell), the other two
// axes 0..n-1.
__global__ void face_coef_kernel(const double* __restrict__ L, double* __restrict__ lfx, double* __restrict__ lfy,
                                 double* __restrict__ lfz, int sy, long sz, int nx, int ny, int nz) {
  const long total = (long)(nx + 1) * (ny + 1) * (nz + 1);
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const int x = (int)(i % (nx + 1)), y = (int)((i / (nx + 1)) % (ny + 1)), z = (int)(i / ((long)(nx + 1) * (ny + 1)));
    const long c = (long)x + (long)sy * y + sz * z;
    const double lc = L[c];
    if (y < ny && z < nz) lfx[c] = L[c - 1] + lc;
    if (x < nx && z < nz) lfy[c] = L[c - sy] + lc;
    if (x < nx && y < ny) lfz[c] = L[c - sz] + lc;
  }
}

// dst = src rounded to FP32 (whole windows of the same layout).
__global__ void to_f32_kernel(const double* __restrict__ src, float* __restrict__ dst, long n) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    dst[i] = fixmath::f64_to_f32_rn(src[i]);
}

// abar_N = T_N - T_target on the interior (+ images); per-block partial sums of (T_N - T_target)^2.
template <typename S>
__global__ void loss_seed_kernel(const S* __restrict__ T, const double* __restrict__ Tt, double* __restrict__ A,
                                 int sy, long sz, int nx, int ny, int nz, double* __restrict__ partial) {
  double acc = 0.0;
  const long total = (long)nx * ny * nz;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < total; i += (long)gridDim.x * blockDim.x) {
    const int x = (int)(i % nx), y = (int)((i / nx) % ny), z = (int)(i / ((long)nx * ny));
    const long c = (long)x + (long)sy * y + sz * z;
    const double d = to_f64(T[c]) - Tt[c];
    acc = fma(d, d, acc);
    store_images1(A, sy, sz, x, y, z, nx, ny, nz, d);
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  __shared__ double sh[32];
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < (int)(blockDim.x + 31) / 32; ++i) t += sh[i];
    partial[blockIdx.x] = t;
  }
}

}  // namespace

int heat_step_dispatch(const nebo_field* T, const nebo_field* To, const nebo_field* L, double dt, const double sp[3],
                       cudaStream_t s);  // heat.cu

}  // namespace nebo

using namespace nebo;

// One reverse step (exposed for tests): Aout, glam from T_k, A_{k+1}; all windows one ghost
// layer, same shape; A_{k+1} and T_k must hold periodic ghost images (lam too).
extern "C" int nebo_heat_adjoint_step(const nebo_field* Tk, const nebo_field* Ain, const nebo_field* Aout,
                                      const nebo_field* lam, const nebo_field* glam, double dt, nebo_stream_t stream) {
  const nebo_field* fs[5] = {Tk, Ain, Aout, lam, glam};
  for (int i = 0; i < 5; ++i) {
    int rc = check_field(fs[i], "nebo_heat_adjoint_step");
    if (rc) return rc;
    if (fs[i]->dtype != NEBO_F64) return fail(NEBO_ERR_UNSUPPORTED, "Nebo error in nebo_heat_adjoint_step: FP64 only");
    if ((rc = check_periodic_patch(fs[i], 1, "nebo_heat_adjoint_step"))) return rc;
    if (i && (rc = check_same_layout(Tk, fs[i], "nebo_heat_adjoint_step"))) return rc;
  }
  int n[3];
  interior_extent(*Tk, n);
  const View<double> vt = make_view<double>(*Tk), va = make_view<double>(*Ain), vo = make_view<double>(*Aout),
                     vl = make_view<double>(*lam), vg = make_view<double>(*glam);
  const int gxb = (n[0] + BX - 1) / BX, gyb = (n[1] + BY - 1) / BY;
  static std::atomic<int> per_sm{0};  // z chunks in whole waves of resident blocks
  const int zchunk = wave_zchunk((long)gxb * gyb,
                                 (long)num_sms() * blocks_per_sm(heat_adjoint_kernel<true, false>, BX * BY, per_sm),
                                 n[2], 1, 8, 1);
  const int chunks = (n[2] + zchunk - 1) / zchunk;
  cudaStream_t s = (cudaStream_t)stream;
  LaunchScope ls("heat_adjoint_step", s);
  heat_adjoint_kernel<true, false><<<dim3(gxb, gyb, chunks), dim3(BX, BY), 0, s>>>(
      vt.base, va.base, vo.base, vl.base, nullptr, nullptr, nullptr, vg.base, vt.sy, vt.sz, n[0], n[1], n[2], zchunk,
      0.5 * dt);
  NEBO_LAUNCH_CHECK("nebo_heat_adjoint_step");
  return NEBO_OK;
}

namespace {
// One reverse step of the gradient driver: precomputed face coefficients (View bases of the
// three face arrays, same layout as T), exact or FP32 face products.
template <typename S>
int adjoint_step_lf(const nebo_field* Tk, const nebo_field* Ain, const nebo_field* Aout, const double* lfx,
                    const double* lfy, const double* lfz, const nebo_field* glam, double dt, bool exact,
                    cudaStream_t s) {
  int n[3];
  interior_extent(*Tk, n);
  const View<S> vt = make_view<S>(*Tk);
  const View<double> va = make_view<double>(*Ain), vo = make_view<double>(*Aout), vg = make_view<double>(*glam);
  const int gxb = (n[0] + BX - 1) / BX, gyb = (n[1] + BY - 1) / BY;
  static std::atomic<int> per_sm[2];  // z chunks in whole waves of resident blocks (zero: not queried)
  const int bps = exact ? blocks_per_sm(heat_adjoint_kernel<true, true, S>, BX * BY, per_sm[1])
                        : blocks_per_sm(heat_adjoint_kernel<false, true, S>, BX * BY, per_sm[0]);
  const int zchunk = wave_zchunk((long)gxb * gyb, (long)num_sms() * bps, n[2], 1, 8, 1);
  const int chunks = (n[2] + zchunk - 1) / zchunk;
  LaunchScope ls("heat_adjoint_step", s);
  if (exact)
    heat_adjoint_kernel<true, true, S><<<dim3(gxb, gyb, chunks), dim3(BX, BY), 0, s>>>(
        vt.base, va.base, vo.base, nullptr, lfx, lfy, lfz, vg.base, vt.sy, vt.sz, n[0], n[1], n[2], zchunk, 0.5 * dt);
  else
    heat_adjoint_kernel<false, true, S><<<dim3(gxb, gyb, chunks), dim3(BX, BY), 0, s>>>(
        vt.base, va.base, vo.base, nullptr, lfx, lfy, lfz, vg.base, vt.sy, vt.sz, n[0], n[1], n[2], zchunk, 0.5 * dt);
  NEBO_LAUNCH_CHECK("nebo_heat_gradient (reverse step)");
  return NEBO_OK;
}
}  // namespace

namespace {
// The state buffers (element type S, `stride` elements apart): [0, nck) checkpoints T_0, T_L, ...;
// [nck, nck+L) segment states; two forward temporaries; for FP32 states one more for the FP32
// copy of lambda.  The FP64 buffers: two adjoint states, three face-coefficient arrays, then 256
// doubles of loss partials.
template <typename S>
int gradient_impl(S* spool, size_t stride, double* dpool, size_t cells, int nck, int L, const nebo_field* T0,
                  const nebo_field* lam, const nebo_field* Ttarget, int steps, double dt, bool exact,
                  const nebo_field* gT0, const nebo_field* glam, double* J, nebo_stream_t stream) {
  constexpr bool f64 = std::is_same<S, double>::value;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t bytes = cells * sizeof(double);
  auto sbuf = [&](size_t i) { return spool + i * stride; };
  auto dbuf = [&](size_t i) { return dpool + i * cells; };
  double* partial = dpool + 5 * cells;
  auto state_at = [&](S* p) {
    nebo_field f = *T0;
    f.data = p;
    f.dtype = f64 ? NEBO_F64 : NEBO_F32;
    return f;
  };
  auto field_at = [&](double* p) {
    nebo_field f = *T0;
    f.data = p;
    return f;
  };
  const double unit[3] = {1.0, 1.0, 1.0};
  int rc = NEBO_OK;
  nebo_field lamf = *lam;
  int n[3];
  interior_extent(*T0, n);
  // lambda's ghosts must be periodic images (they are read at boundary faces); face coefficients
  if ((rc = fill_periodic_any(&lamf, s))) return rc;
  double* A0 = dbuf(0);
  double* A1 = dbuf(1);
  S* tmp0 = sbuf(nck + L);
  S* tmp1 = sbuf(nck + L + 1);
  const View<double> vl = make_view<double>(lamf);
  const long origin = vl.base - (const double*)lamf.data;  // interior origin within a window
  double* lf[3] = {dbuf(2) + origin, dbuf(3) + origin, dbuf(4) + origin};
  {
    LaunchScope ls("face_coef", s);
    face_coef_kernel<<<num_sms() * 4, 256, 0, s>>>(vl.base, lf[0], lf[1], lf[2], vl.sy, vl.sz, n[0], n[1], n[2]);
    NEBO_LAUNCH_CHECK("nebo_heat_gradient (face coefficients)");
  }
  // the forward sweep's lambda and T_0 in the state type
  nebo_field lamS = lamf;
  if constexpr (!f64) {
    lamS = state_at(sbuf(nck + L + 2));
    LaunchScope ls("to_f32", s);
    to_f32_kernel<<<num_sms() * 4, 256, 0, s>>>((const double*)lamf.data, (float*)lamS.data, (long)cells);
    to_f32_kernel<<<num_sms() * 4, 256, 0, s>>>((const double*)T0->data, (float*)sbuf(0), (long)cells);
    NEBO_LAUNCH_CHECK("nebo_heat_gradient (FP32 forward copies)");
  } else {
    NEBO_CUDA_TRY(cudaMemcpyAsync(sbuf(0), T0->data, bytes, cudaMemcpyDeviceToDevice, s));
  }
  // forward sweep: checkpoints every L steps; the last segment's states go straight to the
  // segment buffers (they need no recomputation)
  const int klast = (nck - 1) * L;
  {
    nebo_field c0 = state_at(sbuf(0));
    if ((rc = fill_periodic_any(&c0, s))) return rc;
  }
  S* cur = sbuf(0);
  for (int k = 0; k < steps && !rc; ++k) {
    const int j = k + 1;  // state being written
    S* nxt;
    if (j == steps)
      nxt = cur == tmp0 ? tmp1 : tmp0;
    else if (j % L == 0)
      nxt = sbuf(j / L);
    else if (j > klast)
      nxt = sbuf(nck + (j - klast - 1));
    else
      nxt = cur == tmp0 ? tmp1 : tmp0;
    nebo_field a = state_at(cur), b = state_at(nxt);
    rc = heat_step_dispatch(&a, &b, &lamS, dt, unit, s);
    cur = nxt;
  }
  if (rc) return rc;
  // seed: abar_N = T_N - T_target, J
  const View<S> vt = make_view<S>(state_at(cur));
  const View<double> vtt = make_view<double>(*Ttarget);
  const View<double> va = make_view<double>(field_at(A0));
  {
    LaunchScope ls("loss_seed", s);
    loss_seed_kernel<S><<<256, 256, 0, s>>>(vt.base, vtt.base, va.base, vt.sy, vt.sz, n[0], n[1], n[2], partial);
  }
  NEBO_CUDA_TRY(cudaGetLastError());
  double hp[256];
  NEBO_CUDA_TRY(cudaMemcpyAsync(hp, partial, sizeof(hp), cudaMemcpyDeviceToHost, s));
  NEBO_CUDA_TRY(cudaMemsetAsync(glam->data, 0, bytes, s));
  // reverse sweep, segment by segment
  double* Ain = A0;
  double* Aout = A1;
  for (int seg = nck - 1; seg >= 0 && !rc; --seg) {
    const int k0 = seg * L, k1 = (k0 + L < steps) ? k0 + L : steps;  // states k0 .. k1-1
    // recompute states k0+1 .. k1-1 into the segment buffers (state k0 is the checkpoint)
    for (int k = k0; seg != nck - 1 && k + 1 < k1 && !rc; ++k) {
      nebo_field a = state_at(k == k0 ? sbuf(seg) : sbuf(nck + (k - k0 - 1)));
      nebo_field b = state_at(sbuf(nck + (k - k0)));
      rc = heat_step_dispatch(&a, &b, &lamS, dt, unit, s);
    }
    for (int k = k1 - 1; k >= k0 && !rc; --k) {
      nebo_field tk = state_at(k == k0 ? sbuf(seg) : sbuf(nck + (k - k0 - 1)));
      nebo_field ai = field_at(Ain), ao = field_at(Aout);
      rc = adjoint_step_lf<S>(&tk, &ai, &ao, lf[0], lf[1], lf[2], glam, dt, exact, s);
      double* t = Ain;
      Ain = Aout;
      Aout = t;
    }
  }
  if (rc) return rc;
  NEBO_CUDA_TRY(cudaMemcpyAsync(gT0->data, Ain, bytes, cudaMemcpyDeviceToDevice, s));
  NEBO_CUDA_TRY(cudaStreamSynchronize(s));
  if (J) {
    double t = 0.0;
    for (int i = 0; i < 256; ++i) t += hp[i];
    *J = 0.5 * t;
  }
  return rc;
}

int gradient_entry(const nebo_field* T0, const nebo_field* lam, const nebo_field* Ttarget, int steps, double dt,
                   int checkpoint_every, bool exact, bool forward_f32, const nebo_field* gT0, const nebo_field* glam,
                   double* J, nebo_stream_t stream, const char* what) {
  const nebo_field* fs[5] = {T0, lam, Ttarget, gT0, glam};
  for (int i = 0; i < 5; ++i) {
    int rc = check_field(fs[i], what);
    if (rc) return rc;
    if (fs[i]->dtype != NEBO_F64) return fail(NEBO_ERR_UNSUPPORTED, "Nebo error in %s: FP64 only", what);
    if ((rc = check_periodic_patch(fs[i], 1, what))) return rc;
    if (i && (rc = check_same_layout(T0, fs[i], what))) return rc;
  }
  if (steps < 1) return fail(NEBO_ERR_INVALID, "Nebo error in %s: steps < 1", what);
  cudaStream_t s = (cudaStream_t)stream;
  const size_t cells = (size_t)T0->glob[0] * T0->glob[1] * T0->glob[2];
  const size_t ssize = forward_f32 ? sizeof(float) : sizeof(double);
  const size_t stride = (cells + 63) / 64 * 64;  // state buffers 256-byte aligned
  const size_t dbytes = 5 * cells * sizeof(double) + 256 * sizeof(double);
  int L = checkpoint_every > 0 ? checkpoint_every : (int)std::ceil(std::sqrt((double)steps));
  if (L > steps) L = steps;  // a segment never holds more than the run's states
  if (checkpoint_every == NEBO_CHECKPOINT_AUTO) {
    // every state kept (no recomputation) when all of them fit in 80 % of the free memory
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) == cudaSuccess) {
      if (((size_t)steps + 4) * stride * ssize + dbytes <= free_b / 10 * 8) L = 1;
    } else {
      cudaGetLastError();
    }
  }
  const int nck = (steps + L - 1) / L;  // checkpoints at steps 0, L, 2L, ...
  // state buffers: nck checkpoints + L segment states + 2 forward temporaries (+ FP32 lambda),
  // ~ 2 sqrt(N) fields; FP64: 2 adjoint states + 3 face-coefficient arrays
  const size_t nstate = (size_t)nck + (size_t)L + 2 + (forward_f32 ? 1 : 0);
  void* spool = nullptr;
  double* dpool = nullptr;
  pool_retain();
  NEBO_CUDA_TRY(cudaMallocAsync(&spool, nstate * stride * ssize, s));
  cudaError_t e = cudaMallocAsync((void**)&dpool, dbytes, s);
  if (e != cudaSuccess) {
    cudaFreeAsync(spool, s);
    return cuda_fail(e, what);
  }
  const int rc = forward_f32
                     ? gradient_impl<float>((float*)spool, stride, dpool, cells, nck, L, T0, lam, Ttarget, steps, dt,
                                            exact, gT0, glam, J, stream)
                     : gradient_impl<double>((double*)spool, stride, dpool, cells, nck, L, T0, lam, Ttarget, steps, dt,
                                             exact, gT0, glam, J, stream);
  cudaFreeAsync(spool, s);
  cudaFreeAsync(dpool, s);
  return rc;
}
}  // namespace

// Full gradient with sqrt(N) checkpointing.  T0, lam, Ttarget: windows (1 ghost, periodic patch);
// gT0, glam: outputs (windows; interiors written, glam overwritten); J: host result.
// checkpoint_every 0 (or below, other than NEBO_CHECKPOINT_AUTO) selects ceil(sqrt(steps));
// NEBO_CHECKPOINT_AUTO keeps every state when they fit in device memory.
extern "C" int nebo_heat_gradient(const nebo_field* T0, const nebo_field* lam, const nebo_field* Ttarget, int steps,
                                  double dt, int checkpoint_every, const nebo_field* gT0, const nebo_field* glam,
                                  double* J, nebo_stream_t stream) {
  return gradient_entry(T0, lam, Ttarget, steps, dt, checkpoint_every, true, false, gT0, glam, J, stream,
                        "nebo_heat_gradient");
}

extern "C" int nebo_heat_gradient_ex(const nebo_field* T0, const nebo_field* lam, const nebo_field* Ttarget, int steps,
                                     double dt, int checkpoint_every, int products, const nebo_field* gT0,
                                     const nebo_field* glam, double* J, nebo_stream_t stream) {
  const int prod = products & ~NEBO_FORWARD_F32;
  if (prod != NEBO_PRODUCTS_F64 && prod != NEBO_PRODUCTS_F32)
    return fail(NEBO_ERR_INVALID, "Nebo error in nebo_heat_gradient_ex: products %d", products);
  return gradient_entry(T0, lam, Ttarget, steps, dt, checkpoint_every, prod == NEBO_PRODUCTS_F64,
                        (products & NEBO_FORWARD_F32) != 0, gT0, glam, J, stream, "nebo_heat_gradient_ex");
}
