// Fused heat-equation step: Tout <<= T + dt*( DivX(InterpX(lam)*GradX(T)) + DivY(..) + DivZ(..) )
// on a single periodic SVol patch with one ghost layer, as one sm_103a kernel.
//
// Reference: the expression of examples/heat_equation.cpp:216-220 with the operators of
// spatialops/structured/stencil/StencilBuilder.cpp:60-72 (interp {1/2,1/2} at points (-1,0),
// grad {-1/dx,1/dx} at (-1,0), div {-1/dx,1/dx} at (0,+1)), evaluated by the reference as the
// nested tree of spatialops/NeboStencils.h:407-448 (each face flux recomputed per use).
//
// Design.  Blocks of 32x8 threads own a 32x8 column of cells and march a chunk of z planes.
// Every face flux is computed once: each thread computes the flux of its low x-, y- and
// z-face; high x/y faces come from the neighbour thread through shared memory (one warp of the
// block computes the tile's +x and +y halo faces), and the high z-face is carried in a register
// to the next plane.  The new value is written to the interior and, in the same pass, to its
// periodic ghost images, so no separate ghost-fill kernel runs between steps.
//
// Arithmetic.  FP64 with unit spacing uses the scaled form F' = (la+lb)*(tb-ta) = 2*F and
// T' = T + (dt/2)*(((Dx'+Dy')+Dz')); every scaling is by a power of two, so each rounding is the
// one the reference's serial walk performs and the result is bit-identical.  FP64 with general
// spacing evaluates the reference's own form (same operations, same order).  Both use _rn
// intrinsics so no multiply-add is contracted.  FP32 (storage and arithmetic) uses the scaled
// form with per-direction weights and lets the compiler fuse.
#include <climits>
#include <map>
#include <mutex>
#include <tuple>

#include "common.cuh"
#include "fp64_int.cuh"
#include "bulk.cuh"

namespace nebo {
namespace {

constexpr int BX = 32;
constexpr int BY = 8;

struct ExactD {
  static __device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }
  static __device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
  static __device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
};
struct FastF {
  static __device__ __forceinline__ float add(float a, float b) { return a + b; }
  static __device__ __forceinline__ float sub(float a, float b) { return a - b; }
  static __device__ __forceinline__ float mul(float a, float b) { return a * b; }
};

enum { MODE_UNIT = 0, MODE_REFERENCE = 1, MODE_WEIGHTED = 2 };

template <typename T>
struct HeatParams {
  T dt;       // time step
  T hdt;      // dt/2 (MODE_UNIT)
  T c0[3];    // -1/d per axis (MODE_REFERENCE)
  T c1[3];    // +1/d per axis
  T w[3];     // dt/(2 d^2) per axis (MODE_WEIGHTED)
};

// Flux through the face between cell a (low side) and cell b (high side).
template <typename T, class A, int MODE>
__device__ __forceinline__ T face_flux(T la, T lb, T ta, T tb, T c0, T c1) {
  if (MODE == MODE_REFERENCE) {
    const T interp = A::add(A::mul(la, T(0.5)), A::mul(lb, T(0.5)));
    const T grad = A::add(A::mul(ta, c0), A::mul(tb, c1));
    return A::mul(interp, grad);
  } else {
    return A::mul(A::add(la, lb), A::sub(tb, ta));
  }
}

// The periodic ghost images of boundary cell (x,y,z) (up to 7 cells; n >= 2 per axis).
template <typename T>
__device__ __forceinline__ void store_images_only(T* base, int sy, long sz, int x, int y, int z, int nx, int ny,
                                                  int nz, T v) {
  const int ax = x == 0 ? nx : -1, ay = y == 0 ? ny : -1, az = z == 0 ? nz : -1;
  const int m = (x == 0 || x == nx - 1) | ((y == 0 || y == ny - 1) << 1) | ((z == 0 || z == nz - 1) << 2);
  for (int b = 1; b < 8; ++b) {
    if (b & ~m) continue;
    const int xx = (b & 1) ? ax : x, yy = (b & 2) ? ay : y, zz = (b & 4) ? az : z;
    base[(long)xx + (long)sy * yy + sz * zz] = v;
  }
}

template <typename T>
__device__ __forceinline__ void store_with_images(T* base, int sy, long sz, int x, int y, int z, int nx, int ny,
                                                  int nz, T v) {
  base[(long)x + (long)sy * y + sz * z] = v;
  if (x != 0 && x != nx - 1 && y != 0 && y != ny - 1 && z != 0 && z != nz - 1) return;
  store_images_only(base, sy, sz, x, y, z, nx, ny, nz, v);
}

template <typename T, class A, int MODE>
__global__ void __launch_bounds__(BX* BY) heat_step_kernel(const T* __restrict__ tin, T* __restrict__ tout,
                                                           const T* __restrict__ lam, int sy, long sz, int nx, int ny,
                                                           int nz, int zchunk, HeatParams<T> p) {
  __shared__ T sfx[2][BY][BX + 1];
  __shared__ T sfy[2][BY + 1][BX];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int x0 = blockIdx.x * BX, y0 = blockIdx.y * BY;
  const int x = x0 + tx, y = y0 + ty;
  const int z0 = blockIdx.z * zchunk;
  const int z1 = min(z0 + zchunk, nz);
  const bool active = x < nx && y < ny;
  // inactive threads read the +ghost column/row, which exists, and write nothing
  const int xc = min(x, nx), yc = min(y, ny);
  auto at = [&](int i, int j, int k) { return (long)i + (long)sy * j + sz * k; };

  T tc = __ldg(tin + at(xc, yc, z0));
  T lc = __ldg(lam + at(xc, yc, z0));
  T fzlo = face_flux<T, A, MODE>(__ldg(lam + at(xc, yc, z0 - 1)), lc, __ldg(tin + at(xc, yc, z0 - 1)), tc, p.c0[2],
                                 p.c1[2]);
  for (int z = z0; z < z1; ++z) {
    const int buf = z & 1;
    const T tn = __ldg(tin + at(xc, yc, z + 1));
    const T ln = __ldg(lam + at(xc, yc, z + 1));
    const T fzhi = face_flux<T, A, MODE>(lc, ln, tc, tn, p.c0[2], p.c1[2]);
    const T fx = face_flux<T, A, MODE>(__ldg(lam + at(xc - 1, yc, z)), lc, __ldg(tin + at(xc - 1, yc, z)), tc, p.c0[0],
                                       p.c1[0]);
    const T fy = face_flux<T, A, MODE>(__ldg(lam + at(xc, yc - 1, z)), lc, __ldg(tin + at(xc, yc - 1, z)), tc, p.c0[1],
                                       p.c1[1]);
    sfx[buf][ty][tx] = fx;
    sfy[buf][ty][tx] = fy;
    if (ty == 0) {
      // +y halo face of column x: between rows y0+BY-1 and y0+BY
      const int yh = y0 + BY;
      if (yh <= ny && x <= nx) {
        sfy[buf][BY][tx] = face_flux<T, A, MODE>(__ldg(lam + at(xc, yh - 1, z)), __ldg(lam + at(xc, yh, z)),
                                                 __ldg(tin + at(xc, yh - 1, z)), __ldg(tin + at(xc, yh, z)), p.c0[1],
                                                 p.c1[1]);
      }
    } else if (ty == 1 && tx < BY) {
      // +x halo face of row y0+tx: between columns x0+BX-1 and x0+BX
      const int xh = x0 + BX, yr = y0 + tx;
      if (xh <= nx && yr < ny) {
        sfx[buf][tx][BX] = face_flux<T, A, MODE>(__ldg(lam + at(xh - 1, yr, z)), __ldg(lam + at(xh, yr, z)),
                                                 __ldg(tin + at(xh - 1, yr, z)), __ldg(tin + at(xh, yr, z)), p.c0[0],
                                                 p.c1[0]);
      }
    }
    __syncthreads();
    if (active) {
      const T fxhi = sfx[buf][ty][tx + 1];
      const T fyhi = sfy[buf][ty + 1][tx];
      T v;
      if (MODE == MODE_UNIT) {
        const T s = A::add(A::add(A::sub(fxhi, fx), A::sub(fyhi, fy)), A::sub(fzhi, fzlo));
        v = A::add(tc, A::mul(p.hdt, s));
      } else if (MODE == MODE_REFERENCE) {
        const T dx = A::add(A::mul(fx, p.c0[0]), A::mul(fxhi, p.c1[0]));
        const T dy = A::add(A::mul(fy, p.c0[1]), A::mul(fyhi, p.c1[1]));
        const T dz = A::add(A::mul(fzlo, p.c0[2]), A::mul(fzhi, p.c1[2]));
        v = A::add(tc, A::mul(p.dt, A::add(A::add(dx, dy), dz)));
      } else {
        v = tc + p.w[0] * (fxhi - fx) + p.w[1] * (fyhi - fy) + p.w[2] * (fzhi - fzlo);
      }
      store_with_images(tout, sy, sz, x, y, z, nx, ny, nz, v);
    }
    tc = tn;
    lc = ln;
    fzlo = fzhi;
  }
}


// FP32 heat step with an asynchronous plane pipeline.  FP32 arithmetic is nearly free on this
// GPU, so the kernel is bound by instruction issue and by the bytes it keeps in flight: each block
// streams planes of T and lambda (its 32x32 tile plus a one-cell halo) into a ring of NS shared-
// memory stages with cp.async, using no registers for the loads in flight, and each thread owns a
// column of four y-adjacent cells, so three of its five y faces are interior to it and the per-plane
// overhead (barrier, copies) is shared by four cells.  z chunks are multiples of NS and the z loop is
// unrolled by NS, so every stage index and shared-memory offset is a compile-time constant.  When
// the window's row pitch is even (VEC), halo rows are copied as 8-byte chunks (17 per row).
//
// Ring schedule: plane p (z0-1 <= p <= z1) lives in stage (p - z0 + NS) % NS.  Before the loop,
// planes z0-1 .. z0+NS-3 are issued (one commit group each) and the first two awaited; iteration z
// waits until at most NS-4 groups are pending (so planes up to z+1 have landed), syncs the block,
// issues plane z+NS-2 into the stage of plane z-2 (last read in iteration z-1, before the sync),
// then computes from the stages of planes z and z+1 (plane z-1 enters only through the z faces
// carried in registers).
constexpr int NS = 5;              // pipeline stages (planes resident or in flight)
constexpr int FTY = 32;            // tile y: a column of CPT cells per thread of the 32 x 8 block
constexpr int CPT = FTY / BY;
constexpr int HX = BX + 2, HY = FTY + 2;

__device__ __forceinline__ void cp_async4_s(uint32_t smem, const void* gmem) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async8_s(uint32_t smem, const void* gmem) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

template <bool VEC>
__global__ void __launch_bounds__(BX* BY, 3) heat_step_f32_async_kernel(const float* __restrict__ tin,
                                                                      float* __restrict__ tout,
                                                                      const float* __restrict__ lam, int sy, long sz,
                                                                      int nx, int ny, int nz, int zchunk, float w0,
                                                                      float w1, float w2) {
  constexpr int PLANE = HX * HY;                                // floats per stage and field
  constexpr int UNITS = VEC ? (HX / 2) * HY : PLANE;            // copies per plane and field
  constexpr int NCOPY = (UNITS + BX * BY - 1) / (BX * BY);      // copy slots per thread
  __shared__ __align__(16) float sT[NS * PLANE];
  __shared__ __align__(16) float sL[NS * PLANE];
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * BX + tx;
  const int x0 = blockIdx.x * BX, y0 = blockIdx.y * FTY;
  const int z0 = blockIdx.z * zchunk;  // a multiple of NS
  const int z1 = min(z0 + zchunk, nz);
  // copy slots: unit k of the (HY x HX) halo tile (VEC: 8-byte pairs of columns); units past the
  // +ghost column/row clamp to it (they exist and are never used; VEC keeps pairs aligned since
  // nx is even when the pitch is)
  int goff[NCOPY];  // within a plane (a plane holds fewer than 2^31 cells)
  uint32_t soff[NCOPY];
#pragma unroll
  for (int j = 0; j < NCOPY; ++j) {
    const int k = min(tid + j * BX * BY, UNITS - 1);
    if (VEC) {
      const int r = k / (HX / 2), c = 2 * (k - r * (HX / 2));
      goff[j] = min(x0 - 1 + c, nx - 1) + sy * min(y0 - 1 + r, ny);
      soff[j] = (uint32_t)((r * HX + c) * sizeof(float));
    } else {
      const int r = k / HX, c = k - r * HX;
      goff[j] = min(x0 - 1 + c, nx) + sy * min(y0 - 1 + r, ny);
      soff[j] = (uint32_t)(k * sizeof(float));
    }
  }
  const bool last_slot = tid + (NCOPY - 1) * BX * BY < UNITS;
  const uint32_t sT0 = (uint32_t)__cvta_generic_to_shared(sT), sL0 = (uint32_t)__cvta_generic_to_shared(sL);
  // plane p into stage st (a constant wherever the z loop below is unrolled)
  auto issue = [&](int p, int st) {
    if (p <= z1) {
      const uint32_t so = (uint32_t)st * (PLANE * sizeof(float));
      const float* tp = tin + sz * p;
      const float* lp = lam + sz * p;
#pragma unroll
      for (int j = 0; j < NCOPY; ++j) {
        if (j == NCOPY - 1 && !last_slot) break;
        if (VEC) {
          cp_async8_s(sT0 + so + soff[j], tp + goff[j]);
          cp_async8_s(sL0 + so + soff[j], lp + goff[j]);
        } else {
          cp_async4_s(sT0 + so + soff[j], tp + goff[j]);
          cp_async4_s(sL0 + so + soff[j], lp + goff[j]);
        }
      }
    }
  };
  issue(z0 - 1, NS - 1);
  cp_async_commit();
#pragma unroll
  for (int i = 0; i < NS - 2; ++i) {
    issue(z0 + i, i);
    cp_async_commit();
  }
  const int x = x0 + tx, yt = y0 + CPT * ty;
  const int ci = (CPT * ty + 1) * HX + tx + 1;  // the thread's first cell in a stage
  bool act[CPT], edge[CPT];
#pragma unroll
  for (int k = 0; k < CPT; ++k) {
    act[k] = x < nx && yt + k < ny;
    edge[k] = x == 0 || x == nx - 1 || yt + k == 0 || yt + k == ny - 1;
  }
  // centres and low z faces of plane z0 (planes z0-1 and z0 landed)
  cp_async_wait<NS - 3>();
  __syncthreads();
  float t[CPT], l[CPT], fz[CPT];
  {
    const float* Tm = sT + (NS - 1) * PLANE;
    const float* Lm = sL + (NS - 1) * PLANE;
#pragma unroll
    for (int k = 0; k < CPT; ++k) {
      t[k] = sT[ci + k * HX];
      l[k] = sL[ci + k * HX];
      fz[k] = (Lm[ci + k * HX] + l[k]) * (t[k] - Tm[ci + k * HX]);
    }
  }
  float* out = tout + (long)x + (long)sy * yt + sz * z0;
#pragma unroll 1
  for (int zb = z0; zb < z1; zb += NS) {
#pragma unroll
    for (int i = 0; i < NS; ++i) {
      const int z = zb + i;
      if (z >= z1) break;
      cp_async_wait<NS - 4>();  // planes up to z+1 have landed (this thread's copies)
      __syncthreads();          // ... and everyone's; plane z-2's stage is no longer read
      issue(z + NS - 2, (i + NS - 2) % NS);
      cp_async_commit();
      const float* T0 = sT + i * PLANE;
      const float* L0 = sL + i * PLANE;
      const float* Tn = sT + ((i + 1) % NS) * PLANE;
      const float* Ln = sL + ((i + 1) % NS) * PLANE;
      float tn[CPT], ln[CPT], fy[CPT + 1];
#pragma unroll
      for (int k = 0; k < CPT; ++k) {
        tn[k] = Tn[ci + k * HX];
        ln[k] = Ln[ci + k * HX];
      }
      fy[0] = (L0[ci - HX] + l[0]) * (t[0] - T0[ci - HX]);
#pragma unroll
      for (int k = 1; k < CPT; ++k) fy[k] = (l[k - 1] + l[k]) * (t[k] - t[k - 1]);
      fy[CPT] = (l[CPT - 1] + L0[ci + CPT * HX]) * (T0[ci + CPT * HX] - t[CPT - 1]);
      const bool zedge = z == 0 || z == nz - 1;
#pragma unroll
      for (int k = 0; k < CPT; ++k) {
        const int c = ci + k * HX;
        const float fxl = (L0[c - 1] + l[k]) * (t[k] - T0[c - 1]);
        const float fxh = (l[k] + L0[c + 1]) * (T0[c + 1] - t[k]);
        const float fzh = (l[k] + ln[k]) * (tn[k] - t[k]);
        const float v = t[k] + w0 * (fxh - fxl) + w1 * (fy[k + 1] - fy[k]) + w2 * (fzh - fz[k]);
        if (act[k]) {
          out[(long)sy * k] = v;
          if (edge[k] || zedge) store_images_only(tout, sy, sz, x, yt + k, z, nx, ny, nz, v);
        }
        fz[k] = fzh;
        t[k] = tn[k];
        l[k] = ln[k];
      }
      out += sz;
    }
  }
  cp_async_wait<0>();
}

// FP32 heat step on packed pairs (the 8-byte-aligned case).  Each thread owns two x-adjacent
// cells in two rows (a 2 x 2 block; 256 threads cover the same 32 x 32 tile and the same ring
// of NS stages as heat_step_f32_async_kernel).  The cells x, x+1 (x even) and their x
// neighbours x-1, x+2 are the two aligned pairs A = (x-1, x) and B = (x+1, x+2) of the stage
// row, so two 8-byte loads per field bring all four, and every flux, difference and update runs
// as one packed FP32x2 instruction for both cells (a - b as fma(b, -1, a), exact).  The next
// plane's pairs are loaded one iteration ahead and become the centre plane's.  Same arithmetic
// per cell as the scalar kernel: F = (la + lb)(tb - ta) per face,
//   T' = T + w0 (Fx+ - Fx-) + w1 (Fy+ - Fy-) + w2 (Fz+ - Fz-).
constexpr int QX = 16, QY = 16, QCPT = 2;  // pair-columns, thread rows, rows per thread (32 x 32 tile)
static_assert(2 * QX == BX && QY * QCPT == FTY, "the packed kernel shares the scalar kernel's tile");

__device__ __forceinline__ float2 psub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a); }
__device__ __forceinline__ float2 pflux(float2 la, float2 lb, float2 ta, float2 tb) {
  return __fmul2_rn(__fadd2_rn(la, lb), psub(tb, ta));
}

__global__ void __launch_bounds__(QX* QY, 3) heat_step_f32x2_kernel(const float* __restrict__ tin,
                                                                   float* __restrict__ tout,
                                                                   const float* __restrict__ lam, int sy, long sz,
                                                                   int nx, int ny, int nz, int zchunk, float w0,
                                                                   float w1, float w2) {
  constexpr int PLANE = HX * HY;                  // floats per stage and field
  constexpr int UNITS = (HX / 2) * HY;            // 8-byte pairs per plane and field
  constexpr int NT = QX * QY;
  constexpr int NCOPY = (UNITS + NT - 1) / NT;
  __shared__ __align__(16) float sT[NS * PLANE];
  __shared__ __align__(16) float sL[NS * PLANE];
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * QX + tx;
  const int x0 = blockIdx.x * BX, y0 = blockIdx.y * FTY;
  const int z0 = blockIdx.z * zchunk;  // a multiple of NS
  const int z1 = min(z0 + zchunk, nz);
  int goff[NCOPY];
  uint32_t soff[NCOPY];
#pragma unroll
  for (int j = 0; j < NCOPY; ++j) {
    const int k = min(tid + j * NT, UNITS - 1);
    const int r = k / (HX / 2), c = 2 * (k - r * (HX / 2));
    goff[j] = min(x0 - 1 + c, nx - 1) + sy * min(y0 - 1 + r, ny);
    soff[j] = (uint32_t)((r * HX + c) * sizeof(float));
  }
  const bool last_slot = tid + (NCOPY - 1) * NT < UNITS;
  const uint32_t sT0 = (uint32_t)__cvta_generic_to_shared(sT), sL0 = (uint32_t)__cvta_generic_to_shared(sL);
  auto issue = [&](int p, int st) {
    if (p <= z1) {
      const uint32_t so = (uint32_t)st * (PLANE * sizeof(float));
      const float* tp = tin + sz * p;
      const float* lp = lam + sz * p;
#pragma unroll
      for (int j = 0; j < NCOPY; ++j) {
        if (j == NCOPY - 1 && !last_slot) break;
        cp_async8_s(sT0 + so + soff[j], tp + goff[j]);
        cp_async8_s(sL0 + so + soff[j], lp + goff[j]);
      }
    }
  };
  issue(z0 - 1, NS - 1);
  cp_async_commit();
#pragma unroll
  for (int i = 0; i < NS - 2; ++i) {
    issue(z0 + i, i);
    cp_async_commit();
  }
  const int x = x0 + 2 * tx, yt = y0 + QCPT * ty;
  const int rc = QCPT * ty + 1;  // stage row of the thread's first cell
  const int pc = rc * HX + 2 * tx;  // float index of pair A of that row (cells x-1, x)
  bool act[QCPT], edge[QCPT];
#pragma unroll
  for (int k = 0; k < QCPT; ++k) {
    act[k] = x < nx && yt + k < ny;  // nx is even: x and x+1 are both inside or both outside
    edge[k] = x == 0 || x + 1 == nx - 1 || yt + k == 0 || yt + k == ny - 1;
  }
  auto pair = [](const float* st, int i) { return *reinterpret_cast<const float2*>(st + i); };
  auto centre = [](float2 a, float2 b) { return make_float2(a.y, b.x); };
  cp_async_wait<NS - 3>();
  __syncthreads();
  // centre plane z0: pairs A, B of T and lambda per row; low z faces from plane z0-1
  float2 aT[QCPT], bT[QCPT], aL[QCPT], bL[QCPT], fz[QCPT];
  {
    const float* T0 = sT;
    const float* L0 = sL;
    const float* Tm = sT + (NS - 1) * PLANE;
    const float* Lm = sL + (NS - 1) * PLANE;
#pragma unroll
    for (int k = 0; k < QCPT; ++k) {
      const int i = pc + k * HX;
      aT[k] = pair(T0, i);
      bT[k] = pair(T0, i + 2);
      aL[k] = pair(L0, i);
      bL[k] = pair(L0, i + 2);
      const float2 tm = centre(pair(Tm, i), pair(Tm, i + 2)), lm = centre(pair(Lm, i), pair(Lm, i + 2));
      fz[k] = pflux(lm, centre(aL[k], bL[k]), tm, centre(aT[k], bT[k]));
    }
  }
  const float2 W0 = make_float2(w0, w0), W1 = make_float2(w1, w1), W2 = make_float2(w2, w2);
  float* out = tout + (long)x + (long)sy * yt + sz * z0;
#pragma unroll 1
  for (int zb = z0; zb < z1; zb += NS) {
#pragma unroll
    for (int i = 0; i < NS; ++i) {
      const int z = zb + i;
      if (z >= z1) break;
      cp_async_wait<NS - 4>();  // planes up to z+1 have landed (this thread's copies)
      __syncthreads();          // ... and everyone's; plane z-2's stage is no longer read
      issue(z + NS - 2, (i + NS - 2) % NS);
      cp_async_commit();
      const float* T0 = sT + i * PLANE;
      const float* L0 = sL + i * PLANE;
      const float* Tn = sT + ((i + 1) % NS) * PLANE;
      const float* Ln = sL + ((i + 1) % NS) * PLANE;
      const bool zedge = z == 0 || z == nz - 1;
      // y face below the first row (from the row above the thread's block)
      float2 fyl;
      {
        const int jl = pc - HX;
        fyl = pflux(make_float2(L0[jl + 1], L0[jl + 2]), centre(aL[0], bL[0]), make_float2(T0[jl + 1], T0[jl + 2]),
                    centre(aT[0], bT[0]));
      }
#pragma unroll
      for (int k = 0; k < QCPT; ++k) {
        const int j = pc + k * HX;
        const float2 tc = centre(aT[k], bT[k]), lc = centre(aL[k], bL[k]);
        // y face above row k: row k+1 of this thread (not yet advanced) or the row beyond the block
        float2 fyh;
        if (k + 1 < QCPT) {
          fyh = pflux(lc, centre(aL[k + 1], bL[k + 1]), tc, centre(aT[k + 1], bT[k + 1]));
        } else {
          const int jh = pc + QCPT * HX;
          fyh = pflux(lc, make_float2(L0[jh + 1], L0[jh + 2]), tc, make_float2(T0[jh + 1], T0[jh + 2]));
        }
        const float2 naT = pair(Tn, j), nbT = pair(Tn, j + 2), naL = pair(Ln, j), nbL = pair(Ln, j + 2);
        const float2 fxl = pflux(aL[k], lc, aT[k], tc);  // faces x-1/2 of both cells
        const float2 fxh = pflux(lc, bL[k], tc, bT[k]);  // faces x+1/2
        const float2 fzh = pflux(lc, centre(naL, nbL), tc, centre(naT, nbT));
        float2 v = __ffma2_rn(W0, psub(fxh, fxl), tc);
        v = __ffma2_rn(W1, psub(fyh, fyl), v);
        v = __ffma2_rn(W2, psub(fzh, fz[k]), v);
        if (act[k]) {
          float* o = out + (long)sy * k;
          o[0] = v.x;
          o[1] = v.y;
          if (edge[k] || zedge) {
            store_images_only(tout, sy, sz, x, yt + k, z, nx, ny, nz, v.x);
            store_images_only(tout, sy, sz, x + 1, yt + k, z, nx, ny, nz, v.y);
          }
        }
        fz[k] = fzh;
        fyl = fyh;
        aT[k] = naT;
        bT[k] = nbT;
        aL[k] = naL;
        bL[k] = nbL;
      }
      out += sz;
    }
  }
  cp_async_wait<0>();
}

// ------------------------------------------------------------------ FP64 step in fixed point
// An FP64 heat step (FP64 storage, unit spacing) whose flux arithmetic runs on the integer pipe.
// With |T| < 2^ET and |lambda| < 2^EL over the windows, every value becomes a signed 64-bit
// integer in units of 2^(ET-61) (2^(EL-61)), truncated toward zero.  Per face the sum of the two
// lambdas and the difference of the two T are exact in 64 bits, their product exact in 128 bits,
// and the divergence S = (Fx+ - Fx-) + (Fy+ - Fy-) + (Fz+ - Fz-) exact in 128 bits; then
//   T' = fma(dt/2, RN(S 2^(ET+EL-122)), T)
// rounds twice.  The FP64 pipe runs one FMA per cell instead of the reference form's 16
// operations.  Error: each truncation moves a value by less than 2^(ET-61), so a step's error is
// within a few 2^-60 of max|T| (the reference's FP64 form: a few 2^-53 of each value), i.e. the
// result agrees with the reference to well within 1e-13 relative max-norm, but not bit for bit.
// ET comes from the previous step (each launch folds the largest biased exponent of what it
// writes into an integer in device memory; the first from a reduction pass).  A field with an
// infinity or a NaN, or too small for the scaled divergence to stay a normal double, runs the
// same kernel in plain FP64.
__device__ __forceinline__ long long to_fix61(double v, int E) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  const int e = (int)((b >> 52) & 0x7ff);
  const unsigned long long m = (b & 0xFFFFFFFFFFFFFull) | (e ? (1ull << 52) : 0ull);
  const int sh = (e ? e : 1) - 1014 - E;  // v 2^(61-E) = m 2^sh; sh <= 8 when |v| < 2^E
  const unsigned long long f = sh >= 0 ? m << sh : (sh > -64 ? m >> -sh : 0ull);
  return (b >> 63) ? -(long long)f : (long long)f;
}

// largest biased exponent of n doubles -> atomicMax(*out)
__global__ void max_biased_exp_kernel(const double* __restrict__ f, long n, int* __restrict__ out) {
  int m = 0;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    m = max(m, (int)(((unsigned long long)__double_as_longlong(f[i]) >> 52) & 0x7ff));
  m = __reduce_max_sync(0xffffffffu, m);
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

typedef __int128 i128;

// 64 x 64 -> 128-bit signed product (two 64-bit multiplies on the integer pipe)
__device__ __forceinline__ i128 mul_wide(long long a, long long b) {
  const unsigned long long lo = (unsigned long long)a * (unsigned long long)b;
  const long long hi = __mul64hi(a, b);
  return (i128)(((unsigned __int128)(unsigned long long)hi << 64) | lo);
}

// One plane of a 32 x 8 tile at a time: every value of the tile and of its one-cell x / y halo
// is converted once and staged in shared memory (two buffers, one barrier per plane); each thread
// then forms its cell's six face fluxes from the staged values (an in-plane face is formed by both
// of its cells with the same exact integer operations, so both see the same value), carrying the
// z faces and the next plane's converted values in registers.  In the plain FP64 fallback the
// same slots hold the doubles' bits and the fluxes are the exact form's.
__global__ void __launch_bounds__(BX* BY) heat_step_fix_kernel(const double* __restrict__ tin, double* __restrict__ tout,
                                                              const double* __restrict__ lam, int sy, long sz, int nx,
                                                              int ny, int nz, int zchunk, const int* __restrict__ eT,
                                                              const int* __restrict__ eL, int* __restrict__ eOut,
                                                              double hdt) {
  __shared__ long long cT[2][BY + 2][BX + 2];
  __shared__ long long cL[2][BY + 2][BX + 2];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int x0 = blockIdx.x * BX, y0 = blockIdx.y * BY;
  const int x = x0 + tx, y = y0 + ty;
  const int z0 = blockIdx.z * zchunk;
  const int z1 = min(z0 + zchunk, nz);
  const bool active = x < nx && y < ny;
  // inactive threads convert the +ghost column/row, which exists, and write nothing
  const int xc = min(x, nx), yc = min(y, ny);
  auto at = [&](int i, int j, int k) { return (long)i + (long)sy * j + sz * k; };
  const int bT = *eT, bL = *eL;  // largest biased exponents of T's and lambda's windows
  const int ET = bT - 1022, EL = bL - 1022;
  const int su = ET + EL - 122;  // S counts units of 2^su
  // plain FP64 (the exact unit form) for non-finite values or a scale whose results could leave
  // the normal range
  const bool plain = bT >= 2047 || bL >= 2047 || su < -900 || su > 900;
  auto cvt = [&](double v, int E) -> long long { return plain ? (long long)__double_as_longlong(v) : to_fix61(v, E); };
  auto asd = [](long long b) { return __longlong_as_double(b); };
  // the tile's one-cell halo, staged by three warps per plane: warp 0 the row below (y0 - 1),
  // warp 1 the row above (y0 + 8), lanes 0..15 of warp 2 the columns x0 - 1 and x0 + 32 of the
  // 8 rows; coordinates clamped into the window (a clamped cell is never read by an active cell)
  bool has_halo = false;
  int hx = 0, hy = 0, hsx = 0, hsy = 0;
  if (ty == 0) {
    has_halo = true;
    hx = xc;
    hy = y0 - 1;
    hsx = tx + 1;
    hsy = 0;
  } else if (ty == 1) {
    has_halo = true;
    hx = xc;
    hy = min(y0 + BY, ny);
    hsx = tx + 1;
    hsy = BY + 1;
  } else if (ty == 2 && tx < 2 * BY) {
    has_halo = true;
    const int r = tx % BY;
    hx = tx < BY ? x0 - 1 : min(x0 + BX, nx);
    hy = min(y0 + r, ny);
    hsx = tx < BY ? 0 : BX + 1;
    hsy = r + 1;
  }
  // face flux between staged/registered values (a low, b high)
  auto flux = [&](long long la, long long lb, long long ta, long long tb) -> i128 {
    if (plain) {
      const double f = __dmul_rn(__dadd_rn(asd(la), asd(lb)), __dsub_rn(asd(tb), asd(ta)));
      return (i128)(long long)__double_as_longlong(f);
    }
    return mul_wide(la + lb, tb - ta);
  };
  const long c0 = at(xc, yc, z0);
  long long tc = cvt(__ldg(tin + c0), ET), lc = cvt(__ldg(lam + c0), EL);
  i128 fzlo = flux(cvt(__ldg(lam + c0 - sz), EL), lc, cvt(__ldg(tin + c0 - sz), ET), tc);
  int emax = 0;
  for (int z = z0; z < z1; ++z) {
    const int buf = z & 1;
    const long c = at(xc, yc, z);
    cT[buf][ty + 1][tx + 1] = tc;
    cL[buf][ty + 1][tx + 1] = lc;
    if (has_halo) {
      const long h = at(hx, hy, z);
      cT[buf][hsy][hsx] = cvt(__ldg(tin + h), ET);
      cL[buf][hsy][hsx] = cvt(__ldg(lam + h), EL);
    }
    // the next plane of this cell (its z+1 face and next iteration's centre)
    const long long tn = cvt(__ldg(tin + c + sz), ET), ln = cvt(__ldg(lam + c + sz), EL);
    __syncthreads();
    const i128 fzhi = flux(lc, ln, tc, tn);
    if (active) {
      const long long tw = cT[buf][ty + 1][tx], te = cT[buf][ty + 1][tx + 2];
      const long long ts = cT[buf][ty][tx + 1], tnn = cT[buf][ty + 2][tx + 1];
      const long long lw = cL[buf][ty + 1][tx], le = cL[buf][ty + 1][tx + 2];
      const long long ls = cL[buf][ty][tx + 1], lnn = cL[buf][ty + 2][tx + 1];
      const i128 fx = flux(lw, lc, tw, tc), fxhi = flux(lc, le, tc, te);
      const i128 fy = flux(ls, lc, ts, tc), fyhi = flux(lc, lnn, tc, tnn);
      const double tcd = __ldg(tin + c);
      double v;
      if (plain) {
        auto d = [&](i128 f) { return __longlong_as_double((long long)f); };
        const double sum = __dadd_rn(__dadd_rn(__dsub_rn(d(fxhi), d(fx)), __dsub_rn(d(fyhi), d(fy))),
                                     __dsub_rn(d(fzhi), d(fzlo)));
        v = __dadd_rn(tcd, __dmul_rn(hdt, sum));
      } else {
        const i128 S = ((fxhi - fx) + (fyhi - fy)) + (fzhi - fzlo);
        v = fma(hdt, fixmath::units_to_double0(S, su), tcd);
      }
      store_with_images(tout, sy, sz, x, y, z, nx, ny, nz, v);
      emax = max(emax, (int)(((unsigned long long)__double_as_longlong(v) >> 52) & 0x7ff));
    }
    fzlo = fzhi;
    tc = tn;
    lc = ln;
  }
  emax = __reduce_max_sync(0xffffffffu, emax);
  if ((tx & 31) == 0) atomicMax(eOut, emax);
}

// ------------------------------------------------------------------ FP64 heat, fixed-point state
// NEBO_HEAT_FIXED_STATE: a run converts T once into signed 64-bit integers in units of 2^U and
// lambda once into integers of (dt/2) lambda in units of 2^(k-64); every step then works on
// integers only,
//   F  = hi64((lw_a + lw_b)(T_b - T_a))            (units 2^(U+k): the 128-bit product's high half)
//   T' = (T + (((Fx+ - Fx-) + (Fy+ - Fy-)) + (Fz+ - Fz-)) 2^k) 2^-s,
// and the last state goes back to doubles (one rounding).  No value is converted inside the time
// loop and the FP64 pipe is idle.  Both cells of a face form its flux with the same operations,
// so between rescalings the steps conserve the integer sum of T exactly, and the truncations of
// the high halves (toward -inf) cancel in expectation between a cell's two faces per axis.
// Bounds: with L = 2^(EL-1022) > max|lambda| and g = 1 + 24 |dt/2| L < 2^G, a state with
// |T| <= 2^b gives |T + divergence| < 2^(b+G).  Each launch ORs the ones' complements of the
// values it writes (|v| - 1 for v < 0: |v| <= 2^b for the OR's bit length b) into a device
// word; the next launch rescales what it writes by s = b + G - B (B = 63 - G; rounded to nearest
// when s > 0, exact when s < 0), so every state stays within 2^B, every sum inside 64 bits, and a
// state that neither grows nor decays settles at B - G bits (about 57) with s = 0.  U += s.  k is
// the smallest k >= 0 with |dt/2| L 2^(64-k) <= 2^61, so a sum of two lambda weights stays below
// 2^62; lambda >= 0 (checked), so that sum is unsigned and each face takes one unsigned high
// product and one sign correction for T_b - T_a.
// Error: a truncation (less than 2^(U+k) per face) and a rescaling (half a unit) per step, a few
// 2^-56 of max|T| at most, well inside 1e-13 relative; the final conversion rounds once.  A field
// with an infinity or a NaN, a negative lambda, exponents outside +-900, or a growth bound g
// above 2^20 runs the exact FP64 form on the same buffers (bit-identical to nebo_heat_run).
struct FxState {
  int eT, eL;                // largest biased exponents of T's and lambda's windows
  int negL;                  // some lambda < 0
  int plain, G, k;           // plain: the exact FP64 form; G, k as above (B = 63 - G)
  int U[3];                  // state j counts units of 2^U[j % 3]
  unsigned long long M[3];   // OR of the magnitudes of state j (the bit length of the largest)
};

// ceil(log2 v) for v > 0 (exact: frexp is exact)
__device__ __forceinline__ int ceil_log2(double v) {
  int e;
  const double m = frexp(v, &e);  // v = m 2^e, m in [0.5, 1)
  return m == 0.5 ? e - 1 : e;
}

__global__ void fxs_setup_kernel(FxState* c, double w) {
  const int eT = c->eT, eL = c->eL;
  const double aw = fabs(w);
  const double wl = aw * ldexp(1.0, (eL ? eL : 1) - 1022);  // > max |w lambda|
  const int G = ceil_log2(1.0 + 24.0 * wl);
  const int k = wl > 0.0 ? max(0, ceil_log2(wl) + 3) : 0;
  const int u = (eT ? eT : 1) - 1022;
  c->plain = eT >= 2047 || eL >= 2047 || c->negL || !(aw < INFINITY) || u > 900 || u < -900 || G > 20 || k > 40;
  c->G = G;
  c->k = k;
  c->U[0] = u - (63 - G);  // |T| < 2^u: state 0 has at most B bits
  c->M[0] = c->M[1] = c->M[2] = 0ull;
}

// largest biased exponent of lambda -> atomicMax(c->eL); any lambda < 0 -> c->negL = 1
__global__ void fxs_lambda_scan_kernel(const double* __restrict__ f, long n, FxState* __restrict__ c) {
  int m = 0, neg = 0;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const double v = f[i];
    m = max(m, (int)(((unsigned long long)__double_as_longlong(v) >> 52) & 0x7ff));
    neg |= v < 0.0;
  }
  m = __reduce_max_sync(0xffffffffu, m);
  neg = __reduce_or_sync(0xffffffffu, neg);
  if ((threadIdx.x & 31) == 0) {
    atomicMax(&c->eL, m);
    if (neg) atomicOr(&c->negL, 1);
  }
}

__device__ __forceinline__ unsigned long long or_warp64(unsigned long long v) {
  const unsigned lo = __reduce_or_sync(0xffffffffu, (unsigned)v);
  const unsigned hi = __reduce_or_sync(0xffffffffu, (unsigned)(v >> 32));
  return ((unsigned long long)hi << 32) | lo;
}

// state 0 and the lambda weights (every cell of the windows, ghosts included)
__global__ void fxs_convert_kernel(const double* __restrict__ t, long long* __restrict__ tfix,
                                   const double* __restrict__ lam, long long* __restrict__ lw, long n,
                                   FxState* __restrict__ c, double w) {
  const bool plain = c->plain;
  const int U = c->U[0], k = c->k;
  unsigned long long m = 0;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const double tv = t[i], lv = lam[i];
    if (plain) {
      tfix[i] = __double_as_longlong(tv);
      lw[i] = __double_as_longlong(lv);
    } else {
      const long long a = __double2ll_rn(ldexp(tv, -U));
      tfix[i] = a;
      lw[i] = __double2ll_rn(ldexp(w * lv, 64 - k));
      m |= (unsigned long long)(a ^ (a >> 63));
    }
  }
  m = or_warp64(m);
  if ((threadIdx.x & 31) == 0 && m) atomicOr(&c->M[0], m);
}

__global__ void fxs_finish_kernel(const long long* __restrict__ tfix, double* __restrict__ t, long n,
                                  const FxState* __restrict__ c, int slot) {
  const bool plain = c->plain;
  const int U = c->U[slot];
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    const long long v = tfix[i];
    t[i] = plain ? __longlong_as_double(v) : ldexp(__ll2double_rn(v), U);
  }
}

// One step on a 32 x 8 tile marching z, staged like heat_step_fix_kernel (the tile and its x / y
// halo in shared memory, two buffers, one barrier per plane; z faces in registers), with the
// global loads one plane ahead: iteration z stages plane z (loaded in iteration z-1) and loads the
// halo of plane z+1 and the cell of plane z+2.
// KIND 0: the doubles' bits, exact FP64 form; 1: integers; 2: integers, output rescaled by 2^-s.
typedef long long FxPlane[BY + 2][BX + 2];

template <int KIND>
__device__ __forceinline__ void fxs_step(const long long* __restrict__ tin, long long* __restrict__ tout,
                                         const long long* __restrict__ lw, int sy, long sz, int nx, int ny, int nz,
                                         int zchunk, int s, int k, double hdt, FxPlane* cT, FxPlane* cL,
                                         unsigned long long& mag) {
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int x0 = blockIdx.x * BX, y0 = blockIdx.y * BY;
  const int x = x0 + tx, y = y0 + ty;
  const int z0 = blockIdx.z * zchunk;
  const int z1 = min(z0 + zchunk, nz);
  const bool active = x < nx && y < ny;
  const int xc = min(x, nx), yc = min(y, ny);
  auto at = [&](int i, int j, int kk) { return (long)i + (long)sy * j + sz * kk; };
  auto asd = [](long long b) { return __longlong_as_double(b); };
  auto flux = [&](long long la, long long lb, long long ta, long long tb) -> long long {
    if (KIND == 0) return __double_as_longlong(__dmul_rn(__dadd_rn(asd(la), asd(lb)), __dsub_rn(asd(tb), asd(ta))));
    const unsigned long long kap = (unsigned long long)(la + lb);  // < 2^62, lambda >= 0
    const long long d = tb - ta;
    return (long long)(__umul64hi(kap, (unsigned long long)d) - (d < 0 ? kap : 0ull));
  };
  // halo staging as in heat_step_fix_kernel: warp 0 the row below, warp 1 the row above, lanes
  // 0..15 of warp 2 the columns x0 - 1 and x0 + 32 (coordinates clamped into the window)
  bool has_halo = false;
  int hx = 0, hy = 0, hsx = 0, hsy = 0;
  if (ty == 0) {
    has_halo = true;
    hx = xc;
    hy = y0 - 1;
    hsx = tx + 1;
  } else if (ty == 1) {
    has_halo = true;
    hx = xc;
    hy = min(y0 + BY, ny);
    hsx = tx + 1;
    hsy = BY + 1;
  } else if (ty == 2 && tx < 2 * BY) {
    has_halo = true;
    const int r = tx % BY;
    hx = tx < BY ? x0 - 1 : min(x0 + BX, nx);
    hy = min(y0 + r, ny);
    hsx = tx < BY ? 0 : BX + 1;
    hsy = r + 1;
  }
  const long c0 = at(xc, yc, z0), h0 = at(hx, hy, z0);
  long long tc = __ldg(tin + c0), lc = __ldg(lw + c0);
  long long fzlo = flux(__ldg(lw + c0 - sz), lc, __ldg(tin + c0 - sz), tc);
  long long tn = __ldg(tin + c0 + sz), ln = __ldg(lw + c0 + sz);  // plane z0 + 1 (z0 + 1 <= nz)
  long long ht = 0, hl = 0;
  if (has_halo) {
    ht = __ldg(tin + h0);
    hl = __ldg(lw + h0);
  }
  for (int z = z0; z < z1; ++z) {
    const int buf = z & 1;
    const long dz = (long)(z - z0) * sz;
    cT[buf][ty + 1][tx + 1] = tc;
    cL[buf][ty + 1][tx + 1] = lc;
    if (has_halo) {
      cT[buf][hsy][hsx] = ht;
      cL[buf][hsy][hsx] = hl;
    }
    // the loads of the next iteration: the halo of plane z+1 (<= nz) and the cell of plane
    // z+2 (clamped to the ghost plane nz; the clamped value is never used)
    const long n2 = c0 + dz + (z + 2 <= nz ? 2 : 1) * sz;
    const long long tn2 = __ldg(tin + n2), ln2 = __ldg(lw + n2);
    long long ht2 = 0, hl2 = 0;
    if (has_halo) {
      ht2 = __ldg(tin + h0 + dz + sz);
      hl2 = __ldg(lw + h0 + dz + sz);
    }
    __syncthreads();
    const long long fzhi = flux(lc, ln, tc, tn);
    if (active) {
      const long long tw = cT[buf][ty + 1][tx], te = cT[buf][ty + 1][tx + 2];
      const long long ts = cT[buf][ty][tx + 1], tnn = cT[buf][ty + 2][tx + 1];
      const long long lwe = cL[buf][ty + 1][tx], le = cL[buf][ty + 1][tx + 2];
      const long long ls = cL[buf][ty][tx + 1], lnn = cL[buf][ty + 2][tx + 1];
      const long long fx = flux(lwe, lc, tw, tc), fxhi = flux(lc, le, tc, te);
      const long long fy = flux(ls, lc, ts, tc), fyhi = flux(lc, lnn, tc, tnn);
      long long v;
      if (KIND == 0) {
        const double sum = __dadd_rn(__dadd_rn(__dsub_rn(asd(fxhi), asd(fx)), __dsub_rn(asd(fyhi), asd(fy))),
                                     __dsub_rn(asd(fzhi), asd(fzlo)));
        v = __double_as_longlong(__dadd_rn(asd(tc), __dmul_rn(hdt, sum)));
      } else {
        const long long S = ((fxhi - fx) + (fyhi - fy)) + (fzhi - fzlo);
        v = tc + (long long)((unsigned long long)S << k);
        if (KIND == 2) v = s > 0 ? (v >> s) + ((v >> (s - 1)) & 1) : (long long)((unsigned long long)v << -s);
        mag |= (unsigned long long)(v ^ (v >> 63));
      }
      store_with_images(tout, sy, sz, x, y, z, nx, ny, nz, v);
    }
    fzlo = fzhi;
    tc = tn;
    lc = ln;
    tn = tn2;
    ln = ln2;
    ht = ht2;
    hl = hl2;
  }
}

__global__ void __launch_bounds__(BX* BY) heat_step_fxs_kernel(const long long* __restrict__ tin,
                                                              long long* __restrict__ tout,
                                                              const long long* __restrict__ lw, int sy, long sz,
                                                              int nx, int ny, int nz, int zchunk,
                                                              FxState* __restrict__ c, int j, double hdt) {
  __shared__ long long cT[2][BY + 2][BX + 2];
  __shared__ long long cL[2][BY + 2][BX + 2];
  const int slot = j % 3;
  const bool plain = c->plain != 0;
  const unsigned long long M = c->M[slot];
  const int G = c->G;
  const int s = (plain || M == 0ull) ? 0 : (64 - __clzll((long long)M)) + G - (63 - G);
  if (blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0 && threadIdx.x == 0 && threadIdx.y == 0) {
    c->U[(j + 1) % 3] = c->U[slot] + s;  // read by the next launch
    c->M[(j + 2) % 3] = 0ull;            // the slot the previous launch read; the next one ORs into it
  }
  unsigned long long mag = 0;
  if (plain)
    fxs_step<0>(tin, tout, lw, sy, sz, nx, ny, nz, zchunk, 0, 0, hdt, cT, cL, mag);
  else if (s == 0)
    fxs_step<1>(tin, tout, lw, sy, sz, nx, ny, nz, zchunk, 0, c->k, hdt, cT, cL, mag);
  else
    fxs_step<2>(tin, tout, lw, sy, sz, nx, ny, nz, zchunk, s, c->k, hdt, cT, cL, mag);
  if (!plain) {
    mag = or_warp64(mag);
    if (((threadIdx.y * BX + threadIdx.x) & 31) == 0 && mag) atomicOr(&c->M[(j + 1) % 3], mag);
  }
}

// The time loop of NEBO_HEAT_FIXED_STATE (T's ghosts filled, steps >= 1): state 0 goes into Ttmp,
// the states ping-pong between Ttmp and T (as integers), the last one is converted into T.
int heat_run_fixed_state(const nebo_field* T, const nebo_field* Ttmp, const nebo_field* lam, int steps, double dt,
                         cudaStream_t s, const char* what) {
  int n[3];
  interior_extent(*T, n);
  const long cells = (long)T->glob[0] * T->glob[1] * T->glob[2];
  FxState* c = nullptr;
  long long* lw = nullptr;
  pool_retain();
  NEBO_CUDA_TRY(cudaMallocAsync((void**)&c, sizeof(FxState), s));
  cudaError_t err = cudaMallocAsync((void**)&lw, (size_t)cells * sizeof(long long), s);
  if (err != cudaSuccess) {
    cudaFreeAsync(c, s);
    return cuda_fail(err, what);
  }
  const double w = 0.5 * dt;
  const int rblocks = num_sms() * 4;
  err = cudaMemsetAsync(c, 0, sizeof(FxState), s);
  if (err == cudaSuccess) {
    LaunchScope ls("heat_fixed_state_in", s);
    max_biased_exp_kernel<<<rblocks, 256, 0, s>>>((const double*)T->data, cells, &c->eT);
    fxs_lambda_scan_kernel<<<rblocks, 256, 0, s>>>((const double*)lam->data, cells, c);
    fxs_setup_kernel<<<1, 1, 0, s>>>(c, w);
    fxs_convert_kernel<<<rblocks, 256, 0, s>>>((const double*)T->data, (long long*)Ttmp->data,
                                               (const double*)lam->data, lw, cells, c, w);
    err = cudaGetLastError();
  }
  const View<long long> va = make_view<long long>(*Ttmp), vb = make_view<long long>(*T);
  const long long* lwb = lw + (va.base - (long long*)Ttmp->data);  // lambda weights, same layout
  const int gxb = (n[0] + BX - 1) / BX, gyb = (n[1] + BY - 1) / BY;
  static std::atomic<int> per_sm{0};
  const int zchunk = wave_zchunk((long)gxb * gyb, (long)num_sms() * blocks_per_sm(heat_step_fxs_kernel, BX * BY, per_sm),
                                 n[2], 2, 4, 1);
  const dim3 grid(gxb, gyb, (n[2] + zchunk - 1) / zchunk), block(BX, BY);
  long long* buf[2] = {va.base, vb.base};
  for (int j = 0; j < steps && err == cudaSuccess; ++j) {
    LaunchScope ls("heat_step_fixed_state", s);
    heat_step_fxs_kernel<<<grid, block, 0, s>>>(buf[j & 1], buf[(j + 1) & 1], lwb, va.sy, va.sz, n[0], n[1], n[2],
                                                zchunk, c, j, w);
    err = cudaGetLastError();
  }
  if (err == cudaSuccess) {
    LaunchScope ls("heat_fixed_state_out", s);
    const long long* last = (steps & 1) ? (const long long*)T->data : (const long long*)Ttmp->data;
    fxs_finish_kernel<<<rblocks, 256, 0, s>>>(last, (double*)T->data, cells, c, steps % 3);
    err = cudaGetLastError();
  }
  cudaFreeAsync(lw, s);
  cudaFreeAsync(c, s);
  if (err != cudaSuccess) return cuda_fail(err, what);
  return NEBO_OK;
}

// ------------------------------------------------------------------ FP32 step on bulk-copied slabs
// The FP32 fields' rows are full-width slabs in HBM: rows y0-1 .. y0+8 of a plane (10 x gx floats)
// are one contiguous run that starts on an even row, so with an even row pitch it is 16-byte
// aligned and a multiple of 16 bytes long: one cp.async.bulk per plane and field moves it into
// shared memory, issued by one thread and tracked by an mbarrier (no per-thread copy
// instructions, no per-thread waits on copy groups).  A block of 256 threads owns 8 full rows
// and marches a chunk of z planes through a ring of BK_NS stages: at plane z it computes from the
// stages of planes z and z+1 (the z face below is carried in a register) while the copy of plane
// z+2 is in flight.  Every wait is bounded (about a second of clock cycles); a wait that gives
// up is counted in g_bulk_timeouts, which nebo_stream_sync reports as NEBO_ERR_TIMEOUT.
constexpr int BK_RY = 8;              // interior rows per block
constexpr int BK_ROWS = BK_RY + 2;    // rows per stage (one halo row on each side)
constexpr int BK_NS = 3;              // stages (three blocks per SM)

__device__ unsigned int g_bulk_timeouts;

// Packed pairs: a thread owns the x-adjacent cells (x, x+1), x even, in four rows (two groups of
// 128 pair columns cover the block's 8 rows).  The aligned 8-byte pairs (x-1, x) and (x+1, x+2)
// of a stage row bring both cells and their x neighbours; every face flux and the update run as
// packed FP32x2 operations (the arithmetic of heat_step_f32x2_kernel).  The slab layout needs an
// even row pitch, so nx is even.  Three stages (62 KB) and at most 80 registers let three blocks
// (24 warps) share an SM.
constexpr int BP_PAIRS = 128;  // pair columns per block: nx <= 256
constexpr int BP_RPT = 4;      // rows per thread
constexpr int BP_THREADS = BP_PAIRS * (BK_RY / BP_RPT);
static_assert(BK_RY % BP_RPT == 0, "the block's rows split evenly between the groups");

__global__ void __launch_bounds__(BP_THREADS, 3) heat_step_f32_bulk2_kernel(const float* __restrict__ tin,
                                                                           float* __restrict__ tout,
                                                                           const float* __restrict__ lam, int gx,
                                                                           long sz, int nx, int ny, int nz, int zchunk,
                                                                           float w0, float w1, float w2) {
  extern __shared__ __align__(128) unsigned char bk_smem[];
  const int sf = BK_ROWS * gx;  // floats per stage and field
  const uint32_t bytes = (uint32_t)sf * 4u;
  const float* sb = reinterpret_cast<const float*>(bk_smem);
  const uint32_t s0 = (uint32_t)__cvta_generic_to_shared(bk_smem);
  const uint32_t bar0 = s0 + (uint32_t)(BK_NS * 2) * bytes;
  const int tid = threadIdx.x;
  const int y0 = blockIdx.x * BK_RY;
  const int z0 = blockIdx.y * zchunk, z1 = min(z0 + zchunk, nz);
  if (tid == 0) {
    for (int st = 0; st < BK_NS; ++st) mbar_init(bar0 + 8 * st, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  // plane q of the chunk is interior plane z0 - 1 + q, in stage q % BK_NS, phase (q / BK_NS) & 1
  auto issue = [&](int q) {
    if (z0 - 1 + q > z1) return;
    const int st = q % BK_NS;
    const uint32_t bar = bar0 + 8 * st;
    const long off = (long)(z0 + q) * sz + (long)y0 * gx;
    mbar_expect_tx(bar, 2 * bytes);
    bulk_g2s(s0 + (uint32_t)(2 * st) * bytes, tin + off, bytes, bar);
    bulk_g2s(s0 + (uint32_t)(2 * st + 1) * bytes, lam + off, bytes, bar);
  };
  if (tid == 0)
    for (int q = 0; q < BK_NS; ++q) issue(q);
  const int x = 2 * (tid % BP_PAIRS), g = x + 1;  // cells x, x+1 at glob columns g, g+1
  const int rg = (tid / BP_PAIRS) * BP_RPT;       // the group's first row
  const bool active = x < nx;
  const bool xedge0 = x == 0, xedge1 = x + 1 == nx - 1;
  auto pair = [](const float* row, int i) { return *reinterpret_cast<const float2*>(row + i); };
  auto centre = [](float2 a, float2 b) { return make_float2(a.y, b.x); };
  bool ok = mbar_wait(bar0, 0) & mbar_wait(bar0 + 8, 0);
  float2 fz[BP_RPT];
  {
    const float* Tm = sb;  // stage 0: plane z0 - 1
    const float* Lm = sb + sf;
    const float* Tc = sb + 2 * sf;  // stage 1: plane z0
    const float* Lc = sb + 3 * sf;
#pragma unroll
    for (int r = 0; r < BP_RPT; ++r) {
      const int i = (rg + r + 1) * gx + g;
      fz[r] = active ? pflux(centre(pair(Lm, i - 1), pair(Lm, i + 1)), centre(pair(Lc, i - 1), pair(Lc, i + 1)),
                             centre(pair(Tm, i - 1), pair(Tm, i + 1)), centre(pair(Tc, i - 1), pair(Tc, i + 1)))
                     : make_float2(0.f, 0.f);
    }
  }
  const float2 W0 = make_float2(w0, w0), W1 = make_float2(w1, w1), W2 = make_float2(w2, w2);
  float* out = tout + (long)x + (long)gx * (y0 + rg) + sz * z0;
#pragma unroll 1
  for (int z = z0; z < z1; ++z) {
    const int q = z - z0 + 1;  // centre plane
    __syncthreads();           // plane q-1's stage is no longer read
    if (tid == 0) {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      issue(q - 1 + BK_NS);
    }
    ok &= mbar_wait(bar0 + 8 * ((q + 1) % BK_NS), ((q + 1) / BK_NS) & 1);
    const float* Tc = sb + 2 * (q % BK_NS) * sf;
    const float* Lc = Tc + sf;
    const float* Tn = sb + 2 * ((q + 1) % BK_NS) * sf;
    const float* Ln = Tn + sf;
    if (active) {
      const bool zedge = z == 0 || z == nz - 1;
      const int i0 = (rg + 1) * gx + g;
      float2 aT = pair(Tc, i0 - 1), bT = pair(Tc, i0 + 1), aL = pair(Lc, i0 - 1), bL = pair(Lc, i0 + 1);
      float2 fyl = pflux(centre(pair(Lc, i0 - gx - 1), pair(Lc, i0 - gx + 1)), centre(aL, bL),
                         centre(pair(Tc, i0 - gx - 1), pair(Tc, i0 - gx + 1)), centre(aT, bT));
#pragma unroll
      for (int r = 0; r < BP_RPT; ++r) {
        const int i = i0 + r * gx;
        const float2 uaT = pair(Tc, i + gx - 1), ubT = pair(Tc, i + gx + 1);
        const float2 uaL = pair(Lc, i + gx - 1), ubL = pair(Lc, i + gx + 1);
        const float2 tc = centre(aT, bT), lc = centre(aL, bL);
        const float2 fxl = pflux(aL, lc, aT, tc);  // faces x-1/2 of both cells
        const float2 fxh = pflux(lc, bL, tc, bT);  // faces x+1/2
        const float2 fyh = pflux(lc, centre(uaL, ubL), tc, centre(uaT, ubT));
        const float2 fzh = pflux(lc, centre(pair(Ln, i - 1), pair(Ln, i + 1)), tc,
                                 centre(pair(Tn, i - 1), pair(Tn, i + 1)));
        float2 v = __ffma2_rn(W0, psub(fxh, fxl), tc);
        v = __ffma2_rn(W1, psub(fyh, fyl), v);
        v = __ffma2_rn(W2, psub(fzh, fz[r]), v);
        float* o = out + (long)gx * r;
        o[0] = v.x;
        o[1] = v.y;
        const int y = y0 + rg + r;
        const bool yzedge = zedge || y == 0 || y == ny - 1;
        if (xedge0 || yzedge) store_images_only(tout, gx, sz, x, y, z, nx, ny, nz, v.x);
        if (xedge1 || yzedge) store_images_only(tout, gx, sz, x + 1, y, z, nx, ny, nz, v.y);
        fz[r] = fzh;
        fyl = fyh;
        aT = uaT;
        bT = ubT;
        aL = uaL;
        bL = ubL;
      }
    }
    out += sz;
  }
  if (!ok) atomicAdd(&g_bulk_timeouts, 1u);
}

int check_heat(const nebo_field* T, const nebo_field* To, const nebo_field* L, const char* what) {
  int rc;
  if ((rc = check_field(T, what)) || (rc = check_field(To, what)) || (rc = check_field(L, what))) return rc;
  if ((rc = check_same_layout(T, To, what)) || (rc = check_same_layout(T, L, what))) return rc;
  if ((rc = check_periodic_patch(T, 1, what))) return rc;
  if (T->data == To->data) return fail(NEBO_ERR_INVALID, "Nebo error in %s: in-place stencil update", what);
  return NEBO_OK;
}

template <typename T>
int launch_heat(const nebo_field* Tf, const nebo_field* Tof, const nebo_field* Lf, double dt, const double sp[3],
                cudaStream_t s) {
  int n[3];
  interior_extent(*Tf, n);
  const View<T> vin = make_view<T>(*Tf), vout = make_view<T>(*Tof), vl = make_view<T>(*Lf);
  HeatParams<T> p;
  p.dt = (T)dt;
  p.hdt = (T)(0.5 * dt);
  for (int i = 0; i < 3; ++i) {
    p.c0[i] = (T)(-1.0 / sp[i]);
    p.c1[i] = (T)(1.0 / sp[i]);
    p.w[i] = (T)(0.5 * dt / (sp[i] * sp[i]));
  }
  const int gxb = (n[0] + BX - 1) / BX, gyb = (n[1] + BY - 1) / BY;
  const bool unit = sp[0] == 1.0 && sp[1] == 1.0 && sp[2] == 1.0;
  if constexpr (sizeof(T) == 8) {
    // z chunks in whole waves of resident blocks (a chunk re-reads one plane below it)
    static std::atomic<int> per_sm[2];  // zero: not queried
    const int bps = unit ? blocks_per_sm(heat_step_kernel<double, ExactD, MODE_UNIT>, BX * BY, per_sm[1])
                         : blocks_per_sm(heat_step_kernel<double, ExactD, MODE_REFERENCE>, BX * BY, per_sm[0]);
    const int zchunk = wave_zchunk((long)gxb * gyb, (long)num_sms() * bps, n[2], 1, 4, 1);
    dim3 grid(gxb, gyb, (n[2] + zchunk - 1) / zchunk), block(BX, BY);
    LaunchScope ls("heat_step_f64", s);
    if (unit)
      heat_step_kernel<double, ExactD, MODE_UNIT><<<grid, block, 0, s>>>(vin.base, vout.base, vl.base, vin.sy, vin.sz,
                                                                         n[0], n[1], n[2], zchunk, p);
    else
      heat_step_kernel<double, ExactD, MODE_REFERENCE><<<grid, block, 0, s>>>(vin.base, vout.base, vl.base, vin.sy,
                                                                              vin.sz, n[0], n[1], n[2], zchunk, p);
  } else {
    // bulk-copied slabs: rows of 16-byte aligned windows with an even pitch, 8 rows per block
    const int gx = Tf->glob[0], gy = Tf->glob[1];
    const size_t bk_smem = (size_t)BK_NS * 2 * BK_ROWS * gx * sizeof(float) + BK_NS * sizeof(uint64_t);
    const bool bulk = n[0] <= 2 * BP_PAIRS && n[1] % BK_RY == 0 && gx % 2 == 0 && gy % 2 == 0 &&
                      (uintptr_t)Tf->data % 16 == 0 && (uintptr_t)Lf->data % 16 == 0 && bk_smem <= 113 * 1024;
    if (bulk) {
      // (per device and cheap: the attribute is set on every launch)
      auto kern = heat_step_f32_bulk2_kernel;
      NEBO_CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, 113 * 1024));
      int bps = 0;
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kern, BP_THREADS, bk_smem) != cudaSuccess || bps < 1) {
        cudaGetLastError();
        bps = 1;
      }
      const int yb = n[1] / BK_RY;
      // one wave of resident blocks: as many z chunks as the slots allow
      const int ch = max(1, min(num_sms() * bps / yb, n[2]));
      const int zc = (n[2] + ch - 1) / ch;
      LaunchScope ls("heat_step_f32", s);
      kern<<<dim3(yb, (n[2] + zc - 1) / zc), BP_THREADS, bk_smem, s>>>(
          (const float*)Tf->data, vout.base, (const float*)Lf->data, gx, vin.sz, n[0], n[1], n[2], zc, p.w[0], p.w[1],
          p.w[2]);
      NEBO_LAUNCH_CHECK("nebo_heat_step");
      return NEBO_OK;
    }
    // 8-byte copies when every row of T and lambda starts 8-byte aligned (even pitch, aligned
    // windows); then nx is even too, which keeps the clamped column pairs aligned
    const bool vec = (vin.sy % 2 == 0) && ((uintptr_t)(vin.base - 1) % 8 == 0) && ((uintptr_t)(vl.base - 1) % 8 == 0);
    // one full wave: as many z chunks as the resident blocks allow (each chunk re-reads two
    // halo planes and fills the ring once, so more chunks than slots only cost)
    static std::atomic<int> per_sm[2];  // zero: not queried
    const int bps = vec ? blocks_per_sm(heat_step_f32x2_kernel, QX * QY, per_sm[1])
                        : blocks_per_sm(heat_step_f32_async_kernel<false>, BX * BY, per_sm[0]);
    const int fyb = (n[1] + FTY - 1) / FTY;
    int ch = max(1, min(num_sms() * bps / (gxb * fyb), (n[2] + 7) / 8));
    int zc = (n[2] + ch - 1) / ch;
    zc = (zc + NS - 1) / NS * NS;  // chunks start on a multiple of NS: constant ring stages
    ch = (n[2] + zc - 1) / zc;
    LaunchScope ls("heat_step_f32", s);
    if (vec)
      heat_step_f32x2_kernel<<<dim3(gxb, fyb, ch), dim3(QX, QY), 0, s>>>(vin.base, vout.base, vl.base, vin.sy, vin.sz,
                                                                        n[0], n[1], n[2], zc, p.w[0], p.w[1],
                                                                        p.w[2]);
    else
      heat_step_f32_async_kernel<false><<<dim3(gxb, fyb, ch), dim3(BX, BY), 0, s>>>(vin.base, vout.base, vl.base, vin.sy,
                                                                             vin.sz, n[0], n[1], n[2], zc, p.w[0],
                                                                             p.w[1], p.w[2]);
  }
  NEBO_LAUNCH_CHECK("nebo_heat_step");
  return NEBO_OK;
}

int heat_step_any(const nebo_field* T, const nebo_field* To, const nebo_field* L, double dt, const double sp[3],
                  cudaStream_t s) {
  return T->dtype == NEBO_F64 ? launch_heat<double>(T, To, L, dt, sp, s) : launch_heat<float>(T, To, L, dt, sp, s);
}

// CUDA-graph cache for nebo_heat_run and nebo_heat_run_ex: one instantiated graph per argument set
// (mode -1: nebo_heat_run's steps).
struct GraphKey {
  void *t, *t2, *l;
  int glob[3], dtype, steps, mode;
  double dt, sp[3];
  bool operator<(const GraphKey& o) const {
    return std::tie(t, t2, l, glob[0], glob[1], glob[2], dtype, steps, mode, dt, sp[0], sp[1], sp[2]) <
           std::tie(o.t, o.t2, o.l, o.glob[0], o.glob[1], o.glob[2], o.dtype, o.steps, o.mode, o.dt, o.sp[0],
                    o.sp[1], o.sp[2]);
  }
};
std::mutex g_graph_mu;
std::map<GraphKey, cudaGraphExec_t> g_graphs;

// Launch the graph cached for key on s, capturing body(capture stream) into it the first time.
template <class Body>
int graph_launch(const GraphKey& key, Body body, cudaStream_t s, const char* what) {
  cudaGraphExec_t exec = nullptr;
  {
    std::lock_guard<std::mutex> g(g_graph_mu);
    auto it = g_graphs.find(key);
    if (it != g_graphs.end()) exec = it->second;
  }
  if (!exec) {
    cudaStream_t cap;
    NEBO_CUDA_TRY(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    NEBO_CUDA_TRY(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
    const int rc = body(cap);
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(cap, &graph);
    cudaStreamDestroy(cap);
    if (rc) {
      if (graph) cudaGraphDestroy(graph);
      return rc;
    }
    if (e != cudaSuccess) return cuda_fail(e, what);
    e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) return cuda_fail(e, what);
    std::lock_guard<std::mutex> g(g_graph_mu);
    g_graphs[key] = exec;
  }
  NEBO_CUDA_TRY(cudaGraphLaunch(exec, s));
  return NEBO_OK;
}

// The time loop of NEBO_HEAT_FIXED_POINT (T's ghosts filled, steps >= 1).
int heat_run_fixed_point(const nebo_field* T, const nebo_field* Ttmp, const nebo_field* lam, int steps, double dt,
                         cudaStream_t s, const char* what) {
  int n[3];
  interior_extent(*T, n);
  const size_t cells = (size_t)T->glob[0] * T->glob[1] * T->glob[2];
  int* e = nullptr;  // [0], [1]: T's exponents, ping-pong; [2]: lambda's
  NEBO_CUDA_TRY(cudaMallocAsync((void**)&e, 3 * sizeof(int), s));
  cudaError_t err = cudaMemsetAsync(e, 0, 3 * sizeof(int), s);
  const int rblocks = num_sms() * 4;
  {
    LaunchScope ls("max_exponent", s);
    max_biased_exp_kernel<<<rblocks, 256, 0, s>>>((const double*)T->data, (long)cells, e);
    max_biased_exp_kernel<<<rblocks, 256, 0, s>>>((const double*)lam->data, (long)cells, e + 2);
  }
  if (err == cudaSuccess) err = cudaGetLastError();
  const int gxb = (n[0] + BX - 1) / BX, gyb = (n[1] + BY - 1) / BY;
  static std::atomic<int> per_sm{0};
  const int zchunk = wave_zchunk((long)gxb * gyb, (long)num_sms() * blocks_per_sm(heat_step_fix_kernel, BX * BY, per_sm),
                                 n[2], 2, 4, 1);
  const dim3 grid(gxb, gyb, (n[2] + zchunk - 1) / zchunk), block(BX, BY);
  for (int k = 0; k < steps && err == cudaSuccess; ++k) {
    const nebo_field* a = (k & 1) ? Ttmp : T;
    const nebo_field* b = (k & 1) ? T : Ttmp;
    const View<double> va = make_view<double>(*a), vb = make_view<double>(*b), vl = make_view<double>(*lam);
    err = cudaMemsetAsync(e + ((k + 1) & 1), 0, sizeof(int), s);
    if (err != cudaSuccess) break;
    LaunchScope ls("heat_step_fix", s);
    heat_step_fix_kernel<<<grid, block, 0, s>>>(va.base, vb.base, vl.base, va.sy, va.sz, n[0], n[1], n[2], zchunk,
                                                e + (k & 1), e + 2, e + ((k + 1) & 1), 0.5 * dt);
    err = cudaGetLastError();
  }
  if (err == cudaSuccess && (steps & 1))
    err = cudaMemcpyAsync(T->data, Ttmp->data, cells * sizeof(double), cudaMemcpyDeviceToDevice, s);
  cudaFreeAsync(e, s);
  if (err != cudaSuccess) return cuda_fail(err, what);
  return NEBO_OK;
}

}  // namespace

// Bounded device-side waits that gave up since the last call (cleared by the read).
int bulk_wait_timeouts(unsigned int* count) {
  unsigned int v = 0, zero = 0;
  NEBO_CUDA_TRY(cudaMemcpyFromSymbol(&v, g_bulk_timeouts, sizeof(v)));
  if (v) NEBO_CUDA_TRY(cudaMemcpyToSymbol(g_bulk_timeouts, &zero, sizeof(zero)));
  *count = v;
  return NEBO_OK;
}

// Launch one heat step with no argument checks (callers inside the library have checked).
int heat_step_dispatch(const nebo_field* T, const nebo_field* To, const nebo_field* L, double dt, const double sp[3],
                       cudaStream_t s) {
  return heat_step_any(T, To, L, dt, sp, s);
}

}  // namespace nebo

using namespace nebo;

extern "C" int nebo_heat_step(const nebo_field* T, const nebo_field* Tout, const nebo_field* lam, double dt,
                              const double spacing[3], nebo_stream_t stream) {
  const double unit[3] = {1.0, 1.0, 1.0};
  int rc = check_heat(T, Tout, lam, "nebo_heat_step");
  if (rc) return rc;
  return heat_step_any(T, Tout, lam, dt, spacing ? spacing : unit, (cudaStream_t)stream);
}

extern "C" int nebo_heat_run_ex(const nebo_field* T, const nebo_field* Ttmp, const nebo_field* lam, int steps,
                                double dt, const double spacing[3], int mode, nebo_stream_t stream) {
  const char* what = "nebo_heat_run_ex";
  const bool graph = (mode & NEBO_HEAT_GRAPH) != 0;
  mode &= ~NEBO_HEAT_GRAPH;
  if (mode == NEBO_HEAT_EXACT) return nebo_heat_run(T, Ttmp, lam, steps, dt, spacing, graph ? 1 : 0, stream);
  if (mode != NEBO_HEAT_FIXED_POINT && mode != NEBO_HEAT_FIXED_STATE)
    return fail(NEBO_ERR_INVALID, "Nebo error in %s: mode %d", what, mode);
  int rc = check_heat(T, Ttmp, lam, what);
  if (rc) return rc;
  if (T->dtype != NEBO_F64) return fail(NEBO_ERR_UNSUPPORTED, "Nebo error in %s: fixed point is FP64 only", what);
  if (spacing && (spacing[0] != 1.0 || spacing[1] != 1.0 || spacing[2] != 1.0))
    return fail(NEBO_ERR_UNSUPPORTED, "Nebo error in %s: fixed point takes unit spacing", what);
  if (steps < 0) return fail(NEBO_ERR_INVALID, "Nebo error in %s: negative step count", what);
  cudaStream_t s = (cudaStream_t)stream;
  if ((rc = fill_periodic_any(T, s))) return rc;
  if (steps == 0) return NEBO_OK;
  pool_retain();
  auto body = [&](cudaStream_t st) {
    return mode == NEBO_HEAT_FIXED_STATE ? heat_run_fixed_state(T, Ttmp, lam, steps, dt, st, what)
                                         : heat_run_fixed_point(T, Ttmp, lam, steps, dt, st, what);
  };
  if (!graph) return body(s);
  GraphKey key{T->data, Ttmp->data, lam->data, {T->glob[0], T->glob[1], T->glob[2]}, T->dtype, steps, mode, dt,
               {1.0, 1.0, 1.0}};
  return graph_launch(key, body, s, what);
}

extern "C" int nebo_heat_run(const nebo_field* T, const nebo_field* Ttmp, const nebo_field* lam, int steps, double dt,
                             const double spacing[3], int use_graph, nebo_stream_t stream) {
  const double unit[3] = {1.0, 1.0, 1.0};
  const double* sp = spacing ? spacing : unit;
  int rc = check_heat(T, Ttmp, lam, "nebo_heat_run");
  if (rc) return rc;
  if (steps < 0) return fail(NEBO_ERR_INVALID, "Nebo error in nebo_heat_run: negative step count");
  cudaStream_t s = (cudaStream_t)stream;
  // T's ghosts must hold the periodic images before the first step
  if ((rc = fill_periodic_any(T, s))) return rc;
  if (steps == 0) return NEBO_OK;
  const size_t bytes = (size_t)T->glob[0] * T->glob[1] * T->glob[2] * elem_size(T->dtype);
  if (!use_graph) {
    for (int k = 0; k < steps; ++k) {
      const nebo_field* a = (k & 1) ? Ttmp : T;
      const nebo_field* b = (k & 1) ? T : Ttmp;
      if ((rc = heat_step_any(a, b, lam, dt, sp, s))) return rc;
    }
    if (steps & 1) NEBO_CUDA_TRY(cudaMemcpyAsync(T->data, Ttmp->data, bytes, cudaMemcpyDeviceToDevice, s));
    return NEBO_OK;
  }
  GraphKey key{T->data, Ttmp->data, lam->data, {T->glob[0], T->glob[1], T->glob[2]}, T->dtype, steps, -1, dt,
               {sp[0], sp[1], sp[2]}};
  auto body = [&](cudaStream_t cap) {
    int r = 0;
    for (int k = 0; k < steps && !r; ++k) {
      const nebo_field* a = (k & 1) ? Ttmp : T;
      const nebo_field* b = (k & 1) ? T : Ttmp;
      r = heat_step_any(a, b, lam, dt, sp, cap);
    }
    if (!r && (steps & 1)) {
      cudaError_t e = cudaMemcpyAsync(T->data, Ttmp->data, bytes, cudaMemcpyDeviceToDevice, cap);
      if (e != cudaSuccess) r = cuda_fail(e, "nebo_heat_run capture copy");
    }
    return r;
  };
  return graph_launch(key, body, s, "nebo_heat_run");
}
