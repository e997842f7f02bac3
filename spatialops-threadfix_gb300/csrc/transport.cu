// Variable-coefficient scalar transport on a staggered mesh, Heun's RK2, periodic, two ghost
// layers:  per direction d, on the faces of the SVol cells (XVol/YVol/ZVol locations),
//   F_d = nu * Interp(lambda) * G4_d(phi) - u_d * cond(u_d > 0, phi[i-1])(phi[i])
//   rhs = Grad_{X->S}(F_x) + Grad_{Y->S}(F_y) + Grad_{Z->S}(F_z)
// with G4 the 4th-order staggered gradient {1, -27, 27, -1}/24 at points (-2,-1,0,+1), the
// upwind value chosen by cond on the face velocity, Interp {1/2,1/2} at (-1,0) and the
// divergence {-1, +1} at (0,+1) (user NeboStencilBuilder stencils of the reference's API,
// spatialops/NeboStencilBuilder.h:85-152; the Nebo form is in oracle/ref/ref_driver.cpp).
//
// Precision modes (one template):
//   FP32 storage: phi, u, v, w, lambda are float; the stencil arithmetic is float; the time
//                 state is accumulated in an FP64 field (phi64), and a float copy of the state
//                 is written for the next stencil sweep.  Reductions read phi64.
//   FP64 storage: everything double (the plain path the FP32 form is measured against).
// Each stage is ONE kernel: face fluxes computed once per face (low faces by each thread, high
// faces through shared memory or carried in z), RK combination fused, periodic ghost images of
// the stencil copy written in the same pass.
#include <cuda.h>  // CUtensorMap and its enums (the encoder comes from the runtime's driver entry point)

#include "bulk.cuh"
#include "common.cuh"
#include "fp64_int.cuh"

namespace nebo {

// Bounded mbarrier waits of the tensor-staged FP32 stage kernel that gave up (read and cleared
// by transport_wait_timeouts; nebo_stream_sync reports them).
__device__ unsigned int g_transport_timeouts;

namespace {

constexpr int TX = 32;
constexpr int TY = 8;
constexpr int G = 2;

template <typename T>
struct TrArgs {
  const T* phi;      // stencil source (ghosts valid)
  const double* acc; // FP64 state the stage advances from (phi64 for stage 1, phi1_64 for stage 2)
  const double* base;  // stage 2: phi_n (FP64); unused in stage 1
  double* out64;     // FP64 result (may alias the stencil copy in FP64 mode)
  T* outS;           // stencil copy of the result with periodic images (FP32 mode), or nullptr
  const T* u;
  const T* v;
  const T* w;
  const T* lam;
  int n, sy;
  long sz;
  T nu, q0, q1, q2, q3;  // nu and the G4 coefficients
  double dt;
};

template <typename T>
__device__ __forceinline__ T face_flux(const TrArgs<T>& a, long f, long s, const T* vel) {
  const T* p = a.phi;
  const T il = (__ldg(a.lam + f - s) + __ldg(a.lam + f)) * T(0.5);
  const T g4 = ((__ldg(p + f - 2 * s) * a.q0 + __ldg(p + f - s) * a.q1) + __ldg(p + f) * a.q2) + __ldg(p + f + s) * a.q3;
  const T uf = __ldg(vel + f);
  const T up = (uf > T(0)) ? __ldg(p + f - s) : __ldg(p + f);
  return a.nu * il * g4 - uf * up;
}

// Cells within G of a face: the value and its periodic images (out of line: rare, and its index
// lists live in local memory).
template <typename T>
__device__ __noinline__ void store_images2_edge(T* base, int sy, long sz, int x, int y, int z, int n, T v) {
  int xs[3], ys[3], zs[3];
  int cx = 0, cy = 0, cz = 0;
  xs[cx++] = x;
  if (x < G) xs[cx++] = x + n;
  if (x >= n - G) xs[cx++] = x - n;
  ys[cy++] = y;
  if (y < G) ys[cy++] = y + n;
  if (y >= n - G) ys[cy++] = y - n;
  zs[cz++] = z;
  if (z < G) zs[cz++] = z + n;
  if (z >= n - G) zs[cz++] = z - n;
  for (int k = 0; k < cz; ++k)
    for (int j = 0; j < cy; ++j)
      for (int i = 0; i < cx; ++i) base[(long)xs[i] + (long)sy * ys[j] + sz * zs[k]] = v;
}

// The value at (x, y, z) and, for cells within G of a face, its periodic images.
template <typename T>
__device__ __forceinline__ void store_images2(T* base, int sy, long sz, int x, int y, int z, int n, T v) {
  if (x >= G && x < n - G && y >= G && y < n - G && z >= G && z < n - G)
    base[(long)x + (long)sy * y + sz * z] = v;
  else
    store_images2_edge(base, sy, sz, x, y, z, n, v);
}

// Ask L2 to fetch the line holding p (no register, no wait): planes are requested PFZ steps of
// the z march before the kernel reads them, so DRAM latency overlaps the current plane's work.
__device__ __forceinline__ void prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }
constexpr int PFZ = 6;

template <typename T, bool SECOND>
__global__ void __launch_bounds__(TX* TY) transport_stage_kernel(TrArgs<T> a, int zchunk) {
  __shared__ T sfx[2][TY][TX + 1];
  __shared__ T sfy[2][TY + 1][TX];
  const int tx = threadIdx.x, ty = threadIdx.y;
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
  const int n = a.n;
  const int x = x0 + tx, y = y0 + ty;
  const int z0 = blockIdx.z * zchunk, z1 = min(z0 + zchunk, n);
  const bool active = x < n && y < n;
  const int xc = min(x, n), yc = min(y, n);  // column/row n is a ghost: valid memory
  const int sy = a.sy;
  const long sz = a.sz;
  auto at = [&](int i, int j, int k) { return (long)i + (long)sy * j + sz * k; };
  T fzlo = face_flux(a, at(xc, yc, z0), sz, a.w);
  for (int z = z0; z < z1; ++z) {
    const int buf = z & 1;
    const long c = at(xc, yc, z);
    {
      // the planes this column reads first at step z + PFZ (clamped inside the window)
      const int zp = min(z + PFZ, n + 1);
      const long cp = at(xc, yc, zp);
      prefetch_l2(a.phi + cp);
      prefetch_l2(a.lam + cp);
      prefetch_l2(a.u + cp);
      prefetch_l2(a.v + cp);
      prefetch_l2(a.w + cp);
      if (zp < n) {
        prefetch_l2(a.acc + cp);
        if (SECOND) prefetch_l2(a.base + cp);
      }
    }
    const T fzhi = face_flux(a, c + sz, sz, a.w);
    const T fx = face_flux(a, c, 1, a.u);
    const T fy = face_flux(a, c, sy, a.v);
    sfx[buf][ty][tx] = fx;
    sfy[buf][ty][tx] = fy;
    if (ty == 0) {
      const int yh = y0 + TY;
      if (yh <= n && x <= n) sfy[buf][TY][tx] = face_flux(a, at(xc, yh, z), sy, a.v);
    } else if (ty == 1 && tx < TY) {
      const int xh = x0 + TX, yr = y0 + tx;
      if (xh <= n && yr < n) sfx[buf][tx][TX] = face_flux(a, at(xh, yr, z), 1, a.u);
    }
    __syncthreads();
    if (active) {
      const T rhs = ((sfx[buf][ty][tx + 1] - fx) + (sfy[buf][ty + 1][tx] - fy)) + (fzhi - fzlo);
      // FP32 mode: the float <-> double conversions from the bits (a hardware conversion issues
      // on the FP64 pipe, at the FP64 rate)
      double rd;
      if constexpr (sizeof(T) == 4) rd = fixmath::f32_to_f64(rhs); else rd = rhs;
      double r;
      if (!SECOND)
        r = a.acc[c] + a.dt * rd;
      else
        r = 0.5 * a.base[c] + 0.5 * (a.acc[c] + a.dt * rd);
      T rs;
      if constexpr (sizeof(T) == 4) rs = fixmath::f64_to_f32_rn(r); else rs = r;
      if (a.outS) {
        a.out64[c] = r;
        store_images2(a.outS, sy, sz, x, y, z, n, rs);
      } else {
        store_images2(reinterpret_cast<T*>(a.out64), sy, sz, x, y, z, n, rs);
      }
    }
    fzlo = fzhi;
  }
}

// FP32 stage with staged planes.  phi and lambda planes (the 32 x 8 tile plus a two-cell x/y
// halo, 36 x 12) stream through a ring of SNS shared-memory stages with 8-byte cp.async copies
// (the row pitch is even); each thread computes both x faces and both y faces of its cell from
// the stage, and the z faces from its column's phi window (z-1 .. z+2) carried in registers, so
// the only global reads per cell are the face velocities and the FP64 state.  Face arithmetic as
// face_flux.  Ring: plane p (z0 <= p <= z1+1) lives in stage (p - z0) % SNS; the prologue issues
// planes z0 .. z0+3; iteration z waits until planes up to z+2 have landed (one group pending),
// syncs, issues plane z+4 into the stage of plane z-1 and reads planes z, z+1, z+2.
constexpr int SNS = 5;
constexpr int SPW = TX + 2 * G, SPH = TY + 2 * G;  // staged tile incl. halo
constexpr int SPLANE = SPW * SPH;
constexpr int SUNITS = (SPW / 2) * SPH;            // 8-byte pairs per field and plane
constexpr int SNCOPY = (2 * SUNITS + TX * TY - 1) / (TX * TY);

__device__ __forceinline__ void tcp_async8(uint32_t smem, const void* gmem) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem), "l"(gmem) : "memory");
}
__device__ __forceinline__ void tcp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void tcp_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// face flux from its stencil values: la, lb = lambda[f-s], lambda[f]; pm2, pm1, p0, pp1 =
// phi[f-2s], phi[f-s], phi[f], phi[f+s]; uf = velocity[f] (the order of face_flux)
__device__ __forceinline__ float sflux(const TrArgs<float>& a, float la, float lb, float pm2, float pm1, float p0,
                                       float pp1, float uf) {
  const float il = (la + lb) * 0.5f;
  const float g4 = ((pm2 * a.q0 + pm1 * a.q1) + p0 * a.q2) + pp1 * a.q3;
  const float up = (uf > 0.0f) ? pm1 : p0;
  return a.nu * il * g4 - uf * up;
}

template <bool SECOND>
__global__ void __launch_bounds__(TX* TY) transport_stage_f32_staged_kernel(TrArgs<float> a, int zchunk) {
  __shared__ __align__(16) float sP[SNS * SPLANE];
  __shared__ __align__(16) float sL[SNS * SPLANE];
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * TX + tx;
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
  const int n = a.n, sy = a.sy;
  const long sz = a.sz;
  const int x = x0 + tx, y = y0 + ty;
  const int z0 = blockIdx.z * zchunk, z1 = min(z0 + zchunk, n);
  const bool active = x < n && y < n;
  const int xc = min(x, n), yc = min(y, n);  // column/row n is a ghost: valid memory
  // copy slots: unit u < 2 SUNITS (phi, then lambda) -> tile row r, column pair c (clamped to
  // the window: pairs start at most at column n, rows at most n + 1)
  int goff[SNCOPY];
  uint32_t soff[SNCOPY];
  bool lamf[SNCOPY];
  const uint32_t sP0 = (uint32_t)__cvta_generic_to_shared(sP), sL0 = (uint32_t)__cvta_generic_to_shared(sL);
#pragma unroll
  for (int j = 0; j < SNCOPY; ++j) {
    const int u = min(tid + j * TX * TY, 2 * SUNITS - 1);
    lamf[j] = u >= SUNITS;
    const int k = lamf[j] ? u - SUNITS : u;
    const int r = k / (SPW / 2), c = 2 * (k - r * (SPW / 2));
    goff[j] = min(x0 - G + c, n) + sy * min(y0 - G + r, n + 1);
    soff[j] = (lamf[j] ? sL0 : sP0) + (uint32_t)((r * SPW + c) * sizeof(float));
  }
  const bool last_slot = tid + (SNCOPY - 1) * TX * TY < 2 * SUNITS;
  auto issue = [&](int p, int st) {
    if (p <= z1 + 1) {
      const float* pp = a.phi + sz * p;
      const float* lp = a.lam + sz * p;
      const uint32_t so = (uint32_t)st * (SPLANE * sizeof(float));
#pragma unroll
      for (int j = 0; j < SNCOPY; ++j) {
        if (j == SNCOPY - 1 && !last_slot) break;
        tcp_async8(soff[j] + so, (lamf[j] ? lp : pp) + goff[j]);
      }
    }
  };
#pragma unroll
  for (int i = 0; i < SNS - 1; ++i) {
    issue(z0 + i, i);
    tcp_commit();
  }
  auto at = [&](int i, int j, int k) { return (long)i + (long)sy * j + sz * k; };
  // the column's phi window and the low z face of plane z0, from global memory
  const long c0 = at(xc, yc, z0);
  float pm1 = __ldg(a.phi + c0 - sz), p0 = __ldg(a.phi + c0), p1 = __ldg(a.phi + c0 + sz);
  float fzlo = face_flux(a, c0, sz, a.w);
  const int ci = (ty + G) * SPW + tx + G;
  // this column's global values of plane z (velocities on its faces, the FP64 state), loaded one
  // plane ahead so their latency overlaps the previous plane's work
  struct Col {
    float ul, uh, vl, vh, wh;
    double acc, base;
  };
  auto load_col = [&](int z) {
    Col q;
    const long c = at(xc, yc, z);
    q.ul = __ldg(a.u + c);
    q.uh = __ldg(a.u + c + 1);
    q.vl = __ldg(a.v + c);
    q.vh = __ldg(a.v + c + sy);
    q.wh = __ldg(a.w + c + sz);
    q.acc = a.acc[c];
    q.base = SECOND ? a.base[c] : 0.0;
    return q;
  };
  Col cur = load_col(z0);
  for (int z = z0; z < z1; ++z) {
    const int i = z - z0;
    const Col nxt = load_col(min(z + 1, n));  // plane n is a ghost plane: valid memory
    tcp_wait<1>();
    __syncthreads();
    issue(z + SNS - 1, (i + SNS - 1) % SNS);
    tcp_commit();
    const float* P0 = sP + (i % SNS) * SPLANE;
    const float* L0 = sL + (i % SNS) * SPLANE;
    const float* L1 = sL + ((i + 1) % SNS) * SPLANE;
    const float* P2 = sP + ((i + 2) % SNS) * SPLANE;
    const long c = at(xc, yc, z);
    const float p2 = P2[ci], l0 = L0[ci], l1 = L1[ci];
    const float xm2 = P0[ci - 2], xm1 = P0[ci - 1], xp1 = P0[ci + 1], xp2 = P0[ci + 2];
    const float ym2 = P0[ci - 2 * SPW], ym1 = P0[ci - SPW], yp1 = P0[ci + SPW], yp2 = P0[ci + 2 * SPW];
    const float fxl = sflux(a, L0[ci - 1], l0, xm2, xm1, p0, xp1, cur.ul);
    const float fxh = sflux(a, l0, L0[ci + 1], xm1, p0, xp1, xp2, cur.uh);
    const float fyl = sflux(a, L0[ci - SPW], l0, ym2, ym1, p0, yp1, cur.vl);
    const float fyh = sflux(a, l0, L0[ci + SPW], ym1, p0, yp1, yp2, cur.vh);
    const float fzh = sflux(a, l0, l1, pm1, p0, p1, p2, cur.wh);
    if (active) {
      const float rhs = ((fxh - fxl) + (fyh - fyl)) + (fzh - fzlo);
      const double rd = fixmath::f32_to_f64(rhs);
      double r;
      if (!SECOND)
        r = cur.acc + a.dt * rd;
      else
        r = 0.5 * cur.base + 0.5 * (cur.acc + a.dt * rd);
      a.out64[c] = r;
      store_images2(a.outS, sy, sz, x, y, z, n, fixmath::f64_to_f32_rn(r));
    }
    fzlo = fzh;
    pm1 = p0;
    p0 = p1;
    p1 = p2;
    cur = nxt;
  }
  tcp_wait<0>();
}

// FP32 stage, two x-adjacent cells (x, x+1; x even) per thread: the 32 x 8 tile of the staged
// kernel with 16 x 8 threads, the same plane ring and copy layout, and every face flux, difference
// and stencil value as a packed FP32x2 pair (__ffma2_rn / __fadd2_rn / __fmul2_rn), so one packed
// instruction serves both cells.  Pairs in the stage and in the fields start at even columns
// (8-byte loads): with Pm = (x-2, x-1), P = (x, x+1), Pp = (x+2, x+3) the low x faces of the two
// cells (x-1/2, x+1/2) and their high x faces (x+1/2, x+3/2) each take one packed flux (the
// shared face x+1/2 is evaluated twice, identically); y and z faces take one packed flux each.
// The RK combination, the FP64 state and the stencil copy with its images stay per cell.
// Needs n even (even pitch) and 8-byte aligned field bases.
//
// Two ways to stage the phi and lambda planes (template TMA):
//   false: 8-byte cp.async copies by every thread, one commit group per plane;
//   true:  one thread issues two 3-D tensor-tile loads per plane (cp.async.bulk.tensor, box
//          36 x 12 x 1 floats at glob (x0, y0, z + G): the tile and its two-cell halo) into
//          128-byte-aligned stages; each stage's mbarrier counts the 3456 bytes, and every
//          thread waits on the phase of the newest plane it reads.  The tensor maps cover the
//          whole windows, so the row pitch (n + 4) * 4 bytes must be a multiple of 16 (n a
//          multiple of 4) and the window bases 16-byte aligned.  A tile reaching past the window
//          (n not a multiple of 32 or 8) reads zeros there, which only idle lanes use.  Waits
//          are bounded; one that gives up is counted in g_transport_timeouts.
constexpr int PTX = TX / 2;   // threads per tile row
constexpr int TSTRIDE = 448;  // floats per TMA stage: 36 x 12 = 432, padded to 128 bytes
static_assert(SPW == 36 && SPH == 12 && TSTRIDE * 4 % 128 == 0 && TSTRIDE >= SPLANE, "TMA stage layout");
constexpr uint32_t TMA_STAGE_BYTES = 2u * SPLANE * sizeof(float);  // phi and lambda boxes

// The tensor maps of one stage launch: phi's stencil copy and lambda, each over its whole window.
struct TrMaps {
  CUtensorMap phi, lam;
};

__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap* map, int x, int y, int z, uint32_t bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(bar)
      : "memory");
}

__device__ __forceinline__ float2 tsub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.0f, -1.0f), a); }
__device__ __forceinline__ float2 tld2(const float* p) { return __ldg(reinterpret_cast<const float2*>(p)); }
__device__ __forceinline__ float2 tsh2(const float* p) { return *reinterpret_cast<const float2*>(p); }

// sflux for two faces at once (same operand order).
__device__ __forceinline__ float2 sflux2(float2 nu, float2 q0, float2 q1, float2 q2, float2 q3, float2 la, float2 lb,
                                         float2 pm2, float2 pm1, float2 p0, float2 pp1, float2 uf) {
  const float2 il = __fmul2_rn(__fadd2_rn(la, lb), make_float2(0.5f, 0.5f));
  float2 g4 = __fmul2_rn(pm2, q0);
  g4 = __ffma2_rn(pm1, q1, g4);
  g4 = __ffma2_rn(p0, q2, g4);
  g4 = __ffma2_rn(pp1, q3, g4);
  const float2 up = make_float2(uf.x > 0.0f ? pm1.x : p0.x, uf.y > 0.0f ? pm1.y : p0.y);
  return __ffma2_rn(make_float2(-uf.x, -uf.y), up, __fmul2_rn(__fmul2_rn(nu, il), g4));
}

// The pair (x, x+1) at (y, z) of the stencil copy, with periodic images for cells within G of a face.
__device__ __forceinline__ void store_images2_pair(float* base, int sy, long sz, int x, int y, int z, int n, float v0,
                                                   float v1) {
  if (x >= G && x + 1 < n - G && y >= G && y < n - G && z >= G && z < n - G) {
    *reinterpret_cast<float2*>(base + (long)x + (long)sy * y + sz * z) = make_float2(v0, v1);
  } else {
    store_images2_edge(base, sy, sz, x, y, z, n, v0);
    store_images2_edge(base, sy, sz, x + 1, y, z, n, v1);
  }
}

template <bool SECOND, bool TMA>
__global__ void __launch_bounds__(PTX* TY) transport_stage_f32_pair_kernel(TrArgs<float> a, int zchunk,
                                                                           const __grid_constant__ TrMaps maps) {
  constexpr int NT = PTX * TY;
  constexpr int NCP = (2 * SUNITS + NT - 1) / NT;
  constexpr int STRIDE = TMA ? TSTRIDE : SPLANE;  // floats per stage
  __shared__ __align__(128) float sP[SNS * STRIDE];
  __shared__ __align__(128) float sL[SNS * STRIDE];
  __shared__ __align__(8) uint64_t sbar[TMA ? SNS : 1];
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * PTX + tx;
  const int x0 = blockIdx.x * TX, y0 = blockIdx.y * TY;
  const int n = a.n, sy = a.sy;
  const long sz = a.sz;
  const int x = x0 + 2 * tx, y = y0 + ty;
  const int z0 = blockIdx.z * zchunk, z1 = min(z0 + zchunk, n);
  const bool active = x < n && y < n;            // n even: x + 1 < n as well
  const int xc = min(x, n - 2), yc = min(y, n);  // idle lanes read valid cells (x + 3 <= n + 1)
  int goff[NCP];
  uint32_t soff[NCP];
  bool lamf[NCP];
  const uint32_t sP0 = (uint32_t)__cvta_generic_to_shared(sP), sL0 = (uint32_t)__cvta_generic_to_shared(sL);
#pragma unroll
  for (int j = 0; j < NCP; ++j) {
    const int u = min(tid + j * NT, 2 * SUNITS - 1);
    lamf[j] = u >= SUNITS;
    const int k = lamf[j] ? u - SUNITS : u;
    const int r = k / (SPW / 2), c = 2 * (k - r * (SPW / 2));
    goff[j] = min(x0 - G + c, n) + sy * min(y0 - G + r, n + 1);
    soff[j] = (lamf[j] ? sL0 : sP0) + (uint32_t)((r * SPW + c) * sizeof(float));
  }
  const bool last_slot = tid + (NCP - 1) * NT < 2 * SUNITS;
  const uint32_t bar0 = (uint32_t)__cvta_generic_to_shared(sbar);
  // plane p (z0 <= p <= z1 + 1) into stage st; with TMA thread 0 alone calls this
  auto issue = [&](int p, int st) {
    if (p <= z1 + 1) {
      const uint32_t so = (uint32_t)st * (STRIDE * sizeof(float));
      if constexpr (TMA) {
        const uint32_t bar = bar0 + 8u * (uint32_t)st;
        mbar_expect_tx(bar, TMA_STAGE_BYTES);
        tma_load_3d(sP0 + so, &maps.phi, x0, y0, p + G, bar);
        tma_load_3d(sL0 + so, &maps.lam, x0, y0, p + G, bar);
      } else {
        const float* pp = a.phi + sz * p;
        const float* lp = a.lam + sz * p;
#pragma unroll
        for (int j = 0; j < NCP; ++j) {
          if (j == NCP - 1 && !last_slot) break;
          tcp_async8(soff[j] + so, (lamf[j] ? lp : pp) + goff[j]);
        }
      }
    }
  };
  bool ok = true;
  if constexpr (TMA) {
    if (tid == 0) {
      for (int st = 0; st < SNS; ++st) mbar_init(bar0 + 8u * st, 1);
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (tid == 0)
      for (int i = 0; i < SNS - 1; ++i) issue(z0 + i, i);
  } else {
#pragma unroll
    for (int i = 0; i < SNS - 1; ++i) {
      issue(z0 + i, i);
      tcp_commit();
    }
  }
  auto at = [&](int i, int j, int k) { return (long)i + (long)sy * j + sz * k; };
  const long c0 = at(xc, yc, z0);
  float2 pm1 = tld2(a.phi + c0 - sz), p0 = tld2(a.phi + c0), p1 = tld2(a.phi + c0 + sz);
  float2 fzlo = make_float2(face_flux(a, c0, sz, a.w), face_flux(a, c0 + 1, sz, a.w));
  const int ci = (ty + G) * SPW + 2 * tx + G;  // even: 8-byte aligned pairs
  struct Col {
    float2 ul, vl, vh, wh;
    float u2;
    double acc0, acc1, base0, base1;
  };
  auto load_col = [&](int z) {
    Col q;
    const long c = at(xc, yc, z);
    q.ul = tld2(a.u + c);  // faces x-1/2, x+1/2
    q.u2 = __ldg(a.u + c + 2);  // face x+3/2
    q.vl = tld2(a.v + c);
    q.vh = tld2(a.v + c + sy);
    q.wh = tld2(a.w + c + sz);
    q.acc0 = a.acc[c];
    q.acc1 = a.acc[c + 1];
    q.base0 = SECOND ? a.base[c] : 0.0;
    q.base1 = SECOND ? a.base[c + 1] : 0.0;
    return q;
  };
  const float2 NU = make_float2(a.nu, a.nu), Q0 = make_float2(a.q0, a.q0), Q1 = make_float2(a.q1, a.q1),
               Q2 = make_float2(a.q2, a.q2), Q3 = make_float2(a.q3, a.q3);
  Col cur = load_col(z0);
  for (int z = z0; z < z1; ++z) {
    const int i = z - z0;
    const Col nxt = load_col(min(z + 1, n));  // plane n is a ghost plane: valid memory
    if constexpr (TMA) {
      // planes z and z+1 were waited for as the newest planes of the two previous iterations
      if (i == 0) ok &= mbar_wait(bar0, 0) & mbar_wait(bar0 + 8u, 0);
      const int q = i + 2;  // plane z+2: stage q % SNS, its (q / SNS)-th use
      ok &= mbar_wait(bar0 + 8u * (uint32_t)(q % SNS), (uint32_t)(q / SNS) & 1u);
      __syncthreads();  // the stage of plane z-1 is no longer read
      if (tid == 0) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        issue(z + SNS - 1, (i + SNS - 1) % SNS);
      }
    } else {
      tcp_wait<1>();
      __syncthreads();
      issue(z + SNS - 1, (i + SNS - 1) % SNS);
      tcp_commit();
    }
    const float* P0 = sP + (i % SNS) * STRIDE + ci;
    const float* L0 = sL + (i % SNS) * STRIDE + ci;
    const float* L1 = sL + ((i + 1) % SNS) * STRIDE + ci;
    const float* P2 = sP + ((i + 2) % SNS) * STRIDE + ci;
    const float2 p2 = tsh2(P2), l0 = tsh2(L0), l1 = tsh2(L1);
    const float2 pxm = tsh2(P0 - 2), pxp = tsh2(P0 + 2), lxm = tsh2(L0 - 2), lxp = tsh2(L0 + 2);
    const float2 pym2 = tsh2(P0 - 2 * SPW), pym1 = tsh2(P0 - SPW), pyp1 = tsh2(P0 + SPW), pyp2 = tsh2(P0 + 2 * SPW);
    const float2 lym = tsh2(L0 - SPW), lyp = tsh2(L0 + SPW);
    const float2 pmid = make_float2(pxm.y, p0.x), pmid2 = make_float2(p0.y, pxp.x);  // (x-1, x), (x+1, x+2)
    const float2 fxl = sflux2(NU, Q0, Q1, Q2, Q3, make_float2(lxm.y, l0.x), l0, pxm, pmid, p0, pmid2, cur.ul);
    const float2 fxh = sflux2(NU, Q0, Q1, Q2, Q3, l0, make_float2(l0.y, lxp.x), pmid, p0, pmid2, pxp,
                              make_float2(cur.ul.y, cur.u2));
    const float2 fyl = sflux2(NU, Q0, Q1, Q2, Q3, lym, l0, pym2, pym1, p0, pyp1, cur.vl);
    const float2 fyh = sflux2(NU, Q0, Q1, Q2, Q3, l0, lyp, pym1, p0, pyp1, pyp2, cur.vh);
    const float2 fzh = sflux2(NU, Q0, Q1, Q2, Q3, l0, l1, pm1, p0, p1, p2, cur.wh);
    if (active) {
      const float2 rhs = __fadd2_rn(__fadd2_rn(tsub(fxh, fxl), tsub(fyh, fyl)), tsub(fzh, fzlo));
      const double rd0 = fixmath::f32_to_f64(rhs.x), rd1 = fixmath::f32_to_f64(rhs.y);
      double r0, r1;
      if (!SECOND) {
        r0 = cur.acc0 + a.dt * rd0;
        r1 = cur.acc1 + a.dt * rd1;
      } else {
        r0 = 0.5 * cur.base0 + 0.5 * (cur.acc0 + a.dt * rd0);
        r1 = 0.5 * cur.base1 + 0.5 * (cur.acc1 + a.dt * rd1);
      }
      const long c = at(x, y, z);
      a.out64[c] = r0;
      a.out64[c + 1] = r1;
      store_images2_pair(a.outS, sy, sz, x, y, z, n, fixmath::f64_to_f32_rn(r0), fixmath::f64_to_f32_rn(r1));
    }
    fzlo = fzh;
    pm1 = p0;
    p0 = p1;
    p1 = p2;
    cur = nxt;
  }
  if constexpr (TMA) {
    if (!ok) atomicAdd(&g_transport_timeouts, 1u);
  } else {
    tcp_wait<0>();
  }
}

__global__ void cast_f64_f32_kernel(const double* __restrict__ a, float* __restrict__ b, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    b[i] = fixmath::f64_to_f32_rn(a[i]);
}

int cast_f64_to_f32(const double* a, float* b, size_t n, cudaStream_t s) {
  LaunchScope ls("cast_f64_f32", s);
  cast_f64_f32_kernel<<<num_sms() * 8, 256, 0, s>>>(a, b, n);
  NEBO_LAUNCH_CHECK("nebo_transport_run (cast)");
  return NEBO_OK;
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (no link against libcuda).
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_tiled() {
  static std::atomic<EncodeTiledFn> fn{nullptr};
  EncodeTiledFn f = fn.load(std::memory_order_acquire);
  if (!f) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess)
      return nullptr;
    f = reinterpret_cast<EncodeTiledFn>(p);
    fn.store(f, std::memory_order_release);
  }
  return f;
}

// The tensor map of a float window of gl^3 cells at `base` (16-byte aligned, gl a multiple of 4),
// box 36 x 12 x 1 (the pair kernel's staged tile).  False when the encoder refuses it.
bool window_map(CUtensorMap* m, const float* base, int gl) {
  EncodeTiledFn f = encode_tiled();
  if (!f || ((uintptr_t)base & 15u) || gl % 4) return false;
  const cuuint64_t dims[3] = {(cuuint64_t)gl, (cuuint64_t)gl, (cuuint64_t)gl};
  const cuuint64_t strides[2] = {(cuuint64_t)gl * 4, (cuuint64_t)gl * gl * 4};
  const cuuint32_t box[3] = {(cuuint32_t)SPW, (cuuint32_t)SPH, 1};
  const cuuint32_t estr[3] = {1, 1, 1};
  return f(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base), dims, strides, box, estr,
           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// maps: the tensor maps of a.phi's and a.lam's windows, or nullptr (no tensor staging)
template <typename T>
int transport_launch(TrArgs<T> a, bool second, cudaStream_t s, const TrMaps* maps = nullptr) {
  const int n = a.n;
  const int gxb = (n + TX - 1) / TX, gyb = (n + TY - 1) / TY;
  // FP32 kernels: 3 = cell pairs with tensor-tile staging (kind 2 and tensor maps), 2 = cell
  // pairs (even pitch, every float field 8-byte aligned), 1 = staged planes (even pitch, phi and
  // lambda 8-byte aligned), 0 = the generic kernel
  auto al8 = [](const void* p) { return ((uintptr_t)p & 7u) == 0; };
  int kind = 0;
  if (sizeof(T) == 4 && a.sy % 2 == 0 && al8(a.phi) && al8(a.lam)) {
    kind = 1;
    if (al8(a.u) && al8(a.v) && al8(a.w) && al8(a.outS)) kind = maps ? 3 : 2;
  }
  // z chunks in whole waves of resident blocks (a chunk reads 2G halo planes beyond its own)
  static std::atomic<int> per_sm[4][2];  // zero: not queried
  std::atomic<int>& cache = per_sm[kind][second];
  int ps;
  if (kind == 3)
    ps = second ? blocks_per_sm(transport_stage_f32_pair_kernel<true, true>, PTX * TY, cache)
                : blocks_per_sm(transport_stage_f32_pair_kernel<false, true>, PTX * TY, cache);
  else if (kind == 2)
    ps = second ? blocks_per_sm(transport_stage_f32_pair_kernel<true, false>, PTX * TY, cache)
                : blocks_per_sm(transport_stage_f32_pair_kernel<false, false>, PTX * TY, cache);
  else if (kind == 1)
    ps = second ? blocks_per_sm(transport_stage_f32_staged_kernel<true>, TX * TY, cache)
                : blocks_per_sm(transport_stage_f32_staged_kernel<false>, TX * TY, cache);
  else
    ps = second ? blocks_per_sm(transport_stage_kernel<T, true>, TX * TY, cache)
                : blocks_per_sm(transport_stage_kernel<T, false>, TX * TY, cache);
  const int zchunk = wave_zchunk((long)gxb * gyb, (long)num_sms() * ps, n, 2 * G, 8, 1);
  dim3 grid(gxb, gyb, (n + zchunk - 1) / zchunk), block(TX, TY);
  LaunchScope ls(sizeof(T) == 4 ? "transport_stage_f32" : "transport_stage_f64", s);
  if constexpr (sizeof(T) == 4) {
    if (kind == 3) {
      if (second)
        transport_stage_f32_pair_kernel<true, true><<<grid, dim3(PTX, TY), 0, s>>>(a, zchunk, *maps);
      else
        transport_stage_f32_pair_kernel<false, true><<<grid, dim3(PTX, TY), 0, s>>>(a, zchunk, *maps);
      NEBO_LAUNCH_CHECK("nebo_transport_run");
      return NEBO_OK;
    }
    if (kind == 2) {
      const TrMaps none{};
      if (second)
        transport_stage_f32_pair_kernel<true, false><<<grid, dim3(PTX, TY), 0, s>>>(a, zchunk, none);
      else
        transport_stage_f32_pair_kernel<false, false><<<grid, dim3(PTX, TY), 0, s>>>(a, zchunk, none);
      NEBO_LAUNCH_CHECK("nebo_transport_run");
      return NEBO_OK;
    }
    if (kind == 1) {
      if (second)
        transport_stage_f32_staged_kernel<true><<<grid, block, 0, s>>>(a, zchunk);
      else
        transport_stage_f32_staged_kernel<false><<<grid, block, 0, s>>>(a, zchunk);
      NEBO_LAUNCH_CHECK("nebo_transport_run");
      return NEBO_OK;
    }
  }
  if (second)
    transport_stage_kernel<T, true><<<grid, block, 0, s>>>(a, zchunk);
  else
    transport_stage_kernel<T, false><<<grid, block, 0, s>>>(a, zchunk);
  NEBO_LAUNCH_CHECK("nebo_transport_run");
  return NEBO_OK;
}

}  // namespace

int transport_wait_timeouts(unsigned int* count) {
  unsigned int v = 0, zero = 0;
  NEBO_CUDA_TRY(cudaMemcpyFromSymbol(&v, g_transport_timeouts, sizeof(v)));
  if (v) NEBO_CUDA_TRY(cudaMemcpyToSymbol(g_transport_timeouts, &zero, sizeof(zero)));
  *count = v;
  return NEBO_OK;
}

}  // namespace nebo

using namespace nebo;

// phi: state (FP64 window, 2 ghosts) in/out.  u, v, w, lam: windows of the storage dtype.
// work: caller-provided device scratch of nebo_transport_work_bytes(n, dtype) bytes.
extern "C" size_t nebo_transport_work_bytes(int n, int dtype) {
  const size_t cells = (size_t)(n + 2 * G) * (n + 2 * G) * (n + 2 * G);
  return cells * (2 * sizeof(double) + (dtype == NEBO_F32 ? 2 * sizeof(float) : 0)) + 1024;
}

extern "C" int nebo_transport_run(double* phi, const void* u, const void* v, const void* w, const void* lam, int n,
                                  int steps, double dt, double nu, int dtype, void* work, nebo_stream_t stream) {
  if (!phi || !u || !v || !w || !lam || !work || n < 2 * G || steps < 0)
    return fail(NEBO_ERR_INVALID, "Nebo error in nebo_transport_run: bad arguments");
  if (dtype != NEBO_F64 && dtype != NEBO_F32) return fail(NEBO_ERR_INVALID, "Nebo error in nebo_transport_run: dtype");
  cudaStream_t s = (cudaStream_t)stream;
  const int gl = n + 2 * G;
  const size_t cells = (size_t)gl * gl * gl;
  const long sy = gl, sz = (long)gl * gl;
  const long interior = G + sy * G + sz * G;
  char* wp = static_cast<char*>(work);
  wp = (char*)(((uintptr_t)wp + 255) & ~(uintptr_t)255);
  double* phi1 = reinterpret_cast<double*>(wp);  // stage-1 state (FP64)
  double* phin = phi1 + cells;                   // stage-2 state (FP64)
  nebo_field f;
  for (int i = 0; i < 3; ++i) {
    f.glob[i] = f.extent[i] = gl;
    f.offset[i] = 0;
    f.ghost_minus[i] = f.ghost_plus[i] = G;
    f.has_bc[i] = f.bc_extra[i] = 0;
  }
  int rc;
  if (dtype == NEBO_F64) {
    f.dtype = NEBO_F64;
    f.data = phi;
    if ((rc = fill_periodic_any(&f, s))) return rc;
    for (const void* q : {u, v, w, lam}) {
      f.data = const_cast<void*>(q);
      if ((rc = fill_periodic_any(&f, s))) return rc;
    }
    TrArgs<double> a{};
    a.u = (const double*)u + interior;
    a.v = (const double*)v + interior;
    a.w = (const double*)w + interior;
    a.lam = (const double*)lam + interior;
    a.n = n;
    a.sy = (int)sy;
    a.sz = sz;
    a.nu = nu;
    const double h = 1.0 / 24.0;
    a.q0 = h;
    a.q1 = -27.0 * h;
    a.q2 = 27.0 * h;
    a.q3 = -h;
    a.dt = dt;
    double* cur = phi;
    for (int k = 0; k < steps; ++k) {
      // stage 1: phi1 = cur + dt R(cur)
      a.phi = cur + interior;
      a.acc = cur + interior;
      a.out64 = phi1 + interior;
      a.outS = nullptr;
      if ((rc = transport_launch(a, false, s))) return rc;
      // stage 2: phin = cur/2 + (phi1 + dt R(phi1))/2
      a.phi = phi1 + interior;
      a.acc = phi1 + interior;
      a.base = cur + interior;
      a.out64 = (cur == phi ? phin : phi) + interior;
      if ((rc = transport_launch(a, true, s))) return rc;
      cur = (cur == phi) ? phin : phi;
    }
    if (cur != phi) NEBO_CUDA_TRY(cudaMemcpyAsync(phi, cur, cells * sizeof(double), cudaMemcpyDeviceToDevice, s));
    return NEBO_OK;
  }
  // FP32 storage: float stencil copies + FP64 accumulators
  float* s0 = reinterpret_cast<float*>(phin + cells);
  float* s1 = s0 + cells;
  f.dtype = NEBO_F32;
  for (const void* q : {u, v, w, lam}) {
    f.data = const_cast<void*>(q);
    if ((rc = fill_periodic_any(&f, s))) return rc;
  }
  f.dtype = NEBO_F64;
  f.data = phi;
  if ((rc = fill_periodic_any(&f, s))) return rc;
  if ((rc = cast_f64_to_f32(phi, s0, cells, s))) return rc;
  TrArgs<float> a{};
  a.u = (const float*)u + interior;
  a.v = (const float*)v + interior;
  a.w = (const float*)w + interior;
  a.lam = (const float*)lam + interior;
  a.n = n;
  a.sy = (int)sy;
  a.sz = sz;
  a.nu = (float)nu;
  const float h = 1.0f / 24.0f;
  a.q0 = h;
  a.q1 = -27.0f * h;
  a.q2 = 27.0f * h;
  a.q3 = -h;
  a.dt = dt;
  // tensor-tile staging of the stencil copies and lambda where the windows allow it (n a multiple
  // of 4, 16-byte aligned bases; the encoder available)
  TrMaps m0, m1;  // stage 1 reads s0, stage 2 reads s1
  const bool tma = n % 4 == 0 && window_map(&m0.phi, s0, gl) && window_map(&m1.phi, s1, gl) &&
                   window_map(&m0.lam, (const float*)lam, gl);
  m1.lam = m0.lam;
  double* cur = phi;
  for (int k = 0; k < steps; ++k) {
    a.phi = s0 + interior;
    a.acc = cur + interior;
    a.out64 = phi1 + interior;
    a.outS = s1;
    a.outS += interior;
    if ((rc = transport_launch(a, false, s, tma ? &m0 : nullptr))) return rc;
    a.phi = s1 + interior;
    a.acc = phi1 + interior;
    a.base = cur + interior;
    double* nxt = (cur == phi) ? phin : phi;
    a.out64 = nxt + interior;
    a.outS = s0 + interior;
    if ((rc = transport_launch(a, true, s, tma ? &m1 : nullptr))) return rc;
    cur = nxt;
  }
  if (cur != phi) NEBO_CUDA_TRY(cudaMemcpyAsync(phi, cur, cells * sizeof(double), cudaMemcpyDeviceToDevice, s));
  // the FP64 state's ghosts: periodic images of the result
  f.dtype = NEBO_F64;
  f.data = phi;
  return fill_periodic_any(&f, s);
}
