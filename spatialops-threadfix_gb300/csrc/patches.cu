// Batched patches: many independent periodic heat-equation patches of uneven sizes advanced by
// ONE persistent launch per step over a device patch table, with the steps captured in a CUDA
// graph and the tile shape of each patch picked by a small autotuner.
//
// The reference advances patches one `<<=` at a time from the caller's patch loop (Uintah/
// Wasatch-style; spatialops/NeboLhs.h:29-41 launches a 16x16 grid per expression), paying a
// launch and a tail per patch and expression.  Here:
//   * all patches live in one arena per buffer, each a ghosted window, x fastest: FP64 states,
//     or FP32 states (half the bytes), or two-float states (FP32 arithmetic, ~48-bit state);
//   * a work list enumerates (patch, x-tile, y-tile, z-chunk) items; a fixed grid of blocks
//     (a multiple of the SM count) strides through it, so small and large patches share SMs;
//   * tiles are TX x TY = 256 cells per plane with TX in {16, 32, 64} per patch (the autotuner
//     times each candidate on the patches of each x-extent class and keeps the fastest);
//   * each item is the fused heat step of nebo_heat_step: face fluxes computed once, high
//     faces shared through shared memory, z-face carried in a register, and the new values
//     written to the interior and to their periodic ghost images in the same pass.
// Lambda is a scalar per patch, so each face costs (2 lambda) * (Tb - Ta): exactly twice the flux
// the reference computes for a constant lambda field, (lam*1/2 + lam*1/2) * (Ta*(-1) + Tb*1),
// and with the update scaled by dt/2 the FP64 results are bit-identical to the reference's
// serial walk with such a field.
#include <algorithm>
#include <map>
#include <vector>

#include "common.cuh"
#include "bulk.cuh"

struct nebo_patchset;  // opaque handle of the C ABI

namespace nebo {
namespace {

constexpr int PT_THREADS = 256;
constexpr int PF = 4;  // z planes prefetched ahead per thread
constexpr int PT_MAX_TY = 16;   // TX = 16
constexpr int PT_MAX_TX = 64;   // TY = 4

struct PatchDev {
  long long offset;  // element offset of the patch window in the arena
  long long off32;   // FP32 slab layout: element offset of the patch's interior (0,0,0)
  int nx, ny, nz;
  int log2tx;        // tile x extent = 1 << log2tx
  int pitch32;       // FP32 slab layout: row pitch in floats (nx rounded up to a multiple of 4)
  double lam2;       // 2*lambda
  double hdt;        // dt/2
};

struct WorkItem {
  int patch;
  int x0, y0;
  int z0, z1;
};

// Storage and arithmetic of the three precision modes.
//   PMODE_F64   value = double, fluxes double, round-to-nearest FP64 ops (bit-exact form)
//   PMODE_F32   value = float: FP32 storage and arithmetic (half the bytes of FP64); served by
//               patches_f32_strip_kernel below
//   PMODE_F32X2 value = float2 (hi, lo): the state as an unevaluated sum of two floats (~48-bit
//               significand); differences (hb-ha)+(lb-la), fluxes and the update in float, the
//               update added with an error-free two-sum.  No FP64 operation on the sweep.
enum { PMODE_F64 = 0, PMODE_F32 = 1, PMODE_F32X2 = 2 };

template <int M> struct PM;
template <> struct PM<PMODE_F64> {
  typedef double S;
  typedef double F;
  static __device__ __forceinline__ F diff(S a, S b) { return __dsub_rn(b, a); }
  static __device__ __forceinline__ F add(F a, F b) { return __dadd_rn(a, b); }
  static __device__ __forceinline__ F sub(F a, F b) { return __dsub_rn(a, b); }
  static __device__ __forceinline__ F mul(F a, F b) { return __dmul_rn(a, b); }
};
template <> struct PM<PMODE_F32X2> {
  typedef float2 S;
  typedef float F;
  static __device__ __forceinline__ F diff(S a, S b) { return (b.x - a.x) + (b.y - a.y); }
  static __device__ __forceinline__ F add(F a, F b) { return a + b; }
  static __device__ __forceinline__ F sub(F a, F b) { return a - b; }
  static __device__ __forceinline__ F mul(F a, F b) { return a * b; }
};

// (hi, lo) + inc with Knuth's two-sum, renormalised (Dekker's fast two-sum)
__device__ __forceinline__ float2 ff_add(float2 v, float inc) {
  const float s = __fadd_rn(v.x, inc);
  const float bb = __fsub_rn(s, v.x);
  const float e = __fadd_rn(__fsub_rn(v.x, __fsub_rn(s, bb)), __fsub_rn(inc, bb));
  const float lo = __fadd_rn(v.y, e);
  const float hi = __fadd_rn(s, lo);
  return make_float2(hi, __fsub_rn(lo, __fsub_rn(hi, s)));
}

template <typename T>
__device__ __forceinline__ void store_images(T* base, int sy, long sz, int x, int y, int z, int nx, int ny, int nz,
                                             T v) {
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

template <typename S>
__device__ __forceinline__ S ldg_s(const S* p) { return __ldg(p); }

// One persistent launch = one time step of every patch (mode M, see PM above).
template <int M>
__global__ void __launch_bounds__(PT_THREADS) patches_step_kernel(const PatchDev* __restrict__ patches,
                                                                  const WorkItem* __restrict__ items, int nitems,
                                                                  const typename PM<M>::S* __restrict__ src,
                                                                  typename PM<M>::S* __restrict__ dst) {
  typedef typename PM<M>::S S;
  typedef typename PM<M>::F F;
  __shared__ F sfx[2][PT_MAX_TY * (PT_MAX_TX + 1) / 4 + 64];  // TY*(TX+1) <= 16*17, 8*33, 4*65
  __shared__ F sfy[2][(PT_MAX_TY + 1) * 16 + 64];            // (TY+1)*TX <= 17*16, 9*32, 5*64
  const int tid = threadIdx.x;
  for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
    const WorkItem it = items[w];
    const PatchDev P = patches[it.patch];
    const int lx = P.log2tx, TX = 1 << lx, TY = PT_THREADS >> lx;
    const int tx = tid & (TX - 1), ty = tid >> lx;
    const int nx = P.nx, ny = P.ny, nz = P.nz;
    const int sy = nx + 2;
    const long sz = (long)(nx + 2) * (ny + 2);
    const long interior = (long)1 + sy + sz;  // flat offset of interior (0,0,0)
    const S* tin = src + P.offset + interior;
    S* tout = dst + P.offset + interior;
    const F l2 = (F)P.lam2, hdt = (F)P.hdt;
    const int x = it.x0 + tx, y = it.y0 + ty;
    const bool active = x < nx && y < ny;
    const int xc = min(x, nx), yc = min(y, ny);
    auto at = [&](int i, int j, int k) { return (long)i + (long)sy * j + sz * k; };
    auto flux = [&](S ta, S tb) { return PM<M>::mul(l2, PM<M>::diff(ta, tb)); };
    S tc = ldg_s(tin + at(xc, yc, it.z0));
    F fzlo = flux(ldg_s(tin + at(xc, yc, it.z0 - 1)), tc);
    // register queue of the next PF planes (loads issued PF planes ahead of use; clamped to
    // the +z ghost plane, which exists)
    S q[PF];
#pragma unroll
    for (int i = 0; i < PF; ++i) q[i] = ldg_s(tin + at(xc, yc, min(it.z0 + 1 + i, nz)));
    for (int z = it.z0; z < it.z1; ++z) {
      const int buf = z & 1;
      const S tn = q[0];
#pragma unroll
      for (int i = 0; i < PF - 1; ++i) q[i] = q[i + 1];
      q[PF - 1] = ldg_s(tin + at(xc, yc, min(z + 1 + PF, nz)));
      const F fzhi = flux(tc, tn);
      const F fx = flux(ldg_s(tin + at(xc - 1, yc, z)), tc);
      const F fy = flux(ldg_s(tin + at(xc, yc - 1, z)), tc);
      sfx[buf][ty * (TX + 1) + tx] = fx;
      sfy[buf][ty * TX + tx] = fy;
      if (ty == 0) {  // +y halo faces of the tile
        const int yh = it.y0 + TY;
        if (yh <= ny && x <= nx) sfy[buf][TY * TX + tx] = flux(ldg_s(tin + at(xc, yh - 1, z)), ldg_s(tin + at(xc, yh, z)));
      } else if (ty == 1 && tx < TY) {  // +x halo faces of the tile
        const int xh = it.x0 + TX, yr = it.y0 + tx;
        if (xh <= nx && yr < ny) sfx[buf][tx * (TX + 1) + TX] = flux(ldg_s(tin + at(xh - 1, yr, z)), ldg_s(tin + at(xh, yr, z)));
      }
      __syncthreads();
      if (active) {
        const F fxhi = sfx[buf][ty * (TX + 1) + tx + 1];
        const F fyhi = sfy[buf][(ty + 1) * TX + tx];
        const F s = PM<M>::add(PM<M>::add(PM<M>::sub(fxhi, fx), PM<M>::sub(fyhi, fy)), PM<M>::sub(fzhi, fzlo));
        if constexpr (M == PMODE_F64) {
          store_images(tout, sy, sz, x, y, z, nx, ny, nz, __dadd_rn(tc, __dmul_rn(hdt, s)));
        } else {
          store_images(tout, sy, sz, x, y, z, nx, ny, nz, ff_add(tc, hdt * s));
        }
      }
      tc = tn;
      fzlo = fzhi;
    }
    __syncthreads();  // shared faces are reused by the next item
  }
}

// FP32 mode shares the ring machinery of the FP32 heat step: plane p (z0-1 <= p <= z1) lives in
// stage (p - z0 + PNS) % PNS, iteration z waits for planes up to z+1, syncs, refills the stage of
// plane z-2 with plane z+PNS-2 and computes from the stages of planes z and z+1; the z loop is
// unrolled over the ring so stages are constants.  lambda is a scalar per patch, so each face
// costs (2 lambda) * (Tb - Ta): two FP32 operations.
constexpr int PNS = 5;

// Every ghost cell of every patch of an FP32 arena takes its periodic source's value (one block
// per patch, threads over the six ghost faces: z faces whole, then y faces for the interior z,
// then x faces for the interior y and z).  The strip kernel writes no ghosts during the steps.
__global__ void __launch_bounds__(256) patches_ghosts_f32_kernel(const PatchDev* __restrict__ patches, int npatch,
                                                                 float* __restrict__ arena) {
  for (int p = blockIdx.x; p < npatch; p += gridDim.x) {
    const PatchDev P = patches[p];
    const int nx = P.nx, ny = P.ny, nz = P.nz, gx = nx + 2, gy = ny + 2;
    float* base = arena + P.offset + 1 + gx + (long)gx * gy;  // interior (0, 0, 0)
    const long sz = (long)gx * gy;
    const long A = (long)gx * gy, B = (long)gx * nz, C = (long)ny * nz;
    for (long g = threadIdx.x; g < 2 * (A + B + C); g += blockDim.x) {
      int x, y, z;
      if (g < 2 * A) {
        const long q = g % A;
        z = g < A ? -1 : nz;
        y = (int)(q / gx) - 1;
        x = (int)(q % gx) - 1;
      } else if (g < 2 * (A + B)) {
        const long h = g - 2 * A, q = h % B;
        y = h < B ? -1 : ny;
        z = (int)(q / gx);
        x = (int)(q % gx) - 1;
      } else {
        const long h = g - 2 * (A + B), q = h % C;
        x = h < C ? -1 : nx;
        z = (int)(q / ny);
        y = (int)(q % ny);
      }
      const int sx = x < 0 ? x + nx : (x >= nx ? x - nx : x);
      const int syy = y < 0 ? y + ny : (y >= ny ? y - ny : y);
      const int szz = z < 0 ? z + nz : (z >= nz ? z - nz : z);
      base[x + (long)gx * y + sz * z] = base[sx + (long)gx * syy + sz * szz];
    }
  }
}

__device__ __forceinline__ void pcp_async4(uint32_t smem, const void* gmem) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem), "l"(gmem) : "memory");
}
__device__ __forceinline__ void pcp_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void pcp_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

// FP32 mode, row strips: an item is a strip of R rows of W = min(nx, 512) columns of one patch
// over a z range (R <= 1024 / W, the patch's rows split evenly between its strips), and the
// block's 256 threads own its cells linearly (4 each, strided by 256), so lanes have cells
// whatever the patch's shape (tiles of fixed width leave up to half the lanes idle on patches of
// 16..96 cells).  The strip plus its one-cell halo, at most (R + 2)(W + 2) <= PR_STAGE floats,
// streams through the same ring of PNS stages as the tiled kernel; each cell reads its six
// neighbours from the stage and carries its centre value and the one below it in registers.  The
// halo is read from the periodic images' sources (x = -1 -> nx - 1, ...), so no step writes
// ghost cells: nebo_patchset_run fills them once after its last step.  With lambda constant over
// a patch the six face fluxes sum to 2 lambda (sum of the neighbours - 6 T), so a cell costs 5
// adds and 2 FMAs in FP32, T' = T + (dt lambda) (sum - 6 T) with dt lambda rounded once on the
// host (the FP64 mode keeps the reference's face form, bit for bit).
constexpr int PR_CELLS = 1024;                    // cells per strip plane
constexpr int PR_CPT = PR_CELLS / PT_THREADS;     // cells per thread
constexpr int PR_MAXW = 512;
constexpr int PR_STAGE = 2056;                    // max over W of (1024 / W + 2)(W + 2), W >= 2
constexpr int PR_NCOPY = (PR_STAGE + PT_THREADS - 1) / PT_THREADS;

// strip width and rows (the same on host and device)
__host__ __device__ __forceinline__ void strip_shape(int nx, int ny, int& wfull, int& rows) {
  wfull = nx < PR_MAXW ? nx : PR_MAXW;
  const int rmax = PR_CELLS / wfull, nstrips = (ny + rmax - 1) / rmax;
  rows = (ny + nstrips - 1) / nstrips;
}

__global__ void __launch_bounds__(PT_THREADS, 2) patches_f32_strip_kernel(const PatchDev* __restrict__ patches,
                                                                          const WorkItem* __restrict__ items,
                                                                          int nitems, const float* __restrict__ src,
                                                                          float* __restrict__ dst) {
  __shared__ __align__(16) float ring[PNS * PR_STAGE];
  const int tid = threadIdx.x;
  const uint32_t ring0 = (uint32_t)__cvta_generic_to_shared(ring);
  for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
    const WorkItem it = items[w];
    const PatchDev P = patches[it.patch];
    const int nx = P.nx, ny = P.ny, nz = P.nz;
    int wfull, rfull;
    strip_shape(nx, ny, wfull, rfull);
    const int W = min(wfull, nx - it.x0), R = min(rfull, ny - it.y0);
    const int SW = W + 2, PLANE = SW * (R + 2);  // stage row pitch and size
    const int sy = nx + 2;
    const long sz = (long)(nx + 2) * (ny + 2);
    const long interior = (long)1 + sy + sz;
    const float* tin = src + P.offset + interior;
    float* tout = dst + P.offset + interior;
    const float k = (float)(P.hdt * P.lam2);  // T' = T + k (sum of the 6 neighbours - 6 T)
    const int z0 = it.z0, z1 = it.z1;
    // copy slots: unit k of the (R+2) x (W+2) halo strip, halo cells at the patch's faces taken
    // from their periodic sources
    int goff[PR_NCOPY];
#pragma unroll
    for (int j = 0; j < PR_NCOPY; ++j) {
      const int k = min(tid + j * PT_THREADS, PLANE - 1);
      const int r = k / SW, c = k - r * SW;
      int x = it.x0 - 1 + c, y = it.y0 - 1 + r;
      x = x < 0 ? x + nx : (x >= nx ? x - nx : x);
      y = y < 0 ? y + ny : (y >= ny ? y - ny : y);
      goff[j] = x + sy * y;
    }
    auto issue = [&](int p, int st) {
      if (p <= z1) {
        const float* tp = tin + sz * (p < 0 ? p + nz : (p >= nz ? p - nz : p));
        const uint32_t so = ring0 + (uint32_t)(st * PR_STAGE) * sizeof(float);
#pragma unroll
        for (int j = 0; j < PR_NCOPY; ++j) {
          const int k = tid + j * PT_THREADS;
          if (k < PLANE) pcp_async4(so + (uint32_t)k * sizeof(float), tp + goff[j]);
        }
      }
    };
    issue(z0 - 1, PNS - 1);
    pcp_commit();
#pragma unroll
    for (int i = 0; i < PNS - 2; ++i) {
      issue(z0 + i, i);
      pcp_commit();
    }
    // this thread's cells: strip cell tid + 256 j -> stage index si, window offset gi (x + sy y);
    // bit j of `live`: the cell exists
    int si[PR_CPT], gi[PR_CPT];
    unsigned live = 0;
#pragma unroll
    for (int j = 0; j < PR_CPT; ++j) {
      const int c = tid + j * PT_THREADS;
      const int r = c / W, col = c - r * W;
      if (c < W * R) live |= 1u << j;
      si[j] = c < W * R ? (r + 1) * SW + col + 1 : SW + 1;
      gi[j] = (it.x0 + col) + sy * (it.y0 + r);
    }
    pcp_wait<PNS - 3>();
    __syncthreads();
    float t[PR_CPT], tb[PR_CPT];  // the cell and the one below it
#pragma unroll
    for (int j = 0; j < PR_CPT; ++j) {
      t[j] = ring[si[j]];
      tb[j] = ring[(PNS - 1) * PR_STAGE + si[j]];
    }
    for (int zb = z0; zb < z1; zb += PNS) {
#pragma unroll
      for (int i = 0; i < PNS; ++i) {
        const int z = zb + i;
        if (z >= z1) break;
        pcp_wait<PNS - 4>();
        __syncthreads();
        issue(z + PNS - 2, (i + PNS - 2) % PNS);
        pcp_commit();
        const float* T0 = ring + i * PR_STAGE;
        const float* Tn = ring + ((i + 1) % PNS) * PR_STAGE;
#pragma unroll
        for (int j = 0; j < PR_CPT; ++j) {
          const int c = si[j];
          const float tc = t[j], tn = Tn[c];
          const float nb = ((T0[c - 1] + T0[c + 1]) + (T0[c - SW] + T0[c + SW])) + (tb[j] + tn);
          if ((live >> j) & 1u) tout[(long)gi[j] + sz * z] = fmaf(k, fmaf(-6.0f, tc, nb), tc);
          tb[j] = tc;
          t[j] = tn;
        }
      }
    }
    pcp_wait<0>();
    __syncthreads();  // the ring is refilled by the next item
  }
}

// FP32 mode on bulk-copied slabs (every patch with nx <= PB_CELLS).  The FP32 working state
// holds each patch's interior only, rows padded to a multiple of 4 floats (16 bytes) and each
// patch 256-byte aligned, so every row starts on a 16-byte boundary.  An item is a strip of R
// full rows of one patch over a z range (R nx <= 1024, the rows split evenly between the strips).
// Per plane three cp.async.bulk copies fill a stage of the ring: the row below the strip, its R
// rows (one contiguous run) and the row above, the two halo rows and the halo planes taken from
// their periodic sources (rows ny-1 / 0, planes nz-1 / 0); the x halo is the row's own other end.
// One thread arms the stage's mbarrier and issues the copies; the 256 threads own the strip's
// cells linearly (4 each) and compute what patches_f32_strip_kernel computes, with the same
// operations.  No ghost cells exist in this layout: nebo_patchset_sync writes whole FP64 windows.
constexpr int PB_CELLS = 1024;                 // cells per strip plane
constexpr int PB_CPT = PB_CELLS / PT_THREADS;  // cells per thread
constexpr int PB_NS = 5;                       // stages

__host__ __device__ __forceinline__ int strip_rows_bulk(int nx, int ny) {
  const int rmax = PB_CELLS / nx > 0 ? PB_CELLS / nx : 1;
  const int nstrips = (ny + rmax - 1) / rmax;
  return (ny + nstrips - 1) / nstrips;
}

__device__ unsigned int g_patch_bulk_timeouts;

// stage_floats: floats per stage (a multiple of 4, at least (R + 2) pitch32 for every item)
__global__ void __launch_bounds__(PT_THREADS) patches_f32_bulk_kernel(const PatchDev* __restrict__ patches,
                                                                      const WorkItem* __restrict__ items, int nitems,
                                                                      const float* __restrict__ src,
                                                                      float* __restrict__ dst, int stage_floats) {
  extern __shared__ __align__(128) unsigned char pb_smem[];
  const float* ring = reinterpret_cast<const float*>(pb_smem);
  const uint32_t ring0 = (uint32_t)__cvta_generic_to_shared(pb_smem);
  const uint32_t bar0 = ring0 + (uint32_t)(PB_NS * stage_floats) * 4u;
  const int tid = threadIdx.x;
  bool ok = true;
  for (int w = blockIdx.x; w < nitems; w += gridDim.x) {
    const WorkItem it = items[w];
    const PatchDev P = patches[it.patch];
    const int nx = P.nx, ny = P.ny, nz = P.nz, pitch = P.pitch32;
    const int R = min(strip_rows_bulk(nx, ny), ny - it.y0);
    const long sz = (long)ny * pitch;
    const float* base = src + P.off32;
    float* obase = dst + P.off32;
    const float k = (float)(P.hdt * P.lam2);  // T' = T + k (sum of the 6 neighbours - 6 T)
    const int z0 = it.z0, z1 = it.z1;
    const uint32_t rowb = (uint32_t)pitch * 4u;
    const int ylo = it.y0 == 0 ? ny - 1 : it.y0 - 1;
    const int yhi = it.y0 + R == ny ? 0 : it.y0 + R;
    if (tid == 0) {
      for (int st = 0; st < PB_NS; ++st) mbar_init(bar0 + 8 * st, 1);
      asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    // plane q of the item is z0 - 1 + q (periodic), in stage q % PB_NS, phase (q / PB_NS) & 1
    auto issue = [&](int q) {
      const int p = z0 - 1 + q;
      if (p > z1) return;  // the last plane read is z1 (the +z neighbour of the item's last plane)
      const int pw = p < 0 ? p + nz : (p >= nz ? p - nz : p);
      const int st = q % PB_NS;
      const uint32_t bar = bar0 + 8 * st;
      const uint32_t so = ring0 + (uint32_t)(st * stage_floats) * 4u;
      const float* pl = base + (long)pw * sz;
      mbar_expect_tx(bar, (uint32_t)(R + 2) * rowb);
      bulk_g2s(so, pl + (long)ylo * pitch, rowb, bar);
      bulk_g2s(so + rowb, pl + (long)it.y0 * pitch, (uint32_t)R * rowb, bar);
      bulk_g2s(so + (uint32_t)(R + 1) * rowb, pl + (long)yhi * pitch, rowb, bar);
    };
    if (tid == 0)
      for (int q = 0; q < PB_NS; ++q) issue(q);
    // this thread's cells: strip cell tid + 256 j -> stage indices (centre, x-1, x+1, wrapped
    // within the row) and the output offset in a plane; bit j of `live`: the cell exists
    int si[PB_CPT], sl[PB_CPT], sr[PB_CPT], go[PB_CPT];
    unsigned live = 0;
#pragma unroll
    for (int j = 0; j < PB_CPT; ++j) {
      const int c = tid + j * PT_THREADS;
      const bool in = c < R * nx;
      const int r = in ? c / nx : 0, col = in ? c - r * nx : 0;
      if (in) live |= 1u << j;
      si[j] = (r + 1) * pitch + col;
      sl[j] = (r + 1) * pitch + (col == 0 ? nx - 1 : col - 1);
      sr[j] = (r + 1) * pitch + (col == nx - 1 ? 0 : col + 1);
      go[j] = (it.y0 + r) * pitch + col;
    }
    ok &= mbar_wait(bar0, 0) & mbar_wait(bar0 + 8, 0);
    float t[PB_CPT], tb[PB_CPT];  // the cell and the one below it
#pragma unroll
    for (int j = 0; j < PB_CPT; ++j) {
      t[j] = ring[stage_floats + si[j]];
      tb[j] = ring[si[j]];
    }
    for (int z = z0; z < z1; ++z) {
      const int q = z - z0 + 1;  // centre plane
      __syncthreads();           // plane q-1's stage is no longer read
      if (tid == 0) {
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        issue(q - 1 + PB_NS);
      }
      ok &= mbar_wait(bar0 + 8 * ((q + 1) % PB_NS), ((q + 1) / PB_NS) & 1);
      const float* T0 = ring + (q % PB_NS) * stage_floats;
      const float* Tn = ring + ((q + 1) % PB_NS) * stage_floats;
      float* op = obase + (long)z * sz;
#pragma unroll
      for (int j = 0; j < PB_CPT; ++j) {
        const int c = si[j];
        const float tc = t[j], tn = Tn[c];
        const float nb = ((T0[sl[j]] + T0[sr[j]]) + (T0[c - pitch] + T0[c + pitch])) + (tb[j] + tn);
        if ((live >> j) & 1u) op[go[j]] = fmaf(k, fmaf(-6.0f, tc, nb), tc);
        tb[j] = tc;
        t[j] = tn;
      }
    }
    __syncthreads();  // every copy of the item has landed and been read: the barriers start over
    if (tid == 0)
      for (int st = 0; st < PB_NS; ++st) mbar_inval(bar0 + 8 * st);
  }
  if (!ok) atomicAdd(&g_patch_bulk_timeouts, 1u);
}

// FP64 windows -> FP32 slab layout (interiors only) and back (whole windows: each cell of a
// window takes its periodic interior source, so the ghosts are filled in the same pass).
__global__ void patches_pack_f32_kernel(const PatchDev* __restrict__ patches, int npatch,
                                        const double* __restrict__ a64, float* __restrict__ a32) {
  for (int p = blockIdx.y; p < npatch; p += gridDim.y) {
    const PatchDev P = patches[p];
    const int nx = P.nx, ny = P.ny, gx = nx + 2, gy = ny + 2;
    const long n = (long)nx * ny * P.nz;
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
      const int x = (int)(i % nx), y = (int)((i / nx) % ny), z = (int)(i / ((long)nx * ny));
      a32[P.off32 + ((long)z * ny + y) * P.pitch32 + x] =
          (float)a64[P.offset + (x + 1) + (long)gx * ((y + 1) + (long)gy * (z + 1))];
    }
  }
}
__global__ void patches_unpack_f32_kernel(const PatchDev* __restrict__ patches, int npatch,
                                          const float* __restrict__ a32, double* __restrict__ a64) {
  for (int p = blockIdx.y; p < npatch; p += gridDim.y) {
    const PatchDev P = patches[p];
    const int nx = P.nx, ny = P.ny, nz = P.nz, gx = nx + 2, gy = ny + 2;
    const long n = (long)gx * gy * (nz + 2);
    for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
      int x = (int)(i % gx) - 1, y = (int)((i / gx) % gy) - 1, z = (int)(i / ((long)gx * gy)) - 1;
      x = x < 0 ? nx - 1 : (x == nx ? 0 : x);
      y = y < 0 ? ny - 1 : (y == ny ? 0 : y);
      z = z < 0 ? nz - 1 : (z == nz ? 0 : z);
      a64[P.offset + i] = (double)a32[P.off32 + ((long)z * ny + y) * P.pitch32 + x];
    }
  }
}

}  // namespace

// Bounded waits of the patch kernels that gave up since the last call (cleared by the read).
int patch_wait_timeouts(unsigned int* count) {
  unsigned int v = 0, zero = 0;
  NEBO_CUDA_TRY(cudaMemcpyFromSymbol(&v, g_patch_bulk_timeouts, sizeof(v)));
  if (v) NEBO_CUDA_TRY(cudaMemcpyToSymbol(g_patch_bulk_timeouts, &zero, sizeof(zero)));
  *count = v;
  return NEBO_OK;
}

struct PatchSet {
  int npatch = 0;
  int dtype = NEBO_F64;
  std::vector<int> shape;  // 3 per patch
  std::vector<long long> offset;
  std::vector<double> lam, dt;
  std::vector<int> log2tx;
  long long total = 0;  // elements per arena
  void* arena[2] = {nullptr, nullptr};    // FP64 states
  float* arena32[2] = {nullptr, nullptr};  // FP32 states (FP32 mode)
  float2* arena2[2] = {nullptr, nullptr};  // two-float states (FP32X2 mode)
  PatchDev* d_patches = nullptr;
  WorkItem* d_items = nullptr;
  int nitems = 0;
  int zchunk = 16;
  int grid = 0;
  int grid32 = 0;  // resident blocks of the FP32 ring kernel (one full wave)
  bool bulk32 = false;            // FP32 mode on the slab layout (every nx <= PB_CELLS)
  std::vector<long long> off32;   // slab layout: interior offsets
  std::vector<int> pitch32;       // slab layout: row pitches
  long long total32 = 0;          // slab layout: floats per arena
  int stage32 = 0;                // slab layout: floats per ring stage
  std::map<std::pair<int, int>, cudaGraphExec_t> graphs;  // (steps, parity) -> graph
  ~PatchSet() {
    for (auto& kv : graphs) cudaGraphExecDestroy(kv.second);
    cudaFree(arena[0]);
    cudaFree(arena[1]);
    cudaFree(arena32[0]);
    cudaFree(arena32[1]);
    cudaFree(arena2[0]);
    cudaFree(arena2[1]);
    cudaFree(d_patches);
    cudaFree(d_items);
  }
};

namespace {

std::vector<WorkItem> build_items(const PatchSet& ps, const std::vector<int>& which, int zchunk) {
  std::vector<WorkItem> items;
  for (int p : which) {
    const int nx = ps.shape[3 * p], ny = ps.shape[3 * p + 1], nz = ps.shape[3 * p + 2];
    // FP32: row strips (strip_shape); otherwise tiles, one row per thread row
    int TX = 1 << ps.log2tx[p], TY = PT_THREADS / TX;
    if (ps.dtype == NEBO_F32) {
      if (ps.bulk32) {
        TX = nx;
        TY = strip_rows_bulk(nx, ny);
      } else {
        strip_shape(nx, ny, TX, TY);
      }
    }
    for (int z0 = 0; z0 < nz; z0 += zchunk)
      for (int y0 = 0; y0 < ny; y0 += TY)
        for (int x0 = 0; x0 < nx; x0 += TX) items.push_back(WorkItem{p, x0, y0, z0, std::min(z0 + zchunk, nz)});
  }
  // largest z-extent items first so the strided assignment ends with short items
  std::stable_sort(items.begin(), items.end(), [](const WorkItem& a, const WorkItem& b) { return (a.z1 - a.z0) > (b.z1 - b.z0); });
  return items;
}

int upload_tables(PatchSet& ps, const std::vector<WorkItem>& items, cudaStream_t s) {
  std::vector<PatchDev> pd(ps.npatch);
  for (int p = 0; p < ps.npatch; ++p) {
    pd[p].offset = ps.offset[p];
    pd[p].off32 = ps.bulk32 ? ps.off32[p] : 0;
    pd[p].pitch32 = ps.bulk32 ? ps.pitch32[p] : 0;
    pd[p].nx = ps.shape[3 * p];
    pd[p].ny = ps.shape[3 * p + 1];
    pd[p].nz = ps.shape[3 * p + 2];
    pd[p].log2tx = ps.log2tx[p];
    pd[p].lam2 = ps.lam[p] + ps.lam[p];
    pd[p].hdt = 0.5 * ps.dt[p];
  }
  if (!ps.d_patches) NEBO_CUDA_TRY(cudaMalloc((void**)&ps.d_patches, sizeof(PatchDev) * ps.npatch));
  NEBO_CUDA_TRY(cudaMemcpyAsync(ps.d_patches, pd.data(), sizeof(PatchDev) * ps.npatch, cudaMemcpyHostToDevice, s));
  cudaFree(ps.d_items);
  ps.d_items = nullptr;
  NEBO_CUDA_TRY(cudaMalloc((void**)&ps.d_items, sizeof(WorkItem) * std::max<size_t>(1, items.size())));
  NEBO_CUDA_TRY(cudaMemcpyAsync(ps.d_items, items.data(), sizeof(WorkItem) * items.size(), cudaMemcpyHostToDevice, s));
  NEBO_CUDA_TRY(cudaStreamSynchronize(s));
  ps.nitems = (int)items.size();
  for (auto& kv : ps.graphs) cudaGraphExecDestroy(kv.second);
  ps.graphs.clear();
  return NEBO_OK;
}

int launch_step(const PatchSet& ps, const WorkItem* items, int nitems, int parity, cudaStream_t s) {
  if (nitems == 0) return NEBO_OK;
  LaunchScope ls(ps.dtype == NEBO_F64 ? "patches_step_f64" : (ps.dtype == NEBO_F32 ? "patches_step_f32" : "patches_step_f32x2"), s);
  const int grid = std::min(nitems, ps.grid);
  if (ps.dtype == NEBO_F64)
    patches_step_kernel<PMODE_F64><<<grid, PT_THREADS, 0, s>>>(ps.d_patches, items, nitems,
                                                               (const double*)ps.arena[parity],
                                                               (double*)ps.arena[parity ^ 1]);
  else if (ps.dtype == NEBO_F32 && ps.bulk32)
    patches_f32_bulk_kernel<<<std::min(nitems, ps.grid32), PT_THREADS,
                              (size_t)PB_NS * ps.stage32 * sizeof(float) + PB_NS * sizeof(uint64_t), s>>>(
        ps.d_patches, items, nitems, ps.arena32[parity], ps.arena32[parity ^ 1], ps.stage32);
  else if (ps.dtype == NEBO_F32)
    patches_f32_strip_kernel<<<std::min(nitems, ps.grid32), PT_THREADS, 0, s>>>(ps.d_patches, items, nitems,
                                                                               ps.arena32[parity],
                                                                               ps.arena32[parity ^ 1]);
  else
    patches_step_kernel<PMODE_F32X2><<<grid, PT_THREADS, 0, s>>>(ps.d_patches, items, nitems, ps.arena2[parity],
                                                                 ps.arena2[parity ^ 1]);
  NEBO_LAUNCH_CHECK("nebo_patchset_run");
  return NEBO_OK;
}

int default_log2tx(int nx) { return nx <= 16 ? 4 : (nx <= 40 ? 5 : 6); }

__global__ void patches_cast_kernel(const double* __restrict__ a, float* __restrict__ b, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}
__global__ void patches_split_kernel(const double* __restrict__ a, float2* __restrict__ b, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const float hi = (float)a[i];
    b[i] = make_float2(hi, (float)(a[i] - (double)hi));
  }
}
__global__ void patches_widen_kernel(const float* __restrict__ a, double* __restrict__ b, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    b[i] = (double)a[i];
}
__global__ void patches_join_kernel(const float2* __restrict__ a, double* __restrict__ b, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    b[i] = (double)a[i].x + (double)a[i].y;
}

}  // namespace
}  // namespace nebo

using namespace nebo;

struct nebo_patchset : PatchSet {};

extern "C" int nebo_patchset_create(nebo_patchset** out, int npatch, const int32_t* shapes, const double* lam,
                                    const double* dt, int dtype) {
  if (!out || npatch <= 0 || !shapes || !lam || !dt)
    return fail(NEBO_ERR_INVALID, "Nebo error in nebo_patchset_create: bad arguments");
  if (dtype != NEBO_F64 && dtype != NEBO_F32 && dtype != NEBO_F32X2)
    return fail(NEBO_ERR_INVALID, "Nebo error in nebo_patchset_create: dtype");
  *out = nullptr;
  nebo_patchset* ps = new nebo_patchset();
  ps->npatch = npatch;
  ps->dtype = dtype;
  ps->shape.assign(shapes, shapes + 3 * npatch);
  ps->lam.assign(lam, lam + npatch);
  ps->dt.assign(dt, dt + npatch);
  ps->offset.resize(npatch);
  ps->log2tx.resize(npatch);
  long long off = 0;
  for (int p = 0; p < npatch; ++p) {
    const int nx = shapes[3 * p], ny = shapes[3 * p + 1], nz = shapes[3 * p + 2];
    if (nx < 2 || ny < 2 || nz < 2) {
      delete ps;
      return fail(NEBO_ERR_INVALID, "Nebo error in nebo_patchset_create: patch %d has an edge below 2", p);
    }
    ps->offset[p] = off;
    off += (long long)(nx + 2) * (ny + 2) * (nz + 2);
    off = (off + 31) & ~31LL;  // 256-byte aligned windows
    ps->log2tx[p] = default_log2tx(nx);
  }
  ps->total = off;
  const size_t bytes = (size_t)off * sizeof(double);
  cudaError_t e = cudaMalloc(&ps->arena[0], bytes);
  if (e == cudaSuccess) e = cudaMalloc(&ps->arena[1], bytes);
  if (e == cudaSuccess) e = cudaMemset(ps->arena[0], 0, bytes);
  if (e == cudaSuccess) e = cudaMemset(ps->arena[1], 0, bytes);
  if (dtype == NEBO_F32X2) {
    const size_t b2 = (size_t)off * sizeof(float2);
    if (e == cudaSuccess) e = cudaMalloc((void**)&ps->arena2[0], b2);
    if (e == cudaSuccess) e = cudaMalloc((void**)&ps->arena2[1], b2);
    if (e == cudaSuccess) e = cudaMemset(ps->arena2[0], 0, b2);
    if (e == cudaSuccess) e = cudaMemset(ps->arena2[1], 0, b2);
  }
  if (dtype == NEBO_F32) {
    // the slab layout when every row fits a strip: interiors only, rows padded to 16 bytes
    ps->bulk32 = true;
    for (int p = 0; p < npatch; ++p) ps->bulk32 = ps->bulk32 && shapes[3 * p] <= PB_CELLS;
    if (ps->bulk32) {
      ps->off32.resize(npatch);
      ps->pitch32.resize(npatch);
      long long o32 = 0;
      int stage = 0;
      for (int p = 0; p < npatch; ++p) {
        const int nx = shapes[3 * p], ny = shapes[3 * p + 1], nz = shapes[3 * p + 2];
        const int pitch = (nx + 3) / 4 * 4;
        ps->off32[p] = o32;
        ps->pitch32[p] = pitch;
        o32 += (long long)pitch * ny * nz;
        o32 = (o32 + 63) & ~63LL;  // 256-byte aligned patches
        stage = std::max(stage, (strip_rows_bulk(nx, ny) + 2) * pitch);
      }
      ps->total32 = o32;
      ps->stage32 = stage;
    }
  }
  if (dtype == NEBO_F32) {
    const size_t b32 = (size_t)(ps->bulk32 ? ps->total32 : off) * sizeof(float);
    if (e == cudaSuccess) e = cudaMalloc((void**)&ps->arena32[0], b32);
    if (e == cudaSuccess) e = cudaMalloc((void**)&ps->arena32[1], b32);
    if (e == cudaSuccess) e = cudaMemset(ps->arena32[0], 0, b32);
    if (e == cudaSuccess) e = cudaMemset(ps->arena32[1], 0, b32);
  }
  if (e != cudaSuccess) {
    delete ps;
    return cuda_fail(e, "nebo_patchset_create");
  }
  ps->grid = num_sms() * 8;
  if (dtype == NEBO_F32) {
    ps->zchunk = 1 << 30;  // FP32 items cover the patch's whole z extent
    int per_sm = 0;
    if (ps->bulk32) {
      const size_t smem = (size_t)PB_NS * ps->stage32 * sizeof(float) + PB_NS * sizeof(uint64_t);
      if (smem > 48 * 1024 &&
          cudaFuncSetAttribute(patches_f32_bulk_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
              cudaSuccess) {
        cudaGetLastError();
        delete ps;
        return fail(NEBO_ERR_UNSUPPORTED, "Nebo error in nebo_patchset_create: FP32 strips need %zu bytes of "
                                          "shared memory", smem);
      }
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, patches_f32_bulk_kernel, PT_THREADS, smem) !=
              cudaSuccess ||
          per_sm < 1) {
        cudaGetLastError();
        per_sm = 1;
      }
    } else if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, patches_f32_strip_kernel, PT_THREADS, 0) !=
                   cudaSuccess ||
               per_sm < 1) {
      cudaGetLastError();
      per_sm = 1;
    }
    ps->grid32 = num_sms() * per_sm;
  }
  std::vector<int> all(npatch);
  for (int p = 0; p < npatch; ++p) all[p] = p;
  int rc = upload_tables(*ps, build_items(*ps, all, ps->zchunk), 0);
  if (rc) {
    delete ps;
    return rc;
  }
  *out = ps;
  return NEBO_OK;
}

extern "C" int nebo_patchset_destroy(nebo_patchset* ps) {
  delete ps;
  return NEBO_OK;
}

extern "C" int nebo_patchset_info(const nebo_patchset* ps, int64_t* total_elems, int64_t* offsets, int32_t* log2tx,
                                  int32_t* nitems) {
  if (!ps) return fail(NEBO_ERR_INVALID, "Nebo error in nebo_patchset_info: null handle");
  if (total_elems) *total_elems = ps->total;
  for (int p = 0; p < ps->npatch; ++p) {
    if (offsets) offsets[p] = ps->offset[p];
    if (log2tx) log2tx[p] = ps->log2tx[p];
  }
  if (nitems) *nitems = ps->nitems;
  return NEBO_OK;
}

extern "C" void* nebo_patchset_arena(const nebo_patchset* ps, int which) {
  return (ps && (which == 0 || which == 1)) ? ps->arena[which] : nullptr;
}

// Every patch's ghosts take their periodic images (run once after filling arena 0).
extern "C" int nebo_patchset_fill_ghosts(const nebo_patchset* ps, int which, nebo_stream_t stream) {
  if (!ps || (which != 0 && which != 1)) return fail(NEBO_ERR_INVALID, "Nebo error in nebo_patchset_fill_ghosts");
  for (int p = 0; p < ps->npatch; ++p) {
    nebo_field f;
    f.data = (double*)ps->arena[which] + ps->offset[p];
    for (int i = 0; i < 3; ++i) {
      f.glob[i] = f.extent[i] = ps->shape[3 * p + i] + 2;
      f.offset[i] = 0;
      f.ghost_minus[i] = f.ghost_plus[i] = 1;
      f.has_bc[i] = f.bc_extra[i] = 0;
    }
    f.dtype = NEBO_F64;
    int rc = nebo::fill_periodic_any(&f, (cudaStream_t)stream);
    if (rc) return rc;
  }
  if (ps->dtype == NEBO_F32 && ps->bulk32) {  // the FP32 working state, slab layout
    LaunchScope ls("patches_pack_f32", (cudaStream_t)stream);
    patches_pack_f32_kernel<<<dim3(8, std::min(ps->npatch, 4096)), 256, 0, (cudaStream_t)stream>>>(
        ps->d_patches, ps->npatch, (const double*)ps->arena[which], ps->arena32[which]);
    NEBO_LAUNCH_CHECK("nebo_patchset_fill_ghosts");
  } else if (ps->dtype == NEBO_F32) {  // the FP32 working state
    LaunchScope ls("patches_cast_f32", (cudaStream_t)stream);
    patches_cast_kernel<<<num_sms() * 8, 256, 0, (cudaStream_t)stream>>>((const double*)ps->arena[which],
                                                                         ps->arena32[which], (size_t)ps->total);
    NEBO_LAUNCH_CHECK("nebo_patchset_fill_ghosts");
  } else if (ps->dtype == NEBO_F32X2) {  // split each double into (hi, lo) floats
    LaunchScope ls("patches_split_f32x2", (cudaStream_t)stream);
    patches_split_kernel<<<num_sms() * 8, 256, 0, (cudaStream_t)stream>>>((const double*)ps->arena[which],
                                                                          ps->arena2[which], (size_t)ps->total);
    NEBO_LAUNCH_CHECK("nebo_patchset_fill_ghosts");
  }
  return NEBO_OK;
}

// Bring the state of arena `which` into its FP64 arena (FP32 mode widens, FP32X2 joins hi + lo;
// FP64 mode already keeps its state there).
extern "C" int nebo_patchset_sync(const nebo_patchset* ps, int which, nebo_stream_t stream) {
  if (!ps || (which != 0 && which != 1)) return fail(NEBO_ERR_INVALID, "Nebo error in nebo_patchset_sync");
  if (ps->dtype == NEBO_F64) return NEBO_OK;
  LaunchScope ls("patches_to_f64", (cudaStream_t)stream);
  if (ps->dtype == NEBO_F32X2)
    patches_join_kernel<<<num_sms() * 8, 256, 0, (cudaStream_t)stream>>>(ps->arena2[which], (double*)ps->arena[which],
                                                                         (size_t)ps->total);
  else if (ps->bulk32)
    patches_unpack_f32_kernel<<<dim3(8, std::min(ps->npatch, 4096)), 256, 0, (cudaStream_t)stream>>>(
        ps->d_patches, ps->npatch, ps->arena32[which], (double*)ps->arena[which]);
  else
    patches_widen_kernel<<<num_sms() * 8, 256, 0, (cudaStream_t)stream>>>(ps->arena32[which],
                                                                          (double*)ps->arena[which], (size_t)ps->total);
  NEBO_LAUNCH_CHECK("nebo_patchset_sync");
  return NEBO_OK;
}

// Time each tile width on the patches of each x-extent class and keep the fastest.
// FP32 strips need no tile width; the tuner picks the z extent of the items instead (whole
// patches, or chunks of 32 or 16 planes: shorter items balance the persistent blocks better,
// longer ones refill the plane ring less often) by timing whole steps.
static int autotune_strips(nebo_patchset* ps, cudaStream_t s, int32_t* chosen_log2tx) {
  std::vector<int> all(ps->npatch);
  for (int p = 0; p < ps->npatch; ++p) all[p] = p;
  cudaEvent_t a, b;
  NEBO_CUDA_TRY(cudaEventCreate(&a));
  NEBO_CUDA_TRY(cudaEventCreate(&b));
  int rc = NEBO_OK, bestz = ps->zchunk;
  float best = 1e30f;
  const int cands[3] = {1 << 30, 32, 16};
  for (int zc : cands) {
    rc = upload_tables(*ps, build_items(*ps, all, zc), s);
    if (rc) break;
    float ms = 0.f;
    for (int rep = 0; rep < 4 && !rc; ++rep) {
      cudaEventRecord(a, s);
      rc = launch_step(*ps, ps->d_items, ps->nitems, rep & 1, s);
      cudaEventRecord(b, s);
      cudaEventSynchronize(b);
      float t = 0.f;
      cudaEventElapsedTime(&t, a, b);
      if (rep > 0) ms += t;  // first launch warms up
    }
    if (!rc && ms < best) {
      best = ms;
      bestz = zc;
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (rc) return rc;
  ps->zchunk = bestz;
  rc = upload_tables(*ps, build_items(*ps, all, ps->zchunk), s);
  if (rc) return rc;
  if (chosen_log2tx)
    for (int p = 0; p < ps->npatch; ++p) chosen_log2tx[p] = ps->log2tx[p];
  return NEBO_OK;
}

extern "C" int nebo_patchset_autotune(nebo_patchset* ps, nebo_stream_t stream, int32_t* chosen_log2tx) {
  if (!ps) return fail(NEBO_ERR_INVALID, "Nebo error in nebo_patchset_autotune: null handle");
  cudaStream_t s = (cudaStream_t)stream;
  if (ps->dtype == NEBO_F32) return autotune_strips(ps, s, chosen_log2tx);
  std::map<int, std::vector<int>> classes;  // class by nx bucket of 8
  for (int p = 0; p < ps->npatch; ++p) classes[(ps->shape[3 * p] + 7) / 8].push_back(p);
  cudaEvent_t a, b;
  NEBO_CUDA_TRY(cudaEventCreate(&a));
  NEBO_CUDA_TRY(cudaEventCreate(&b));
  WorkItem* d_tmp = nullptr;
  int rc = NEBO_OK;
  for (auto& kv : classes) {
    float best = 1e30f;
    int bestl = default_log2tx(ps->shape[3 * kv.second[0]]);
    for (int l = 4; l <= 6 && !rc; ++l) {
      for (int p : kv.second) ps->log2tx[p] = l;
      std::vector<WorkItem> items = build_items(*ps, kv.second, ps->zchunk);
      cudaFree(d_tmp);
      d_tmp = nullptr;
      if (cudaMalloc((void**)&d_tmp, sizeof(WorkItem) * items.size()) != cudaSuccess) { rc = NEBO_ERR_ALLOC; break; }
      cudaMemcpyAsync(d_tmp, items.data(), sizeof(WorkItem) * items.size(), cudaMemcpyHostToDevice, s);
      // patch table must carry the candidate tile width
      std::vector<int> keep = ps->log2tx;
      rc = upload_tables(*ps, std::vector<WorkItem>(), s);
      if (rc) break;
      float ms = 0.f;
      for (int rep = 0; rep < 4 && !rc; ++rep) {
        cudaEventRecord(a, s);
        rc = launch_step(*ps, d_tmp, (int)items.size(), rep & 1, s);
        cudaEventRecord(b, s);
        cudaEventSynchronize(b);
        float t = 0.f;
        cudaEventElapsedTime(&t, a, b);
        if (rep > 0) ms += t;  // first launch warms up
      }
      if (ms < best) {
        best = ms;
        bestl = l;
      }
    }
    for (int p : kv.second) ps->log2tx[p] = bestl;
  }
  cudaFree(d_tmp);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  if (rc) return rc;
  std::vector<int> all(ps->npatch);
  for (int p = 0; p < ps->npatch; ++p) all[p] = p;
  rc = upload_tables(*ps, build_items(*ps, all, ps->zchunk), s);
  if (rc) return rc;
  if (chosen_log2tx)
    for (int p = 0; p < ps->npatch; ++p) chosen_log2tx[p] = ps->log2tx[p];
  // the timing runs overwrote the arenas: callers autotune before loading data
  return NEBO_OK;
}

// After the steps of a run: the FP32 strip kernel writes no ghost cells, so the arena that holds
// the result gets them here (one launch).
int finish_run(const PatchSet& ps, int which, cudaStream_t s) {
  if (ps.dtype != NEBO_F32 || ps.bulk32) return NEBO_OK;  // the slab layout has no ghost cells
  LaunchScope ls("patches_ghosts_f32", s);
  patches_ghosts_f32_kernel<<<std::min(ps.npatch, num_sms() * 8), 256, 0, s>>>(ps.d_patches, ps.npatch,
                                                                               ps.arena32[which]);
  NEBO_LAUNCH_CHECK("nebo_patchset_run ghosts");
  return NEBO_OK;
}

// steps time steps starting from arena `start`; returns (via *final) the arena holding the result.
extern "C" int nebo_patchset_run(nebo_patchset* ps, int start, int steps, int use_graph, int* final_arena,
                                 nebo_stream_t stream) {
  if (!ps || (start != 0 && start != 1) || steps < 0) return fail(NEBO_ERR_INVALID, "Nebo error in nebo_patchset_run");
  cudaStream_t s = (cudaStream_t)stream;
  if (final_arena) *final_arena = (start + steps) & 1;
  if (steps == 0) return NEBO_OK;
  if (!use_graph) {
    for (int k = 0; k < steps; ++k) {
      int rc = launch_step(*ps, ps->d_items, ps->nitems, (start + k) & 1, s);
      if (rc) return rc;
    }
    return finish_run(*ps, (start + steps) & 1, s);
  }
  const std::pair<int, int> key(steps, start);
  auto it = ps->graphs.find(key);
  if (it == ps->graphs.end()) {
    cudaStream_t cap;
    NEBO_CUDA_TRY(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
    NEBO_CUDA_TRY(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
    int rc = NEBO_OK;
    for (int k = 0; k < steps && !rc; ++k) rc = launch_step(*ps, ps->d_items, ps->nitems, (start + k) & 1, cap);
    if (!rc) rc = finish_run(*ps, (start + steps) & 1, cap);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(cap, &g);
    cudaStreamDestroy(cap);
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (e != cudaSuccess) return cuda_fail(e, "nebo_patchset_run capture");
    cudaGraphExec_t exec;
    e = cudaGraphInstantiate(&exec, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(e, "nebo_patchset_run instantiate");
    it = ps->graphs.emplace(key, exec).first;
  }
  NEBO_CUDA_TRY(cudaGraphLaunch(it->second, s));
  return NEBO_OK;
}
