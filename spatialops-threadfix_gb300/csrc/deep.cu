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
// Kernel 1 evaluates exp and sin mostly on the integer pipe (fp64_int.cuh); kernel 2 sums the 27
// points separably (x, then y from shared memory, then z from registers while marching in z),
// optionally folding the four reductions of filt into the same pass.
#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "fp64_int.cuh"
#include "reduce4.cuh"

namespace nebo {
namespace {

constexpr int FX = 32;  // filter tile x
constexpr int FY = 8;   // filter tile y

// A thread walks z in steps of gridDim.z; the loads of its next cell (the four a values, b, c
// and the mask word) are issued one step ahead, so their latency overlaps this cell's exp/sin.
__global__ void __launch_bounds__(256) deep_out_kernel(const double* __restrict__ a, const double* __restrict__ b,
                                                       const double* __restrict__ c, const uint32_t* __restrict__ mask,
                                                       long mask_base, double* __restrict__ out, int sy, long sz,
                                                       int nx, int ny, int nz, double q) {
  // region: x in [1, nx), y in [-1, ny+1), z in [-1, nz+1)
  const int x = 1 + blockIdx.x * blockDim.x + threadIdx.x;
  const int y = -1 + (int)(blockIdx.y * blockDim.y + threadIdx.y);
  if (x >= nx || y > ny) return;
  const int zs = gridDim.z;
  const long row = (long)x + (long)sy * y;
  struct Cell {
    double am2, am1, a0, ap1, b, c;
    uint32_t w;
  };
  auto load = [&](int z) {
    Cell v;
    const long i = row + sz * z;
    const long bit = mask_base + i;  // flat index in the window
    v.w = __ldg(mask + (bit >> 5)) >> (bit & 31);
    v.am2 = __ldg(a + i - 2);
    v.am1 = __ldg(a + i - 1);
    v.a0 = __ldg(a + i);
    v.ap1 = __ldg(a + i + 1);
    v.b = __ldg(b + i);
    v.c = __ldg(c + i);
    return v;
  };
  int z = -1 + (int)blockIdx.z;
  if (z > nz) return;
  Cell cur = load(z);
  for (; z <= nz; z += zs) {
    const int zn = z + zs;
    const Cell nxt = load(zn <= nz ? zn : z);  // the last step reloads its own cell
    double v;
    if (cur.w & 1u) {
      v = 0.0;
    } else {
      const double igi = q * ((cur.ap1 - cur.am1) + (cur.a0 - cur.am2));
      v = fma(igi, fixmath::exp_i(cur.b), fixmath::sin_i(cur.c));
    }
    out[row + sz * z] = v;
    cur = nxt;
  }
}

__device__ __forceinline__ void cp_async8(uint32_t smem, const void* gmem) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(smem), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory"); }

struct ShellArgs {
  int on;              // 1: the shell is not empty
  const double* base;  // filt's allocation
  int gx;
  long gxy;
  int lx, hx, ly, hy, lz, hz;        // reduction box [lo, hi) (glob coordinates)
  int ix0, ix1, iy0, iy1, iz0, iz1;  // the filter's written box, excluded
};

// The four reductions over the cells of box [lo, hi) that are not in the box [ilo, ihi): the
// valid ghost cells of `filt`, which the filter does not write but nebo_sum/max/min/norm
// include.  Two parts: the rows entirely outside the inner box (planes z outside it, and rows y
// outside it within the inner z range), a warp per row; and the x ends of the rows that cross
// the inner box, a thread per cell.  Block sb of nsb, 256 threads (tid linear).
__device__ __forceinline__ void shell_part(Acc4& acc, const ShellArgs& sa, int sb, int nsb, int tid) {
  const int lane = tid & 31;
  const int nyr = sa.hy - sa.ly;
  const int zout = (sa.iz0 - sa.lz) + (sa.hz - sa.iz1);        // planes outside the inner z range
  const int yout = (sa.iy0 - sa.ly) + (sa.hy - sa.iy1);        // rows per inner plane outside in y
  const int nfull = zout * nyr + (sa.iz1 - sa.iz0) * yout;
  for (int r = sb * 8 + (tid >> 5); r < nfull; r += nsb * 8) {
    int y, z;
    if (r < zout * nyr) {
      const int pz = r / nyr;
      z = pz < sa.iz0 - sa.lz ? sa.lz + pz : sa.iz1 + (pz - (sa.iz0 - sa.lz));
      y = sa.ly + r % nyr;
    } else {
      const int t = r - zout * nyr, py = t % yout;
      z = sa.iz0 + t / yout;
      y = py < sa.iy0 - sa.ly ? sa.ly + py : sa.iy1 + (py - (sa.iy0 - sa.ly));
    }
    const double* row = sa.base + (long)sa.gx * y + sa.gxy * z;
    for (int xx = sa.lx + lane; xx < sa.hx; xx += 32) acc4_add(acc, __ldg(row + xx));
  }
  const int xout = (sa.ix0 - sa.lx) + (sa.hx - sa.ix1);
  const long nedge = (long)(sa.iz1 - sa.iz0) * (sa.iy1 - sa.iy0) * xout;
  for (long e = sb * 256L + tid; e < nedge; e += nsb * 256L) {
    const int px = (int)(e % xout);
    const long rr = e / xout;
    const int y = sa.iy0 + (int)(rr % (sa.iy1 - sa.iy0)), z = sa.iz0 + (int)(rr / (sa.iy1 - sa.iy0));
    const int xx = px < sa.ix0 - sa.lx ? sa.lx + px : sa.ix1 + (px - (sa.ix0 - sa.lx));
    acc4_add(acc, __ldg(sa.base + xx + (long)sa.gx * y + sa.gxy * z));
  }
}

// Writes this block's partial; the last block to do so merges all n partials into out4
// ({sum, max, min, norm}) and resets the ticket.  No block waits for another: each fences its
// partial before taking a ticket, and only the holder of the last ticket reads them all.
__device__ __forceinline__ void partial_and_finish(Acc4 acc, Acc4* partials, int idx, int n, unsigned* ticket,
                                                   double* out4, int tid, int nthreads) {
  __shared__ bool last;
  acc = block_reduce4(acc);
  if (tid == 0) {
    partials[idx] = acc;
    __threadfence();
    last = atomicAdd(ticket, 1u) == (unsigned)(n - 1);
  }
  __syncthreads();
  if (!last) return;
  __threadfence();
  Acc4 a = acc4_identity();
  for (int i = tid; i < n; i += nthreads) {
    const Acc4* q = partials + i;  // written by other blocks: read through L2
    Acc4 b;
    b.s = __ldcg(&q->s);
    b.sc = __ldcg(&q->sc);
    b.q = __ldcg(&q->q);
    b.qc = __ldcg(&q->qc);
    b.mx = __ldcg(&q->mx);
    b.mn = __ldcg(&q->mn);
    merge4(a, b);
  }
  a = block_reduce4(a);
  if (tid == 0) {
    out4[0] = a.s + a.sc;
    out4[1] = a.mx == LLONG_MIN ? -INFINITY : from_key(a.mx);
    out4[2] = a.mn == LLONG_MAX ? INFINITY : from_key(a.mn);
    out4[3] = sqrt(a.q + a.qc);
  }
}

constexpr int FNS = 5;   // filter ring stages
constexpr int FTY = 16;  // filter tile y (each thread of the 32 x 8 block owns two y-adjacent cells)

// filt[x,y,z] = (sum over the 27 neighbours of out) / 27 on the interior, and with RED the
// four reductions of the values written (one Acc4 partial per block).
//
// Planes of `out` (the 32 x 16 tile plus a one-cell halo) stream through a ring of FNS
// shared-memory stages with cp.async.  Ring schedule: plane p (-1..nz) lives in stage
// (p+1) % FNS; the prologue issues planes z0-1 .. z0+FNS-3; iteration p waits until plane p has
// landed (at most FNS-2 groups pending), syncs, issues plane p+FNS-1 into the stage of plane p-1
// (consumed in iteration p-1, before the sync), then sums plane p: x-sums of 3 into `rows`
// (two neighbouring sums share their middle pair), a sync, y-sums of 3 for the thread's two
// cells; the 2-D sums of planes p-2, p-1, p give the outputs of plane p-1.
//
// The 9-point (x, y) sums of a plane run on the integer pipe, exactly, in 128-bit fixed point
// (fp64_int.cuh).  A plane whose largest biased exponent is E converts each value to an integer
// in units of 2^(E-1144), rounded to nearest: every value down to 2^-69 of the plane's largest
// keeps its 53 bits, each term is below 2^122 and 9 of them stay below 2^126.  Each cell's plane
// sum is rounded once to a double; an output adds its three plane sums in FP64 and multiplies
// by RN(1/27): four roundings of up to 2^-53 of the partial sums (plus 9 units of 2^-122 of the
// plane's largest |value|), against the reference's 27 roundings.  A plane holding an infinity
// or NaN, only values below 2^-893 (all-zero planes included) or values above 2^1017 sums in
// FP64 instead (the adds of the reference, reassociated; IEEE overflow to infinity).
// Work split: the output planes of all FX x FTY tiles in a flat order (tile-major, z innermost);
// block b of gridDim.x takes the range [b total / gridDim.x, (b+1) total / gridDim.x), one or
// more z runs of consecutive tiles, so every resident block gets the same number of planes.
// With RED every block also reduces a share of filt's ghost shell (shell_part) after its runs,
// leaves its partial, and the last block merges them into out4.
template <bool RED>
__global__ void __launch_bounds__(FX* FY, 4) box_filter_kernel(const double* __restrict__ src, double* __restrict__ dst,
                                                            int sy, long sz, int nx, int ny, int nz, int tiles_x,
                                                            long total, Acc4* __restrict__ partials, ShellArgs sa,
                                                            unsigned* __restrict__ ticket, double* __restrict__ out4) {
  constexpr int PW = FX + 2, PH = FTY + 2, PLANE = PW * PH;
  constexpr int NCOPY = (PLANE + FX * FY - 1) / (FX * FY);
  constexpr int XTASKS = PH * (FX / 2);  // x-sum pairs per plane
  __shared__ __align__(16) double ring[FNS * PLANE];
  __shared__ fixmath::fix128 fplane[PLANE];  // the plane in fixed point (once per value)
  __shared__ fixmath::fix128 rows[PH * FX];  // fixed-point x-sums (or FP64 bits on a special plane)
  __shared__ unsigned plane_exp[2];
  const int tx = threadIdx.x, ty = threadIdx.y, tid = ty * FX + tx;
  const int lane = tid & 31;
  // total < 2^31 (checked by the host)
  const int beg = (int)((long)blockIdx.x * total / gridDim.x), end = (int)((long)(blockIdx.x + 1) * total / gridDim.x);
  Acc4 acc = acc4_identity();
#pragma unroll 1
  for (int run = beg; run < end;) {
    const int tile = run / nz;
    const int x0 = (tile % tiles_x) * FX, y0 = (tile / tiles_x) * FTY;
    const int x = x0 + tx, ya = y0 + 2 * ty;
    const int z0 = run - tile * nz, z1 = min(nz, z0 + (end - run));
    run += z1 - z0;
    int goff[NCOPY];  // within a plane (fewer than 2^31 cells)
    uint32_t soff[NCOPY];
#pragma unroll
    for (int j = 0; j < NCOPY; ++j) {
      const int k = min(tid + j * FX * FY, PLANE - 1);
      const int r = k / PW, c = k - r * PW;
      goff[j] = min(x0 - 1 + c, nx) + sy * min(y0 - 1 + r, ny);
      soff[j] = (uint32_t)(k * sizeof(double));
    }
    const uint32_t ring0 = (uint32_t)__cvta_generic_to_shared(ring);
    auto issue = [&](int p) {
      if (p > z1) return;
      const uint32_t st = ring0 + (uint32_t)((p + 1) % FNS) * (PLANE * sizeof(double));
      const double* sp = src + sz * p;
#pragma unroll
      for (int j = 0; j < NCOPY; ++j) {
        if (j == NCOPY - 1 && tid + j * FX * FY >= PLANE) break;
        cp_async8(st + soff[j], sp + goff[j]);
      }
    };
    if (tid < 2) plane_exp[tid] = 0u;
#pragma unroll 1
    for (int i = 0; i < FNS - 1; ++i) {
      issue(z0 - 1 + i);
      cp_async_commit();
    }
    const bool act0 = x < nx && ya < ny, act1 = x < nx && ya + 1 < ny;
    // 9-point (x, y) sums of planes p-2 (p*) and p-1 (c*) for both cells
    double p0 = 0.0, c0 = 0.0, p1 = 0.0, c1 = 0.0;
    double* out = dst + (long)x + (long)sy * ya + sz * (z0 - 1);
#pragma unroll 1
    for (int p = z0 - 1; p <= z1; ++p, out += sz) {
      cp_async_wait<FNS - 2>();
      __syncthreads();
      issue(p + FNS - 1);
      cp_async_commit();
      const double* pl = ring + ((p + 1) % FNS) * PLANE;
      // the plane's largest biased exponent; this thread's values stay in registers
      constexpr int PER = (PLANE + FX * FY - 1) / (FX * FY);
      double val[PER];
      unsigned e = 0;
#pragma unroll
      for (int j = 0; j < PER; ++j) {
        const int t = tid + j * FX * FY;
        val[j] = t < PLANE ? pl[t] : 0.0;
        e = max(e, ((unsigned)__double2hiint(val[j]) >> 20) & 0x7ffu);
      }
      e = __reduce_max_sync(0xffffffffu, e);
      if (lane == 0) atomicMax(&plane_exp[p & 1], e);
      __syncthreads();
      const int E = (int)plane_exp[p & 1];
      if (tid == 0) plane_exp[(p + 1) & 1] = 0u;  // the slot of plane p+1 (last read in iteration p-1)
      const bool special = E == 0x7ff || E < 130 || E > 2040;
      const int u = E - 1144;
      if (!special) {
#pragma unroll
        for (int j = 0; j < PER; ++j) {
          const int t = tid + j * FX * FY;
          if (t < PLANE) fplane[t] = fixmath::to_units(val[j], E);
        }
        __syncthreads();
      }
      for (int t = tid; t < XTASKS; t += FX * FY) {
        const int r = t / (FX / 2), c = 2 * (t % (FX / 2));
        if (!special) {
          const fixmath::fix128* f = fplane + r * PW + c;
          const fixmath::fix128 mid = f[1] + f[2];
          rows[r * FX + c] = f[0] + mid;
          rows[r * FX + c + 1] = mid + f[3];
        } else {
          const double* q = pl + r * PW + c;
          const double mid = q[1] + q[2];
          rows[r * FX + c] = __double_as_longlong(q[0] + mid);
          rows[r * FX + c + 1] = __double_as_longlong(mid + q[3]);
        }
      }
      __syncthreads();
      const fixmath::fix128* col = rows + 2 * ty * FX + tx;
      double s0, s1;
      if (!special) {
        const fixmath::fix128 mid = col[FX] + col[2 * FX];
        s0 = fixmath::units_to_double0(col[0] + mid, u);
        s1 = fixmath::units_to_double0(mid + col[3 * FX], u);
      } else {
        auto d = [](fixmath::fix128 f) { return __longlong_as_double((long long)f); };
        const double mid = __dadd_rn(d(col[FX]), d(col[2 * FX]));
        s0 = __dadd_rn(d(col[0]), mid);
        s1 = __dadd_rn(mid, d(col[3 * FX]));
      }
      if (p >= z0 + 1) {
        constexpr double C27 = 1.0 / 27.0;
        if (act0) {
          const double v = __dmul_rn(__dadd_rn(__dadd_rn(p0, c0), s0), C27);
          out[-sz] = v;  // plane p-1
          if (RED) acc4_add(acc, v);
        }
        if (act1) {
          const double v = __dmul_rn(__dadd_rn(__dadd_rn(p1, c1), s1), C27);
          out[sy - sz] = v;
          if (RED) acc4_add(acc, v);
        }
      }
      p0 = c0;
      c0 = s0;
      p1 = c1;
      c1 = s1;
    }
    cp_async_wait<0>();
    __syncthreads();  // the ring and plane_exp are free for the next run
  }
  if (RED) {
    if (sa.on) shell_part(acc, sa, blockIdx.x, gridDim.x, tid);
    partial_and_finish(acc, partials, blockIdx.x, gridDim.x, ticket, out4, tid, FX * FY);
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

namespace nebo {
void reduction_region(const nebo_field& f, int interior, int lo[3], int hi[3]);
namespace {

int filter_impl(const nebo_field* out, const nebo_field* filt, bool reduce, int interior, double* d_out4,
                cudaStream_t s, const char* what);

int deep_impl(const nebo_field* a, const nebo_field* b, const nebo_field* c, const uint32_t* mask_words,
              const nebo_field* out, const nebo_field* filt, double dx, bool reduce, int interior, double* d_out4,
              cudaStream_t s, const char* what) {
  int rc = check_deep(a, b, c, out, filt);
  if (rc) return rc;
  if (!mask_words) return fail(NEBO_ERR_INVALID, "Nebo error in %s: null mask", what);
  if (reduce && !d_out4) return fail(NEBO_ERR_INVALID, "Nebo error in %s: null result pointer", what);
  int n[3];
  interior_extent(*a, n);
  const View<const double> va = make_view<const double>(*a), vb = make_view<const double>(*b),
                           vc = make_view<const double>(*c);
  const View<double> vo = make_view<double>(*out);
  // flat window index of interior (0,0,0): used to locate mask bits
  const long mask_base = (long)(out->offset[0] + 1) + (long)out->glob[0] * (out->offset[1] + 1) +
                         (long)out->glob[0] * out->glob[1] * (out->offset[2] + 1);
  const double q = 0.25 * (1.0 / dx);
  if (n[0] > 1) {
    // z split: the whole number of resident-block waves (at most 8) with the smallest idle tail
    static std::atomic<int> per_sm_cache{0};
    const int per_sm = blocks_per_sm(deep_out_kernel, 256, per_sm_cache);
    dim3 block(32, 8);
    dim3 grid((n[0] - 1 + 31) / 32, (n[1] + 2 + 7) / 8, 1);
    const long planes_blocks = (long)grid.x * grid.y, slots = (long)num_sms() * per_sm;
    int zsplit = 1;
    double best = -1.0;
    for (int zs = 1; zs <= n[2] + 2 && planes_blocks * zs <= 8 * slots; ++zs) {
      const double waves = (double)(planes_blocks * zs) / slots;
      const double fill = waves / std::ceil(waves);  // fraction of the slot-waves that hold a block
      if (fill > best + 1e-3) {
        best = fill;
        zsplit = zs;
      }
    }
    grid.z = zsplit;
    LaunchScope ls("deep_chain", s);
    deep_out_kernel<<<grid, block, 0, s>>>(va.base, vb.base, vc.base, mask_words, mask_base, vo.base, vo.sy, vo.sz,
                                           n[0], n[1], n[2], q);
    NEBO_LAUNCH_CHECK(what);
  }
  return filter_impl(out, filt, reduce, interior, d_out4, s, what);
}

// filt <<= BoxFilter(out) on the interior, optionally with sum/max/min/norm of filt.
int filter_impl(const nebo_field* out, const nebo_field* filt, bool reduce, int interior, double* d_out4,
                cudaStream_t s, const char* what) {
  int n[3];
  interior_extent(*out, n);
  const View<double> vo = make_view<double>(*out), vf = make_view<double>(*filt);
  // filter: resident blocks per SM
  static std::atomic<int> per_sm_cache[2];  // zero: not queried
  const int per_sm = reduce ? blocks_per_sm(box_filter_kernel<true>, FX * FY, per_sm_cache[1])
                            : blocks_per_sm(box_filter_kernel<false>, FX * FY, per_sm_cache[0]);
  // one wave of resident blocks, each at least 8 planes of a tile
  const int tiles_x = (n[0] + FX - 1) / FX, tiles_y = (n[1] + FTY - 1) / FTY;
  const long total = (long)tiles_x * tiles_y * n[2];
  if (total >= (1L << 31)) return fail(NEBO_ERR_UNSUPPORTED, "Nebo error in %s: more than 2^31 filter tile planes", what);
  const int blocks = (int)std::max(1L, std::min((long)num_sms() * per_sm, (total + 7) / 8));
  if (!reduce) {
    LaunchScope ls("box_filter", s);
    box_filter_kernel<false><<<blocks, dim3(FX, FY), 0, s>>>(vo.base, vf.base, vo.sy, vo.sz, n[0], n[1], n[2], tiles_x,
                                                            total, nullptr, ShellArgs{}, nullptr, nullptr);
    NEBO_LAUNCH_CHECK(what);
    return NEBO_OK;
  }
  // reduction region (valid ghosts included unless interior) and the filter's written box
  int lo[3], hi[3], ilo[3], ihi[3];
  reduction_region(*filt, interior, lo, hi);
  for (int i = 0; i < 3; ++i) {
    ilo[i] = filt->offset[i] + filt->ghost_minus[i];
    ihi[i] = ilo[i] + n[i];
  }
  const bool shell = lo[0] != ilo[0] || hi[0] != ihi[0] || lo[1] != ilo[1] || hi[1] != ihi[1] || lo[2] != ilo[2] ||
                     hi[2] != ihi[2];
  const ShellArgs sa{shell ? 1 : 0, (const double*)filt->data, filt->glob[0], (long)filt->glob[0] * filt->glob[1],
                     lo[0], hi[0], lo[1], hi[1], lo[2], hi[2], ilo[0], ihi[0], ilo[1], ihi[1], ilo[2], ihi[2]};
  const long nblocks = blocks;
  // one allocation: the partials, then the ticket
  const size_t pbytes = sizeof(Acc4) * nblocks;
  char* scratch = nullptr;
  pool_retain();
  NEBO_CUDA_TRY(cudaMallocAsync((void**)&scratch, pbytes + 16, s));
  Acc4* partials = (Acc4*)scratch;
  unsigned* ticket = (unsigned*)(scratch + pbytes);
  cudaError_t le = cudaMemsetAsync(ticket, 0, sizeof(unsigned), s);
  if (le == cudaSuccess) {
    LaunchScope ls("box_filter_reduce", s);
    box_filter_kernel<true><<<blocks, dim3(FX, FY), 0, s>>>(vo.base, vf.base, vo.sy, vo.sz, n[0], n[1], n[2], tiles_x,
                                                           total, partials, sa, ticket, d_out4);
    le = cudaGetLastError();
  }
  cudaFreeAsync(scratch, s);
  if (le != cudaSuccess) return cuda_fail(le, what);
  return NEBO_OK;
}

}  // namespace
}  // namespace nebo

extern "C" int nebo_box_filter(const nebo_field* src, const nebo_field* dst, int interior, double* d_out4,
                               nebo_stream_t stream) {
  const char* w = "nebo_box_filter";
  int rc;
  const nebo_field* fs[2] = {src, dst};
  for (int i = 0; i < 2; ++i) {
    if ((rc = check_field(fs[i], w))) return rc;
    if (fs[i]->dtype != NEBO_F64) return fail(NEBO_ERR_UNSUPPORTED, "Nebo error in %s: FP64 fields only", w);
    if ((rc = check_periodic_patch(fs[i], 1, w))) return rc;
  }
  if ((rc = check_same_layout(src, dst, w))) return rc;
  if (src->data == dst->data) return fail(NEBO_ERR_INVALID, "Nebo error in %s: output aliases input", w);
  return filter_impl(src, dst, d_out4 != nullptr, interior, d_out4, (cudaStream_t)stream, w);
}

extern "C" int nebo_deep_chain(const nebo_field* a, const nebo_field* b, const nebo_field* c,
                               const uint32_t* mask_words, const nebo_field* out, const nebo_field* filt, double dx,
                               nebo_stream_t stream) {
  return deep_impl(a, b, c, mask_words, out, filt, dx, false, 0, nullptr, (cudaStream_t)stream, "nebo_deep_chain");
}

extern "C" int nebo_deep_chain_reduce(const nebo_field* a, const nebo_field* b, const nebo_field* c,
                                      const uint32_t* mask_words, const nebo_field* out, const nebo_field* filt,
                                      double dx, int interior, double* d_out4, nebo_stream_t stream) {
  return deep_impl(a, b, c, mask_words, out, filt, dx, true, interior, d_out4, (cudaStream_t)stream,
                   "nebo_deep_chain_reduce");
}

// Element-wise FP64 exp / sin of the integer-pipe functions (fn 0: exp, 1: sin).
namespace nebo {
namespace {
__global__ void fastmath_kernel(int fn, const double* __restrict__ x, double* __restrict__ y, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    if (fn == 0) {
      y[i] = fixmath::exp_i(x[i]);
    } else if (fn == 1) {
      y[i] = fixmath::sin_i(x[i]);
    } else {
      const double a = x[2 * i], b = x[2 * i + 1];
      y[i] = fn == 2 ? fixmath::div_by(a, b, __drcp_rn(b), fixmath::divisor_ok(b)) : __ddiv_rn(a, b);
    }
  }
}
}  // namespace
}  // namespace nebo

extern "C" int nebo_fastmath_eval(int fn, const double* x, double* y, size_t n, nebo_stream_t stream) {
  if (fn < 0 || fn > 3 || (n && (!x || !y))) return fail(NEBO_ERR_INVALID, "Nebo error in nebo_fastmath_eval");
  if (!n) return NEBO_OK;
  cudaStream_t s = (cudaStream_t)stream;
  LaunchScope ls("fastmath_eval", s);
  fastmath_kernel<<<num_sms() * 8, 256, 0, s>>>(fn, x, y, n);
  NEBO_LAUNCH_CHECK("nebo_fastmath_eval");
  return NEBO_OK;
}
