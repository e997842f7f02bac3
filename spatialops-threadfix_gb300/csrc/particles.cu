// Particle <-> cell operators (the kernels behind Particle::CellToParticle::apply_to_field,
// spatialops/particles/ParticleOperators.h:313-398, and ParticleToCell::apply_to_field, :186-273).
//
// A particle p is a cube of edge size[p] centred at (px, py, pz)[p].  A null coordinate array
// switches an axis off: the particle then covers one cell along it with weight 1.  For each cell
// (i, j, k) of the cell field's window the particle overlaps, its weight is
//     w = ((xcont * ycont) * zcont) / pvol,   xcont = min(xcp, pxhi) - max(xcm, pxlo), ...
// with every operation of the reference evaluated in the reference's order and rounded once (no
// contraction), so that both directions reproduce the reference's bits:
//     cell -> particle  dest[p] = ((+0 + src(c1) * w1) + src(c2) * w2) + ...  box in (k, j, i) order
//     particle -> cell  dest(c) = ((+0 + v[p1] * w) + v[p2] * w) + ...        particles in index order
//
// The scatter keeps the reference's order without a serial loop:
//   1. count  every particle adds 1 to the counter of each cell of its box (and its box size to a
//             64-bit total), and is filed under the 4 x 4 x 4 block of cells its box starts in;
//   2. scan   an exclusive prefix sum of the counters gives each cell a slice of one entry list;
//             a prefix sum of the per-block counts and one scatter give the particles in block
//             order;
//   3. fill   every (particle, cell) pair writes a 16-byte entry (particle index, v * w) into a
//             free slot of its cell's slice, the particles taken in block order so that a warp's
//             stores land in nearby slices (random particle order scatters them over the list:
//             8.2 ms against 4.2 for 16.8 M particles on 256^3);
//   4. fold   each window cell sorts its slice by particle index (an insertion sort: slots are
//             taken in nearly increasing index order) and sums it from +0 in that order; a cell
//             with no entry gets +0 (the reference's `dest <<= 0` before it adds).
// CellToParticle and the fill spread a warp's (particle, cell) pairs evenly over its lanes, so
// box sizes that differ between particles cost no divergence.  The floating-point work stays
// on the FP64 pipe where the reference's bits require it (products, the weights' quotients,
// the sums); box indices, min/max and range checks run on the integer pipe.
//
// Boxes that leave the window: the reference clips the high end of a box to the window and
// leaves the low end to a double -> size_t conversion that is undefined below -1 cells; here
// both ends are clipped, so a particle partly outside adds to the window cells it overlaps.
#include "common.cuh"
#include "fp64_int.cuh"

namespace nebo {
namespace {

struct PGeom {
  double d[3];     // mesh spacing dx_, dy_, dz_
  double face[3];  // low face of window cell 0: xlo_ - dx_*ngm - dx_/2 (ParticleOperators.h:197-199)
  double inv[3];   // RN(1/d)
  int nmax[3];     // window extent (ghosts included)
  int glob[3];     // allocation
  int off[3];      // window offset in the allocation
  int on[3];       // axis has coordinates
};

// trunc(q), saturated to +-2^31, from q's bits (integer pipe).  near: q lies within 2^-29 |q|
// (at least 2^-30) of an integer, or |q| >= 2^30.  nan: q is a NaN.
__device__ __forceinline__ long long trunc_near(double q, bool& near, bool& nan) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(q);
  const int e = (int)((b >> 52) & 0x7ff);
  const unsigned long long frac = b & 0xFFFFFFFFFFFFFull;
  const bool neg = (b >> 63) != 0;
  nan = e == 0x7ff && frac != 0;
  if (e < 1023) {  // |q| < 1: within 2^-30 of 0, or of +-1
    near = e < 1023 - 30 || (e == 1022 && frac >= (1ull << 52) - (1ull << 23));
    return 0;
  }
  if (e >= 1023 + 31) {
    near = false;
    return neg ? -(1ll << 31) : (1ll << 31);
  }
  const int shift = 52 - (e - 1023);  // fraction bits: 22 .. 52
  const unsigned long long m = frac | (1ull << 52);
  const unsigned long long f = m & ((1ull << shift) - 1);
  near = f <= (1ull << 23) || f + (1ull << 23) >= (1ull << shift);
  const long long t = (long long)(m >> shift);
  return neg ? -t : t;
}

// trunc(RN(x / d)) (saturated to +-2^31) and whether RN(x / d) is a NaN.  The product with
// RN(1/d) is within two ulps of RN(x / d); unless it lies near an integer both have the same
// integer part, otherwise the quotient is computed by division.
__device__ __forceinline__ long long index_quot(double x, const PGeom& g, int a, bool& nan) {
  bool near;
  long long t = trunc_near(__dmul_rn(x, g.inv[a]), near, nan);
  if (near) t = trunc_near(__ddiv_rn(x, g.d[a]), near, nan);
  return t;
}

struct Axis {
  int lo, hi;       // window cells [lo, hi) along this axis
  double plo, phi;  // particle's low and high coordinate
};

// std::min / std::max of two finite doubles: (b < a) ? b : a and (a < b) ? b : a, compared as
// order-preserving integer keys (integer pipe).  Unlike IEEE comparison the keys order -0
// below +0; an overlap can then come out as -0 instead of +0, which changes no sum that starts
// from +0 (every sum here does).
__device__ __forceinline__ long long okey(double v) {
  const long long b = __double_as_longlong(v);
  return b ^ ((b >> 63) & 0x7fffffffffffffffll);
}
__device__ __forceinline__ double dmin(double a, double b) { return okey(b) < okey(a) ? b : a; }
__device__ __forceinline__ double dmax(double a, double b) { return okey(a) < okey(b) ? b : a; }

// The cells [lo, hi) of the window the particle covers along one axis (ParticleOperators.h:
// 214-234 / 337-357, both ends clipped to the window).
__device__ __forceinline__ void make_axis(Axis& ax, double pos, double size, const PGeom& g, int a) {
  const double rp = __dmul_rn(size, 0.5);
  const bool on = g.on[a];
  ax.plo = on ? __dsub_rn(pos, rp) : 0.0;
  ax.phi = on ? __dadd_rn(ax.plo, size) : 0.0;
  const long long n = g.nmax[a];
  bool nan;
  const long long tl = index_quot(__dsub_rn(ax.plo, g.face[a]), g, a, nan);
  // lo: the truncated quotient; (-1, 0) gives 0 as in the reference, lower values are clipped;
  // past the window's high end (or NaN) the box is empty
  long long lo = nan || tl >= n ? n : (tl > 0 ? tl : 0);
  long long hi;
  if (on) {
    const long long th = index_quot(__dsub_rn(ax.phi, g.face[a]), g, a, nan);
    // int() + 1 clipped to the window (ParticleOperators.h:232-234); below -1 (or NaN): empty
    hi = nan || th < 0 ? 0 : (th + 1 < n ? th + 1 : n);
  } else if (g.glob[a] == 1) {
    lo = 0;  // the reference's one cell along an off axis; an allocation extent of 1 maps every
    hi = 1;  // index to 0 (MemoryWindow::flat_index)
  } else {
    hi = lo + 1 < n ? lo + 1 : n;
  }
  ax.lo = (int)lo;
  ax.hi = (int)hi;
}

// Overlap of the particle with window cell i along one axis (1 when the axis is off).
__device__ __forceinline__ double axis_cont(const Axis& ax, const PGeom& g, int a, int i) {
  if (!g.on[a]) return 1.0;
  const double cm = __dadd_rn(g.face[a], __dmul_rn(fixmath::i32_to_f64(i), g.d[a]));
  const double cp = __dadd_rn(cm, g.d[a]);
  return __dsub_rn(dmin(cp, ax.phi), dmax(cm, ax.plo));
}

// One (particle, value) entry of a cell's slice: 16 bytes, written with one store.
struct __align__(16) Entry {
  double val;
  long long pid;
};

__device__ __forceinline__ void put_entry(Entry* e, long long pid, double val) {
  Entry t;
  t.val = val;
  t.pid = pid;
  *e = t;
}

struct Box {
  Axis a[3];
  double pvol;
  __device__ __forceinline__ int count(int k) const { return a[k].hi > a[k].lo ? a[k].hi - a[k].lo : 0; }
};

__device__ __forceinline__ void make_box(Box& b, const PGeom& g, const double* __restrict__ px,
                                         const double* __restrict__ py, const double* __restrict__ pz,
                                         const double* __restrict__ psize, long p) {
  const double size = psize[p];
  make_axis(b.a[0], g.on[0] ? px[p] : 0.0, size, g, 0);
  make_axis(b.a[1], g.on[1] ? py[p] : 0.0, size, g, 1);
  make_axis(b.a[2], g.on[2] ? pz[p] : 0.0, size, g, 2);
  const double two_rp = __dmul_rn(2.0, __dmul_rn(size, 0.5));
  b.pvol = __dmul_rn(__dmul_rn(g.on[0] ? two_rp : 1.0, g.on[1] ? two_rp : 1.0), g.on[2] ? two_rp : 1.0);
}

using fixmath::div_by;
using fixmath::divisor_ok;

// Window cell (i, j, k) -> element of the allocation (MemoryWindow::flat_index: an axis of
// allocation extent 1 is always index 0).
__device__ __forceinline__ long glob_flat(const PGeom& g, int i, int j, int k) {
  const long x = g.glob[0] > 1 ? i + g.off[0] : 0;
  const long y = g.glob[1] > 1 ? j + g.off[1] : 0;
  const long z = g.glob[2] > 1 ? k + g.off[2] : 0;
  return x + (long)g.glob[0] * (y + (long)g.glob[1] * z);
}
__device__ __forceinline__ long win_flat(const PGeom& g, int i, int j, int k) {
  return (long)i + (long)g.nmax[0] * ((long)j + (long)g.nmax[1] * k);
}

// ---- warp-cooperative particle kernels
//
// A warp takes 32 consecutive particles.  Each lane builds its particle's box and the overlaps
// along each axis (at most PB cells per axis; larger boxes go to the lane's own serial loop).
// The warp then spreads the (particle, cell) pairs, particle-major and (k, j, i) within a
// particle, over its lanes 32 at a time, so every lane does the same work per pair whatever the
// box sizes.  For CellToParticle the owner lane then adds its pairs' products in that order.
constexpr int PB = 4;
constexpr int PWARPS = 8;  // warps per block
constexpr int PCAP = 512;  // CellToParticle: products held per warp before the owners add them
enum { PM_C2P = 0, PM_FILL = 2 };

template <int MODE>
struct WarpShared {
  double cont[3][PB][32];  // overlap of lane's particle with its box's t-th cell along each axis
  double pvol[32], rcp[32];
  double val[32];          // FILL: the particles' values
  long long pid[32];       // FILL: the particles' indices (the entries' keys)
  double prod[MODE == PM_C2P ? PCAP : 1];  // C2P: products of pairs [S, S + PCAP) of the warp's list
  int lo[3][32];
  int n[3][32];
  unsigned mxy[32], mx[32];  // 2^16 / (nx ny) + 1 and 2^16 / nx + 1: division of small pair indices
  int start[33];           // exclusive prefix of the pair counts
};

// One particle by its own lane, in the reference's loop order (boxes wider than PB cells).
template <int MODE>
__device__ __noinline__ double serial_particle(const PGeom& g, const double* __restrict__ px,
                                               const double* __restrict__ py, const double* __restrict__ pz,
                                               const double* __restrict__ psize, long p,
                                               const double* __restrict__ cell, const double* __restrict__ src,
                                               const int* __restrict__ off, int* __restrict__ cnt,
                                               Entry* __restrict__ ent) {
  Box b;
  make_box(b, g, px, py, pz, psize, p);
  const bool fast = divisor_ok(b.pvol);
  const double y = __drcp_rn(b.pvol);
  double acc = 0.0;
  for (int k = b.a[2].lo; k < b.a[2].hi; ++k) {
    const double zc = axis_cont(b.a[2], g, 2, k);
    for (int j = b.a[1].lo; j < b.a[1].hi; ++j) {
      const double yc = axis_cont(b.a[1], g, 1, j);
      for (int i = b.a[0].lo; i < b.a[0].hi; ++i) {
        const double xc = axis_cont(b.a[0], g, 0, i);
        const double w = div_by(__dmul_rn(__dmul_rn(xc, yc), zc), b.pvol, y, fast);
        if (MODE == PM_C2P) {
          acc = __dadd_rn(acc, __dmul_rn(cell[glob_flat(g, i, j, k)], w));
        } else {
          const long cc = win_flat(g, i, j, k);
          const int slot = off[cc + 1] - atomicSub(cnt + cc, 1);
          put_entry(ent + slot, p, __dmul_rn(src[p], w));
        }
      }
    }
  }
  return acc;
}

template <int MODE>
__global__ void __launch_bounds__(PWARPS * 32, 2) particles_kernel(
    PGeom g, const double* __restrict__ px, const double* __restrict__ py, const double* __restrict__ pz,
    const double* __restrict__ psize, long np, const double* __restrict__ cell, double* __restrict__ dest,
    const double* __restrict__ src, const int* __restrict__ off, int* __restrict__ cnt, Entry* __restrict__ ent,
    const int* __restrict__ order) {
  extern __shared__ __align__(16) unsigned char particle_smem[];
  WarpShared<MODE>* smem = reinterpret_cast<WarpShared<MODE>*>(particle_smem);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  WarpShared<MODE>& sm = smem[warp];
  for (long base = ((long)blockIdx.x * PWARPS + warp) * 32; base < np; base += (long)gridDim.x * PWARPS * 32) {
    // FILL with an order: the warp's particles in that order (particles of nearby cells together,
    // so the entries' stores land near each other); the entries keep the particles' indices
    const long p = (MODE == PM_FILL && order && base + lane < np) ? (long)order[base + lane] : base + lane;
    int npairs = 0;
    bool big = false;
    if (base + lane < np) {
      Box b;
      make_box(b, g, px, py, pz, psize, p);
      const int n0 = b.count(0), n1 = b.count(1), n2 = b.count(2);
      const long cells = (long)n0 * n1 * n2;
      big = cells > 0 && (n0 > PB || n1 > PB || n2 > PB);
      if (cells > 0 && !big) {
        npairs = (int)cells;
        sm.n[0][lane] = n0;
        sm.n[1][lane] = n1;
        sm.lo[0][lane] = b.a[0].lo;
        sm.lo[1][lane] = b.a[1].lo;
        sm.lo[2][lane] = b.a[2].lo;
        sm.mxy[lane] = 65536u / (unsigned)(n0 * n1) + 1u;
        sm.mx[lane] = 65536u / (unsigned)n0 + 1u;
        sm.pvol[lane] = b.pvol;
        sm.rcp[lane] = __drcp_rn(b.pvol);
        for (int t = 0; t < n0; ++t) sm.cont[0][t][lane] = axis_cont(b.a[0], g, 0, b.a[0].lo + t);
        for (int t = 0; t < n1; ++t) sm.cont[1][t][lane] = axis_cont(b.a[1], g, 1, b.a[1].lo + t);
        for (int t = 0; t < n2; ++t) sm.cont[2][t][lane] = axis_cont(b.a[2], g, 2, b.a[2].lo + t);
        if (MODE == PM_FILL) {
          sm.val[lane] = src[p];
          sm.pid[lane] = p;
        }
      }
    }
    // exclusive prefix of the pair counts
    int incl = npairs;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += v;
    }
    sm.start[lane] = incl - npairs;
    if (lane == 31) sm.start[32] = incl;
    __syncwarp();
    const int total_pairs = sm.start[32];
    const int my0 = sm.start[lane], my1 = sm.start[lane + 1];
    double acc = 0.0;
    for (int c0 = 0; c0 < total_pairs; c0 += 32) {
      const int t = c0 + lane;
      const int S = c0 & ~(PCAP - 1);  // first pair of the current product batch
      if (t < total_pairs) {
        int o = 0;
#pragma unroll
        for (int s = 16; s > 0; s >>= 1)
          if (sm.start[o + s] <= t) o += s;
        const unsigned local = (unsigned)(t - sm.start[o]);
        const unsigned nx = (unsigned)sm.n[0][o], nxy = nx * (unsigned)sm.n[1][o];
        const unsigned k = (local * sm.mxy[o]) >> 16;
        const unsigned r = local - k * nxy;
        const unsigned j = (r * sm.mx[o]) >> 16;
        const unsigned i = r - j * nx;
        const int ci = sm.lo[0][o] + (int)i, cj = sm.lo[1][o] + (int)j, ck = sm.lo[2][o] + (int)k;
        const double pv = sm.pvol[o];
        const double w = div_by(__dmul_rn(__dmul_rn(sm.cont[0][i][o], sm.cont[1][j][o]), sm.cont[2][k][o]), pv,
                                sm.rcp[o], divisor_ok(pv));
        if (MODE == PM_C2P) {
          sm.prod[t - S] = __dmul_rn(cell[glob_flat(g, ci, cj, ck)], w);
        } else {
          const long cc = win_flat(g, ci, cj, ck);
          const int slot = off[cc + 1] - atomicSub(cnt + cc, 1);
          put_entry(ent + slot, sm.pid[o], __dmul_rn(sm.val[o], w));
        }
      }
      if (MODE == PM_C2P && (c0 + 32 == S + PCAP || c0 + 32 >= total_pairs)) {
        // the batch is complete: each owner adds its products of the batch in pair order (the
        // loads of four products go out together; the additions stay in order)
        __syncwarp();
        const int s1 = min(my1, S + PCAP);
        int s = max(my0, S);
        for (; s + 4 <= s1; s += 4) {
          const double v0 = sm.prod[s - S], v1 = sm.prod[s + 1 - S], v2 = sm.prod[s + 2 - S], v3 = sm.prod[s + 3 - S];
          acc = __dadd_rn(__dadd_rn(__dadd_rn(__dadd_rn(acc, v0), v1), v2), v3);
        }
        for (; s < s1; ++s) acc = __dadd_rn(acc, sm.prod[s - S]);
        __syncwarp();
      }
    }
    if (big) acc = serial_particle<MODE>(g, px, py, pz, psize, p, cell, src, off, cnt, ent);
    if (MODE == PM_C2P && base + lane < np) dest[p] = acc;
    __syncwarp();
  }
}

// Counting pass of ParticleToCell: one lane per particle adds 1 to each cell of its box.  The
// pairs need no floating-point work here, so the lane's own loop beats spreading them.  It also
// files each particle under the 4 x 4 x 4 block of cells that holds its box's first cell (key;
// nkey for an empty box) and counts the particles per key (hist), from which the fill's order is
// built.
__global__ void __launch_bounds__(256) p2c_count_kernel(PGeom g, const double* __restrict__ px,
                                                        const double* __restrict__ py, const double* __restrict__ pz,
                                                        const double* __restrict__ psize, long np,
                                                        int* __restrict__ cnt, unsigned long long* __restrict__ total,
                                                        int* __restrict__ key, int* __restrict__ hist, int kbx,
                                                        int kby, int nkey) {
  unsigned long long mine = 0;
  for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < np; p += (long)gridDim.x * blockDim.x) {
    Box b;
    make_box(b, g, px, py, pz, psize, p);
    const int n0 = b.count(0), n1 = b.count(1), n2 = b.count(2);
    mine += (unsigned long long)((long)n0 * n1 * n2);
    const int k = (n0 && n1 && n2) ? (b.a[0].lo >> 2) + kbx * ((b.a[1].lo >> 2) + kby * (b.a[2].lo >> 2)) : nkey;
    key[p] = k;
    atomicAdd(hist + k, 1);
    if (!n0 || !n1 || !n2) continue;
    for (int k = b.a[2].lo; k < b.a[2].hi; ++k)
      for (int j = b.a[1].lo; j < b.a[1].hi; ++j)
        for (int i = b.a[0].lo; i < b.a[0].hi; ++i) atomicAdd(cnt + win_flat(g, i, j, k), 1);
  }
  for (int o = 16; o > 0; o >>= 1) mine += __shfl_xor_sync(0xffffffffu, mine, o);
  if ((threadIdx.x & 31) == 0 && mine) atomicAdd(total, mine);
}

// The fill's order: the particles grouped by key (pos: the keys' exclusive prefix, advanced as
// the slots are taken; the order within a key does not matter, the fold sorts by index).
__global__ void __launch_bounds__(256) p2c_order_kernel(const int* __restrict__ key, long np, int* __restrict__ pos,
                                                        int* __restrict__ order) {
  for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < np; p += (long)gridDim.x * blockDim.x)
    order[atomicAdd(pos + key[p], 1)] = (int)p;
}

// Fold of ParticleToCell: a warp takes 32 consecutive window cells, whose slices form one
// contiguous run of the entry list.  It stages the run in shared memory with coalesced loads,
// in groups of consecutive lanes whose slices fit in FCAP entries, and each lane of a group
// sorts its cell's slice by particle index (an insertion sort: the slots were taken in nearly
// increasing order) and adds it from +0 in that order.  A single slice longer than FCAP is
// sorted and added where it lies, in global memory.
constexpr int FCAP = 512;
constexpr int FWARPS = 4;

__device__ __forceinline__ void fold_slice(Entry* e, int n, double& acc) {
  for (int s = 1; s < n; ++s) {
    const Entry key = e[s];
    int t = s - 1;
    while (t >= 0 && e[t].pid > key.pid) {
      e[t + 1] = e[t];
      --t;
    }
    e[t + 1] = key;
  }
  for (int s = 0; s < n; ++s) acc = __dadd_rn(acc, e[s].val);
}

__global__ void __launch_bounds__(FWARPS * 32) p2c_fold_kernel(PGeom g, long ncell, const int* __restrict__ off,
                                                               Entry* __restrict__ ent, double* __restrict__ dest) {
  __shared__ Entry stage[FWARPS][FCAP];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long nxy = (long)g.nmax[0] * g.nmax[1];
  for (long c0 = ((long)blockIdx.x * FWARPS + warp) * 32; c0 < ncell; c0 += (long)gridDim.x * FWARPS * 32) {
    const long c = c0 + lane;
    const bool live = c < ncell;
    const int r_end = off[c0 + 32 < ncell ? c0 + 32 : ncell];
    const int b = live ? off[c] : r_end, e = live ? off[c + 1] : r_end;
    double acc = 0.0;
    int first = 0;  // first lane of the current group (warp-uniform)
    while (first < 32) {
      const int r0 = __shfl_sync(0xffffffffu, b, first);
      // lanes first.. whose slices end within FCAP entries of r0 (a prefix: e grows with the lane)
      const unsigned fits = __ballot_sync(0xffffffffu, lane >= first && e - r0 <= FCAP);
      const int last = fits ? 31 - __clz(fits) : first;  // last lane of the group
      const bool mine = lane >= first && lane <= last;
      if (!fits) {
        if (lane == first) fold_slice(ent + b, e - b, acc);  // one slice longer than FCAP
      } else {
        const int r1 = __shfl_sync(0xffffffffu, e, last);
        for (int t = r0 + lane; t < r1; t += 128) {
          Entry v[4];
#pragma unroll
          for (int u = 0; u < 4; ++u)
            if (t + 32 * u < r1) v[u] = ent[t + 32 * u];
#pragma unroll
          for (int u = 0; u < 4; ++u)
            if (t + 32 * u < r1) stage[warp][t + 32 * u - r0] = v[u];
        }
        __syncwarp();
        if (mine) fold_slice(&stage[warp][b - r0], e - b, acc);
        __syncwarp();
      }
      first = last + 1;
    }
    if (live) {
      int i, j, k;
      if (ncell < (1L << 31)) {
        const unsigned cu = (unsigned)c, nx = (unsigned)g.nmax[0], nxyu = (unsigned)nxy;
        k = (int)(cu / nxyu);
        const unsigned r = cu - (unsigned)k * nxyu;
        j = (int)(r / nx);
        i = (int)(r - (unsigned)j * nx);
      } else {
        k = (int)(c / nxy);
        const long r = c - (long)k * nxy;
        j = (int)(r / g.nmax[0]);
        i = (int)(r - (long)j * g.nmax[0]);
      }
      dest[glob_flat(g, i, j, k)] = acc;
    }
  }
}

// ---- exclusive prefix sum of n int counters into off[0..n] (off[n] = total < 2^31)
constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

__device__ __forceinline__ int block_exclusive_sum(int v, int* total) {
  __shared__ int warp_sums[SCAN_THREADS / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_sums[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int w = lane < SCAN_THREADS / 32 ? warp_sums[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < SCAN_THREADS / 32) warp_sums[lane] = w;
  }
  __syncthreads();
  const int before = (warp ? warp_sums[warp - 1] : 0) + x - v;
  *total = warp_sums[SCAN_THREADS / 32 - 1];
  __syncthreads();
  return before;
}

__global__ void __launch_bounds__(SCAN_THREADS) scan_tile_sums_kernel(const int* __restrict__ in, long n,
                                                                      int* __restrict__ bsum) {
  const long base = (long)blockIdx.x * SCAN_TILE;
  int s = 0;
  for (int t = 0; t < SCAN_ITEMS; ++t) {
    const long i = base + (long)t * SCAN_THREADS + threadIdx.x;
    if (i < n) s += in[i];
  }
  int total;
  block_exclusive_sum(s, &total);
  if (threadIdx.x == 0) bsum[blockIdx.x] = total;
}

__global__ void __launch_bounds__(SCAN_THREADS) scan_block_sums_kernel(int* __restrict__ bsum, int nb,
                                                                       int* __restrict__ grand) {
  int carry = 0;
  for (int b0 = 0; b0 < nb; b0 += SCAN_THREADS) {
    const int i = b0 + threadIdx.x;
    const int v = i < nb ? bsum[i] : 0;
    int total;
    const int ex = block_exclusive_sum(v, &total);
    if (i < nb) bsum[i] = carry + ex;
    carry += total;
  }
  if (threadIdx.x == 0) *grand = carry;
}

__global__ void __launch_bounds__(SCAN_THREADS) scan_tile_apply_kernel(const int* __restrict__ in, long n,
                                                                       const int* __restrict__ bsum,
                                                                       int* __restrict__ out) {
  // thread t owns items [base + t*ITEMS, base + (t+1)*ITEMS) of the tile
  const long base = (long)blockIdx.x * SCAN_TILE + (long)threadIdx.x * SCAN_ITEMS;
  int v[SCAN_ITEMS];
  int s = 0;
#pragma unroll
  for (int t = 0; t < SCAN_ITEMS; ++t) {
    v[t] = base + t < n ? in[base + t] : 0;
    s += v[t];
  }
  int total;
  int run = bsum[blockIdx.x] + block_exclusive_sum(s, &total);
#pragma unroll
  for (int t = 0; t < SCAN_ITEMS; ++t) {
    if (base + t < n) out[base + t] = run;
    run += v[t];
  }
}

int particle_geom(const nebo_particle_mesh* mesh, const nebo_field* cell, const void* px, const void* py,
                  const void* pz, PGeom& g, const char* who) {
  if (!mesh) return fail(NEBO_ERR_INVALID, "Nebo error in %s: null mesh", who);
  if (int rc = check_field(cell, who)) return rc;
  if (cell->dtype != NEBO_F64)
    return fail(NEBO_ERR_UNSUPPORTED, "Nebo error in %s: the cell field must hold doubles", who);
  const void* pos[3] = {px, py, pz};
  for (int a = 0; a < 3; ++a) {
    if (!(mesh->spacing[a] > 0.0)) return fail(NEBO_ERR_INVALID, "Nebo error in %s: mesh spacing must be > 0", who);
    const double d = mesh->spacing[a];
    g.d[a] = d;
    // xlo_ - dx_*ngm - dx_/2 with each operation rounded on its own (volatile keeps the host
    // compiler from fusing the product into the subtraction)
    volatile double t = d * (double)mesh->ghost_minus[a];
    volatile double u = mesh->low[a] - t;
    g.face[a] = u - d * 0.5;
    g.inv[a] = 1.0 / d;
    g.nmax[a] = cell->extent[a];
    g.glob[a] = cell->glob[a];
    g.off[a] = cell->offset[a];
    g.on[a] = pos[a] != nullptr;
  }
  return NEBO_OK;
}

int particle_blocks(long np, int per_sm = 6) {
  long b = (np + PWARPS * 32 - 1) / (PWARPS * 32);
  const long cap = (long)num_sms() * per_sm;
  if (b > cap) b = cap;
  return (int)(b < 1 ? 1 : b);
}

// CellToParticle's shared memory exceeds the 48 KB default; opt in once per device.
int c2p_prepare() {
  static std::atomic<unsigned long long> done{0};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return cuda_fail(cudaGetLastError(), "nebo_cell_to_particle");
  if (dev < 64 && (done.load() & (1ull << dev))) return NEBO_OK;
  NEBO_CUDA_TRY(cudaFuncSetAttribute(particles_kernel<PM_C2P>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)(PWARPS * sizeof(WarpShared<PM_C2P>))));
  if (dev < 64) done.fetch_or(1ull << dev);
  return NEBO_OK;
}

}  // namespace
}  // namespace nebo

using namespace nebo;

extern "C" int nebo_cell_to_particle(const nebo_particle_mesh* mesh, const double* px, const double* py,
                                     const double* pz, const double* psize, int64_t nparticles,
                                     const nebo_field* cell, double* dest, nebo_stream_t stream) {
  const char* who = "CellToParticle::apply_to_field";
  PGeom g;
  if (int rc = particle_geom(mesh, cell, px, py, pz, g, who)) return rc;
  if (nparticles < 0) return fail(NEBO_ERR_INVALID, "Nebo error in %s: negative particle count", who);
  if (nparticles == 0) return NEBO_OK;
  if (!psize || !dest) return fail(NEBO_ERR_INVALID, "Nebo error in %s: null particle size or destination", who);
  cudaStream_t s = (cudaStream_t)stream;
  if (int rc = c2p_prepare()) return rc;
  {
    LaunchScope ls("cell_to_particle", s);
    particles_kernel<PM_C2P><<<particle_blocks(nparticles), PWARPS * 32, PWARPS * sizeof(WarpShared<PM_C2P>), s>>>(
        g, px, py, pz, psize, (long)nparticles, static_cast<const double*>(cell->data), dest, nullptr, nullptr,
        nullptr, nullptr, nullptr);
  }
  NEBO_LAUNCH_CHECK("nebo_cell_to_particle");
  return NEBO_OK;
}

extern "C" int nebo_particle_to_cell(const nebo_particle_mesh* mesh, const double* px, const double* py,
                                     const double* pz, const double* psize, int64_t nparticles,
                                     const double* src, const nebo_field* cell, nebo_stream_t stream) {
  const char* who = "ParticleToCell::apply_to_field";
  PGeom g;
  if (int rc = particle_geom(mesh, cell, px, py, pz, g, who)) return rc;
  if (nparticles < 0) return fail(NEBO_ERR_INVALID, "Nebo error in %s: negative particle count", who);
  if (nparticles > 0 && (!psize || !src))
    return fail(NEBO_ERR_INVALID, "Nebo error in %s: null particle size or source", who);
  if (nparticles >= (1L << 31))
    return fail(NEBO_ERR_UNSUPPORTED, "Nebo error in %s: at most 2^31-1 particles", who);
  const long ncell = (long)g.nmax[0] * g.nmax[1] * g.nmax[2];
  if (ncell <= 0) return NEBO_OK;
  if (ncell >= (1L << 31) - 1) return fail(NEBO_ERR_UNSUPPORTED, "Nebo error in %s: window above 2^31-2 cells", who);
  cudaStream_t s = (cudaStream_t)stream;
  // the scan runs over ncell + 1 counters (the last one stays 0), so off[ncell] is the total
  const long nscan = ncell + 1;
  const long ntile = (nscan + SCAN_TILE - 1) / SCAN_TILE;
  // one allocation: counters, offsets, tile sums, grand total, 64-bit box total, then the fill's
  // order: particles per key (a key is a box's first cell, or ncell), their prefix, each
  // particle's key and the order
  auto up16 = [](size_t b) { return (b + 15) & ~(size_t)15; };
  const size_t cnt_b = (size_t)nscan * 4, off_b = (size_t)nscan * 4, bs_b = (size_t)ntile * 4;
  const size_t cnt_o = 0, off_o = up16(cnt_b), bs_o = off_o + up16(off_b);
  const size_t gr_o = bs_o + up16(bs_b), tot_o = gr_o + 16;
  // keys: 4 x 4 x 4 blocks of window cells
  const int kbx = (g.nmax[0] + 3) >> 2, kby = (g.nmax[1] + 3) >> 2, kbz = (g.nmax[2] + 3) >> 2;
  const int nkey = kbx * kby * kbz;
  const long nkscan = (long)nkey + 1, nktile = (nkscan + SCAN_TILE - 1) / SCAN_TILE;
  const size_t hist_b = (size_t)nkscan * 4;
  const size_t hist_o = tot_o + 16, hpos_o = hist_o + up16(hist_b), key_o = hpos_o + up16(hist_b);
  const size_t ord_o = key_o + up16((size_t)nparticles * 4), ws_b = ord_o + up16((size_t)nparticles * 4);
  char* ws = nullptr;
  pool_retain();
  NEBO_CUDA_TRY(cudaMallocAsync((void**)&ws, ws_b, s));
  int* cnt = (int*)(ws + cnt_o);
  int* off = (int*)(ws + off_o);
  int* bsum = (int*)(ws + bs_o);
  int* grand = (int*)(ws + gr_o);
  unsigned long long* total = (unsigned long long*)(ws + tot_o);
  int* hist = (int*)(ws + hist_o);
  int* hpos = (int*)(ws + hpos_o);
  int* key = (int*)(ws + key_o);
  int* order = (int*)(ws + ord_o);
  Entry* ent = nullptr;
  unsigned long long htotal = 0;
  int rc = NEBO_OK;
  cudaError_t e = cudaMemsetAsync(cnt, 0, cnt_b, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(total, 0, 8, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(hist, 0, hist_b, s);
  if (e != cudaSuccess) {
    rc = cuda_fail(e, "nebo_particle_to_cell workspace");
    goto done;
  }
  if (nparticles > 0) {
    {
      LaunchScope ls("particle_to_cell_count", s);
      p2c_count_kernel<<<particle_blocks(nparticles, 16), 256, 0, s>>>(g, px, py, pz, psize, (long)nparticles, cnt,
                                                                   total, key, hist, kbx, kby, nkey);
    }
    if ((e = cudaGetLastError()) != cudaSuccess) {
      rc = cuda_fail(e, "nebo_particle_to_cell count");
      goto done;
    }
    if ((e = cudaMemcpyAsync(&htotal, total, 8, cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess) {
      rc = cuda_fail(e, "nebo_particle_to_cell count");
      goto done;
    }
    if (htotal >= (1ULL << 31)) {
      rc = fail(NEBO_ERR_UNSUPPORTED, "Nebo error in %s: %llu particle-cell overlaps (at most 2^31-1)", who, htotal);
      goto done;
    }
  }
  {
    LaunchScope ls("particle_to_cell_scan_tiles", s);
    scan_tile_sums_kernel<<<(unsigned)ntile, SCAN_THREADS, 0, s>>>(cnt, nscan, bsum);
  }
  {
    LaunchScope ls("particle_to_cell_scan_sums", s);
    scan_block_sums_kernel<<<1, SCAN_THREADS, 0, s>>>(bsum, (int)ntile, grand);
  }
  {
    LaunchScope ls("particle_to_cell_scan_apply", s);
    scan_tile_apply_kernel<<<(unsigned)ntile, SCAN_THREADS, 0, s>>>(cnt, nscan, bsum, off);
  }
  if ((e = cudaGetLastError()) != cudaSuccess) {
    rc = cuda_fail(e, "nebo_particle_to_cell scan");
    goto done;
  }
  if (htotal > 0) {
    {
      // the fill's order: the particles grouped by key (the tile sums and total of the scan above
      // are free again)
      LaunchScope ls("particle_to_cell_order", s);
      scan_tile_sums_kernel<<<(unsigned)nktile, SCAN_THREADS, 0, s>>>(hist, nkscan, bsum);
      scan_block_sums_kernel<<<1, SCAN_THREADS, 0, s>>>(bsum, (int)nktile, grand);
      scan_tile_apply_kernel<<<(unsigned)nktile, SCAN_THREADS, 0, s>>>(hist, nkscan, bsum, hpos);
      p2c_order_kernel<<<particle_blocks(nparticles, 16), 256, 0, s>>>(key, (long)nparticles, hpos, order);
    }
    if ((e = cudaGetLastError()) != cudaSuccess) {
      rc = cuda_fail(e, "nebo_particle_to_cell order");
      goto done;
    }
    if ((e = cudaMallocAsync((void**)&ent, htotal * sizeof(Entry), s)) != cudaSuccess) {
      rc = fail(NEBO_ERR_ALLOC, "Nebo error in %s: %llu entries do not fit on the device", who, htotal);
      goto done;
    }
    {
      LaunchScope ls("particle_to_cell_fill", s);
      particles_kernel<PM_FILL><<<particle_blocks(nparticles), PWARPS * 32, PWARPS * sizeof(WarpShared<PM_FILL>), s>>>(
          g, px, py, pz, psize, (long)nparticles, nullptr, nullptr, src, off, cnt, ent, order);
    }
    if ((e = cudaGetLastError()) != cudaSuccess) {
      rc = cuda_fail(e, "nebo_particle_to_cell fill");
      goto done;
    }
  }
  {
    long nb = (ncell + FWARPS * 32 - 1) / (FWARPS * 32);
    const long cap = (long)num_sms() * 8;
    if (nb > cap) nb = cap;
    LaunchScope ls("particle_to_cell_fold", s);
    p2c_fold_kernel<<<(unsigned)nb, FWARPS * 32, 0, s>>>(g, ncell, off, ent, static_cast<double*>(cell->data));
  }
  if ((e = cudaGetLastError()) != cudaSuccess) rc = cuda_fail(e, "nebo_particle_to_cell fold");
done:
  if (ent) cudaFreeAsync(ent, s);
  cudaFreeAsync(ws, s);
  return rc;
}
