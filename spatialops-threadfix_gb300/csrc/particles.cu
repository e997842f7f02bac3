// Particle <-> cell operators (the kernels behind Particle::CellToParticle and
// Particle::ParticleToCell, spatialops/particles/ParticleOperators.h:183-246 and :319-398).
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
//             64-bit total);
//   2. scan   an exclusive prefix sum of the counters gives each cell a slice of one entry list;
//   3. fill   every particle writes (index, v * w) into a free slot of each of its cells' slices;
//   4. fold   one thread per window cell sorts its slice by particle index (an insertion sort:
//             slots are taken in nearly increasing index order) and sums it from +0 in that
//             order; a cell with no entry gets +0 (the reference's `dest <<= 0` before it adds).
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
  double lo[3];    // xlo_, ylo_, zlo_
  int ngm[3];      // cell field's ghost cells on - faces
  int nmax[3];     // window extent (ghosts included)
  int glob[3];     // allocation
  int off[3];      // window offset in the allocation
  int on[3];       // axis has coordinates
};

struct Axis {
  int lo, hi;       // window cells [lo, hi) along this axis
  double plo, phi;  // particle's low and high coordinate
  double face;      // low face of window cell 0
  double d;
  int on;
};

// std::min / std::max on doubles (the second argument wins ties and unordered pairs as in
// <algorithm>)
__device__ __forceinline__ double dmin(double a, double b) { return (b < a) ? b : a; }
__device__ __forceinline__ double dmax(double a, double b) { return (a < b) ? b : a; }

__device__ __forceinline__ void make_axis(Axis& ax, const double* __restrict__ pos, long p, double size,
                                          const PGeom& g, int a) {
  ax.on = g.on[a];
  ax.d = g.d[a];
  // xloface = xlo_ - dx_*ngm - dx_/2 (ParticleOperators.h:202-204, 329-331)
  ax.face = __dsub_rn(__dsub_rn(g.lo[a], __dmul_rn(g.d[a], fixmath::i32_to_f64(g.ngm[a]))), __dmul_rn(g.d[a], 0.5));
  const double rp = __dmul_rn(size, 0.5);
  ax.plo = ax.on ? __dsub_rn(pos[p], rp) : 0.0;
  ax.phi = ax.on ? __dadd_rn(ax.plo, size) : 0.0;
  const int n = g.nmax[a];
  const double ql = __ddiv_rn(__dsub_rn(ax.plo, ax.face), ax.d);
  int lo;
  if (!(ql < (double)n))
    lo = n;  // past the window's high end (or NaN): empty
  else
    lo = ql > 0.0 ? (int)ql : 0;  // truncation; (-1, 0) gives 0 as in the reference, below is clipped
  int hi;
  if (ax.on) {
    const double qh = __ddiv_rn(__dsub_rn(ax.phi, ax.face), ax.d);
    if (!(qh > -1.0))
      hi = 0;  // wholly below the window (or NaN)
    else if (qh >= (double)n)
      hi = n;
    else
      hi = min(n, (int)qh + 1);  // int() + 1, clipped to the window (ParticleOperators.h:228-230)
  } else if (g.glob[a] == 1) {
    lo = 0;  // the reference's one cell along an off axis; an allocation extent of 1 maps every
    hi = 1;  // index to 0 (MemoryWindow::flat_index)
  } else {
    hi = min(n, lo + 1);
  }
  ax.lo = lo;
  ax.hi = hi;
}

// Overlap of the particle with window cell i along one axis (1 when the axis is off).
__device__ __forceinline__ double axis_cont(const Axis& ax, int i) {
  if (!ax.on) return 1.0;
  const double cm = __dadd_rn(ax.face, __dmul_rn(fixmath::i32_to_f64(i), ax.d));
  const double cp = __dadd_rn(cm, ax.d);
  return __dsub_rn(dmin(cp, ax.phi), dmax(cm, ax.plo));
}

struct Box {
  Axis a[3];
  double pvol;
  __device__ __forceinline__ bool empty() const {
    return a[0].lo >= a[0].hi || a[1].lo >= a[1].hi || a[2].lo >= a[2].hi;
  }
  __device__ __forceinline__ long cells() const {
    return empty() ? 0 : (long)(a[0].hi - a[0].lo) * (a[1].hi - a[1].lo) * (a[2].hi - a[2].lo);
  }
};

__device__ __forceinline__ void make_box(Box& b, const PGeom& g, const double* __restrict__ px,
                                         const double* __restrict__ py, const double* __restrict__ pz,
                                         const double* __restrict__ psize, long p) {
  const double size = psize[p];
  make_axis(b.a[0], px, p, size, g, 0);
  make_axis(b.a[1], py, p, size, g, 1);
  make_axis(b.a[2], pz, p, size, g, 2);
  const double two_rp = __dmul_rn(2.0, __dmul_rn(size, 0.5));
  b.pvol = __dmul_rn(__dmul_rn(g.on[0] ? two_rp : 1.0, g.on[1] ? two_rp : 1.0), g.on[2] ? two_rp : 1.0);
}

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

__global__ void __launch_bounds__(256) c2p_kernel(PGeom g, const double* __restrict__ px, const double* __restrict__ py,
                                                  const double* __restrict__ pz, const double* __restrict__ psize,
                                                  long np, const double* __restrict__ cell,
                                                  double* __restrict__ dest) {
  for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < np; p += (long)gridDim.x * blockDim.x) {
    Box b;
    make_box(b, g, px, py, pz, psize, p);
    double acc = 0.0;
    for (int k = b.a[2].lo; k < b.a[2].hi; ++k) {
      const double zc = axis_cont(b.a[2], k);
      for (int j = b.a[1].lo; j < b.a[1].hi; ++j) {
        const double yc = axis_cont(b.a[1], j);
        for (int i = b.a[0].lo; i < b.a[0].hi; ++i) {
          const double xc = axis_cont(b.a[0], i);
          const double w = __ddiv_rn(__dmul_rn(__dmul_rn(xc, yc), zc), b.pvol);
          acc = __dadd_rn(acc, __dmul_rn(cell[glob_flat(g, i, j, k)], w));
        }
      }
    }
    dest[p] = acc;
  }
}

__global__ void __launch_bounds__(256) p2c_count_kernel(PGeom g, const double* __restrict__ px,
                                                        const double* __restrict__ py, const double* __restrict__ pz,
                                                        const double* __restrict__ psize, long np,
                                                        int* __restrict__ cnt, unsigned long long* __restrict__ total) {
  unsigned long long mine = 0;
  for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < np; p += (long)gridDim.x * blockDim.x) {
    Box b;
    make_box(b, g, px, py, pz, psize, p);
    mine += (unsigned long long)b.cells();
    if (b.empty()) continue;
    for (int k = b.a[2].lo; k < b.a[2].hi; ++k)
      for (int j = b.a[1].lo; j < b.a[1].hi; ++j)
        for (int i = b.a[0].lo; i < b.a[0].hi; ++i) atomicAdd(cnt + win_flat(g, i, j, k), 1);
  }
  for (int o = 16; o > 0; o >>= 1) mine += __shfl_xor_sync(0xffffffffu, mine, o);
  if ((threadIdx.x & 31) == 0 && mine) atomicAdd(total, mine);
}

__global__ void __launch_bounds__(256) p2c_fill_kernel(PGeom g, const double* __restrict__ px,
                                                       const double* __restrict__ py, const double* __restrict__ pz,
                                                       const double* __restrict__ psize, long np,
                                                       const double* __restrict__ src, const int* __restrict__ off,
                                                       int* __restrict__ cnt, int* __restrict__ epid,
                                                       double* __restrict__ eval) {
  for (long p = blockIdx.x * (long)blockDim.x + threadIdx.x; p < np; p += (long)gridDim.x * blockDim.x) {
    Box b;
    make_box(b, g, px, py, pz, psize, p);
    if (b.empty()) continue;
    const double v = src[p];
    for (int k = b.a[2].lo; k < b.a[2].hi; ++k) {
      const double zc = axis_cont(b.a[2], k);
      for (int j = b.a[1].lo; j < b.a[1].hi; ++j) {
        const double yc = axis_cont(b.a[1], j);
        for (int i = b.a[0].lo; i < b.a[0].hi; ++i) {
          const double xc = axis_cont(b.a[0], i);
          const double w = __ddiv_rn(__dmul_rn(__dmul_rn(xc, yc), zc), b.pvol);
          const long c = win_flat(g, i, j, k);
          // the counter runs down from the cell's count: slots are taken from the slice's start
          const int slot = off[c + 1] - atomicSub(cnt + c, 1);
          epid[slot] = (int)p;
          eval[slot] = __dmul_rn(v, w);
        }
      }
    }
  }
}

__global__ void __launch_bounds__(256) p2c_fold_kernel(PGeom g, long ncell, const int* __restrict__ off,
                                                       int* __restrict__ epid, double* __restrict__ eval,
                                                       double* __restrict__ dest) {
  const long nxy = (long)g.nmax[0] * g.nmax[1];
  for (long c = blockIdx.x * (long)blockDim.x + threadIdx.x; c < ncell; c += (long)gridDim.x * blockDim.x) {
    const int b = off[c], e = off[c + 1];
    for (int s = b + 1; s < e; ++s) {
      const int key = epid[s];
      const double v = eval[s];
      int t = s - 1;
      while (t >= b && epid[t] > key) {
        epid[t + 1] = epid[t];
        eval[t + 1] = eval[t];
        --t;
      }
      epid[t + 1] = key;
      eval[t + 1] = v;
    }
    double acc = 0.0;
    for (int s = b; s < e; ++s) acc = __dadd_rn(acc, eval[s]);
    const int k = (int)(c / nxy);
    const long r = c - (long)k * nxy;
    const int j = (int)(r / g.nmax[0]);
    const int i = (int)(r - (long)j * g.nmax[0]);
    dest[glob_flat(g, i, j, k)] = acc;
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
    g.d[a] = mesh->spacing[a];
    g.lo[a] = mesh->low[a];
    g.ngm[a] = mesh->ghost_minus[a];
    g.nmax[a] = cell->extent[a];
    g.glob[a] = cell->glob[a];
    g.off[a] = cell->offset[a];
    g.on[a] = pos[a] != nullptr;
  }
  return NEBO_OK;
}

int particle_blocks(long np) {
  long b = (np + 255) / 256;
  const long cap = (long)num_sms() * 8;
  if (b > cap) b = cap;
  return (int)(b < 1 ? 1 : b);
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
  {
    LaunchScope ls("cell_to_particle", s);
    c2p_kernel<<<particle_blocks(nparticles), 256, 0, s>>>(g, px, py, pz, psize, (long)nparticles,
                                                           static_cast<const double*>(cell->data), dest);
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
  cudaStream_t s = (cudaStream_t)stream;
  // the scan runs over ncell + 1 counters (the last one stays 0), so off[ncell] is the total
  const long nscan = ncell + 1;
  const long ntile = (nscan + SCAN_TILE - 1) / SCAN_TILE;
  // one allocation: counters, offsets, tile sums, grand total, 64-bit box total
  const size_t cnt_b = (size_t)nscan * 4, off_b = (size_t)nscan * 4, bs_b = (size_t)ntile * 4;
  const size_t cnt_o = 0, off_o = (cnt_b + 15) & ~(size_t)15, bs_o = off_o + ((off_b + 15) & ~(size_t)15);
  const size_t gr_o = bs_o + ((bs_b + 15) & ~(size_t)15), tot_o = gr_o + 16, ws_b = tot_o + 16;
  char* ws = nullptr;
  NEBO_CUDA_TRY(cudaMallocAsync((void**)&ws, ws_b, s));
  int* cnt = (int*)(ws + cnt_o);
  int* off = (int*)(ws + off_o);
  int* bsum = (int*)(ws + bs_o);
  int* grand = (int*)(ws + gr_o);
  unsigned long long* total = (unsigned long long*)(ws + tot_o);
  int* epid = nullptr;
  double* eval = nullptr;
  unsigned long long htotal = 0;
  int rc = NEBO_OK;
  cudaError_t e = cudaMemsetAsync(cnt, 0, cnt_b, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(total, 0, 8, s);
  if (e != cudaSuccess) {
    rc = cuda_fail(e, "nebo_particle_to_cell workspace");
    goto done;
  }
  if (nparticles > 0) {
    {
      LaunchScope ls("particle_to_cell_count", s);
      p2c_count_kernel<<<particle_blocks(nparticles), 256, 0, s>>>(g, px, py, pz, psize, (long)nparticles, cnt,
                                                                   total);
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
    LaunchScope ls("particle_to_cell_scan", s);
    scan_tile_sums_kernel<<<(unsigned)ntile, SCAN_THREADS, 0, s>>>(cnt, nscan, bsum);
    scan_block_sums_kernel<<<1, SCAN_THREADS, 0, s>>>(bsum, (int)ntile, grand);
    scan_tile_apply_kernel<<<(unsigned)ntile, SCAN_THREADS, 0, s>>>(cnt, nscan, bsum, off);
  }
  if ((e = cudaGetLastError()) != cudaSuccess) {
    rc = cuda_fail(e, "nebo_particle_to_cell scan");
    goto done;
  }
  if (htotal > 0) {
    if ((e = cudaMallocAsync((void**)&epid, htotal * 4, s)) != cudaSuccess ||
        (e = cudaMallocAsync((void**)&eval, htotal * 8, s)) != cudaSuccess) {
      rc = fail(NEBO_ERR_ALLOC, "Nebo error in %s: %llu entries do not fit on the device", who, htotal);
      goto done;
    }
    {
      LaunchScope ls("particle_to_cell_fill", s);
      p2c_fill_kernel<<<particle_blocks(nparticles), 256, 0, s>>>(g, px, py, pz, psize, (long)nparticles, src, off,
                                                                  cnt, epid, eval);
    }
    if ((e = cudaGetLastError()) != cudaSuccess) {
      rc = cuda_fail(e, "nebo_particle_to_cell fill");
      goto done;
    }
  }
  {
    long nb = (ncell + 255) / 256;
    const long cap = (long)num_sms() * 16;
    if (nb > cap) nb = cap;
    LaunchScope ls("particle_to_cell_fold", s);
    p2c_fold_kernel<<<(unsigned)nb, 256, 0, s>>>(g, ncell, off, epid, eval, static_cast<double*>(cell->data));
  }
  if ((e = cudaGetLastError()) != cudaSuccess) rc = cuda_fail(e, "nebo_particle_to_cell fold");
done:
  if (eval) cudaFreeAsync(eval, s);
  if (epid) cudaFreeAsync(epid, s);
  cudaFreeAsync(ws, s);
  return rc;
}
