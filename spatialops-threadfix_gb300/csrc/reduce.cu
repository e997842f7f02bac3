// Reductions nebo_sum / nebo_max / nebo_min / nebo_norm (and _interior) over one field
// (spatialops/NeboReductions.h:45-240).  The reference folds serially on the CPU; here a
// two-pass, deterministic tree runs on the device:
//   pass 1: a warp per row, 8 independent loads per lane, pairwise sums of each batch folded
//           into per-thread Neumaier-compensated FP64 sums (or max/min), warp shuffles, one
//           partial per block;
//   pass 2: one block combines the partials in a fixed order.
// FP32 fields are accumulated in FP64.  max/min use the reference's comparisons
// ((r < v) ? v : r and (r > v) ? v : r), so they are exact.
#include <cmath>
#include <climits>
#include <mutex>

#include "common.cuh"
#include "fp64_int.cuh"
#include "reduce4.cuh"

namespace nebo {
namespace {

constexpr int RED_THREADS = 256;
constexpr int RED_MAX_BLOCKS = 1024;

struct Acc {
  double s, c;  // sum and running compensation (sum/norm), or the extremum in s
};

__device__ __forceinline__ void two_sum_add(Acc& a, double v) {
  const double t = a.s + v;
  if (fabs(a.s) >= fabs(v))
    a.c += (a.s - t) + v;
  else
    a.c += (v - t) + a.s;
  a.s = t;
}

__device__ __forceinline__ void merge(Acc& a, const Acc& b, int op) {
  if (op == NEBO_RED_MAX) {
    a.s = (a.s < b.s) ? b.s : a.s;
  } else if (op == NEBO_RED_MIN) {
    a.s = (a.s > b.s) ? b.s : a.s;
  } else {
    two_sum_add(a, b.s);
    a.c += b.c;
  }
}

__device__ __forceinline__ Acc identity(int op) {
  Acc a;
  a.s = op == NEBO_RED_MAX ? -INFINITY : (op == NEBO_RED_MIN ? INFINITY : 0.0);
  a.c = 0.0;
  return a;
}

__device__ Acc block_reduce(Acc a, int op) {
  __shared__ Acc sh[32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int o = 16; o > 0; o >>= 1) {
    Acc b;
    b.s = __shfl_down_sync(0xffffffffu, a.s, o);
    b.c = __shfl_down_sync(0xffffffffu, a.c, o);
    merge(a, b, op);
  }
  if (lane == 0) sh[wid] = a;
  __syncthreads();
  const int nw = (blockDim.x + 31) >> 5;
  a = (threadIdx.x < nw) ? sh[threadIdx.x] : identity(op);
  if (wid == 0) {
    for (int o = 16; o > 0; o >>= 1) {
      Acc b;
      b.s = __shfl_down_sync(0xffffffffu, a.s, o);
      b.c = __shfl_down_sync(0xffffffffu, a.c, o);
      merge(a, b, op);
    }
  }
  return a;
}

// FP32 elements widen exactly through integer operations (a hardware f32 -> f64 conversion issues
// on the FP64 pipe, which the accumulation itself needs).
__device__ __forceinline__ double widen(double v) { return v; }
__device__ __forceinline__ double widen(float v) { return fixmath::f32_to_f64(v); }

// Every element of the region's rows, a warp per row (rows strided over all warps of the grid),
// each lane issuing 8 independent loads before it uses them; f8(v[8]) gets each full batch of 8
// (lanes 32 apart), f1(v) each element of the row tails.
template <typename T, class F8, class F1>
__device__ __forceinline__ void walk_rows(const T* __restrict__ base, int sy, long sz, int x0, int x1, int y0, int ny,
                                          int z0, int nrows, F8&& f8, F1&& f1) {
  const int lane = threadIdx.x & 31;
  const int nwarps = gridDim.x * (blockDim.x >> 5);
  for (int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); r < nrows; r += nwarps) {
    const int z = r / ny, y = r - z * ny;
    const T* row = base + (long)sy * (y0 + y) + sz * (z0 + z);
    int x = x0 + lane;
    for (; x + 7 * 32 < x1; x += 8 * 32) {
      double v[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) v[i] = widen(__ldg(row + x + 32 * i));
      f8(v);
    }
    for (; x < x1; x += 32) f1(widen(__ldg(row + x)));
  }
}

// Sum of 8 in pairs (7 FP64 adds), and of their squares (4 multiplies folded into 4 FMAs).
__device__ __forceinline__ double sum8(const double* v) {
  return ((v[0] + v[1]) + (v[2] + v[3])) + ((v[4] + v[5]) + (v[6] + v[7]));
}
__device__ __forceinline__ double sumsq8(const double* v) {
  const double a = fma(v[0], v[0], v[1] * v[1]), b = fma(v[2], v[2], v[3] * v[3]);
  const double c = fma(v[4], v[4], v[5] * v[5]), d = fma(v[6], v[6], v[7] * v[7]);
  return (a + b) + (c + d);
}

// Pass 1 of one reduction: each thread folds its batches (pairwise within a batch, then into a
// Neumaier-compensated running sum; max/min with the reference's comparisons).
template <typename T>
__global__ void __launch_bounds__(RED_THREADS) reduce_rows_kernel(const T* __restrict__ base, int sy, long sz, int x0,
                                                                  int x1, int y0, int ny, int z0, long nrows, int op,
                                                                  Acc* __restrict__ partials) {
  Acc a = identity(op);
  auto one = [&](double v) {
    if (op == NEBO_RED_MAX)
      a.s = (a.s < v) ? v : a.s;
    else if (op == NEBO_RED_MIN)
      a.s = (a.s > v) ? v : a.s;
    else
      two_sum_add(a, op == NEBO_RED_NORM ? v * v : v);
  };
  walk_rows(base, sy, sz, x0, x1, y0, ny, z0, (int)nrows,
            [&](const double* v) {
              if (op == NEBO_RED_SUM)
                two_sum_add(a, sum8(v));
              else if (op == NEBO_RED_NORM)
                two_sum_add(a, sumsq8(v));
              else
                for (int i = 0; i < 8; ++i) one(v[i]);
            },
            one);
  a = block_reduce(a, op);
  if (threadIdx.x == 0) partials[blockIdx.x] = a;
}

__global__ void __launch_bounds__(RED_THREADS) reduce_final_kernel(const Acc* __restrict__ partials, int n, int op,
                                                                   double* __restrict__ out) {
  Acc a = identity(op);
  // fixed assignment of partials to threads -> deterministic result
  for (int i = threadIdx.x; i < n; i += blockDim.x) merge(a, partials[i], op);
  a = block_reduce(a, op);
  if (threadIdx.x == 0) {
    double r = (op == NEBO_RED_SUM || op == NEBO_RED_NORM) ? a.s + a.c : a.s;
    if (op == NEBO_RED_NORM) r = sqrt(r);
    *out = r;
  }
}

// Per-call scratch from the stream-ordered pool: concurrent reductions on different streams
// never share partials.
int scratch_alloc(Acc** partials, double** result, cudaStream_t s) {
  void* p = nullptr;
  pool_retain();
  NEBO_CUDA_TRY(cudaMallocAsync(&p, RED_MAX_BLOCKS * sizeof(Acc) + 64, s));
  *partials = (Acc*)p;
  *result = (double*)((char*)p + RED_MAX_BLOCKS * sizeof(Acc));
  return NEBO_OK;
}

}  // namespace

// Region of a field reduction in glob coordinates: whole window (valid ghosts included) or the
// window minus its valid ghosts (interior, BC cells included), as nebo_fold does.
void reduction_region(const nebo_field& f, int interior, int lo[3], int hi[3]) {
  for (int i = 0; i < 3; ++i) {
    const int gm = f.extent[i] <= 1 ? 0 : f.ghost_minus[i];
    const int gp = f.extent[i] <= 1 ? 0 : f.ghost_plus[i];
    lo[i] = f.offset[i] + (interior ? gm : 0);
    hi[i] = f.offset[i] + f.extent[i] - (interior ? gp : 0);
  }
}

int reduce_field_into(const nebo_field* f, int op, int interior, double* d_result, Acc* partials, cudaStream_t s) {
  int lo[3], hi[3];
  reduction_region(*f, interior, lo, hi);
  const long nrows = (long)(hi[1] - lo[1]) * (hi[2] - lo[2]);
  if (nrows <= 0 || hi[0] <= lo[0]) return fail(NEBO_ERR_INVALID, "Nebo error in nebo_reduce: empty region");
  int blocks = (int)(nrows < (long)num_sms() * 4 ? nrows : (long)num_sms() * 4);
  if (blocks > RED_MAX_BLOCKS) blocks = RED_MAX_BLOCKS;
  const int sy = f->glob[0];
  const long sz = (long)f->glob[0] * f->glob[1];
  {
    LaunchScope ls("reduce_rows", s);
    if (f->dtype == NEBO_F64)
    reduce_rows_kernel<double><<<blocks, RED_THREADS, 0, s>>>((const double*)f->data, sy, sz, lo[0], hi[0], lo[1],
                                                              hi[1] - lo[1], lo[2], nrows, op, partials);
  else
    reduce_rows_kernel<float><<<blocks, RED_THREADS, 0, s>>>((const float*)f->data, sy, sz, lo[0], hi[0], lo[1],
                                                             hi[1] - lo[1], lo[2], nrows, op, partials);
  }
  {
    LaunchScope ls("reduce_final", s);
    reduce_final_kernel<<<1, RED_THREADS, 0, s>>>(partials, blocks, op, d_result);
  }
  NEBO_LAUNCH_CHECK("nebo_reduce");
  return NEBO_OK;
}

static int check_reduce_args(const nebo_field* f, int op) {
  int rc = check_field(f, "nebo_reduce");
  if (rc) return rc;
  if (op < NEBO_RED_SUM || op > NEBO_RED_NORM) return fail(NEBO_ERR_INVALID, "Nebo error in nebo_reduce: bad op %d", op);
  return NEBO_OK;
}

}  // namespace nebo

using namespace nebo;

extern "C" int nebo_reduce_async(const nebo_field* f, int op, int interior, double* d_result, nebo_stream_t stream) {
  int rc = check_reduce_args(f, op);
  if (rc) return rc;
  if (!d_result) return fail(NEBO_ERR_INVALID, "Nebo error in nebo_reduce_async: null result pointer");
  Acc* partials;
  double* dres;
  cudaStream_t s = (cudaStream_t)stream;
  if ((rc = scratch_alloc(&partials, &dres, s))) return rc;
  rc = reduce_field_into(f, op, interior, d_result, partials, s);
  cudaFreeAsync(partials, s);
  return rc;
}

extern "C" int nebo_reduce(const nebo_field* f, int op, int interior, double* result, nebo_stream_t stream) {
  int rc = check_reduce_args(f, op);
  if (rc) return rc;
  if (!result) return fail(NEBO_ERR_INVALID, "Nebo error in nebo_reduce: null result pointer");
  Acc* partials;
  double* dres;
  cudaStream_t s = (cudaStream_t)stream;
  if ((rc = scratch_alloc(&partials, &dres, s))) return rc;
  rc = reduce_field_into(f, op, interior, dres, partials, s);
  if (!rc) {
    cudaError_t e = cudaMemcpyAsync(result, dres, sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) rc = cuda_fail(e, "nebo_reduce copy");
  }
  cudaFreeAsync(partials, s);
  if (rc) return rc;
  NEBO_CUDA_TRY(cudaStreamSynchronize(s));
  return NEBO_OK;
}

// ------------------------------------------------------------------------------------------
// Reduction without any allocation.
//
// nebo_reduce / nebo_reduce_async take their block partials from the stream-ordered pool on
// every call.  Callers that must not enter the CUDA allocator at that point (a host framework
// that has reserved the device memory up front in its own pool, so a further cudaMalloc fails or
// breaks its accounting; code that runs where the allocator may not be entered) use
// nebo_reduce_noalloc instead: the same two kernels, with the partials in the fixed array below.
//
// The array lives in this module's device memory for every GPU that loads the library, until the
// process exits.  Host code cannot use the symbol's name as a device address, so the first call
// on each device (with that device current) looks the address up with cudaGetSymbolAddress and
// caches it (a cudaDeviceReset voids the cached address: a process that resets a device must not
// call this entry point on it afterwards); that first call should come before any stream capture.
// A reduction takes at most 1024 blocks, one slot each.  All calls share the array
// and it keeps the last call's contents: pass 1 writes every slot that pass 2 reads, so nothing
// needs clearing, but calls whose kernels overlap on the GPU (different streams, no ordering
// between them) race on it.
namespace nebo {
namespace {

constexpr int NOALLOC_MAX_PARTIALS = 1024;  // 16 KiB: one (sum, compensation) pair per block
constexpr long NOALLOC_MAX_ROWS = 2147483647L;  // rows (y * z) of the reduced region
constexpr int NOALLOC_MAX_DEVICES = 64;
static __device__ __align__(256) Acc g_noalloc_partials[NOALLOC_MAX_PARTIALS];

std::mutex g_noalloc_mu;
Acc* g_noalloc_addr[NOALLOC_MAX_DEVICES] = {nullptr};

int noalloc_partials(Acc** out) {
  int dev = 0;
  NEBO_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= NOALLOC_MAX_DEVICES)
    return fail(NEBO_ERR_UNSUPPORTED, "Nebo error in nebo_reduce_noalloc: device index %d beyond %d", dev,
                NOALLOC_MAX_DEVICES);
  std::lock_guard<std::mutex> g(g_noalloc_mu);
  if (!g_noalloc_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partials);
    if (e != cudaSuccess) return cuda_fail(e, "nebo_reduce_noalloc (cudaGetSymbolAddress)");
    g_noalloc_addr[dev] = static_cast<Acc*>(p);
  }
  *out = g_noalloc_addr[dev];
  return NEBO_OK;
}

}  // namespace
}  // namespace nebo

extern "C" int nebo_reduce_noalloc(const nebo_field* f, int op, int interior, double* d_result,
                                   nebo_stream_t stream) {
  int rc = check_reduce_args(f, op);
  if (rc) return rc;
  if (!d_result) return fail(NEBO_ERR_INVALID, "Nebo error in nebo_reduce_noalloc: null result pointer");
  int lo[3], hi[3];
  reduction_region(*f, interior, lo, hi);
  const long nrows = (long)(hi[1] - lo[1]) * (hi[2] - lo[2]);
  if (nrows <= 0 || hi[0] <= lo[0]) return fail(NEBO_ERR_INVALID, "Nebo error in nebo_reduce_noalloc: empty region");
  // The row walk takes an int row count; larger regions are refused before any CUDA call.
  if (nrows > NOALLOC_MAX_ROWS)
    return fail(NEBO_ERR_INVALID,
                "Nebo error in nebo_reduce_noalloc: the region has %ld rows, more than the %ld this entry point takes",
                nrows, (long)NOALLOC_MAX_ROWS);
  // One partial slot per block, and never more blocks than slots: the grid-stride row walk covers
  // any region with fewer blocks, so the fixed array suffices whatever the SM count.
  long want = nrows < (long)num_sms() * 4 ? nrows : (long)num_sms() * 4;
  if (want > NOALLOC_MAX_PARTIALS) want = NOALLOC_MAX_PARTIALS;
  const int blocks = (int)want;
  Acc* partials = nullptr;
  if ((rc = noalloc_partials(&partials))) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  const int sy = f->glob[0];
  const long sz = (long)f->glob[0] * f->glob[1];
  {
    LaunchScope ls("reduce_rows", s);
    if (f->dtype == NEBO_F64)
      reduce_rows_kernel<double><<<blocks, RED_THREADS, 0, s>>>((const double*)f->data, sy, sz, lo[0], hi[0], lo[1],
                                                                hi[1] - lo[1], lo[2], nrows, op, partials);
    else
      reduce_rows_kernel<float><<<blocks, RED_THREADS, 0, s>>>((const float*)f->data, sy, sz, lo[0], hi[0], lo[1],
                                                               hi[1] - lo[1], lo[2], nrows, op, partials);
  }
  {
    LaunchScope ls("reduce_final", s);
    reduce_final_kernel<<<1, RED_THREADS, 0, s>>>(partials, blocks, op, d_result);
  }
  NEBO_LAUNCH_CHECK("nebo_reduce_noalloc");
  return NEBO_OK;
}

// ------------------------------------------------------------------------------------------
// All four reductions in one pass over the field (nebo_sum, nebo_max, nebo_min, nebo_norm of
// the same region), for callers that need several of them: the field is read once instead of
// four times.  FP64 is the scarce unit on this GPU, so each element costs two FP64 operations
// (one add for the sum, one fused multiply-add for the sum of squares); max and min compare
// order-preserving 64-bit integer keys of the doubles on the integer pipe.  Per-thread partial
// sums are plain (at most a few hundred terms each); partials are combined with Neumaier
// compensation.  NaNs are skipped by max/min, as the reference's comparisons skip them; equal
// zeros of opposite sign may come back with either sign.
namespace nebo {
namespace {

template <typename T>
__global__ void __launch_bounds__(RED_THREADS) reduce4_rows_kernel(const T* __restrict__ base, int sy, long sz, int x0,
                                                                   int x1, int y0, int ny, int z0, long nrows,
                                                                   Acc4* __restrict__ partials) {
  double s = 0.0, q = 0.0;
  long long mx = LLONG_MIN, mn = LLONG_MAX;
  auto keys = [&](double v) { keys_add(mx, mn, order_key(v)); };  // NaNs never win a comparison
  walk_rows(base, sy, sz, x0, x1, y0, ny, z0, (int)nrows,
            [&](const double* v) {
              s += sum8(v);
              q += sumsq8(v);
#pragma unroll
              for (int i = 0; i < 8; ++i) keys(v[i]);
            },
            [&](double v) {
              s += v;
              q = fma(v, v, q);
              keys(v);
            });
  Acc4 a{s, 0.0, q, 0.0, mx, mn};
  a = block_reduce4(a);
  if (threadIdx.x == 0) partials[blockIdx.x] = a;
}


}  // namespace
}  // namespace nebo

extern "C" int nebo_reduce_all(const nebo_field* f, int interior, double* d_out4, nebo_stream_t stream) {
  int rc = check_reduce_args(f, NEBO_RED_SUM);
  if (rc) return rc;
  if (!d_out4) return fail(NEBO_ERR_INVALID, "Nebo error in nebo_reduce_all: null result pointer");
  int lo[3], hi[3];
  reduction_region(*f, interior, lo, hi);
  const long nrows = (long)(hi[1] - lo[1]) * (hi[2] - lo[2]);
  if (nrows <= 0 || hi[0] <= lo[0]) return fail(NEBO_ERR_INVALID, "Nebo error in nebo_reduce_all: empty region");
  int blocks = (int)(nrows < (long)num_sms() * 4 ? nrows : (long)num_sms() * 4);
  if (blocks > RED_MAX_BLOCKS) blocks = RED_MAX_BLOCKS;
  cudaStream_t s = (cudaStream_t)stream;
  Acc4* partials = nullptr;
  pool_retain();
  NEBO_CUDA_TRY(cudaMallocAsync((void**)&partials, sizeof(Acc4) * blocks, s));
  const int sy = f->glob[0];
  const long sz = (long)f->glob[0] * f->glob[1];
  {
    LaunchScope ls("reduce4_rows", s);
    if (f->dtype == NEBO_F64)
      reduce4_rows_kernel<double><<<blocks, RED_THREADS, 0, s>>>((const double*)f->data, sy, sz, lo[0], hi[0], lo[1],
                                                                 hi[1] - lo[1], lo[2], nrows, partials);
    else
      reduce4_rows_kernel<float><<<blocks, RED_THREADS, 0, s>>>((const float*)f->data, sy, sz, lo[0], hi[0], lo[1],
                                                                hi[1] - lo[1], lo[2], nrows, partials);
  }
  {
    LaunchScope ls("reduce4_final", s);
    reduce4_final_kernel<<<1, RED_THREADS, 0, s>>>(partials, blocks, d_out4);
  }
  cudaError_t le = cudaGetLastError();
  cudaFreeAsync(partials, s);
  if (le != cudaSuccess) return cuda_fail(le, "nebo_reduce_all");
  return NEBO_OK;
}
