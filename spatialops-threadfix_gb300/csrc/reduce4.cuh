// The four reductions nebo_sum, nebo_max, nebo_min and nebo_norm of one region in a single
// accumulator (spatialops/NeboReductions.h:114-240 fold each of them serially): per-thread plain
// FP64 sums of the values and of their squares, max/min as order-preserving 64-bit integer keys of
// the doubles (NaNs never win, as in the reference's comparisons; equal zeros of opposite sign may
// come back with either sign), Neumaier-compensated merges of the partial accumulators, and a
// one-block final pass in a fixed order (deterministic).
#pragma once

#include <climits>
#include <cmath>

#include "common.cuh"

namespace nebo {
namespace {

struct Acc4 {
  double s, sc, q, qc;  // sum and compensation, sum of squares and compensation
  long long mx, mn;     // order-preserving keys of max and min
};

__device__ __forceinline__ double from_key(long long k) {
  return __longlong_as_double(k ^ ((k >> 63) & 0x7fffffffffffffffLL));
}
__device__ __forceinline__ void comp_add(double& s, double& c, double v) {
  const double t = s + v;
  c += (fabs(s) >= fabs(v)) ? ((s - t) + v) : ((v - t) + s);
  s = t;
}
__device__ __forceinline__ void merge4(Acc4& a, const Acc4& b) {
  comp_add(a.s, a.sc, b.s);
  a.sc += b.sc;
  comp_add(a.q, a.qc, b.q);
  a.qc += b.qc;
  a.mx = a.mx > b.mx ? a.mx : b.mx;
  a.mn = a.mn < b.mn ? a.mn : b.mn;
}
__device__ __forceinline__ Acc4 shfl_down4(const Acc4& a, int o) {
  Acc4 b;
  b.s = __shfl_down_sync(0xffffffffu, a.s, o);
  b.sc = __shfl_down_sync(0xffffffffu, a.sc, o);
  b.q = __shfl_down_sync(0xffffffffu, a.q, o);
  b.qc = __shfl_down_sync(0xffffffffu, a.qc, o);
  b.mx = __shfl_down_sync(0xffffffffu, a.mx, o);
  b.mn = __shfl_down_sync(0xffffffffu, a.mn, o);
  return b;
}
// Merge without compensation (inside a warp: 32 partials pairwise, a few ulp at most).
__device__ __forceinline__ void merge4_plain(Acc4& a, const Acc4& b) {
  a.s += b.s;
  a.sc += b.sc;
  a.q += b.q;
  a.qc += b.qc;
  a.mx = a.mx > b.mx ? a.mx : b.mx;
  a.mn = a.mn < b.mn ? a.mn : b.mn;
}

// Block-wide merge (plain inside each warp, compensated across warps); valid in thread 0.
__device__ __forceinline__ Acc4 block_reduce4(Acc4 a) {
  __shared__ Acc4 sh[32];
  const int tid = threadIdx.x + blockDim.x * (threadIdx.y + blockDim.y * threadIdx.z);
  const int lane = tid & 31, wid = tid >> 5;
  for (int o = 16; o > 0; o >>= 1) merge4_plain(a, shfl_down4(a, o));
  if (lane == 0) sh[wid] = a;
  __syncthreads();
  const int nw = (blockDim.x * blockDim.y * blockDim.z + 31) >> 5;
  if (wid == 0) {
    if (lane < nw) {
      a = sh[lane];
    } else {
      a.s = a.sc = a.q = a.qc = 0.0;
      a.mx = LLONG_MIN;
      a.mn = LLONG_MAX;
    }
    for (int o = 16; o > 0; o >>= 1) merge4(a, shfl_down4(a, o));
  }
  return a;
}


__device__ __forceinline__ Acc4 acc4_identity() { return Acc4{0.0, 0.0, 0.0, 0.0, LLONG_MIN, LLONG_MAX}; }

// Order-preserving key of a double; NaN keys fall outside [key(-inf), key(+inf)] (positive
// NaNs above, negative NaNs below).
__device__ __forceinline__ long long order_key(double v) {
  const long long b = __double_as_longlong(v);
  return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}
constexpr long long KEY_PINF = 0x7ff0000000000000LL, KEY_NINF = (long long)0x800fffffffffffffULL;

// Fold a key into max/min, NaNs skipped (integer compares only).
__device__ __forceinline__ void keys_add(long long& mx, long long& mn, long long k) {
  const long long kx = k > KEY_PINF ? LLONG_MIN : k;  // a positive NaN never wins max
  const long long kn = k < KEY_NINF ? LLONG_MAX : k;  // a negative NaN never wins min
  mx = kx > mx ? kx : mx;
  mn = kn < mn ? kn : mn;
}

// Fold one value into a thread's accumulator (two FP64 operations; the keys on the integer pipe).
__device__ __forceinline__ void acc4_add(Acc4& a, double v) {
  a.s += v;
  a.q = fma(v, v, a.q);
  keys_add(a.mx, a.mn, order_key(v));
}

// out = {sum, max, min, norm} of the partial accumulators (one block).
__global__ void __launch_bounds__(256) reduce4_final_kernel(const Acc4* __restrict__ partials, int n,
                                                                    double* __restrict__ out) {
  Acc4 a{0.0, 0.0, 0.0, 0.0, LLONG_MIN, LLONG_MAX};
  for (int i = threadIdx.x; i < n; i += blockDim.x) merge4(a, partials[i]);
  a = block_reduce4(a);
  if (threadIdx.x == 0) {
    out[0] = a.s + a.sc;
    out[1] = a.mx == LLONG_MIN ? -INFINITY : from_key(a.mx);
    out[2] = a.mn == LLONG_MAX ? INFINITY : from_key(a.mn);
    out[3] = sqrt(a.q + a.qc);
  }
}

}  // namespace
}  // namespace nebo
