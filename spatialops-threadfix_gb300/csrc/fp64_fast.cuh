// FP64 exp and sin with fewer FP64 instructions, for kernels bound by the FP64 pipe (about 1/60
// of the FP32 rate on this GPU).  Both are table driven, so the polynomials are short:
//
// exp(x)  Tang's method (P. T. P. Tang, "Table-driven implementation of the exponential
//         function in IEEE floating-point arithmetic", ACM TOMS 15(2), 1989):
//           x = (64 m + j) ln2/64 + r,  |r| <= ln2/128,
//           exp(x) = 2^m * 2^(j/64) * exp(r),
//           exp(r) - 1 = r + r^2 (1/2 + r/6 + r^2/24 + r^3/120 + r^4/720)
//         (Taylor; the first omitted term r^7/5040 < 2^-64 relative), 2^(j/64) held as a
//         lead + trail pair, ln2/64 split in two so k*L1 is exact.  |x| >= 700 and NaN go to
//         CUDA's exp.
// sin(x)  x = k pi/64 + r,  |r| <= pi/128 (pi/64 split in three for an exact-enough reduction),
//           sin(x) = S_k cos r + C_k sin r,  S_k, C_k = sin, cos(k pi/64) from a 128-entry table,
//           sin r = r + r^3 (-1/6 + r^2/120 - r^4/5040),  cos r - 1 = r^2 (-1/2 + r^2/24 - r^4/720)
//         (Taylor; omitted terms below 2^-60).  |x| >= 2^20 and non-finite x go to CUDA's sin.
// The tables are computed on the host in long double from the C library (tables_init), the
// coefficients are the Taylor series.  Errors (tests/test_gpu_fastmath.py, against CUDA's exp
// and sin on random and edge inputs): a few tenths of an ulp typical, at most 2 ulp.
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

namespace nebo {
namespace fastmath {

// [0,64): exp lead, [64,128): exp trail, [128,256): sin(k pi/64), [256,384): cos(k pi/64)
static __device__ double g_tables[384];

inline int tables_init() {
  static std::mutex mu;
  static bool done[64] = {false};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 1;
  std::lock_guard<std::mutex> g(mu);
  if (done[dev]) return 0;
  double h[384];
  for (int j = 0; j < 64; ++j) {
    const long double v = std::exp2((long double)j / 64.0L);
    h[j] = (double)v;
    h[64 + j] = (double)(v - (long double)h[j]);
  }
  const long double pi = 3.141592653589793238462643383279502884L;
  for (int k = 0; k < 128; ++k) {
    h[128 + k] = (double)std::sin((long double)k * pi / 64.0L);
    h[256 + k] = (double)std::cos((long double)k * pi / 64.0L);
  }
  // exact values at multiples of pi/2 (a long double pi leaves ~1e-20 residues there, which
  // would dominate the result when sin(x) itself is that small)
  const double q_sin[4] = {0.0, 1.0, 0.0, -1.0}, q_cos[4] = {1.0, 0.0, -1.0, 0.0};
  for (int i = 0; i < 4; ++i) {
    h[128 + 32 * i] = q_sin[i];
    h[256 + 32 * i] = q_cos[i];
  }
  if (cudaMemcpyToSymbol(g_tables, h, sizeof(h)) != cudaSuccess) return 1;
  done[dev] = true;
  return 0;
}

__device__ __forceinline__ double exp_fast(double x) {
  if (!(fabs(x) < 700.0)) return exp(x);
  const double inv_l = 92.33248261689366;            // 64 / ln2
  const double l1 = 0.010830424696905538;            // ln2/64 rounded to 32 significant bits:
                                                     // k*l1 is exact for |k| < 2^21
  const double l2 = -6.563929801064195e-13;          // ln2/64 - l1 (to 2e-29)
  const double shifter = 6755399441055744.0;         // 1.5 * 2^52
  const double t = fma(x, inv_l, shifter);
  const double kd = t - shifter;
  const long long k = __double_as_longlong(t) - __double_as_longlong(shifter);
  double r = fma(-kd, l1, x);
  r = fma(-kd, l2, r);
  double q = fma(r, 1.0 / 720.0, 1.0 / 120.0);
  q = fma(r, q, 1.0 / 24.0);
  q = fma(r, q, 1.0 / 6.0);
  q = fma(r, q, 0.5);
  const double p = fma(r * r, q, r);  // exp(r) - 1
  const int j = (int)(k & 63);
  const long long m = k >> 6;
  const double tl = __ldg(g_tables + j), tt = __ldg(g_tables + 64 + j);
  const double v = tl + fma(tl, p, tt);
  return __longlong_as_double(__double_as_longlong(v) + (m << 52));
}

__device__ __forceinline__ double sin_fast(double x) {
  if (!(fabs(x) < 1048576.0)) return sin(x);
  const double inv_a = 20.371832715762604;           // 64 / pi
  const double a1 = 0.049087385181337595;            // pi/64 in three parts; a1 and a2 carry
  const double a2 = 3.100292418622974e-11;           // 27-bit significands, so k*a1 and k*a2
  const double a3 = 1.7878714769093224e-19;          // are exact for |k| < 2^26 (|x| < 2^20)
  const double shifter = 6755399441055744.0;
  const double t = fma(x, inv_a, shifter);
  const double kd = t - shifter;
  const long long k = __double_as_longlong(t) - __double_as_longlong(shifter);
  double r = fma(-kd, a1, x);
  r = fma(-kd, a2, r);
  r = fma(-kd, a3, r);
  const double r2 = r * r;
  double sp = fma(r2, -1.0 / 5040.0, 1.0 / 120.0);
  sp = fma(r2, sp, -1.0 / 6.0);
  const double sr = fma(r2 * r, sp, r);               // sin r
  double cp = fma(r2, -1.0 / 720.0, 1.0 / 24.0);
  cp = fma(r2, cp, -0.5);
  const double cm1 = r2 * cp;                         // cos r - 1
  const int idx = (int)(k & 127);
  const double sk = __ldg(g_tables + 128 + idx), ck = __ldg(g_tables + 256 + idx);
  return sk + fma(sk, cm1, ck * sr);
}

}  // namespace fastmath
}  // namespace nebo
