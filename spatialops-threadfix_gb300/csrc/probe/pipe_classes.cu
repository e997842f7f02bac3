// Instruction-class throughput probe for this GPU: one kernel per class, four data-dependent
// chains per thread (nothing folds at compile time), one full wave of blocks; prints operations
// per clock per SM.  Run under ncu with the sm__inst_executed_pipe_* metrics to see which pipe
// each class issues on.  Not part of the library build.
#include <cstdio>
#include <cstdint>
#include <cuda_runtime.h>
#define ITERS 2048
template <int OP>
__global__ void __launch_bounds__(256) probe(const uint64_t* __restrict__ in, uint64_t* __restrict__ out) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  uint64_t a0 = in[t & 1023], a1 = in[(t + 1) & 1023], a2 = in[(t + 2) & 1023], a3 = in[(t + 3) & 1023];
  double d0 = (double)(a0 & 0xffff) * 1e-3, d1 = (double)(a1 & 0xffff), d2 = d0 + 2, d3 = d0 + 3;
#pragma unroll 2
  for (int i = 0; i < ITERS; ++i) {
    if (OP == 0) { d0 = d0 + d1; d1 = d1 + d2; d2 = d2 + d3; d3 = d3 + d0; }
    if (OP == 1) { d0 = fma(d0, d1, d2); d1 = fma(d1, d2, d3); d2 = fma(d2, d3, d0); d3 = fma(d3, d0, d1); }
    if (OP == 2) { a0 += a1; a1 += a2; a2 += a3; a3 += a0; }
    if (OP == 3) { a0 = (int64_t)a0 > (int64_t)a1 ? a0 : a2; a1 = (int64_t)a1 > (int64_t)a2 ? a1 : a3;
                   a2 = (int64_t)a2 > (int64_t)a3 ? a2 : a0; a3 = (int64_t)a3 > (int64_t)a0 ? a3 : a1; a0 ^= i; }
    if (OP == 4) { a0 = __umul64hi(a0, a1) ^ a2; a1 = __umul64hi(a1, a2) ^ a3; a2 = __umul64hi(a2, a3) ^ a0; a3 = __umul64hi(a3, a0) ^ a1; }
    if (OP == 5) { a0 = a0 * a1; a1 = a1 * a2; a2 = a2 * a3; a3 = a3 * a0; }
    if (OP == 6) { a0 = (a0 << (a1 & 31)) | 1; a1 = (a1 >> (a2 & 31)) | 2; a2 = (a2 << (a3 & 31)) | 3; a3 = (a3 >> (a0 & 31)) | 4; }
    if (OP == 7) { a0 += __clzll(a1 | 1); a1 += __clzll(a2 | 1); a2 += __clzll(a3 | 1); a3 += __clzll(a0 | 1); }
    if (OP == 8) { d0 = __longlong_as_double(__double_as_longlong((double)((float)d0 + 1.5f)) ^ 1);
                   d1 = __longlong_as_double(__double_as_longlong((double)((float)d1 + 1.5f)) ^ 1); }
    if (OP == 9) { uint32_t x0 = (uint32_t)a0, x1 = (uint32_t)a1; x0 = x0 * x1 + (uint32_t)i; x1 = x1 * x0 + 7u;
                   a0 = x0; a1 = x1; }
    if (OP == 10) { a0 = (a0 & a1) ^ (a2 | 5); a1 = (a1 & a2) ^ (a3 | 6); a2 = (a2 & a3) ^ (a0 | 7); a3 = (a3 & a0) ^ (a1 | 9); }
    if (OP == 11) { uint32_t x0 = (uint32_t)a0, x1 = (uint32_t)a1; a0 = (uint64_t)x0 * x1 + a2; a1 = (uint64_t)x1 * (uint32_t)a0 + a3; }
    if (OP == 12) { int k = (int)a0; d0 = (double)k; a0 = __double_as_longlong(d0) + a1; }
    if (OP == 13) { a0 = (uint64_t)(int64_t)(__double_as_longlong(d0) >> 3) + a1; d0 = (double)(int64_t)a0 * 1e-300; }
  }
  out[t] = a0 + a1 + a2 + a3 + __double_as_longlong(d0 + d1 + d2 + d3);
}
template <int OP>
void run(const char* name, double ops_per_iter, const uint64_t* in, uint64_t* out, int sms) {
  dim3 grid(sms * 8), block(256);
  probe<OP><<<grid, block>>>(in, out);
  cudaEvent_t a, b; cudaEventCreate(&a); cudaEventCreate(&b);
  cudaEventRecord(a);
  probe<OP><<<grid, block>>>(in, out);
  cudaEventRecord(b); cudaEventSynchronize(b);
  float ms; cudaEventElapsedTime(&ms, a, b);
  int clk; cudaDeviceGetAttribute(&clk, cudaDevAttrClockRate, 0);
  double ops = (double)grid.x * block.x * ITERS * ops_per_iter;
  printf("%2d %-22s %8.3f ms %8.2f per clk per SM\n", OP, name, ms, ops / (ms * 1e-3) / (clk * 1e3) / sms);
}
int main() {
  int sms; cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, 0);
  uint64_t *in, *out;
  cudaMalloc(&in, 1024 * 8); cudaMalloc(&out, sizeof(uint64_t) * sms * 8 * 256);
  uint64_t h[1024]; for (int i = 0; i < 1024; ++i) h[i] = 0x9E3779B97F4A7C15ULL * (i + 1);
  cudaMemcpy(in, h, sizeof(h), cudaMemcpyHostToDevice);
  run<0>("DADD", 4, in, out, sms); run<1>("DFMA", 4, in, out, sms); run<2>("IADD64", 4, in, out, sms);
  run<3>("cmp+sel 64", 4, in, out, sms); run<4>("umul64hi+xor", 4, in, out, sms); run<5>("mul64 lo", 4, in, out, sms);
  run<6>("var shift 64 +or", 4, in, out, sms); run<7>("clz64 + add", 4, in, out, sms); run<8>("F2F f64>f32>f64", 2, in, out, sms);
  run<9>("IMAD32", 2, in, out, sms); run<10>("LOP 64", 4, in, out, sms); run<11>("IMAD.WIDE 32x32+64", 2, in, out, sms);
  run<12>("I2F.F64.S32", 1, in, out, sms); run<13>("I2F.F64.S64", 1, in, out, sms);
  cudaError_t e = cudaDeviceSynchronize();
  printf("status %s\n", cudaGetErrorString(e));
  return e == cudaSuccess ? 0 : 1;
}
