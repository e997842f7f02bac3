// Tensor Memory Accelerator (TMA) and mbarrier helpers for sm_103a kernels (inline PTX).
//
// Host: encode a 3-D tiled tensor map of a ghosted window (x fastest) through the driver entry
// point cuTensorMapEncodeTiled, fetched at run time with cudaGetDriverEntryPoint (so the library
// does not link libcuda).  Device: mbarrier init / expect-tx / bounded wait, and
// cp.async.bulk.tensor 3-D loads into shared memory (no cluster multicast).
//
// Every wait is bounded: after NEBO_TMA_SPIN_LIMIT polls a wait gives up and returns false; the
// kernel then records an error code in a device word, drains its own copies (also bounded) and
// returns, so a fault in the copy engine ends the launch with a status instead of a hang.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

#include "common.cuh"

#define NEBO_TMA_SPIN_LIMIT (1u << 24)

namespace nebo {
namespace tma {

// ------------------------------------------------------------------ host
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

inline EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  static bool tried = false;
  if (!tried) {
    tried = true;
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &p, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  }
  return fn;
}

// 3-D map over an allocation of gx*gy*gz elements (x fastest); box = bx*by*bz elements.
// The base must be 16-byte aligned and gx*elem_bytes a multiple of 16 for the strides.
inline int encode_3d(CUtensorMap* map, void* base, int elem_bytes, int gx, int gy, int gz, int bx, int by, int bz) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return fail(NEBO_ERR_UNSUPPORTED, "Nebo error: cuTensorMapEncodeTiled is not available");
  const cuuint64_t dims[3] = {(cuuint64_t)gx, (cuuint64_t)gy, (cuuint64_t)gz};
  const cuuint64_t strides[2] = {(cuuint64_t)gx * elem_bytes, (cuuint64_t)gx * gy * elem_bytes};
  const cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)by, (cuuint32_t)bz};
  const cuuint32_t estr[3] = {1, 1, 1};
  const CUtensorMapDataType dt = elem_bytes == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
  const CUresult r = fn(map, dt, 3, base, dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return fail(NEBO_ERR_INVALID, "Nebo error: tensor map encoding failed (%d)", (int)r);
  return NEBO_OK;
}

// ------------------------------------------------------------------ device
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count));
}

__device__ __forceinline__ void fence_barrier_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t phase) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(phase)
      : "memory");
  return ok != 0;
}

// Wait for the barrier's phase to complete; false if it did not within the spin limit.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t phase) {
  for (uint32_t i = 0; i < NEBO_TMA_SPIN_LIMIT; ++i)
    if (mbar_try_wait(bar, phase)) return true;
  return false;
}

__device__ __forceinline__ void load_3d(void* dst, const CUtensorMap* map, int x, int y, int z, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::
          "r"(smem_addr(dst)),
      "l"(map), "r"(x), "r"(y), "r"(z), "r"(smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ void prefetch_map(const CUtensorMap* map) {
  asm volatile("prefetch.tensormap [%0];" ::"l"(map) : "memory");
}

}  // namespace tma
}  // namespace nebo
