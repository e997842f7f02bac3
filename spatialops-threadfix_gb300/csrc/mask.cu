// SpatialMask bit words from a point list (spatialops/structured/BitField.h:291-333,
// SpatialMask.h:99-181): bit (flat % 32) of word (flat / 32), flat = x + gx*(y + gy*z) in the
// ghosted window with the window's interior offset added to each interior-relative point.
// Points of one word may come from different threads, so bits are set with atomicOr.
#include "common.cuh"

namespace nebo {
namespace {

__global__ void mask_from_points_kernel(uint32_t* __restrict__ words, int gx, int gy, int gz, int ox, int oy, int oz,
                                        const int32_t* __restrict__ pts, int npts, int* __restrict__ bad) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < npts; i += gridDim.x * blockDim.x) {
    const int x = ox + pts[3 * i], y = oy + pts[3 * i + 1], z = oz + pts[3 * i + 2];
    if (x < 0 || x >= gx || y < 0 || y >= gy || z < 0 || z >= gz) {
      atomicExch(bad, 1);  // out-of-window point: skipped and reported
      continue;
    }
    const long flat = (long)x + (long)gx * (y + (long)gy * z);
    atomicOr(words + flat / 32, 1u << (flat % 32));
  }
}

}  // namespace
}  // namespace nebo

using namespace nebo;

extern "C" int nebo_mask_from_points(uint32_t* words, const int32_t glob[3], const int32_t offset[3],
                                     const int32_t* points, int32_t npoints, nebo_stream_t stream) {
  if (!words || !glob || !offset || (npoints > 0 && !points))
    return fail(NEBO_ERR_INVALID, "Nebo error in nebo_mask_from_points: null pointer");
  if (npoints < 0) return fail(NEBO_ERR_INVALID, "Nebo error in nebo_mask_from_points: negative point count");
  if (npoints == 0) return NEBO_OK;
  cudaStream_t s = (cudaStream_t)stream;
  int* bad = nullptr;
  pool_retain();
  NEBO_CUDA_TRY(cudaMallocAsync((void**)&bad, sizeof(int), s));
  NEBO_CUDA_TRY(cudaMemsetAsync(bad, 0, sizeof(int), s));
  const int threads = 256;
  int blocks = (npoints + threads - 1) / threads;
  if (blocks > num_sms() * 8) blocks = num_sms() * 8;
  {
    LaunchScope ls("mask_from_points", s);
    mask_from_points_kernel<<<blocks, threads, 0, s>>>(words, glob[0], glob[1], glob[2], offset[0], offset[1], offset[2],
                                                     points, npoints, bad);
  }
  cudaError_t le = cudaGetLastError();
  int hbad = 0;
  cudaError_t ce = cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, s);
  cudaFreeAsync(bad, s);
  if (le != cudaSuccess) return cuda_fail(le, "nebo_mask_from_points");
  if (ce != cudaSuccess) return cuda_fail(ce, "nebo_mask_from_points copy");
  NEBO_CUDA_TRY(cudaStreamSynchronize(s));
  if (hbad) return fail(NEBO_ERR_INVALID, "Nebo error in nebo_mask_from_points: a point lies outside the mask window");
  return NEBO_OK;
}
