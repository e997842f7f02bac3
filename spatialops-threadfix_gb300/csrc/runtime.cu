// Runtime part of the C ABI: status text, per-thread error messages, device selection,
// stream-ordered allocation and copies, descriptor validation, and the host-side ghost
// bookkeeping (calculate_actual_ghost, spatialops/NeboBasic.h:61-100).
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "common.cuh"

namespace nebo {

static thread_local char g_last_error[1024] = "";

int fail(int status, const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(g_last_error, sizeof(g_last_error), fmt, ap);
  va_end(ap);
  return status;
}

int cuda_fail(cudaError_t e, const char* where) {
  if (e == cudaSuccess) return NEBO_OK;
  if (e == cudaErrorMemoryAllocation) return fail(NEBO_ERR_ALLOC, "Nebo error in %s: %s", where, cudaGetErrorString(e));
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver)
    return fail(NEBO_ERR_NO_DEVICE, "Nebo error in %s: %s", where, cudaGetErrorString(e));
  return fail(NEBO_ERR_LAUNCH, "Nebo error in %s: %s", where, cudaGetErrorString(e));
}

int check_field(const nebo_field* f, const char* what) {
  if (!f) return fail(NEBO_ERR_INVALID, "Nebo error in %s: null field descriptor", what);
  if (!f->data) return fail(NEBO_ERR_INVALID, "Nebo error in %s: field has no device memory", what);
  if (f->dtype != NEBO_F64 && f->dtype != NEBO_F32)
    return fail(NEBO_ERR_INVALID, "Nebo error in %s: unknown dtype %d", what, f->dtype);
  for (int i = 0; i < 3; ++i) {
    if (f->glob[i] < 1 || f->extent[i] < 1 || f->offset[i] < 0 || f->offset[i] + f->extent[i] > f->glob[i])
      return fail(NEBO_ERR_INVALID, "Nebo error in %s: window outside allocation on axis %d", what, i);
    if (f->ghost_minus[i] < 0 || f->ghost_plus[i] < 0 || f->ghost_minus[i] + f->ghost_plus[i] >= f->extent[i] + (f->extent[i] == 1))
      return fail(NEBO_ERR_INVALID, "Nebo error in %s: ghosts do not fit the window on axis %d", what, i);
  }
  return NEBO_OK;
}

int check_same_layout(const nebo_field* a, const nebo_field* b, const char* what) {
  for (int i = 0; i < 3; ++i)
    if (a->glob[i] != b->glob[i] || a->extent[i] != b->extent[i] || a->offset[i] != b->offset[i] ||
        a->ghost_minus[i] != b->ghost_minus[i] || a->ghost_plus[i] != b->ghost_plus[i])
      return fail(NEBO_ERR_INVALID, "Nebo error in %s: fields differ in shape or ghosts", what);
  if (a->dtype != b->dtype) return fail(NEBO_ERR_INVALID, "Nebo error in %s: fields differ in dtype", what);
  return NEBO_OK;
}

int check_periodic_patch(const nebo_field* f, int g, const char* what) {
  for (int i = 0; i < 3; ++i) {
    if (f->ghost_minus[i] != g || f->ghost_plus[i] != g)
      return fail(NEBO_ERR_INVALID, "Nebo error in %s: needs %d ghost layer(s) on every face", what, g);
    if (f->bc_extra[i] != 0 || f->has_bc[i] != 0)
      return fail(NEBO_ERR_INVALID, "Nebo error in %s: periodic patch cannot carry BC cells", what);
    if (f->offset[i] != 0 || f->extent[i] != f->glob[i])
      return fail(NEBO_ERR_INVALID, "Nebo error in %s: window must cover the allocation", what);
    if (f->extent[i] - 2 * g < (g > 2 ? g : 2))
      return fail(NEBO_ERR_INVALID, "Nebo error in %s: periodic interior needs at least max(2, ghosts) cells", what);
  }
  return NEBO_OK;
}


void pool_retain() {
  static std::atomic<unsigned long long> done{0};  // one bit per device (first 64)
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return;
  if (done.load() & (1ull << dev)) return;
  cudaMemPool_t pool;
  unsigned long long thr = ~0ull;
  cudaError_t e = cudaDeviceGetDefaultMemPool(&pool, dev);
  if (e == cudaSuccess) e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  if (e != cudaSuccess) cudaGetLastError();  // not fatal: allocations still work, only slower
  done.fetch_or(1ull << dev);
}
}  // namespace nebo

using namespace nebo;

extern "C" {

const char* nebo_status_string(int s) {
  switch (s) {
    case NEBO_OK: return "ok";
    case NEBO_ERR_INVALID: return "invalid argument";
    case NEBO_ERR_GHOST: return "not enough valid ghost cells";
    case NEBO_ERR_ALLOC: return "device allocation failed";
    case NEBO_ERR_LAUNCH: return "kernel launch or CUDA runtime error";
    case NEBO_ERR_TIMEOUT: return "bounded device wait timed out";
    case NEBO_ERR_UNSUPPORTED: return "unsupported";
    case NEBO_ERR_NO_DEVICE: return "no CUDA device";
  }
  return "unknown status";
}

const char* nebo_last_error(void) { return g_last_error; }

int nebo_device_count(int* count) {
  if (!count) return fail(NEBO_ERR_INVALID, "Nebo error in nebo_device_count: null pointer");
  int n = 0;
  cudaError_t e = cudaGetDeviceCount(&n);
  if (e != cudaSuccess) {
    *count = 0;
    cudaGetLastError();
    return cuda_fail(e, "nebo_device_count");
  }
  *count = n;
  return NEBO_OK;
}


int nebo_device_init(int device) {
  int n = 0;
  int rc = nebo_device_count(&n);
  if (rc) return rc;
  if (device < 0 || device >= n) return fail(NEBO_ERR_NO_DEVICE, "Nebo error in nebo_device_init: device %d of %d", device, n);
  NEBO_CUDA_TRY(cudaSetDevice(device));
  NEBO_CUDA_TRY(cudaFree(0));
  return NEBO_OK;
}

int nebo_alloc(size_t bytes, void** ptr, nebo_stream_t stream) {
  if (!ptr) return fail(NEBO_ERR_INVALID, "Nebo error in nebo_alloc: null output pointer");
  *ptr = nullptr;
  if (bytes == 0) return NEBO_OK;
  nebo::pool_retain();
  NEBO_CUDA_TRY(cudaMallocAsync(ptr, bytes, (cudaStream_t)stream));
  return NEBO_OK;
}

int nebo_free(void* ptr, nebo_stream_t stream) {
  if (!ptr) return NEBO_OK;
  NEBO_CUDA_TRY(cudaFreeAsync(ptr, (cudaStream_t)stream));
  return NEBO_OK;
}

int nebo_memcpy_h2d(void* dst, const void* src, size_t bytes, nebo_stream_t stream) {
  if (bytes && (!dst || !src)) return fail(NEBO_ERR_INVALID, "Nebo error in nebo_memcpy_h2d: null pointer");
  NEBO_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, (cudaStream_t)stream));
  return NEBO_OK;
}

int nebo_memcpy_d2h(void* dst, const void* src, size_t bytes, nebo_stream_t stream) {
  if (bytes && (!dst || !src)) return fail(NEBO_ERR_INVALID, "Nebo error in nebo_memcpy_d2h: null pointer");
  NEBO_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, (cudaStream_t)stream));
  return NEBO_OK;
}

int nebo_memcpy_d2d(void* dst, const void* src, size_t bytes, nebo_stream_t stream) {
  if (bytes && (!dst || !src)) return fail(NEBO_ERR_INVALID, "Nebo error in nebo_memcpy_d2d: null pointer");
  NEBO_CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToDevice, (cudaStream_t)stream));
  return NEBO_OK;
}

int nebo_memset(void* dst, int byte, size_t bytes, nebo_stream_t stream) {
  if (bytes && !dst) return fail(NEBO_ERR_INVALID, "Nebo error in nebo_memset: null pointer");
  NEBO_CUDA_TRY(cudaMemsetAsync(dst, byte, bytes, (cudaStream_t)stream));
  return NEBO_OK;
}

int nebo_stream_sync(nebo_stream_t stream) {
  NEBO_CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
  unsigned int timeouts = 0, more = 0;
  int rc = nebo::bulk_wait_timeouts(&timeouts);
  if (rc) return rc;
  if ((rc = nebo::patch_wait_timeouts(&more))) return rc;
  timeouts += more;
  if ((rc = nebo::transport_wait_timeouts(&more))) return rc;
  timeouts += more;
  if (timeouts)
    return nebo::fail(NEBO_ERR_TIMEOUT, "Nebo error in nebo_stream_sync: %u bounded device wait(s) gave up", timeouts);
  return NEBO_OK;
}

// calculate_actual_ghost + the limits of NeboField<Initial>::assign.
int nebo_write_limits(const nebo_field* lhs, int use_ghost, const int32_t rhs_minus[3], const int32_t rhs_plus[3],
                      int32_t limits[6]) {
  if (!lhs || !rhs_minus || !rhs_plus || !limits) return fail(NEBO_ERR_INVALID, "Nebo error in nebo_write_limits: null pointer");
  static const char* axis[3] = {"X", "Y", "Z"};
  int extra[3], lg_m[3], lg_p[3];
  for (int i = 0; i < 3; ++i) {
    // BC extra cells exist only on axes of extent > 1 that have a boundary
    extra[i] = (lhs->has_bc[i] && lhs->extent[i] != 1) ? lhs->bc_extra[i] : 0;
    lg_m[i] = lhs->extent[i] <= 1 ? 0 : lhs->ghost_minus[i];
    lg_p[i] = lhs->extent[i] <= 1 ? 0 : lhs->ghost_plus[i];
    if (lhs->has_bc[i] && rhs_plus[i] < extra[i])
      return fail(NEBO_ERR_GHOST,
                  "Nebo error in Nebo Ghost Checking:\nNot enough valid extra cells to validate all interior cells in the %s direction",
                  axis[i]);
  }
  for (int i = 0; i < 3; ++i) {
    int gm, gp;
    if (use_ghost) {
      gm = rhs_minus[i] < lg_m[i] ? rhs_minus[i] : lg_m[i];
      gp = rhs_plus[i] < lg_p[i] + extra[i] ? rhs_plus[i] : lg_p[i] + extra[i];
    } else {
      gm = 0;
      gp = extra[i];
    }
    gp -= extra[i];
    const int n = lhs->extent[i] - lg_m[i] - lg_p[i];
    limits[2 * i] = -gm;
    limits[2 * i + 1] = n + gp;
  }
  return NEBO_OK;
}

}  // extern "C"
