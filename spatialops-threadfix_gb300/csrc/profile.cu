// Launch accounting and per-kernel CUDA-event timing (the library's tracing hook; the reference
// has NEBO_REPORT_BACKEND prints and TimeLogger wall-clock timers, spatialops/NeboLhs.h:321-392,
// util/TimeLogger.h:85-263).  Every kernel launch site counts itself; when profiling is on,
// it also brackets the launch with events on its own stream, and nebo_profile_report() sums the
// elapsed times per kernel name.
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"

namespace nebo {
namespace {
std::atomic<unsigned long long> g_launches{0};
std::atomic<int> g_profile_on{0};
std::mutex g_prof_mu;
struct Rec {
  std::string name;
  cudaEvent_t a, b;
};
std::vector<Rec> g_pending;
struct Agg {
  unsigned long long launches = 0;
  double ms = 0.0;
};
std::map<std::string, Agg> g_agg;
}  // namespace

LaunchScope::LaunchScope(const char* name, cudaStream_t s) : name_(name), s_(s), a_(nullptr), b_(nullptr) {
  g_launches.fetch_add(1, std::memory_order_relaxed);
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (g_profile_on.load(std::memory_order_relaxed) && cudaStreamIsCapturing(s_, &cs) == cudaSuccess &&
      cs == cudaStreamCaptureStatusNone) {
    if (cudaEventCreate((cudaEvent_t*)&a_) == cudaSuccess && cudaEventCreate((cudaEvent_t*)&b_) == cudaSuccess) {
      cudaEventRecord((cudaEvent_t)a_, s_);
    } else {
      a_ = b_ = nullptr;
    }
  }
}

LaunchScope::~LaunchScope() {
  if (a_ && b_) {
    cudaEventRecord((cudaEvent_t)b_, s_);
    std::lock_guard<std::mutex> g(g_prof_mu);
    g_pending.push_back(Rec{name_, (cudaEvent_t)a_, (cudaEvent_t)b_});
  }
}

}  // namespace nebo

using namespace nebo;

extern "C" unsigned long long nebo_kernel_launch_count(void) { return g_launches.load(); }

extern "C" int nebo_profile_enable(int on) {
  g_profile_on.store(on ? 1 : 0);
  return NEBO_OK;
}

extern "C" int nebo_profile_report(char* buf, size_t len, int reset) {
  std::lock_guard<std::mutex> g(g_prof_mu);
  for (Rec& r : g_pending) {
    float ms = 0.f;
    if (cudaEventSynchronize(r.b) == cudaSuccess && cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) {
      Agg& a = g_agg[r.name];
      a.launches += 1;
      a.ms += ms;
    }
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  g_pending.clear();
  std::string s = "{";
  bool first = true;
  char tmp[256];
  for (auto& kv : g_agg) {
    std::snprintf(tmp, sizeof(tmp), "%s\"%s\": {\"launches\": %llu, \"ms\": %.6f}", first ? "" : ", ", kv.first.c_str(),
                  kv.second.launches, kv.second.ms);
    s += tmp;
    first = false;
  }
  s += "}";
  if (reset) g_agg.clear();
  if (buf && len) {
    std::strncpy(buf, s.c_str(), len - 1);
    buf[len - 1] = 0;
  }
  return s.size() + 1 > len ? NEBO_ERR_INVALID : NEBO_OK;
}
