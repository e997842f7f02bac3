#pragma once
#include <atomic>
namespace boost {
using std::atomic;
using std::atomic_thread_fence;
using std::memory_order_acquire;
using std::memory_order_relaxed;
using std::memory_order_release;
}
