#pragma once
#include <thread>
namespace boost {
// The pool's worker threads spin forever; interrupt() is never reached because the
// Threading singleton is never destroyed by the drivers that use this stand-in.
struct thread : std::thread {
  template <class F> explicit thread(F f) : std::thread(f) {}
  void interrupt() {}
};
}
