// host_parallel.h -- the host loops of the batched caller-side entry points (align_pairs,
// align_chains) split over threads.  Each item's work is independent and writes only its own
// outputs, so results do not depend on the thread count.
#pragma once
#include <stdint.h>
#include <stdlib.h>

#include <algorithm>
#include <thread>
#include <vector>

namespace ksw2g {

// KSW2G_HOST_THREADS, else the hardware threads (at most 64)
inline int host_threads() {
  static const int n = [] {
    const char *s = getenv("KSW2G_HOST_THREADS");
    int v = s ? atoi(s) : (int)std::thread::hardware_concurrency();
    return std::max(1, std::min(v, 64));
  }();
  return n;
}

// f(lo, hi) over [0, n) in contiguous ranges of at least `grain` items, one per thread
template <class F>
void parallel_for(int64_t n, int64_t grain, F &&f) {
  if (n <= 0) return;
  const int64_t nt = std::min<int64_t>(host_threads(), (n + grain - 1) / std::max<int64_t>(grain, 1));
  if (nt <= 1) {
    f((int64_t)0, n);
    return;
  }
  std::vector<std::thread> th;
  th.reserve(nt - 1);
  for (int64_t t = 1; t < nt; ++t) th.emplace_back([&f, t, nt, n] { f(n * t / nt, n * (t + 1) / nt); });
  f((int64_t)0, n / nt);
  for (std::thread &x : th) x.join();
}

}  // namespace ksw2g
