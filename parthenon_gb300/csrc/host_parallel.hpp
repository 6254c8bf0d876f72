// Host-side parallel loop over independent items (table building on the host cores).
#pragma once

#include <algorithm>
#include <atomic>
#include <exception>
#include <mutex>
#include <thread>
#include <vector>

namespace pgb {

// Runs f(i) for i in [0, n) on the host's cores (work handed out in chunks of 16). The
// first exception thrown by any f is rethrown on the calling thread. Small n runs
// inline.
template <class F>
void parallel_for(int n, F &&f) {
  const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
  const int nt = std::min({hw, 32, n / 64});
  if (nt <= 1) {
    for (int i = 0; i < n; ++i) f(i);
    return;
  }
  std::atomic<int> next{0};
  std::exception_ptr err;
  std::mutex mu;
  auto work = [&] {
    try {
      for (;;) {
        const int s = next.fetch_add(16);
        if (s >= n) break;
        const int e = std::min(n, s + 16);
        for (int i = s; i < e; ++i) f(i);
      }
    } catch (...) {
      std::lock_guard<std::mutex> lk(mu);
      if (!err) err = std::current_exception();
      next.store(n);
    }
  };
  std::vector<std::thread> th;
  for (int t = 1; t < nt; ++t) th.emplace_back(work);
  work();
  for (auto &t : th) t.join();
  if (err) std::rethrow_exception(err);
}

}  // namespace pgb
