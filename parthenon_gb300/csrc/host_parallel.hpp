// Host-side parallel loop over independent items (table building on the host cores).
//
// A remesh builds its tables in a few parallel loops of a millisecond or two each, so
// the workers are created once and kept: a loop wakes them, they take chunks of items
// from a shared counter, and the caller works alongside. The pool is never destroyed
// (its workers sleep until process exit).
#pragma once

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstdint>
#include <exception>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

#include <unistd.h>

namespace pgb {

class HostPool {
 public:
  static HostPool &get() {
    static HostPool *p = new HostPool();  // intentionally never deleted
    return *p;
  }
  int workers() const { return (int)threads_.size(); }

  // Runs f(i) for i in [0, n) on the pool and the calling thread; rethrows the first
  // exception. A second caller while a loop runs does its loop inline.
  void run(int n, const std::function<void(int)> &f) {
    // a forked child has none of the workers; another thread's loop keeps the pool
    std::unique_lock<std::mutex> busy(run_mu_, std::defer_lock);
    if (getpid() != pid_ || threads_.empty() || !busy.try_lock()) {
      for (int i = 0; i < n; ++i) f(i);
      return;
    }
    {
      std::lock_guard<std::mutex> lk(mu_);
      job_ = &f;
      n_ = n;
      next_.store(0);
      err_ = nullptr;
      pending_ = (int)threads_.size();
      ++gen_;
    }
    cv_.notify_all();
    work();
    std::unique_lock<std::mutex> lk(mu_);
    done_cv_.wait(lk, [&] { return pending_ == 0; });
    job_ = nullptr;
    if (err_) std::rethrow_exception(err_);
  }

 private:
  HostPool() : pid_(getpid()) {
    const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
    const int nw = std::min(hw, 32) - 1;
    for (int t = 0; t < nw; ++t) {
      threads_.emplace_back([this] { loop(); });
      threads_.back().detach();
    }
  }
  void work() {
    const std::function<void(int)> *f = job_;
    try {
      for (;;) {
        const int s = next_.fetch_add(16);
        if (s >= n_) break;
        const int e = std::min(n_, s + 16);
        for (int i = s; i < e; ++i) (*f)(i);
      }
    } catch (...) {
      std::lock_guard<std::mutex> lk(mu_);
      if (!err_) err_ = std::current_exception();
      next_.store(n_);
    }
  }
  void loop() {
    uint64_t seen = 0;
    for (;;) {
      {
        std::unique_lock<std::mutex> lk(mu_);
        cv_.wait(lk, [&] { return gen_ != seen; });
        seen = gen_;
      }
      work();
      std::lock_guard<std::mutex> lk(mu_);
      if (--pending_ == 0) done_cv_.notify_one();
    }
  }

  const pid_t pid_;
  std::vector<std::thread> threads_;
  std::mutex run_mu_, mu_;
  std::condition_variable cv_, done_cv_;
  const std::function<void(int)> *job_ = nullptr;
  int n_ = 0;
  std::atomic<int> next_{0};
  int pending_ = 0;
  uint64_t gen_ = 0;
  std::exception_ptr err_;
};

// Set while this thread runs a pool loop: a loop inside a loop runs inline (one flag
// for every instantiation of parallel_for).
inline bool &in_pool_loop() {
  thread_local bool inside = false;
  return inside;
}

// Runs f(i) for i in [0, n); loops of fewer than 128 items run inline.
template <class F>
void parallel_for(int n, F &&f) {
  bool &inside = in_pool_loop();
  if (n < 128 || inside) {
    for (int i = 0; i < n; ++i) f(i);
    return;
  }
  const std::function<void(int)> fn = [&f](int i) { f(i); };
  inside = true;
  try {
    HostPool::get().run(n, fn);
  } catch (...) {
    inside = false;
    throw;
  }
  inside = false;
}

}  // namespace pgb
