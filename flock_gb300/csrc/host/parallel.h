// A small persistent host thread pool for the O(m * 2^k)-sized prover work that stays on
// the host (the Frobenius multipoint assist). Sums over GF(2^k) are XORs, so splitting a
// sum across threads gives the same bits in any order.
#pragma once
#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <functional>
#include <mutex>
#include <thread>
#include <vector>

namespace flock {

class ThreadPool {
 public:
  static ThreadPool& instance() {
    static ThreadPool pool;
    return pool;
  }
  size_t workers() const { return threads_.size(); }

  // Runs fn(i) for i in [0, n); the caller takes part. If the pool is already running a
  // job for another caller, the tasks run inline on the calling thread.
  void run(size_t n, const std::function<void(size_t)>& fn) {
    if (n == 0) return;
    std::unique_lock<std::mutex> busy(busy_, std::try_to_lock);
    if (!busy.owns_lock() || threads_.empty() || n == 1) {
      for (size_t i = 0; i < n; ++i) fn(i);
      return;
    }
    {
      std::lock_guard<std::mutex> g(mu_);
      fn_ = &fn;
      n_ = n;
      next_.store(0);
      active_ = threads_.size();
      ++gen_;
    }
    cv_.notify_all();
    work();
    std::unique_lock<std::mutex> g(mu_);
    done_cv_.wait(g, [&] { return active_ == 0; });
    fn_ = nullptr;
  }

  ~ThreadPool() {
    {
      std::lock_guard<std::mutex> g(mu_);
      stop_ = true;
      ++gen_;
    }
    cv_.notify_all();
    for (auto& t : threads_) t.join();
  }

 private:
  ThreadPool() {
    unsigned hc = std::thread::hardware_concurrency();
    unsigned n = hc > 2 ? std::min(hc - 2, 15u) : 0u;
    for (unsigned i = 0; i < n; ++i) threads_.emplace_back([this] { loop(); });
  }
  void work() {
    for (;;) {
      size_t i = next_.fetch_add(1);
      if (i >= n_) break;
      (*fn_)(i);
    }
  }
  void loop() {
    uint64_t seen = 0;
    for (;;) {
      {
        std::unique_lock<std::mutex> g(mu_);
        cv_.wait(g, [&] { return gen_ != seen; });
        seen = gen_;
        if (stop_) return;
      }
      work();
      std::lock_guard<std::mutex> g(mu_);
      if (--active_ == 0) done_cv_.notify_all();
    }
  }

  std::vector<std::thread> threads_;
  std::mutex mu_, busy_;
  std::condition_variable cv_, done_cv_;
  const std::function<void(size_t)>* fn_ = nullptr;
  size_t n_ = 0;
  std::atomic<size_t> next_{0};
  size_t active_ = 0;
  uint64_t gen_ = 0;
  bool stop_ = false;
};

inline void parallel_for(size_t n, const std::function<void(size_t)>& fn) { ThreadPool::instance().run(n, fn); }

}  // namespace flock
