// A small persistent host thread pool for the O(m * 2^k)-sized prover work that stays on
// the host (the Frobenius multipoint assist, the linearised ring-switch coefficients).
// Several callers may run jobs at once (concurrent proofs of a batch): jobs queue, idle
// workers take chunks of items from the oldest job first, and every caller also works on
// its own job. Sums over GF(2^k) are XORs, so splitting a sum across threads gives the same bits
// in any order.
#pragma once
#include <algorithm>
#include <cstdlib>
#include <atomic>
#include <condition_variable>
#include <deque>
#include <functional>
#include <memory>
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

  // Runs fn(i) for i in [0, n) and returns when all have finished. Items are handed out
  // in chunks (a few per participant), so tiny items do not contend on the counters.
  void run(size_t n, const std::function<void(size_t)>& fn) {
    if (n == 0) return;
    if (n == 1 || threads_.empty()) {
      for (size_t i = 0; i < n; ++i) fn(i);
      return;
    }
    auto job = std::make_shared<Job>();
    job->fn = &fn;
    job->n = n;
    job->chunk = std::max<size_t>(1, n / (4 * (threads_.size() + 1)));
    {
      std::lock_guard<std::mutex> g(mu_);
      jobs_.push_back(job);
      gen_.fetch_add(1, std::memory_order_release);
    }
    if (sleepers_.load(std::memory_order_acquire) > 0) cv_.notify_all();
    work_on(*job);
    // the last items are usually microseconds away: spin briefly before blocking
    for (uint32_t i = 0; i < SPIN && job->done.load(std::memory_order_acquire) != n; ++i) {
    }
    if (job->done.load(std::memory_order_acquire) != n) {
      std::unique_lock<std::mutex> g(job->m);
      job->cv.wait(g, [&] { return job->done.load() == n; });
    }
  }

  ~ThreadPool() {
    {
      std::lock_guard<std::mutex> g(mu_);
      stop_ = true;
      gen_.fetch_add(1, std::memory_order_release);
    }
    cv_.notify_all();
    for (auto& t : threads_) t.join();
  }

 private:
  // Idle workers poll for a new job this many times (tens of microseconds) before they
  // sleep on the condition variable: back-to-back parallel loops then start without a
  // wake-up system call.
  static constexpr uint32_t SPIN = 1u << 15;
  struct Job {
    const std::function<void(size_t)>* fn = nullptr;
    size_t n = 0, chunk = 1;
    std::atomic<size_t> next{0}, done{0};
    std::mutex m;
    std::condition_variable cv;
  };

  // Workers: all but two of the host's hardware threads (at most 15), or
  // FLOCK_GB300_HOST_THREADS - 1 when that variable is set (the caller is the last one).
  ThreadPool() {
    unsigned hc = std::thread::hardware_concurrency();
    unsigned n = hc > 2 ? std::min(hc - 2, 15u) : 0u;
    if (const char* e = std::getenv("FLOCK_GB300_HOST_THREADS")) {
      const long v = std::strtol(e, nullptr, 10);
      if (v >= 1 && v <= 256) n = (unsigned)(v - 1);
    }
    for (unsigned i = 0; i < n; ++i) threads_.emplace_back([this] { loop(); });
  }
  static void work_on(Job& j) {
    for (;;) {
      const size_t i = j.next.fetch_add(j.chunk);
      if (i >= j.n) return;
      const size_t e = std::min(j.n, i + j.chunk);
      for (size_t k = i; k < e; ++k) (*j.fn)(k);
      if (j.done.fetch_add(e - i) + (e - i) == j.n) {
        std::lock_guard<std::mutex> g(j.m);
        j.cv.notify_all();
      }
    }
  }
  void loop() {
    uint64_t seen = gen_.load(std::memory_order_acquire);
    for (;;) {
      for (uint32_t i = 0; i < SPIN && gen_.load(std::memory_order_acquire) == seen; ++i) {
      }
      {
        std::unique_lock<std::mutex> g(mu_);
        if (gen_.load(std::memory_order_acquire) == seen) {
          sleepers_.fetch_add(1);
          cv_.wait(g, [&] { return gen_.load(std::memory_order_acquire) != seen; });
          sleepers_.fetch_sub(1);
        }
        if (stop_) return;
        seen = gen_.load(std::memory_order_acquire);
      }
      for (;;) {  // every queued job with items left, oldest first
        std::shared_ptr<Job> job;
        {
          std::lock_guard<std::mutex> g(mu_);
          while (!jobs_.empty() && jobs_.front()->next.load() >= jobs_.front()->n) jobs_.pop_front();
          if (jobs_.empty()) break;
          job = jobs_.front();
        }
        work_on(*job);
      }
    }
  }

  std::vector<std::thread> threads_;
  std::mutex mu_;
  std::condition_variable cv_;
  std::deque<std::shared_ptr<Job>> jobs_;
  std::atomic<uint64_t> gen_{0};
  std::atomic<uint32_t> sleepers_{0};
  bool stop_ = false;
};

inline void parallel_for(size_t n, const std::function<void(size_t)>& fn) { ThreadPool::instance().run(n, fn); }

}  // namespace flock
