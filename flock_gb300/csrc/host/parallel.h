// A small persistent host thread pool for the O(m * 2^k)-sized prover work that stays on
// the host (the Frobenius multipoint assist, the linearised ring-switch coefficients).
// Several callers may run jobs at once (concurrent proofs of a batch): jobs queue, idle
// workers take items from the oldest job first, and every caller also works on its own
// job. Sums over GF(2^k) are XORs, so splitting a sum across threads gives the same bits
// in any order.
#pragma once
#include <algorithm>
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

  // Runs fn(i) for i in [0, n) and returns when all have finished.
  void run(size_t n, const std::function<void(size_t)>& fn) {
    if (n == 0) return;
    if (n == 1 || threads_.empty()) {
      for (size_t i = 0; i < n; ++i) fn(i);
      return;
    }
    auto job = std::make_shared<Job>();
    job->fn = &fn;
    job->n = n;
    {
      std::lock_guard<std::mutex> g(mu_);
      jobs_.push_back(job);
    }
    cv_.notify_all();
    work_on(*job);
    std::unique_lock<std::mutex> g(job->m);
    job->cv.wait(g, [&] { return job->done.load() == n; });
  }

  ~ThreadPool() {
    {
      std::lock_guard<std::mutex> g(mu_);
      stop_ = true;
    }
    cv_.notify_all();
    for (auto& t : threads_) t.join();
  }

 private:
  struct Job {
    const std::function<void(size_t)>* fn = nullptr;
    size_t n = 0;
    std::atomic<size_t> next{0}, done{0};
    std::mutex m;
    std::condition_variable cv;
  };

  ThreadPool() {
    unsigned hc = std::thread::hardware_concurrency();
    unsigned n = hc > 2 ? std::min(hc - 2, 15u) : 0u;
    for (unsigned i = 0; i < n; ++i) threads_.emplace_back([this] { loop(); });
  }
  static void work_on(Job& j) {
    for (;;) {
      size_t i = j.next.fetch_add(1);
      if (i >= j.n) return;
      (*j.fn)(i);
      if (j.done.fetch_add(1) + 1 == j.n) {
        std::lock_guard<std::mutex> g(j.m);
        j.cv.notify_all();
      }
    }
  }
  void loop() {
    for (;;) {
      std::shared_ptr<Job> job;
      {
        std::unique_lock<std::mutex> g(mu_);
        cv_.wait(g, [&] { return stop_ || !jobs_.empty(); });
        if (stop_) return;
        job = jobs_.front();
        if (job->next.load() >= job->n) {  // every item taken: retire it from the queue
          jobs_.pop_front();
          continue;
        }
      }
      work_on(*job);
    }
  }

  std::vector<std::thread> threads_;
  std::mutex mu_;
  std::condition_variable cv_;
  std::deque<std::shared_ptr<Job>> jobs_;
  bool stop_ = false;
};

inline void parallel_for(size_t n, const std::function<void(size_t)>& fn) { ThreadPool::instance().run(n, fn); }

}  // namespace flock
