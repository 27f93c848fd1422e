// Host thread pool stress: several callers run parallel loops of varying sizes at once
// (as concurrent proofs of a batch do); every item must run exactly once per loop.
#include "../../flock_gb300/csrc/host/parallel.h"
#include <atomic>
#include <cstdio>
#include <thread>
#include <vector>

int main() {
  using flock::parallel_for;
  const int callers = 4, loops = 300;
  std::atomic<int> failures{0};
  std::vector<std::thread> ts;
  for (int c = 0; c < callers; ++c) {
    ts.emplace_back([&, c] {
      for (int k = 0; k < loops; ++k) {
        const size_t n = (size_t)((k * 37 + c * 11) % 1500);
        std::vector<std::atomic<uint32_t>> hits(n);
        for (auto& h : hits) h.store(0);
        parallel_for(n, [&](size_t i) { hits[i].fetch_add(1, std::memory_order_relaxed); });
        for (size_t i = 0; i < n; ++i)
          if (hits[i].load() != 1) { failures.fetch_add(1); break; }
        // a loop issued from inside a loop item (nested use) must also complete
        if (k % 50 == 0) {
          std::atomic<uint64_t> sum{0};
          parallel_for(8, [&](size_t i) {
            parallel_for(100, [&](size_t j) { sum.fetch_add(i * 100 + j, std::memory_order_relaxed); });
          });
          if (sum.load() != 799ull * 800 / 2) failures.fetch_add(1);
        }
      }
    });
  }
  for (auto& t : ts) t.join();
  printf("workers %zu failures %d\n", flock::ThreadPool::instance().workers(), failures.load());
  return failures.load() == 0 ? 0 : 1;
}
