// Batched and served proving: many independent proofs in flight on one GPU.
//
// A pool of host workers each drives its own GpuBackend (own CUDA stream, own device
// buffers) per statement shape, so the kernels and round trips of different proofs
// overlap on the device: most of a small proof's time is latency (one round trip per
// sumcheck round), which other proofs' kernels fill. Requests are admitted against a
// device-memory budget: a worker takes a request only when the backend it needs is
// already cached or fits in the budget next to everything else held; idle cached backends
// of other shapes are evicted first. Results are byte-identical to one prove_fast call.
//
// Admission is first fit over the queue in arrival order, with aging: a request that later
// requests have overtaken MAX_BYPASS times becomes a barrier, and nothing behind it is
// admitted until it is, so a large request (a Keccak-f 2^18 proof needs about 35 GB) is not
// starved by a stream of small ones. Statements (and their device-byte estimates) are
// built by the submitting thread, and evicted backends are released by the worker that
// evicted them after it leaves the engine lock, so neither a statement build nor a
// cudaFree stalls the other workers' round trips.
#include "../../../include/flock_gb300.h"
#include "backend.h"
#include <condition_variable>
#include <deque>
#include <list>
#include <memory>
#include <thread>
#include <unordered_map>

using namespace flock;

namespace flock {
std::shared_ptr<Statement> statement_for_shape(HashKind h, uint32_t n);  // capi.cu
std::vector<uint8_t> make_bundle(const ProveResult& R);                 // capi.cu
void set_last_error(const std::string& msg);
}  // namespace flock

namespace {

struct Job {
  uint64_t ticket = 0;
  int hash = 0;
  uint64_t n = 0;
  std::vector<uint8_t> inputs;
  std::vector<uint8_t> domain;
  double t_submit = 0;
  std::shared_ptr<Statement> stmt;  // built at submission, outside the engine lock
  uint64_t need = 0;                // device bytes of a new backend of this shape
  uint32_t bypassed = 0;            // times a later request was admitted before this one
  // result
  bool done = false;
  int status = 0;
  std::string error;
  std::vector<uint8_t> bundle;
  double latency_ms = 0;
};

struct CachedBackend {
  std::shared_ptr<Statement> stmt;
  std::unique_ptr<gpu::GpuBackend> backend;
  uint64_t bytes = 0;
  bool busy = false;
  uint64_t last_use = 0;
};

class Engine {
 public:
  Engine(uint64_t budget, int workers) : budget_(budget) {
    CUDA_OK(cudaGetDevice(&device_));
    if (workers < 1) workers = 1;
    for (int i = 0; i < workers; ++i) threads_.emplace_back([this] { loop(); });
  }
  ~Engine() {
    {
      std::lock_guard<std::mutex> g(mu_);
      stop_ = true;
    }
    cv_.notify_all();
    for (auto& t : threads_) t.join();
  }

  uint64_t submit(std::shared_ptr<Job> j) {
    j->stmt = statement_for_shape((HashKind)j->hash, (uint32_t)j->n);
    j->need = gpu::GpuBackend::estimate_device_bytes(*j->stmt);
    std::lock_guard<std::mutex> g(mu_);
    j->ticket = ++next_ticket_;
    j->t_submit = now_ms();
    jobs_[j->ticket] = j;
    queue_.push_back(j);
    cv_.notify_all();
    return j->ticket;
  }
  // Waits up to wait_ms (negative: forever) for a ticket; returns the job when done.
  std::shared_ptr<Job> wait(uint64_t ticket, int wait_ms) {
    std::unique_lock<std::mutex> g(mu_);
    auto it = jobs_.find(ticket);
    if (it == jobs_.end()) return nullptr;
    auto j = it->second;
    auto pred = [&] { return j->done; };
    if (wait_ms < 0) done_cv_.wait(g, pred);
    else done_cv_.wait_for(g, std::chrono::milliseconds(wait_ms), pred);
    if (j->done) jobs_.erase(ticket);
    return j;
  }

 private:
  using Key = std::pair<int, uint64_t>;
  struct KeyHash {
    size_t operator()(const Key& k) const { return std::hash<uint64_t>()(k.second * 4 + (uint64_t)k.first); }
  };

  // Picks the first queued job whose backend is available (cached idle, or admissible
  // within the budget after evicting idle backends), in arrival order; an aged job (see
  // MAX_BYPASS) stops the scan. Evicted backends move to `evicted` for the caller to
  // release outside the lock. Called with mu_ held.
  static constexpr uint32_t MAX_BYPASS = 4;
  std::shared_ptr<Job> take(CachedBackend*& cb, bool& create, uint64_t& need,
                            std::vector<std::unique_ptr<CachedBackend>>& evicted) {
    for (auto it = queue_.begin(); it != queue_.end(); ++it) {
      auto j = *it;
      auto admit = [&]() {
        for (auto b = queue_.begin(); b != it; ++b) (*b)->bypassed++;
        queue_.erase(it);
        return j;
      };
      Key key{j->hash, j->n};
      auto& lst = cache_[key];
      for (auto& c : lst)
        if (!c->busy) {
          cb = c.get();
          create = false;
          return admit();
        }
      need = j->need;
      if (held_ + reserved_ + need > budget_) {
        // evict only when that admits this job: idle backends (least recently used first)
        // until it fits, or all of them when it then runs alone
        uint64_t idle = 0;
        for (auto& kv : cache_)
          for (auto& c : kv.second)
            if (!c->busy) idle += c->bytes;
        const uint64_t after = held_ - idle + reserved_;
        if (after + need > budget_ && after != 0) {
          if (j->bypassed >= MAX_BYPASS) break;  // aged: wait for room rather than admit around it
          continue;
        }
      }
      while (held_ + reserved_ + need > budget_) {
        CachedBackend* victim = nullptr;
        Key vkey;
        for (auto& kv : cache_)
          for (auto& c : kv.second)
            if (!c->busy && (!victim || c->last_use < victim->last_use)) {
              victim = c.get();
              vkey = kv.first;
            }
        if (!victim) break;
        auto& vl = cache_[vkey];
        for (auto vi = vl.begin(); vi != vl.end(); ++vi)
          if (vi->get() == victim) {
            held_ -= victim->bytes;
            evicted.push_back(std::move(*vi));
            vl.erase(vi);
            break;
          }
      }
      reserved_ += need;
      create = true;
      return admit();
    }
    return nullptr;
  }

  void loop() {
    CUDA_OK(cudaSetDevice(device_));
    for (;;) {
      std::shared_ptr<Job> j;
      CachedBackend* cb = nullptr;
      bool create = false;
      uint64_t need = 0;
      std::vector<std::unique_ptr<CachedBackend>> evicted;
      {
        std::unique_lock<std::mutex> g(mu_);
        cv_.wait(g, [&] {
          if (stop_) return true;
          j = take(cb, create, need, evicted);
          return j != nullptr;
        });
        if (stop_ && !j) return;
        if (!create) {
          cb->busy = true;
          cb->last_use = ++clock_;
        }
      }
      // device memory of evicted backends is released here, outside the lock and before this
      // worker allocates the admitted job's backend
      evicted.clear();
      try {
        if (create) {
          auto owned = std::make_unique<CachedBackend>();
          owned->stmt = j->stmt;
          owned->backend = std::make_unique<gpu::GpuBackend>(*owned->stmt);
          owned->busy = true;
          std::lock_guard<std::mutex> g(mu_);
          cb = owned.get();
          cb->bytes = need;
          cb->last_use = ++clock_;
          reserved_ -= need;
          held_ += need;
          cache_[Key{j->hash, j->n}].push_back(std::move(owned));
        }
        cb->backend->begin_prove(nullptr);
        ProveResult R = prove_fast(*cb->stmt, *cb->backend, j->inputs.data(), j->domain.data(), j->domain.size());
        j->bundle = make_bundle(R);
        j->status = FLOCK_GB300_OK;
      } catch (const std::exception& e) {
        std::string w = e.what();
        j->status = w.rfind("CUDA error", 0) == 0 ? FLOCK_GB300_ECUDA : FLOCK_GB300_EINTERNAL;
        j->error = w;
        if (create && !cb) {
          std::lock_guard<std::mutex> g(mu_);
          reserved_ -= need;
        }
      }
      {
        std::lock_guard<std::mutex> g(mu_);
        if (cb) cb->busy = false;
        j->latency_ms = now_ms() - j->t_submit;
        j->done = true;
        j->inputs.clear();
        j->inputs.shrink_to_fit();
      }
      done_cv_.notify_all();
      cv_.notify_all();
    }
  }

  uint64_t budget_;
  int device_ = 0;
  std::mutex mu_;
  std::condition_variable cv_, done_cv_;
  std::deque<std::shared_ptr<Job>> queue_;
  std::unordered_map<uint64_t, std::shared_ptr<Job>> jobs_;
  std::unordered_map<Key, std::list<std::unique_ptr<CachedBackend>>, KeyHash> cache_;
  uint64_t held_ = 0, reserved_ = 0, clock_ = 0, next_ticket_ = 0;
  bool stop_ = false;
  std::vector<std::thread> threads_;
};

int check_request(const flock_gb300_request* r) {
  if (!r) return FLOCK_GB300_EINVAL;
  if (r->hash_kind < 0 || r->hash_kind > 2) return FLOCK_GB300_EINVAL;
  if (r->n_blocks < 8 || (r->n_blocks & (r->n_blocks - 1)) || r->n_blocks > (uint64_t(1) << 24)) return FLOCK_GB300_EINVAL;
  if (!r->inputs || (!r->domain && r->domain_len)) return FLOCK_GB300_EINVAL;
  return FLOCK_GB300_OK;
}

std::shared_ptr<Job> make_job(const flock_gb300_request* r) {
  auto j = std::make_shared<Job>();
  j->hash = r->hash_kind;
  j->n = r->n_blocks;
  size_t bytes = r->n_blocks * input_record_bytes((HashKind)r->hash_kind);
  j->inputs.assign(static_cast<const uint8_t*>(r->inputs), static_cast<const uint8_t*>(r->inputs) + bytes);
  j->domain.assign(r->domain, r->domain + r->domain_len);
  return j;
}

void fill_result(const Job& j, flock_gb300_result* out) {
  out->status = j.status;
  out->bundle = nullptr;
  out->bundle_len = 0;
  out->latency_ms = j.latency_ms;
  if (j.status == FLOCK_GB300_OK) {
    out->bundle = static_cast<uint8_t*>(malloc(j.bundle.size()));
    if (!out->bundle) {
      out->status = FLOCK_GB300_EINTERNAL;
      return;
    }
    memcpy(out->bundle, j.bundle.data(), j.bundle.size());
    out->bundle_len = j.bundle.size();
  }
}

// Submits every request (larger proofs first: the small ones fill in around them) and
// waits for all; results[i] answers reqs[i].
int run_batch(Engine& e, const flock_gb300_request* reqs, size_t n, flock_gb300_result* results) {
  for (size_t i = 0; i < n; ++i)
    if (check_request(&reqs[i]) != FLOCK_GB300_OK) {
      set_last_error("invalid request " + std::to_string(i));
      return FLOCK_GB300_EINVAL;
    }
  std::vector<size_t> order(n);
  for (size_t i = 0; i < n; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](size_t x, size_t y) {
    return (reqs[x].n_blocks << (2 * reqs[x].hash_kind)) > (reqs[y].n_blocks << (2 * reqs[y].hash_kind));
  });
  std::vector<uint64_t> tickets(n);
  for (size_t i : order) tickets[i] = e.submit(make_job(&reqs[i]));
  int rc = FLOCK_GB300_OK;
  for (size_t i = 0; i < n; ++i) {
    auto j = e.wait(tickets[i], -1);
    fill_result(*j, &results[i]);
    if (results[i].status != FLOCK_GB300_OK && rc == FLOCK_GB300_OK) {
      rc = results[i].status;
      set_last_error(j->error);
    }
  }
  return rc;
}

}  // namespace

struct flock_gb300_server {
  std::unique_ptr<Engine> engine;
};

extern "C" {

int flock_gb300_prove_batch(const flock_gb300_request* reqs, size_t n, int workers, uint64_t hbm_budget_bytes,
                            flock_gb300_result* results) {
  if ((!reqs && n) || (!results && n)) return FLOCK_GB300_EINVAL;
  try {
    Engine e(hbm_budget_bytes, workers);
    return run_batch(e, reqs, n, results);
  } catch (const std::exception& ex) {
    set_last_error(ex.what());
    return FLOCK_GB300_ECUDA;
  }
}

int flock_gb300_server_new(uint64_t hbm_budget_bytes, int workers, flock_gb300_server** out) {
  if (!out) return FLOCK_GB300_EINVAL;
  try {
    auto s = std::make_unique<flock_gb300_server>();
    s->engine = std::make_unique<Engine>(hbm_budget_bytes, workers);
    *out = s.release();
    return FLOCK_GB300_OK;
  } catch (const std::exception& ex) {
    set_last_error(ex.what());
    return FLOCK_GB300_ECUDA;
  }
}

int flock_gb300_server_submit(flock_gb300_server* s, const flock_gb300_request* req, uint64_t* ticket) {
  if (!s || !ticket) return FLOCK_GB300_EINVAL;
  if (check_request(req) != FLOCK_GB300_OK) {
    set_last_error("invalid request");
    return FLOCK_GB300_EINVAL;
  }
  *ticket = s->engine->submit(make_job(req));
  return FLOCK_GB300_OK;
}

int flock_gb300_server_poll(flock_gb300_server* s, uint64_t ticket, int wait_ms, flock_gb300_result* result) {
  if (!s || !result) return FLOCK_GB300_EINVAL;
  auto j = s->engine->wait(ticket, wait_ms);
  if (!j) {
    set_last_error("unknown ticket");
    return FLOCK_GB300_EINVAL;
  }
  if (!j->done) return FLOCK_GB300_PENDING;
  fill_result(*j, result);
  if (result->status != FLOCK_GB300_OK) set_last_error(j->error);
  return FLOCK_GB300_OK;
}

int flock_gb300_server_prove_batch(flock_gb300_server* s, const flock_gb300_request* reqs, size_t n,
                                   flock_gb300_result* results) {
  if (!s || (!reqs && n) || (!results && n)) return FLOCK_GB300_EINVAL;
  try {
    return run_batch(*s->engine, reqs, n, results);
  } catch (const std::exception& ex) {
    set_last_error(ex.what());
    return FLOCK_GB300_ECUDA;
  }
}

void flock_gb300_server_free(flock_gb300_server* s) { delete s; }

}  // extern "C"
