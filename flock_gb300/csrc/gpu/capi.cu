// extern "C" entry points declared in include/flock_gb300.h.
#include "../../../include/flock_gb300.h"
#include "backend.h"
#include "../host/proof_io.h"
#include <cstdlib>
#include <map>
#include <memory>
#include <mutex>

using namespace flock;

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg) {
  g_last_error = msg;
  return code;
}

}  // namespace

namespace flock {
// Statements are shared by every setup of the same (kind, n_blocks): building the
// matrices and the registry digest is the expensive part of Setup::new.
std::shared_ptr<Statement> statement_for_shape(HashKind h, uint32_t n) {
  static std::mutex mu;
  static std::map<std::pair<int, uint32_t>, std::shared_ptr<Statement>> cache;
  std::lock_guard<std::mutex> g(mu);
  auto key = std::make_pair((int)h, n);
  auto it = cache.find(key);
  if (it != cache.end()) return it->second;
  auto s = std::make_shared<Statement>(make_statement(h, n));
  compute_registry_digest(*s);
  cache[key] = s;
  return s;
}
// u64 proof_len | bincode proof | u64 cap_len | cap | ab_value | c_value
std::vector<uint8_t> make_bundle(const ProveResult& R) {
  Bincode bc;
  bc.u64(0);  // proof length, patched below
  bc.merged(R.proof);
  Bincode::put64(bc.out.data(), bc.out.size() - 8);
  bc.vh(R.cap);
  bc.f128(R.claims.ab_value);
  bc.f128(R.claims.c_value);
  return std::move(bc.out);
}
}  // namespace flock

namespace {

template <class F>
int guarded(F&& f) {
  try {
    return f();
  } catch (const std::invalid_argument& e) {
    return fail(FLOCK_GB300_EINVAL, e.what());
  } catch (const std::runtime_error& e) {
    std::string w = e.what();
    return fail(w.rfind("CUDA error", 0) == 0 ? FLOCK_GB300_ECUDA : FLOCK_GB300_EINTERNAL, w);
  } catch (const std::exception& e) {
    return fail(FLOCK_GB300_EINTERNAL, e.what());
  } catch (...) {
    return fail(FLOCK_GB300_EINTERNAL, "unknown error");
  }
}

}  // namespace

namespace flock {
void set_last_error(const std::string& msg) { g_last_error = msg; }
}  // namespace flock

struct flock_gb300_setup {
  std::shared_ptr<Statement> stmt;
  std::unique_ptr<gpu::GpuBackend> backend;
  std::mutex mu;
  ProveTimings last;
};

extern "C" {

size_t flock_gb300_input_record_bytes(int hash_kind) {
  if (hash_kind < 0 || hash_kind > 2) return 0;
  return input_record_bytes((HashKind)hash_kind);
}

int flock_gb300_setup_new(int hash_kind, uint64_t n_blocks, flock_gb300_setup** out) {
  g_last_error.clear();
  if (!out) return fail(FLOCK_GB300_EINVAL, "null output pointer");
  *out = nullptr;
  if (hash_kind < 0 || hash_kind > 2) return fail(FLOCK_GB300_EINVAL, "unknown hash kind");
  if (n_blocks < 8 || (n_blocks & (n_blocks - 1)) || n_blocks > (uint64_t(1) << 24))
    return fail(FLOCK_GB300_EINVAL, "n_blocks must be a power of two in [8, 2^24]");
  return guarded([&] {
    auto s = std::make_unique<flock_gb300_setup>();
    s->stmt = statement_for_shape((HashKind)hash_kind, (uint32_t)n_blocks);
    s->backend = std::make_unique<gpu::GpuBackend>(*s->stmt);
    *out = s.release();
    return FLOCK_GB300_OK;
  });
}

void flock_gb300_setup_free(flock_gb300_setup* setup) { delete setup; }

int flock_gb300_setup_info(const flock_gb300_setup* setup, uint32_t* m, uint32_t* lanes, uint32_t* log_code_len,
                           uint8_t digest[32]) {
  if (!setup) return fail(FLOCK_GB300_EINVAL, "null setup");
  if (m) *m = setup->stmt->m;
  if (lanes) *lanes = setup->stmt->lanes;
  if (log_code_len) *log_code_len = setup->stmt->k_code;
  if (digest) memcpy(digest, setup->stmt->registry_digest.data(), 32);
  return FLOCK_GB300_OK;
}

static int prove_common(flock_gb300_setup* setup, const void* inputs, const void* d_inputs, size_t n_inputs,
                        const uint8_t* domain, size_t domain_len, uint8_t** out, size_t* out_len) {
  g_last_error.clear();
  if (!setup || !(inputs || d_inputs) || !out || !out_len || (!domain && domain_len))
    return fail(FLOCK_GB300_EINVAL, "null argument");
  *out = nullptr;
  *out_len = 0;
  if (n_inputs != setup->stmt->n_blocks)
    return fail(FLOCK_GB300_EINVAL, "input count " + std::to_string(n_inputs) + " != setup n_blocks " +
                                        std::to_string(setup->stmt->n_blocks));
  return guarded([&] {
    std::lock_guard<std::mutex> g(setup->mu);
    CUDA_OK(cudaSetDevice(setup->backend->device()));
    setup->backend->begin_prove(d_inputs);
    ProveResult R = prove_fast(*setup->stmt, *setup->backend, static_cast<const uint8_t*>(inputs), domain, domain_len);
    setup->last = R.t;
    std::vector<uint8_t> bundle = make_bundle(R);
    size_t len = bundle.size();
    uint8_t* buf = static_cast<uint8_t*>(malloc(len));
    if (!buf) return fail(FLOCK_GB300_EINTERNAL, "out of host memory");
    memcpy(buf, bundle.data(), len);
    *out = buf;
    *out_len = len;
    return FLOCK_GB300_OK;
  });
}

int flock_gb300_prove_fast(flock_gb300_setup* setup, const void* inputs, size_t n_inputs, const uint8_t* domain,
                           size_t domain_len, uint8_t** out, size_t* out_len) {
  return prove_common(setup, inputs, nullptr, n_inputs, domain, domain_len, out, out_len);
}

int flock_gb300_prove_fast_device(flock_gb300_setup* setup, const void* d_inputs, size_t n_inputs,
                                  const uint8_t* domain, size_t domain_len, uint8_t** out, size_t* out_len) {
  if (!d_inputs) return fail(FLOCK_GB300_EINVAL, "null device inputs");
  return prove_common(setup, nullptr, d_inputs, n_inputs, domain, domain_len, out, out_len);
}

int flock_gb300_setup_stream(const flock_gb300_setup* setup, void** stream) {
  if (!setup || !stream) return fail(FLOCK_GB300_EINVAL, "null argument");
  *stream = (void*)setup->backend->stream();
  return FLOCK_GB300_OK;
}

int flock_gb300_set_stage_timing(flock_gb300_setup* setup, uint32_t stage_mask) {
  if (!setup) return fail(FLOCK_GB300_EINVAL, "null setup");
  std::lock_guard<std::mutex> g(setup->mu);
  setup->backend->set_stage_timing(stage_mask);
  return FLOCK_GB300_OK;
}

int flock_gb300_last_stage_ms(flock_gb300_setup* setup, double* ms, uint32_t* launches, int cap) {
  if (!setup) return fail(FLOCK_GB300_EINVAL, "null setup");
  return guarded([&] {
    std::lock_guard<std::mutex> g(setup->mu);
    double t[gpu::GpuBackend::ST_COUNT];
    uint32_t l[gpu::GpuBackend::ST_COUNT];
    setup->backend->stage_ms(t, l);
    for (int i = 0; i < cap && i < gpu::GpuBackend::ST_COUNT; ++i) {
      if (ms) ms[i] = t[i];
      if (launches) launches[i] = l[i];
    }
    return (int)gpu::GpuBackend::ST_COUNT;
  });
}

const char* flock_gb300_stage_name(int stage) { return gpu::GpuBackend::stage_name(stage); }

int flock_gb300_last_transfer_bytes(const flock_gb300_setup* setup, uint64_t* h2d, uint64_t* d2h) {
  if (!setup) return fail(FLOCK_GB300_EINVAL, "null setup");
  if (h2d) *h2d = setup->backend->h2d_bytes();
  if (d2h) *d2h = setup->backend->d2h_bytes();
  return FLOCK_GB300_OK;
}

uint64_t flock_gb300_launch_count(void) { return gpu::launch_count(); }

int flock_gb300_last_phase_ms(const flock_gb300_setup* setup, double out[8]) {
  if (!setup || !out) return fail(FLOCK_GB300_EINVAL, "null argument");
  const ProveTimings& t = setup->last;
  out[0] = t.witness; out[1] = t.commit; out[2] = t.zerocheck; out[3] = t.lincheck; out[4] = t.open; out[5] = t.total;
  out[6] = t.assist; out[7] = t.assist_wait;
  return FLOCK_GB300_OK;
}

void flock_gb300_free(uint8_t* p) { free(p); }

int flock_gb300_proof_io(int hash_kind, uint64_t n_blocks, const uint8_t* bundle, size_t bundle_len, uint8_t** out,
                         size_t* out_len) {
  g_last_error.clear();
  if (!bundle || !out || !out_len) return fail(FLOCK_GB300_EINVAL, "null argument");
  if (hash_kind < 0 || hash_kind > 2) return fail(FLOCK_GB300_EINVAL, "unknown hash kind");
  if (n_blocks < 8 || (n_blocks & (n_blocks - 1)) || n_blocks > (uint64_t(1) << 24))
    return fail(FLOCK_GB300_EINVAL, "n_blocks must be a power of two in [8, 2^24]");
  *out = nullptr;
  *out_len = 0;
  return guarded([&] {
    auto st = statement_for_shape((HashKind)hash_kind, (uint32_t)n_blocks);
    std::vector<uint8_t> v = proof_io_from_bundle(*st, bundle, bundle_len);
    uint8_t* buf = static_cast<uint8_t*>(malloc(v.size()));
    if (!buf) return fail(FLOCK_GB300_EINTERNAL, "out of host memory");
    memcpy(buf, v.data(), v.size());
    *out = buf;
    *out_len = v.size();
    return FLOCK_GB300_OK;
  });
}

int flock_gb300_estimate_device_bytes(int hash_kind, uint64_t n_blocks, uint64_t* bytes) {
  g_last_error.clear();
  if (!bytes) return fail(FLOCK_GB300_EINVAL, "null argument");
  if (hash_kind < 0 || hash_kind > 2) return fail(FLOCK_GB300_EINVAL, "unknown hash kind");
  if (n_blocks < 8 || (n_blocks & (n_blocks - 1)) || n_blocks > (uint64_t(1) << 24))
    return fail(FLOCK_GB300_EINVAL, "n_blocks must be a power of two in [8, 2^24]");
  return guarded([&] {
    *bytes = gpu::GpuBackend::estimate_device_bytes(*statement_for_shape((HashKind)hash_kind, (uint32_t)n_blocks));
    return FLOCK_GB300_OK;
  });
}

}  // extern "C"

struct flock_gb300_union_setup {
  std::vector<HashKind> kinds;  // slot order
  uint32_t nu = 0;
  std::array<uint8_t, 32> digest{};
  std::mutex mu;
  struct Prover {
    std::shared_ptr<Statement> stmt;
    std::unique_ptr<gpu::GpuBackend> backend;
  };
  std::map<std::vector<uint64_t>, Prover> provers;  // per counts vector
  std::shared_ptr<Statement> statement(const std::vector<uint64_t>& counts) {
    auto s = std::make_shared<Statement>(make_union_statement(kinds, nu, counts));
    s->registry_digest = digest;
    return s;
  }
};

extern "C" {

int flock_gb300_union_setup_new(const int* hash_kinds, size_t n_types, uint32_t nu, flock_gb300_union_setup** out,
                                int* slot_kinds) {
  g_last_error.clear();
  if (!out || !hash_kinds || !n_types) return fail(FLOCK_GB300_EINVAL, "null argument");
  *out = nullptr;
  if (n_types > 3) return fail(FLOCK_GB300_EINVAL, "at most three hash types");
  if (nu < 3 || nu > 24) return fail(FLOCK_GB300_EINVAL, "nu must be in [3, 24]");
  std::vector<HashKind> kinds;
  for (size_t i = 0; i < n_types; ++i) {
    if (hash_kinds[i] < 0 || hash_kinds[i] > 2) return fail(FLOCK_GB300_EINVAL, "unknown hash kind");
    for (HashKind k : kinds)
      if (k == (HashKind)hash_kinds[i]) return fail(FLOCK_GB300_EINVAL, "registry types must be distinct");
    kinds.push_back((HashKind)hash_kinds[i]);
  }
  return guarded([&] {
    auto u = std::make_unique<flock_gb300_union_setup>();
    for (size_t i : registry_slot_order(kinds)) u->kinds.push_back(kinds[i]);
    u->nu = nu;
    // the registry digest does not depend on the counts
    Statement s = make_union_statement(u->kinds, nu, std::vector<uint64_t>(u->kinds.size(), 0));
    compute_registry_digest(s);
    u->digest = s.registry_digest;
    if (slot_kinds)
      for (size_t i = 0; i < u->kinds.size(); ++i) slot_kinds[i] = (int)u->kinds[i];
    *out = u.release();
    return FLOCK_GB300_OK;
  });
}

void flock_gb300_union_setup_free(flock_gb300_union_setup* setup) { delete setup; }

int flock_gb300_prove_union(flock_gb300_union_setup* setup, const uint64_t* counts, const void* const* inputs,
                            const uint8_t* domain, size_t domain_len, uint8_t** out, size_t* out_len) {
  g_last_error.clear();
  if (!setup || !counts || !inputs || !out || !out_len || (!domain && domain_len))
    return fail(FLOCK_GB300_EINVAL, "null argument");
  *out = nullptr;
  *out_len = 0;
  std::vector<uint64_t> cv(counts, counts + setup->kinds.size());
  for (size_t t = 0; t < cv.size(); ++t) {
    if (cv[t] > (uint64_t(1) << setup->nu)) return fail(FLOCK_GB300_EINVAL, "declared count exceeds 2^nu");
    if (cv[t] && !inputs[t]) return fail(FLOCK_GB300_EINVAL, "null input records for a non-empty slot");
  }
  return guarded([&] {
    std::lock_guard<std::mutex> g(setup->mu);
    auto it = setup->provers.find(cv);
    if (it == setup->provers.end()) {
      if (setup->provers.size() >= 4) setup->provers.erase(setup->provers.begin());
      flock_gb300_union_setup::Prover p;
      p.stmt = setup->statement(cv);
      p.backend = std::make_unique<gpu::GpuBackend>(*p.stmt);
      it = setup->provers.emplace(cv, std::move(p)).first;
    }
    auto& P = it->second;
    CUDA_OK(cudaSetDevice(P.backend->device()));
    P.backend->begin_prove(nullptr);
    std::vector<const uint8_t*> in;
    for (size_t t = 0; t < cv.size(); ++t) in.push_back(static_cast<const uint8_t*>(inputs[t]));
    ProveResult R = prove_fast(*P.stmt, *P.backend, in, domain, domain_len);
    std::vector<uint8_t> bundle = make_bundle(R);
    *out = static_cast<uint8_t*>(malloc(bundle.size()));
    if (!*out) return fail(FLOCK_GB300_EINTERNAL, "out of host memory");
    memcpy(*out, bundle.data(), bundle.size());
    *out_len = bundle.size();
    return FLOCK_GB300_OK;
  });
}

int flock_gb300_mixed_proof_io(const flock_gb300_union_setup* setup, const uint64_t* counts, const uint8_t* bundle,
                               size_t bundle_len, uint8_t** out, size_t* out_len) {
  g_last_error.clear();
  if (!setup || !counts || !bundle || !out || !out_len) return fail(FLOCK_GB300_EINVAL, "null argument");
  return guarded([&] {
    auto u = const_cast<flock_gb300_union_setup*>(setup);
    std::vector<uint64_t> cv(counts, counts + u->kinds.size());
    for (uint64_t c : cv)
      if (c > (uint64_t(1) << u->nu)) return fail(FLOCK_GB300_EINVAL, "declared count exceeds 2^nu");
    auto s = u->statement(cv);
    std::vector<uint8_t> v = mixed_proof_io_from_bundle(*s, bundle, bundle_len);
    *out = static_cast<uint8_t*>(malloc(v.size()));
    if (!*out) return fail(FLOCK_GB300_EINTERNAL, "out of host memory");
    memcpy(*out, v.data(), v.size());
    *out_len = v.size();
    return FLOCK_GB300_OK;
  });
}

int flock_gb300_device_count(void) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) return 0;
  return n;
}

const char* flock_gb300_last_error(void) { return g_last_error.c_str(); }

}  // extern "C"
