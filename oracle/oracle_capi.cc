// ORACLE — test infrastructure only. C ABI over the CPU restatement (cpu_backend.h) so
// the Python tests and the benchmark's CPU-baseline leg can run the same prove_fast on
// the host and compare bundles byte for byte. Built as oracle/_build/liboracle.so; the
// product library never links it.
//
// The bundle format is the one of flock_gb300_prove_fast:
//   u64 proof_len | bincode proof | u64 cap_len | cap x 32 | ab_value (16) | c_value (16)
#include "cpu_backend.h"
#include <cstdlib>
#include <map>
#include <memory>
#include <mutex>

using namespace flock;

namespace {
thread_local std::string g_err;

std::shared_ptr<Statement> statement_for(int h, uint32_t n) {
  static std::mutex mu;
  static std::map<std::pair<int, uint32_t>, std::shared_ptr<Statement>> cache;
  std::lock_guard<std::mutex> g(mu);
  auto key = std::make_pair(h, n);
  auto it = cache.find(key);
  if (it != cache.end()) return it->second;
  auto s = std::make_shared<Statement>(make_statement((HashKind)h, n));
  compute_registry_digest(*s);
  cache[key] = s;
  return s;
}
}  // namespace

extern "C" {

const char* oracle_last_error(void) { return g_err.c_str(); }

int oracle_registry_digest(int hash_kind, uint64_t n_blocks, uint8_t out[32]) {
  try {
    auto s = statement_for(hash_kind, (uint32_t)n_blocks);
    memcpy(out, s->registry_digest.data(), 32);
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return 1;
  }
}

// Phase times (ms) of the last oracle prove on this thread: witness, commit, zc, lc, open, total.
thread_local double g_last_ms[6];
int oracle_last_phase_ms(double out[6]) {
  memcpy(out, g_last_ms, sizeof(g_last_ms));
  return 0;
}

int oracle_prove_fast(int hash_kind, uint64_t n_blocks, const void* inputs, const uint8_t* domain, size_t domain_len,
                      uint8_t** out, size_t* out_len) {
  try {
    auto s = statement_for(hash_kind, (uint32_t)n_blocks);
    oracle::CpuBackend B(*s);
    ProveResult R = prove_fast(*s, B, static_cast<const uint8_t*>(inputs), domain, domain_len);
    g_last_ms[0] = R.t.witness; g_last_ms[1] = R.t.commit; g_last_ms[2] = R.t.zerocheck;
    g_last_ms[3] = R.t.lincheck; g_last_ms[4] = R.t.open; g_last_ms[5] = R.t.total;
    std::vector<uint8_t> pb = proof_bytes(R.proof);
    size_t len = 8 + pb.size() + 8 + 32 * R.cap.size() + 32;
    uint8_t* buf = static_cast<uint8_t*>(malloc(len));
    size_t o = 0;
    auto u64 = [&](uint64_t v) { for (int i = 0; i < 8; ++i) buf[o++] = (uint8_t)(v >> (8 * i)); };
    u64(pb.size());
    memcpy(buf + o, pb.data(), pb.size());
    o += pb.size();
    u64(R.cap.size());
    for (auto& h : R.cap) { memcpy(buf + o, h.data(), 32); o += 32; }
    for (F128 v : {R.claims.ab_value, R.claims.c_value}) { u64(v.lo); u64(v.hi); }
    *out = buf;
    *out_len = len;
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return 1;
  }
}

void oracle_free(uint8_t* p) { free(p); }

// Registry digests of the two small registries pinned by
// crates/flock-core/src/schedule.rs:1160-1189 (boolean_only_digest_is_byte_identical):
//   which = 0: types (k_log 10, useful 700), (9, 300), stub matrices, nu = 3
//   which = 1: (10, 700) stub; (9, 300) with A_0 = rows [[0, 3], [7]] x 512 cols, pin 2
int oracle_registry_digest_kat(int which, uint8_t out[32]) {
  static SparseRows a;
  a.num_rows = 2;
  a.num_cols = 512;
  a.rows = {{0, 3}, {7}};
  TableType t0, t1;
  t0.k_log = 10; t0.useful_bits = 700;
  t1.k_log = 9; t1.useful_bits = 300;
  if (which == 1) { t1.a0 = &a; t1.const_pin = 2; }
  auto d = registry_digest(3, {t0, t1});
  memcpy(out, d.data(), 32);
  return 0;
}

}  // extern "C"
