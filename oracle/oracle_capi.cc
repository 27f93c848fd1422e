// ORACLE — test infrastructure only. C ABI over the CPU restatement (cpu_backend.h) so
// the Python tests and the benchmark's CPU-baseline leg can run the same prove_fast on
// the host and compare bundles byte for byte. Built as oracle/_build/liboracle.so; the
// product library never links it.
//
// The bundle format is the one of flock_gb300_prove_fast:
//   u64 proof_len | bincode proof | u64 cap_len | cap x 32 | ab_value (16) | c_value (16)
#include "cpu_backend.h"
#include "verifier.h"
#include "../flock_gb300/csrc/host/proof_io.h"
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

static int emit_bundle(const ProveResult& R, uint8_t** out, size_t* out_len) {
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
}

int oracle_prove_fast(int hash_kind, uint64_t n_blocks, const void* inputs, const uint8_t* domain, size_t domain_len,
                      uint8_t** out, size_t* out_len) {
  try {
    auto s = statement_for(hash_kind, (uint32_t)n_blocks);
    oracle::CpuBackend B(*s);
    ProveResult R = prove_fast(*s, B, static_cast<const uint8_t*>(inputs), domain, domain_len);
    return emit_bundle(R, out, out_len);
  } catch (const std::exception& e) {
    g_err = e.what();
    return 1;
  }
}

namespace {
std::shared_ptr<Statement> union_statement_for(const int* kinds, size_t n_types, uint32_t nu, const uint64_t* counts) {
  static std::mutex mu;
  static std::map<std::vector<uint64_t>, std::shared_ptr<Statement>> cache;
  std::vector<uint64_t> key{nu};
  for (size_t i = 0; i < n_types; ++i) { key.push_back((uint64_t)kinds[i]); key.push_back(counts[i]); }
  std::lock_guard<std::mutex> g(mu);
  auto it = cache.find(key);
  if (it != cache.end()) return it->second;
  std::vector<HashKind> types;
  for (size_t i = 0; i < n_types; ++i) types.push_back((HashKind)kinds[i]);
  auto s = std::make_shared<Statement>(make_union_statement(types, nu, std::vector<uint64_t>(counts, counts + n_types)));
  compute_registry_digest(*s);
  cache[key] = s;
  return s;
}
}  // namespace

// prove_fast_ligerito_union (prover.rs:587-620) of a registry given in slot order
// (kinds[t], k_log descending) at row capacity 2^nu, declared counts and per-slot input
// records in slot order. Output: the bundle format above.
int oracle_prove_union(const int* kinds, size_t n_types, uint32_t nu, const uint64_t* counts,
                       const void* const* inputs, const uint8_t* domain, size_t domain_len, uint8_t** out,
                       size_t* out_len) {
  try {
    auto s = union_statement_for(kinds, n_types, nu, counts);
    std::vector<const uint8_t*> in;
    for (size_t i = 0; i < n_types; ++i) in.push_back(static_cast<const uint8_t*>(inputs[i]));
    oracle::CpuBackend B(*s);
    ProveResult R = prove_fast(*s, B, in, domain, domain_len);
    return emit_bundle(R, out, out_len);
  } catch (const std::exception& e) {
    g_err = e.what();
    return 1;
  }
}

// MixedProofBundleLigerito::to_bytes of a union bundle (proof_io.rs:254-282).
int oracle_mixed_proof_io(const int* kinds, size_t n_types, uint32_t nu, const uint64_t* counts, const uint8_t* bundle,
                          size_t len, uint8_t** out, size_t* out_len) {
  try {
    auto s = union_statement_for(kinds, n_types, nu, counts);
    auto v = mixed_proof_io_from_bundle(*s, bundle, len);
    *out = static_cast<uint8_t*>(malloc(v.size()));
    memcpy(*out, v.data(), v.size());
    *out_len = v.size();
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return 1;
  }
}

// Verifies a union bundle for the registry (slot order), nu and counts: 0 = accepted,
// 1 = rejected (reason written), 2 = internal error.
int oracle_verify_union(const int* kinds, size_t n_types, uint32_t nu, const uint64_t* counts, const uint8_t* bundle,
                        size_t len, const uint8_t* domain, size_t domain_len, char* reason, size_t reason_len) {
  auto say = [&](const std::string& m) {
    if (reason && reason_len) {
      size_t n = std::min(reason_len - 1, m.size());
      memcpy(reason, m.data(), n);
      reason[n] = 0;
    }
  };
  try {
    auto s = union_statement_for(kinds, n_types, nu, counts);
    oracle::Bundle b = oracle::parse_bundle(bundle, len);
    oracle::verify_bundle(*s, b, domain, domain_len);
    say("accepted");
    return 0;
  } catch (const oracle::Reject& e) {
    say(e.what());
    return 1;
  } catch (const std::exception& e) {
    g_err = e.what();
    say(std::string("internal error: ") + e.what());
    return 2;
  }
}

void oracle_free(uint8_t* p) { free(p); }

// Verifies a bundle (the format above) for the statement (hash_kind, n_blocks) and the
// transcript domain: 0 = accepted, 1 = rejected (the failed check is written to
// `reason`), 2 = internal error.
int oracle_verify(int hash_kind, uint64_t n_blocks, const uint8_t* bundle, size_t len, const uint8_t* domain,
                  size_t domain_len, char* reason, size_t reason_len) {
  auto say = [&](const std::string& m) {
    if (reason && reason_len) {
      size_t n = std::min(reason_len - 1, m.size());
      memcpy(reason, m.data(), n);
      reason[n] = 0;
    }
  };
  try {
    auto s = statement_for(hash_kind, (uint32_t)n_blocks);
    oracle::Bundle b = oracle::parse_bundle(bundle, len);
    oracle::verify_bundle(*s, b, domain, domain_len);
    say("accepted");
    return 0;
  } catch (const oracle::Reject& e) {
    say(e.what());
    return 1;
  } catch (const std::exception& e) {
    g_err = e.what();
    say(std::string("internal error: ") + e.what());
    return 2;
  }
}

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

// R1CS self-checks of one block per hash on seeded inputs (the encoders' satisfiability
// and, for the walker-based Keccak type, the transpose identity <eq, A z> = <eq^T A, z>
// of the oracle's column folds):
//   out[0] = rows where a != A z, out[1] = rows where b != B z (BLAKE3 / SHA-256, the
//            materialised matrices; Keccak: 0 / 1 walker identity failures),
//   out[2] = rows where a AND b != z (C = I),
//   out[3] = Keccak only: 1 if Keccak-f of the zero state starts with lane 0xf1258f7940e1dde7.
extern "C" int oracle_r1cs_check(int hash_kind, uint64_t seed, uint64_t out[4]) {
  try {
    out[0] = out[1] = out[2] = out[3] = 0;
    uint64_t s = seed;
    auto next = [&]() {
      s += 0x9E3779B97F4A7C15ull;
      uint64_t z = s;
      z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
      z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
      return z ^ (z >> 31);
    };
    auto bit = [](const std::vector<uint64_t>& v, uint32_t i) { return (uint32_t)((v[i >> 6] >> (i & 63)) & 1); };
    if (hash_kind == HASH_KECCAK) {
      const uint32_t K = kr1cs::K;
      std::vector<uint64_t> z(K / 64), a(K / 64), b(K / 64);
      uint64_t w[25] = {0};
      kr1cs::witness_block(w, z.data(), a.data(), b.data());
      out[3] = z[kr1cs::STATE24_BIT_BASE / 64] == 0xf1258f7940e1dde7ull ? 1 : 0;
      for (auto& x : w) x = next();
      std::fill(z.begin(), z.end(), 0); std::fill(a.begin(), a.end(), 0); std::fill(b.begin(), b.end(), 0);
      kr1cs::witness_block(w, z.data(), a.data(), b.data());
      std::vector<F128> eq(K);
      for (auto& e : eq) e = F128(next(), next());
      std::vector<F128> ca, cb;
      oracle::keccak_columns_forward(eq.data(), ca, cb);
      F128 l1, r1, l2, r2;
      for (uint32_t i = 0; i < K; ++i) {
        if (bit(a, i)) l1 += eq[i];
        if (bit(z, i)) r1 += ca[i];
        if (bit(b, i)) l2 += eq[i];
        if (bit(z, i)) r2 += cb[i];
      }
      out[0] = l1 == r1 ? 0 : 1;
      out[1] = l2 == r2 ? 0 : 1;
      for (uint32_t i = 0; i < K; ++i) out[2] += (bit(a, i) & bit(b, i)) != bit(z, i);
      return 0;
    }
    MatrixCache& mc = matrices_for((HashKind)hash_kind);
    const uint32_t K = mc.a->num_rows;
    std::vector<uint64_t> z(K / 64), a(K / 64), b(K / 64);
    if (hash_kind == HASH_BLAKE3) {
      b3r1cs::Compression c;
      for (auto& x : c.cv) x = (uint32_t)next();
      for (auto& x : c.m) x = (uint32_t)next();
      c.counter = next();
      c.block_len = 64;
      c.flags = 11;
      b3r1cs::witness_block(c, z.data(), a.data(), b.data());
    } else {
      s2r1cs::Compression c;
      for (auto& x : c.h) x = (uint32_t)next();
      for (auto& x : c.w) x = (uint32_t)next();
      s2r1cs::witness_block(c, z.data(), a.data(), b.data());
    }
    for (uint32_t r = 0; r < K; ++r) {
      uint32_t pa = 0, pb = 0;
      for (uint32_t col : mc.a->rows[r]) pa ^= bit(z, col);
      for (uint32_t col : mc.b->rows[r]) pb ^= bit(z, col);
      out[0] += pa != bit(a, r);
      out[1] += pb != bit(b, r);
      out[2] += (bit(a, r) & bit(b, r)) != bit(z, r);
    }
    return 0;
  } catch (const std::exception& e) {
    g_err = e.what();
    return 1;
  }
}
