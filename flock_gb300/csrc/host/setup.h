// Per-statement setup of prove_fast: the hash's block R1CS, its single-slot union
// registry and digest, the committed geometry and the Ligerito configuration —
// the work of Blake3Setup / Sha256HybridSetup / KeccakSetup ::new
// (crates/flock-prover/src/r1cs_hashes/blake3.rs:1589-1652, sha2.rs:1185-1268,
// keccak.rs:847-909) and PcsParams (crates/flock-core/src/pcs/commit.rs:32-300).
#pragma once
#include "field.h"
#include "statement.h"
#include "r1cs_blake3.h"
#include "r1cs_sha2.h"
#include "r1cs_keccak.h"
#include "ligerito_configs.h"
#include <memory>
#include <stdexcept>
#include <string>

namespace flock {

enum HashKind : int { HASH_BLAKE3 = 0, HASH_SHA256 = 1, HASH_KECCAK = 2 };

inline size_t input_record_bytes(HashKind h) {
  switch (h) {
    case HASH_BLAKE3: return sizeof(b3r1cs::Compression);  // cv[8] m[16] u64 counter u32 blen u32 flags = 112
    case HASH_SHA256: return sizeof(s2r1cs::Compression);  // h[8] w[16] = 96
    case HASH_KECCAK: return 25 * 8;                       // 25 state words = 200
  }
  return 0;
}
static_assert(sizeof(b3r1cs::Compression) == 112, "BLAKE3 input record is 112 bytes");
static_assert(sizeof(s2r1cs::Compression) == 96, "SHA-256 input record is 96 bytes");

// Stratified query schedule (crates/flock-core/src/pcs/stratified.rs:70-140).
struct LevelSchedule {
  uint32_t log_block_len = 0;
  std::vector<uint32_t> depths;  // summand stratum depths, descending
  static LevelSchedule decompose(uint32_t q, uint32_t log_block) {
    LevelSchedule s;
    s.log_block_len = log_block;
    uint32_t rem = q;
    while (rem) {
      uint32_t c = 31 - (uint32_t)__builtin_clz(rem);
      if (c > log_block) c = log_block;
      s.depths.push_back(c);
      rem -= 1u << c;
    }
    return s;
  }
  uint32_t cap_depth() const { return depths.empty() ? 0 : depths[0]; }
  uint32_t queries() const { uint32_t n = 0; for (auto c : depths) n += 1u << c; return n; }
};

struct LigeritoParams {
  uint32_t initial_k = 0, log_n = 0, r = 0;          // r = recursive steps
  std::vector<uint32_t> log_inv_rates, recursive_ks, recursive_log_msg_cols, queries, grinding_bits,
      claim_bits, consistency_bits, ood_samples;
  uint32_t initial_log_msg_cols = 0;
  std::vector<LevelSchedule> sched;
};

inline LigeritoParams ligerito_params_for(uint32_t m) {
  int n = 0;
  const LigeritoFastConfig* t = ligerito_fast_configs(&n);
  for (int i = 0; i < n; ++i) {
    if (t[i].m != m) continue;
    const LigeritoFastConfig& c = t[i];
    LigeritoParams p;
    p.initial_k = c.initial_k;
    p.log_n = c.log_n;
    p.r = c.n_levels - 1;
    p.initial_log_msg_cols = c.levels[0].log_msg_cols;
    for (uint32_t l = 0; l < c.n_levels; ++l) {
      const LigeritoLevelParams& L = c.levels[l];
      p.log_inv_rates.push_back(L.log_inv_rate);
      p.queries.push_back(L.queries);
      p.grinding_bits.push_back(L.grinding_bits);
      p.claim_bits.push_back(L.claim_batch_grinding_bits);
      p.consistency_bits.push_back(L.consistency_batch_grinding_bits);
      p.ood_samples.push_back(L.ood_samples);
      if (L.fold_grinding_bits != 0) throw std::runtime_error("fold grinding is not used by the Fast profile");
      if (l >= 1) { p.recursive_ks.push_back(L.k_recursive); p.recursive_log_msg_cols.push_back(L.log_msg_cols); }
    }
    // level block logs (stratified.rs:171-188)
    std::vector<uint32_t> blog;
    blog.push_back(p.initial_log_msg_cols + p.log_inv_rates[0]);
    for (uint32_t l = 0; l < p.r; ++l) blog.push_back(p.recursive_log_msg_cols[l] + p.log_inv_rates[l + 1]);
    for (uint32_t l = 0; l <= p.r; ++l) p.sched.push_back(LevelSchedule::decompose(p.queries[l], blog[l]));
    return p;
  }
  throw std::runtime_error("no Ligerito Fast configuration for m=" + std::to_string(m));
}

// Everything a prove of `n_blocks` instances of `hash` needs besides the inputs.
struct Statement {
  HashKind hash = HASH_BLAKE3;
  uint32_t n_blocks = 0;     // declared count (= 2^nu: full utilisation)
  uint32_t k_log = 0, nu = 0, m = 0;
  uint64_t useful_bits = 0;
  uint32_t const_pin = 0;
  UnionGeometry geo;
  uint32_t log_batch = 0, lanes = 0, log_dim = 0, k_code = 0;
  LigeritoParams lig;
  std::array<uint8_t, 32> registry_digest{};
  // Matrices: BLAKE3 / SHA-256 materialise (A_0, B_0); Keccak uses the walker.
  std::shared_ptr<SparseRows> a0, b0;
  std::shared_ptr<Csc> csc_a, csc_b;
};

inline uint32_t log2_exact(uint64_t n) {
  uint32_t l = 0;
  while ((uint64_t(1) << l) < n) ++l;
  if ((uint64_t(1) << l) != n) throw std::runtime_error("size must be a power of two");
  return l;
}

struct MatrixCache {
  std::shared_ptr<SparseRows> a, b;
  std::shared_ptr<Csc> ca, cb;
};
inline MatrixCache& matrices_for(HashKind h) {
  static MatrixCache cache[3];
  MatrixCache& c = cache[h];
  if (!c.a && h != HASH_KECCAK) {
    c.a = std::make_shared<SparseRows>();
    c.b = std::make_shared<SparseRows>();
    if (h == HASH_BLAKE3) b3r1cs::build_matrices(*c.a, *c.b);
    else s2r1cs::build_matrices(*c.a, *c.b);
    c.ca = std::make_shared<Csc>(csc_from_rows(*c.a));
    c.cb = std::make_shared<Csc>(csc_from_rows(*c.b));
  }
  return c;
}

// Builds the statement. Only full-utilisation counts (n_blocks a power of two, >= 8)
// are supported: every shipped configuration and every power-of-two batch is one.
inline Statement make_statement(HashKind h, uint32_t n_blocks) {
  if (n_blocks < 8 || (n_blocks & (n_blocks - 1)))
    throw std::runtime_error("n_blocks must be a power of two >= 8");
  Statement s;
  s.hash = h;
  s.n_blocks = n_blocks;
  s.nu = log2_exact(n_blocks);
  switch (h) {
    case HASH_BLAKE3: s.k_log = b3r1cs::K_LOG; s.useful_bits = b3r1cs::USEFUL_BITS; s.const_pin = b3r1cs::Z_CONST_POS; break;
    case HASH_SHA256: s.k_log = s2r1cs::K_LOG; s.useful_bits = s2r1cs::USEFUL_BITS; s.const_pin = s2r1cs::Z_CONST_POS; break;
    case HASH_KECCAK: s.k_log = kr1cs::K_LOG; s.useful_bits = kr1cs::USEFUL_BITS; s.const_pin = kr1cs::Z_CONST; break;
  }
  s.m = s.k_log + s.nu;
  s.geo = union_geometry(s.k_log, s.useful_bits, s.nu);
  if (!s.geo.identity) throw std::runtime_error("only identity-compaction (full utilisation) shapes are supported");
  s.lig = ligerito_params_for(s.geo.dense_m);
  s.log_batch = s.lig.initial_k;
  s.lanes = s.geo.commit_lanes(s.log_batch);
  s.log_dim = s.geo.dense_m - 7 - s.log_batch;
  s.k_code = s.log_dim + 1;
  if (s.lig.log_n != s.geo.dense_m - 7 || s.lig.initial_log_msg_cols != s.log_dim)
    throw std::runtime_error("Ligerito configuration does not match the committed geometry");
  if (h != HASH_KECCAK) {
    MatrixCache& mc = matrices_for(h);
    s.a0 = mc.a; s.b0 = mc.b; s.csc_a = mc.ca; s.csc_b = mc.cb;
  }
  return s;
}

// Registry digest of the single-slot registry (computed once per statement; the
// matrices make it a few hundred MB of BLAKE3 input).
inline void compute_registry_digest(Statement& s) {
  TableType ty;
  ty.k_log = s.k_log;
  ty.useful_bits = s.useful_bits;
  ty.const_pin = s.const_pin;
  ty.c0_identity = true;
  if (s.hash == HASH_KECCAK) { ty.a0 = &kr1cs::empty_stub(); ty.b0 = &kr1cs::empty_stub(); }
  else { ty.a0 = s.a0.get(); ty.b0 = s.b0.get(); }
  s.registry_digest = registry_digest(s.nu, {ty});
}

}  // namespace flock
