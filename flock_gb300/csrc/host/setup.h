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
#include <algorithm>
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

// One type's slot of a union registry (crates/flock-core/src/schedule.rs:246-270, the
// slot layout of Registry::new :337-468) with this proof's declared count n_t.
struct SlotInfo {
  HashKind hash = HASH_BLAKE3;
  uint32_t k_log = 0;          // block width 2^k_log bits
  uint64_t useful_bits = 0;
  uint32_t const_pin = 0;      // column of the constant-one wire
  uint64_t used_cols = 0;      // leading chunk-columns that carry data
  uint32_t m_slot = 0;         // nu + k_log: the slot's capacity area is 2^m_slot bits
  uint64_t offset = 0;         // slot offset in the union address space (bits), 2^m_slot-aligned
  uint64_t prefix = 0;         // offset >> m_slot
  uint64_t count = 0;          // declared invocations n_t <= 2^nu
  std::shared_ptr<SparseRows> a0, b0;  // materialised A_0, B_0 (BLAKE3 / SHA-256; Keccak: walker)
  std::shared_ptr<Csc> csc_a, csc_b;
  uint64_t col_offset(uint32_t nu) const { return offset >> (7 + nu); }  // first union chunk-column
};

// Everything a prove needs besides the inputs. A single-hash statement (the *Setup path)
// is the one-slot union at full utilisation; a mixed statement has several slots with
// arbitrary declared counts (crates/flock-core/src/union.rs). For both, m is the union
// variable count M, k_log = M - nu is the union's column-variable count, and the
// committed stack q is the height-n_t compaction of the padded union buffer.
struct Statement {
  HashKind hash = HASH_BLAKE3;   // the first slot's hash (single-hash statements)
  uint32_t n_blocks = 0;         // single-hash statements: the declared count (= 2^nu)
  uint32_t k_log = 0, nu = 0, m = 0;
  uint64_t useful_bits = 0;
  uint32_t const_pin = 0;
  UnionGeometry geo;
  uint32_t log_batch = 0, lanes = 0, log_dim = 0, k_code = 0;
  LigeritoParams lig;
  std::array<uint8_t, 32> registry_digest{};
  // Matrices of the single slot: BLAKE3 / SHA-256 materialise (A_0, B_0); Keccak uses the walker.
  std::shared_ptr<SparseRows> a0, b0;
  std::shared_ptr<Csc> csc_a, csc_b;
  // Union layout (every statement; one slot for single-hash statements).
  bool mixed = false;                  // built by make_union_statement (several types)
  std::vector<SlotInfo> slots;         // slot order
  std::vector<uint64_t> col_prefix;    // jagged prefix sums over the 2^col_log union chunk-columns
  uint64_t dense_words = 0, committed_words = 0;
  bool identity = true;                // the committed stack is the padded buffer itself
  uint64_t packed_words() const { return uint64_t(1) << (m - 7); }
  uint64_t area() const { return col_prefix.empty() ? 0 : col_prefix.back(); }
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

inline void type_params(HashKind h, uint32_t& k_log, uint64_t& useful, uint32_t& pin) {
  switch (h) {
    case HASH_BLAKE3: k_log = b3r1cs::K_LOG; useful = b3r1cs::USEFUL_BITS; pin = b3r1cs::Z_CONST_POS; return;
    case HASH_SHA256: k_log = s2r1cs::K_LOG; useful = s2r1cs::USEFUL_BITS; pin = s2r1cs::Z_CONST_POS; return;
    case HASH_KECCAK: k_log = kr1cs::K_LOG; useful = kr1cs::USEFUL_BITS; pin = kr1cs::Z_CONST; return;
  }
  throw std::runtime_error("unknown hash kind");
}

// Jagged heights, dense / committed sizes and the identity test of a slot layout
// (union.rs:293-420): used chunk-columns of slot t have height n_t, everything else 0.
inline void finish_union_layout(Statement& s) {
  const uint32_t nu = s.nu, col_log = s.m - 7 - nu;
  std::vector<uint64_t> h(size_t(1) << col_log, 0);
  s.dense_words = 0;
  uint64_t cursor = 0;
  bool ident = true;
  for (const SlotInfo& t : s.slots) {
    const uint64_t c0 = t.col_offset(nu);
    for (uint64_t c = 0; c < t.used_cols; ++c) h[c0 + c] = t.count;
    s.dense_words += t.used_cols * t.count;
    if (cursor != (t.offset >> 7) || t.count != (uint64_t(1) << nu)) ident = false;
    cursor += t.used_cols << nu;
  }
  s.col_prefix.assign(h.size() + 1, 0);
  for (size_t y = 0; y < h.size(); ++y) s.col_prefix[y + 1] = s.col_prefix[y] + h[y];
  uint64_t p2 = 1;
  while (p2 < s.dense_words) p2 <<= 1;
  const uint64_t floor_words = uint64_t(1) << (22 - 7);  // MIN_DENSE_M = 22 (union.rs:43)
  s.committed_words = std::min(std::max(p2, floor_words), s.packed_words());
  uint32_t lg = 0;
  while ((uint64_t(1) << lg) < s.committed_words) ++lg;
  s.identity = ident && s.committed_words == s.packed_words();
  s.geo.k_log = s.k_log;
  s.geo.nu = nu;
  s.geo.m = s.m;
  s.geo.col_log = col_log;
  s.geo.dense_m = lg + 7;
  s.geo.identity = s.identity;
  s.geo.used_cols = s.slots.size() == 1 ? s.slots[0].used_cols : 0;
  s.lig = ligerito_params_for(s.geo.dense_m);
  s.log_batch = s.lig.initial_k;
  s.log_dim = s.geo.dense_m - 7 - s.log_batch;
  s.k_code = s.log_dim + 1;
  // integer lanes t = ceil(dense_words / 2^log_dim), in [1, 2^log_batch] (commit.rs:409-414)
  const uint64_t d = uint64_t(1) << s.log_dim;
  uint64_t t = (s.dense_words + d - 1) / d;
  s.lanes = (uint32_t)std::min<uint64_t>(std::max<uint64_t>(t, 1), uint64_t(1) << s.log_batch);
  if (s.lig.log_n != s.geo.dense_m - 7 || s.lig.initial_log_msg_cols != s.log_dim)
    throw std::runtime_error("Ligerito configuration does not match the committed geometry");
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
  SlotInfo t;
  t.hash = h;
  t.k_log = s.k_log;
  t.useful_bits = s.useful_bits;
  t.const_pin = s.const_pin;
  t.used_cols = s.geo.used_cols;
  t.m_slot = s.m;
  t.count = n_blocks;
  t.a0 = s.a0; t.b0 = s.b0; t.csc_a = s.csc_a; t.csc_b = s.csc_b;
  s.slots.push_back(t);
  const UnionGeometry g = s.geo;
  const uint32_t lanes = s.lanes;
  finish_union_layout(s);
  if (s.geo.dense_m != g.dense_m || s.lanes != lanes || !s.identity)
    throw std::runtime_error("single-slot union layout disagrees with the full-utilisation geometry");
  return s;
}

// Slot order of a registry's types: k_log descending, stable (schedule.rs:400-410).
inline std::vector<size_t> registry_slot_order(const std::vector<HashKind>& types) {
  std::vector<size_t> order(types.size());
  for (size_t i = 0; i < order.size(); ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) {
    uint32_t ka, kb, pa, pb;
    uint64_t ua, ub;
    type_params(types[a], ka, ua, pa);
    type_params(types[b], kb, ub, pb);
    return ka > kb;
  });
  return order;
}

// A mixed (multi-type) union statement: registry of `types_slot_order` (already in slot
// order, see registry_slot_order) at uniform row capacity 2^nu, with declared counts in
// slot order (Registry::new, Instance::new, UnionInstance: schedule.rs:337-468, 654-690;
// union.rs:293-420). Boolean types only (the three hash encoders).
inline Statement make_union_statement(const std::vector<HashKind>& types_slot_order, uint32_t nu,
                                      const std::vector<uint64_t>& counts) {
  if (types_slot_order.empty() || types_slot_order.size() != counts.size())
    throw std::runtime_error("one declared count per registry type");
  if (nu < 3) throw std::runtime_error("the union lincheck needs nu >= 3");
  Statement s;
  s.mixed = true;
  s.nu = nu;
  uint64_t offset = 0;
  uint32_t prev_k = 64;
  for (size_t i = 0; i < types_slot_order.size(); ++i) {
    SlotInfo t;
    t.hash = types_slot_order[i];
    type_params(t.hash, t.k_log, t.useful_bits, t.const_pin);
    if (t.k_log > prev_k) throw std::runtime_error("registry types must be given in slot order (k_log descending)");
    prev_k = t.k_log;
    if (counts[i] > (uint64_t(1) << nu)) throw std::runtime_error("declared count exceeds the row capacity 2^nu");
    t.used_cols = std::min<uint64_t>((t.useful_bits + 127) / 128, uint64_t(1) << (t.k_log - 7));
    t.m_slot = nu + t.k_log;
    t.offset = offset;
    t.prefix = offset >> t.m_slot;
    t.count = counts[i];
    if (t.hash != HASH_KECCAK) {
      MatrixCache& mc = matrices_for(t.hash);
      t.a0 = mc.a; t.b0 = mc.b; t.csc_a = mc.ca; t.csc_b = mc.cb;
    }
    offset += uint64_t(1) << t.m_slot;
    s.slots.push_back(t);
  }
  uint32_t M = 0;
  while ((uint64_t(1) << M) < offset) ++M;
  s.m = M;
  for (auto& t : s.slots) {
    if (t.offset % (uint64_t(1) << t.m_slot)) throw std::runtime_error("slot offset not aligned");
  }
  s.k_log = M - nu;
  s.hash = s.slots[0].hash;
  s.const_pin = s.slots[0].const_pin;
  s.useful_bits = 0;
  finish_union_layout(s);
  return s;
}

// Registry digest of the single-slot registry (computed once per statement; the
// matrices make it a few hundred MB of BLAKE3 input).
inline void compute_registry_digest(Statement& s) {
  std::vector<TableType> types;
  for (const SlotInfo& t : s.slots) {
    TableType ty;
    ty.k_log = t.k_log;
    ty.useful_bits = t.useful_bits;
    ty.const_pin = t.const_pin;
    ty.c0_identity = true;
    if (t.hash == HASH_KECCAK) { ty.a0 = &kr1cs::empty_stub(); ty.b0 = &kr1cs::empty_stub(); }
    else { ty.a0 = t.a0.get(); ty.b0 = t.b0.get(); }
    types.push_back(ty);
  }
  s.registry_digest = registry_digest(s.nu, types);
}

}  // namespace flock
