// Statement binding data: the union registry digest (crates/flock-core/src/schedule.rs:
// 542-578, absorb_matrix at crates/flock-core/src/r1cs.rs:419-433) and the union
// geometry of a single-slot, full-utilisation instance (crates/flock-core/src/union.rs:
// 293-420): dense_m, commit lanes and the jagged column heights.
#pragma once
#include "hashes.h"
#include "r1cs_common.h"
#include <optional>

namespace flock {

struct TableType {
  uint32_t k_log = 0;
  uint64_t useful_bits = 0;
  std::optional<uint64_t> const_pin;
  const SparseRows* a0 = nullptr;  // nullptr = 0x0 stub matrix
  const SparseRows* b0 = nullptr;
  const SparseRows* c0 = nullptr;
  bool c0_identity = false;        // C_0 = I_{2^k_log} without materialising it
};

namespace detail {
inline void put_u64(std::vector<uint8_t>& buf, uint64_t v) {
  for (int i = 0; i < 8; ++i) buf.push_back((uint8_t)(v >> (8 * i)));
}
inline void put_u32(std::vector<uint8_t>& buf, uint32_t v) {
  for (int i = 0; i < 4; ++i) buf.push_back((uint8_t)(v >> (8 * i)));
}
// Length-prefixed matrix absorption: (num_rows, num_cols, [(row_len, cols...)...]), u64 LE.
inline void absorb_matrix(Blake3Hasher& h, const SparseRows* m) {
  std::vector<uint8_t> buf;
  buf.reserve(1 << 20);
  if (!m) { put_u64(buf, 0); put_u64(buf, 0); h.update(buf.data(), buf.size()); return; }
  put_u64(buf, m->num_rows);
  put_u64(buf, m->num_cols);
  for (auto& row : m->rows) {
    put_u64(buf, row.size());
    for (uint32_t c : row) put_u64(buf, c);
    if (buf.size() > (1u << 20) - 8 * 8192) { h.update(buf.data(), buf.size()); buf.clear(); }
  }
  h.update(buf.data(), buf.size());
}
inline void absorb_identity(Blake3Hasher& h, uint32_t k) {
  std::vector<uint8_t> buf;
  buf.reserve(16 + 16 * (size_t)k);
  put_u64(buf, k); put_u64(buf, k);
  for (uint32_t r = 0; r < k; ++r) { put_u64(buf, 1); put_u64(buf, r); }
  h.update(buf.data(), buf.size());
}
}  // namespace detail

// BLAKE3("flock-registry-v1" || 1 || nu u32 || n_types u32 || per type ...). Types must be
// given in registry slot order (class-major, k_log descending, stable).
inline std::array<uint8_t, 32> registry_digest(uint32_t nu, const std::vector<TableType>& types) {
  Blake3Hasher h;
  std::vector<uint8_t> head;
  const char* label = "flock-registry-v1";
  head.insert(head.end(), label, label + strlen(label));
  head.push_back(1);
  detail::put_u32(head, nu);
  detail::put_u32(head, (uint32_t)types.size());
  h.update(head.data(), head.size());
  for (auto& ty : types) {
    std::vector<uint8_t> b;
    detail::put_u32(b, ty.k_log);
    detail::put_u64(b, ty.useful_bits);
    b.push_back(ty.const_pin ? 1 : 0);
    detail::put_u64(b, ty.const_pin ? *ty.const_pin : 0);
    h.update(b.data(), b.size());
    detail::absorb_matrix(h, ty.a0);
    detail::absorb_matrix(h, ty.b0);
    if (ty.c0_identity) detail::absorb_identity(h, 1u << ty.k_log);
    else detail::absorb_matrix(h, ty.c0);
  }
  return h.finalize();
}

// Geometry of a single-slot union at full utilisation (n_t = 2^nu), the shape every
// power-of-two batch takes. `used_cols = ceil(useful_bits / 128)` chunk-columns of
// 2^nu words each; the committed stack is the padded buffer itself when
// next_pow2(used_cols * 2^nu) equals 2^(k_log - 7 + nu) (identity compaction).
struct UnionGeometry {
  uint32_t k_log = 0, nu = 0, m = 0;       // m = k_log + nu
  uint64_t used_cols = 0;                   // chunk-columns carrying data
  uint32_t col_log = 0;                     // k_log - 7
  uint32_t dense_m = 0;                     // log2(committed words) + 7
  bool identity = false;
  uint64_t dense_words() const { return used_cols << nu; }
  // Integer-lane count t = ceil(dense_words / 2^log_dim) (commit.rs:409-414, union.rs:386-390).
  uint32_t commit_lanes(uint32_t log_batch) const {
    uint32_t log_dim = dense_m - 7 - log_batch;
    uint64_t d = uint64_t(1) << log_dim;
    uint64_t t = (dense_words() + d - 1) / d;
    if (t < 1) t = 1;
    if (t > (uint64_t(1) << log_batch)) t = uint64_t(1) << log_batch;
    return (uint32_t)t;
  }
};

inline UnionGeometry union_geometry(uint32_t k_log, uint64_t useful_bits, uint32_t nu) {
  UnionGeometry g;
  g.k_log = k_log; g.nu = nu; g.m = k_log + nu;
  g.col_log = k_log - 7;
  uint64_t n_cols = uint64_t(1) << (k_log - 7);
  g.used_cols = std::min<uint64_t>((useful_bits + 127) / 128, n_cols);
  uint64_t packed_len = uint64_t(1) << (g.m - 7);
  uint64_t dw = g.dense_words(), p2 = 1;
  while (p2 < dw) p2 <<= 1;
  uint64_t floor_words = uint64_t(1) << (22 - 7);  // MIN_DENSE_M = 22 (union.rs:43)
  uint64_t committed = std::min(std::max(p2, floor_words), packed_len);
  uint32_t lg = 0;
  while ((uint64_t(1) << lg) < committed) lg++;
  g.dense_m = lg + 7;
  g.identity = committed == packed_len;
  return g;
}

}  // namespace flock
