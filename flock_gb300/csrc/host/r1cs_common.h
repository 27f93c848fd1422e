// Shared R1CS plumbing for the hash encoders: sparse boolean matrices, the GF(2)
// cancellation used to keep rows canonical, and the 32-bit adder witness parts.
//
// References: crates/flock-core/src/r1cs.rs:12-20 (SparseBinaryMatrix),
// crates/flock-prover/src/r1cs_hashes/common.rs:94-210 (adder parts) and
// :500-515 (xor_dedup).
#pragma once
#include <cstdint>
#include <vector>
#include <algorithm>

namespace flock {

// Rows of a k x k boolean matrix; row r lists the columns holding a 1, sorted.
struct SparseRows {
  uint32_t num_rows = 0, num_cols = 0;
  std::vector<std::vector<uint32_t>> rows;
  size_t nnz() const {
    size_t n = 0;
    for (auto& r : rows) n += r.size();
    return n;
  }
};

// Sort and cancel equal pairs (x + x = 0 over GF(2)).
inline std::vector<uint32_t> xor_dedup(std::vector<uint32_t> v) {
  std::sort(v.begin(), v.end());
  std::vector<uint32_t> out;
  out.reserve(v.size());
  size_t i = 0;
  while (i < v.size()) {
    uint32_t x = v[i];
    size_t c = 0;
    while (i < v.size() && v[i] == x) { ++c; ++i; }
    if (c & 1) out.push_back(x);
  }
  return out;
}

// CSC transpose of a SparseRows matrix: rows having a 1 in column c are
// rows_flat[col_ptr[c] .. col_ptr[c+1]) (crates/flock-core/src/lincheck.rs:366-389).
struct Csc {
  uint32_t n_cols = 0;
  std::vector<uint32_t> col_ptr;
  std::vector<uint32_t> rows_flat;
};
inline Csc csc_from_rows(const SparseRows& m) {
  Csc c;
  c.n_cols = m.num_cols;
  c.col_ptr.assign(m.num_cols + 1, 0);
  for (auto& r : m.rows)
    for (uint32_t col : r) c.col_ptr[col + 1]++;
  for (uint32_t i = 0; i < m.num_cols; ++i) c.col_ptr[i + 1] += c.col_ptr[i];
  std::vector<uint32_t> next(c.col_ptr.begin(), c.col_ptr.end() - 1);
  c.rows_flat.resize(c.col_ptr.back());
  for (uint32_t r = 0; r < m.rows.size(); ++r)
    for (uint32_t col : m.rows[r]) c.rows_flat[next[col]++] = r;
  return c;
}

// ---- adder witness parts (common.rs:94-210) ------------------------------------------
struct AddParts { uint32_t sum, left, right, carry; };
// 2-operand add: carry_aux[i] = (x_i ^ cin_i)(y_i ^ cin_i) for bits 0..30.
inline AddParts add_carry_parts(uint32_t x, uint32_t y) {
  uint32_t sum = x + y;
  uint32_t cin = sum ^ x ^ y;
  uint32_t l = (x ^ cin) & 0x7FFFFFFFu, r = (y ^ cin) & 0x7FFFFFFFu;
  return {sum, l, r, l & r};
}
// 3-operand carry-save add x + y + m: majority products (31 bits) and ripple products
// (bits 1..30, shifted down to 30 bits).
struct Add3Parts { uint32_t sum; uint32_t maj[3]; uint32_t rip[3]; };
inline Add3Parts fused_add3_parts(uint32_t x, uint32_t y, uint32_t m) {
  uint32_t xm = x ^ m, ym = y ^ m, w = xm & ym, p = x ^ y ^ m, bw = (w ^ m) << 1;
  uint32_t sum = p + bw, cin = sum ^ p ^ bw;
  uint32_t rl = p ^ cin, rr = bw ^ cin;
  Add3Parts o;
  o.sum = sum;
  o.maj[0] = xm & 0x7FFFFFFFu; o.maj[1] = ym & 0x7FFFFFFFu; o.maj[2] = w & 0x7FFFFFFFu;
  o.rip[0] = (rl >> 1) & 0x3FFFFFFFu; o.rip[1] = (rr >> 1) & 0x3FFFFFFFu; o.rip[2] = ((rl & rr) >> 1) & 0x3FFFFFFFu;
  return o;
}
// 4-operand add x + y + z + w: two carry-save layers plus a ripple (common.rs:160-195).
struct Add4Parts { uint32_t sum; uint32_t maj1[3]; uint32_t maj2[3]; uint32_t rip[3]; };
inline Add4Parts fused_add4_parts(uint32_t x, uint32_t y, uint32_t z, uint32_t w) {
  uint32_t xz = x ^ z, yz = y ^ z, w1 = xz & yz, p1 = x ^ y ^ z, b1 = (w1 ^ z) << 1;
  uint32_t pw = p1 ^ w, bw = b1 ^ w, w2 = pw & bw, p2 = p1 ^ b1 ^ w, b2 = (w2 ^ w) << 1;
  uint32_t sum = p2 + b2, cin = sum ^ p2 ^ b2;
  uint32_t rl = p2 ^ cin, rr = b2 ^ cin;
  Add4Parts o;
  o.sum = sum;
  o.maj1[0] = xz & 0x7FFFFFFFu; o.maj1[1] = yz & 0x7FFFFFFFu; o.maj1[2] = w1 & 0x7FFFFFFFu;
  o.maj2[0] = pw & 0x7FFFFFFFu; o.maj2[1] = bw & 0x7FFFFFFFu; o.maj2[2] = w2 & 0x7FFFFFFFu;
  o.rip[0] = (rl >> 1) & 0x3FFFFFFFu; o.rip[1] = (rr >> 1) & 0x3FFFFFFFu; o.rip[2] = ((rl & rr) >> 1) & 0x3FFFFFFFu;
  return o;
}
// Constant-operand add k + y: product rows for bits t..30 only, t = tz(k) + 1.
inline AddParts const_add_parts(uint32_t k, uint32_t y) {
  uint32_t t = (uint32_t)__builtin_ctz(k) + 1;
  AddParts p = add_carry_parts(k, y);
  uint32_t mask = (1u << (31 - t)) - 1;
  return {p.sum, (p.left >> t) & mask, (p.right >> t) & mask, (p.carry >> t) & mask};
}

// OR the low bits of `val` into a little-endian bit buffer at bit offset `bit`.
inline void or_u32_at(uint64_t* buf, size_t bit, uint32_t val) {
  size_t w = bit >> 6, s = bit & 63;
  buf[w] |= (uint64_t)val << s;
  if (s > 32) buf[w + 1] |= (uint64_t)val >> (64 - s);
}
inline void or_bit_at(uint64_t* buf, size_t bit) { buf[bit >> 6] |= 1ull << (bit & 63); }

}  // namespace flock
