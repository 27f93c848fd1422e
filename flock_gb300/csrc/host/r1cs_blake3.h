// BLAKE3 compression as a block R1CS over GF(2) with C = I — the "Option F" encoding
// of crates/flock-prover/src/r1cs_hashes/blake3.rs:1-120 (fused 3-operand adders,
// constant-operand adders for round 1's column G's, no sum-bit or lin-id slots).
//
// Layout of one 2^14-bit block (blake3.rs:40-60, :210-247):
//   [0,256) cv | [256,512) out_lo | [512,1024) m | [1024,1152) t_lo t_hi blen flags
//   [1152,1408) out_hi | [1408,11706) 56 G blocks | 11706 the constant one.
// The matrix builder follows build_matrices (blake3.rs:659-782); the witness
// follows build_group_batch_major (blake3.rs:1929-2040), one instance at a time.
#pragma once
#include "r1cs_common.h"
#include "hashes.h"
#include <array>

namespace flock {
namespace b3r1cs {

constexpr int K_LOG = 14;
constexpr uint32_t K = 1u << K_LOG;
constexpr int N_ROUNDS = 7, N_G_PER_ROUND = 8, N_G = 56, WORD_BITS = 32;
constexpr int CARRY_BITS = 31, RIPPLE_BITS = 30, FADD_BITS = 61;

constexpr int g_c1_rows(int g) { return g < 2 ? 30 : (g < 4 ? 29 : 31); }
constexpr int g_block_bits(int g) { return 2 * FADD_BITS + CARRY_BITS + g_c1_rows(g); }

constexpr uint32_t CV_BASE = 0, OUT_LO_BASE = 256, M_BASE = 512, T_LO_BASE = 1024, T_HI_BASE = 1056,
                   BLEN_BASE = 1088, FLAGS_BASE = 1120, OUT_HI_BASE = 1152, GS_BASE = 1408;

struct GBase {
  uint32_t v[N_G + 1];
  constexpr GBase() : v() {
    uint32_t acc = GS_BASE;
    for (int g = 0; g < N_G; ++g) { v[g] = acc; acc += g_block_bits(g); }
    v[N_G] = acc;
  }
};
constexpr GBase G_BASE{};
constexpr uint32_t Z_CONST_POS = G_BASE.v[N_G];  // 11,706
constexpr uint32_t USEFUL_BITS = Z_CONST_POS + 1;  // 11,707
static_assert(Z_CONST_POS == 11706, "BLAKE3 constant wire position");

constexpr int G_LANES[8][4] = {{0, 4, 8, 12}, {1, 5, 9, 13}, {2, 6, 10, 14}, {3, 7, 11, 15},
                               {0, 5, 10, 15}, {1, 6, 11, 12}, {2, 7, 8, 13}, {3, 4, 9, 14}};

constexpr uint32_t off_maj1() { return 0; }
constexpr uint32_t off_rip1() { return CARRY_BITS; }
constexpr uint32_t off_c1() { return FADD_BITS; }
constexpr uint32_t off_maj2(int g) { return FADD_BITS + g_c1_rows(g); }
constexpr uint32_t off_rip2(int g) { return off_maj2(g) + CARRY_BITS; }
constexpr uint32_t off_c2(int g) { return off_rip2(g) + RIPPLE_BITS; }

// per_round_msg_idx (blake3.rs:364-384): message word indices consumed by G g of round r.
inline std::array<std::array<std::array<int, 2>, 8>, 7> msg_idx() {
  std::array<std::array<std::array<int, 2>, 8>, 7> out{};
  int perm[16];
  for (int i = 0; i < 16; ++i) perm[i] = i;
  for (int r = 0; r < 7; ++r) {
    for (int g = 0; g < 8; ++g) { out[r][g][0] = perm[2 * g]; out[r][g][1] = perm[2 * g + 1]; }
    int nx[16];
    for (int i = 0; i < 16; ++i) nx[i] = perm[B3_MSG_PERM[i]];
    for (int i = 0; i < 16; ++i) perm[i] = nx[i];
  }
  return out;
}

// ---- symbolic words for the matrix builder -------------------------------------------
struct Word {
  std::array<std::vector<uint32_t>, 32> bits;
  static Word slot(uint32_t base) {
    Word w;
    for (int i = 0; i < 32; ++i) w.bits[i] = {base + (uint32_t)i};
    return w;
  }
  static Word constant(uint32_t v) {
    Word w;
    for (int i = 0; i < 32; ++i) if ((v >> i) & 1) w.bits[i] = {Z_CONST_POS};
    return w;
  }
  Word xor_dedup_with(const Word& o) const {
    Word w;
    for (int i = 0; i < 32; ++i) {
      std::vector<uint32_t> v = bits[i];
      v.insert(v.end(), o.bits[i].begin(), o.bits[i].end());
      w.bits[i] = xor_dedup(std::move(v));
    }
    return w;
  }
  Word rotr(int n) const {
    Word w;
    for (int i = 0; i < 32; ++i) w.bits[i] = bits[(i + n) % 32];
    return w;
  }
};

inline Word add_sum(const Word& x, const Word& y, uint32_t carry_base) {
  Word o;
  for (int i = 0; i < 32; ++i) {
    std::vector<uint32_t> v = x.bits[i];
    v.insert(v.end(), y.bits[i].begin(), y.bits[i].end());
    for (int j = 0; j < i; ++j) v.push_back(carry_base + j);
    o.bits[i] = xor_dedup(std::move(v));
  }
  return o;
}
inline Word fused_add_sum(const Word& x, const Word& y, const Word& m, uint32_t maj, uint32_t rip) {
  Word o;
  for (int i = 0; i < 32; ++i) {
    std::vector<uint32_t> v = x.bits[i];
    v.insert(v.end(), y.bits[i].begin(), y.bits[i].end());
    v.insert(v.end(), m.bits[i].begin(), m.bits[i].end());
    if (i >= 1) {
      v.push_back(maj + i - 1);
      v.insert(v.end(), m.bits[i - 1].begin(), m.bits[i - 1].end());
      int lim = std::min(i, RIPPLE_BITS + 1);
      for (int l = 1; l < lim; ++l) v.push_back(rip + l - 1);
    }
    o.bits[i] = xor_dedup(std::move(v));
  }
  return o;
}
inline Word const_add_sum(uint32_t k, const Word& y, uint32_t base, int n_rows) {
  int t = CARRY_BITS - n_rows;
  Word o;
  for (int i = 0; i < 32; ++i) {
    std::vector<uint32_t> v = y.bits[i];
    if ((k >> i) & 1) v.push_back(Z_CONST_POS);
    if (i >= t) {
      v.insert(v.end(), y.bits[t - 1].begin(), y.bits[t - 1].end());
      for (int j = t; j < i; ++j) v.push_back(base + j - t);
    }
    o.bits[i] = xor_dedup(std::move(v));
  }
  return o;
}

inline Word write_add(SparseRows& A, SparseRows& B, const Word& x, const Word& y, uint32_t cb) {
  for (int i = 0; i < CARRY_BITS; ++i) {
    std::vector<uint32_t> a = x.bits[i], b = y.bits[i];
    for (int j = 0; j < i; ++j) { a.push_back(cb + j); b.push_back(cb + j); }
    A.rows[cb + i] = xor_dedup(std::move(a));
    B.rows[cb + i] = xor_dedup(std::move(b));
  }
  return add_sum(x, y, cb);
}
inline Word write_fused_add(SparseRows& A, SparseRows& B, const Word& x, const Word& y, const Word& m,
                            uint32_t maj, uint32_t rip) {
  for (int i = 0; i < CARRY_BITS; ++i) {
    std::vector<uint32_t> a = x.bits[i], b = y.bits[i];
    a.insert(a.end(), m.bits[i].begin(), m.bits[i].end());
    b.insert(b.end(), m.bits[i].begin(), m.bits[i].end());
    A.rows[maj + i] = xor_dedup(std::move(a));
    B.rows[maj + i] = xor_dedup(std::move(b));
  }
  for (int j = 1; j <= RIPPLE_BITS; ++j) {
    std::vector<uint32_t> a = x.bits[j];
    a.insert(a.end(), y.bits[j].begin(), y.bits[j].end());
    a.insert(a.end(), m.bits[j].begin(), m.bits[j].end());
    for (int l = 1; l < j; ++l) a.push_back(rip + l - 1);
    std::vector<uint32_t> b = {maj + (uint32_t)j - 1};
    b.insert(b.end(), m.bits[j - 1].begin(), m.bits[j - 1].end());
    for (int l = 1; l < j; ++l) b.push_back(rip + l - 1);
    A.rows[rip + j - 1] = xor_dedup(std::move(a));
    B.rows[rip + j - 1] = xor_dedup(std::move(b));
  }
  return fused_add_sum(x, y, m, maj, rip);
}
inline Word write_const_add(SparseRows& A, SparseRows& B, uint32_t k, const Word& y, uint32_t base, int n_rows) {
  int t = CARRY_BITS - n_rows;
  for (int i = t; i < WORD_BITS - 1; ++i) {
    std::vector<uint32_t> carry = y.bits[t - 1];
    for (int j = t; j < i; ++j) carry.push_back(base + j - t);
    std::vector<uint32_t> a = carry;
    if ((k >> i) & 1) a.push_back(Z_CONST_POS);
    std::vector<uint32_t> b = y.bits[i];
    b.insert(b.end(), carry.begin(), carry.end());
    A.rows[base + i - t] = xor_dedup(std::move(a));
    B.rows[base + i - t] = xor_dedup(std::move(b));
  }
  return const_add_sum(k, y, base, n_rows);
}

// (A_0, B_0) of one compression block (blake3.rs:659-782). C_0 = I.
inline void build_matrices(SparseRows& A, SparseRows& B) {
  A.num_rows = A.num_cols = B.num_rows = B.num_cols = K;
  A.rows.assign(K, {});
  B.rows.assign(K, {});
  A.rows[Z_CONST_POS] = {Z_CONST_POS};
  B.rows[Z_CONST_POS] = {Z_CONST_POS};
  auto input = [&](uint32_t base, uint32_t len) {
    for (uint32_t j = 0; j < len; ++j) { A.rows[base + j] = {base + j}; B.rows[base + j] = {Z_CONST_POS}; }
  };
  input(CV_BASE, 256); input(M_BASE, 512); input(T_LO_BASE, 32); input(T_HI_BASE, 32);
  input(BLEN_BASE, 32); input(FLAGS_BASE, 32);

  auto mi = msg_idx();
  std::array<Word, 16> st;
  for (int w = 0; w < 8; ++w) st[w] = Word::slot(CV_BASE + 32 * w);
  for (int i = 0; i < 4; ++i) st[8 + i] = Word::constant(BLAKE3_IV[i]);
  st[12] = Word::slot(T_LO_BASE); st[13] = Word::slot(T_HI_BASE);
  st[14] = Word::slot(BLEN_BASE); st[15] = Word::slot(FLAGS_BASE);

  for (int r = 0; r < N_ROUNDS; ++r) {
    for (int gi = 0; gi < 8; ++gi) {
      int g = r * 8 + gi;
      int la = G_LANES[gi][0], lb = G_LANES[gi][1], lc = G_LANES[gi][2], ld = G_LANES[gi][3];
      Word a = st[la], b = st[lb], c = st[lc], d = st[ld];
      Word mx = Word::slot(M_BASE + 32 * mi[r][gi][0]);
      Word my = Word::slot(M_BASE + 32 * mi[r][gi][1]);
      uint32_t gb = G_BASE.v[g];
      Word a1 = write_fused_add(A, B, a, b, mx, gb + off_maj1(), gb + off_rip1());
      Word d1 = d.xor_dedup_with(a1).rotr(16);
      Word c1 = g < 4 ? write_const_add(A, B, BLAKE3_IV[g], d1, gb + off_c1(), g_c1_rows(g))
                      : write_add(A, B, c, d1, gb + off_c1());
      Word b1 = b.xor_dedup_with(c1).rotr(12);
      Word a2 = write_fused_add(A, B, a1, b1, my, gb + off_maj2(g), gb + off_rip2(g));
      Word d2 = d1.xor_dedup_with(a2).rotr(8);
      Word c2 = write_add(A, B, c1, d2, gb + off_c2(g));
      Word bn = b1.xor_dedup_with(c2).rotr(7);
      st[la] = std::move(a2); st[lb] = std::move(bn); st[lc] = std::move(c2); st[ld] = std::move(d2);
    }
  }
  for (int w = 0; w < 8; ++w) {
    Word lo = st[w].xor_dedup_with(st[w + 8]);
    for (int i = 0; i < 32; ++i) { A.rows[OUT_LO_BASE + 32 * w + i] = lo.bits[i]; B.rows[OUT_LO_BASE + 32 * w + i] = {Z_CONST_POS}; }
    Word hi = st[w + 8].xor_dedup_with(Word::slot(CV_BASE + 32 * w));
    for (int i = 0; i < 32; ++i) { A.rows[OUT_HI_BASE + 32 * w + i] = hi.bits[i]; B.rows[OUT_HI_BASE + 32 * w + i] = {Z_CONST_POS}; }
  }
}

// One compression input (blake3.rs:1232): (cv, m, counter, block_len, flags).
struct Compression {
  uint32_t cv[8];
  uint32_t m[16];
  uint64_t counter;
  uint32_t block_len;
  uint32_t flags;
};

// Witness bits z, a = A_0 z, b = B_0 z of one block (K bits each, little-endian u64
// words, caller-zeroed). Mirrors build_group_batch_major for a single lane.
inline void witness_block(const Compression& in, uint64_t* z, uint64_t* a, uint64_t* b) {
  auto lin = [&](uint32_t bit, uint32_t v) { or_u32_at(z, bit, v); or_u32_at(a, bit, v); or_u32_at(b, bit, 0xFFFFFFFFu); };
  or_bit_at(z, Z_CONST_POS); or_bit_at(a, Z_CONST_POS); or_bit_at(b, Z_CONST_POS);
  for (int w = 0; w < 8; ++w) lin(CV_BASE + 32 * w, in.cv[w]);
  for (int i = 0; i < 16; ++i) lin(M_BASE + 32 * i, in.m[i]);
  uint32_t tlo = (uint32_t)in.counter, thi = (uint32_t)(in.counter >> 32);
  lin(T_LO_BASE, tlo); lin(T_HI_BASE, thi); lin(BLEN_BASE, in.block_len); lin(FLAGS_BASE, in.flags);
  uint32_t s[16] = {in.cv[0], in.cv[1], in.cv[2], in.cv[3], in.cv[4], in.cv[5], in.cv[6], in.cv[7],
                    BLAKE3_IV[0], BLAKE3_IV[1], BLAKE3_IV[2], BLAKE3_IV[3], tlo, thi, in.block_len, in.flags};
  auto mi = msg_idx();
  for (int r = 0; r < N_ROUNDS; ++r) {
    for (int gi = 0; gi < 8; ++gi) {
      int g = r * 8 + gi;
      int la = G_LANES[gi][0], lb = G_LANES[gi][1], lc = G_LANES[gi][2], ld = G_LANES[gi][3];
      uint32_t mx = in.m[mi[r][gi][0]], my = in.m[mi[r][gi][1]];
      uint32_t gb = G_BASE.v[g];
      Add3Parts f1 = fused_add3_parts(s[la], s[lb], mx);
      or_u32_at(z, gb + off_maj1(), f1.maj[2]); or_u32_at(a, gb + off_maj1(), f1.maj[0]); or_u32_at(b, gb + off_maj1(), f1.maj[1]);
      or_u32_at(z, gb + off_rip1(), f1.rip[2]); or_u32_at(a, gb + off_rip1(), f1.rip[0]); or_u32_at(b, gb + off_rip1(), f1.rip[1]);
      uint32_t a1 = f1.sum;
      uint32_t d1 = rotr32(s[ld] ^ a1, 16);
      uint32_t c1;
      if (g < 4) {
        int nr = g_c1_rows(g), t = CARRY_BITS - nr;
        uint32_t mask = (1u << nr) - 1;
        AddParts p = add_carry_parts(BLAKE3_IV[g], d1);
        or_u32_at(z, gb + off_c1(), (p.carry >> t) & mask);
        or_u32_at(a, gb + off_c1(), (p.left >> t) & mask);
        or_u32_at(b, gb + off_c1(), (p.right >> t) & mask);
        c1 = p.sum;
      } else {
        AddParts p = add_carry_parts(s[lc], d1);
        or_u32_at(z, gb + off_c1(), p.carry); or_u32_at(a, gb + off_c1(), p.left); or_u32_at(b, gb + off_c1(), p.right);
        c1 = p.sum;
      }
      uint32_t b1 = rotr32(s[lb] ^ c1, 12);
      Add3Parts f2 = fused_add3_parts(a1, b1, my);
      or_u32_at(z, gb + off_maj2(g), f2.maj[2]); or_u32_at(a, gb + off_maj2(g), f2.maj[0]); or_u32_at(b, gb + off_maj2(g), f2.maj[1]);
      or_u32_at(z, gb + off_rip2(g), f2.rip[2]); or_u32_at(a, gb + off_rip2(g), f2.rip[0]); or_u32_at(b, gb + off_rip2(g), f2.rip[1]);
      uint32_t a2 = f2.sum;
      uint32_t d2 = rotr32(d1 ^ a2, 8);
      AddParts p2 = add_carry_parts(c1, d2);
      or_u32_at(z, gb + off_c2(g), p2.carry); or_u32_at(a, gb + off_c2(g), p2.left); or_u32_at(b, gb + off_c2(g), p2.right);
      uint32_t c2 = p2.sum;
      uint32_t bn = rotr32(b1 ^ c2, 7);
      s[la] = a2; s[lb] = bn; s[lc] = c2; s[ld] = d2;
    }
  }
  for (int w = 0; w < 8; ++w) {
    lin(OUT_LO_BASE + 32 * w, s[w] ^ s[w + 8]);
    lin(OUT_HI_BASE + 32 * w, s[w + 8] ^ in.cv[w]);
  }
}

}  // namespace b3r1cs
}  // namespace flock
