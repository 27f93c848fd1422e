// SHA-256 compression as a block R1CS over GF(2) with C = I — the I/O-aligned
// "Option F" encoding of crates/flock-prover/src/r1cs_hashes/sha2.rs:1-200
// (h + K[r] as a constant add, T1 as one fused 4-operand carry-save tree, a_new as a
// fused 3-operand tree, schedule steps as fused 4-operand trees, E_NEW/A_NEW
// materialised every second round).
//
// Layout of one 2^15-bit block (sha2.rs:100-194):
//   [0,256) H_in | [256,512) H_out | [512,1024) M | [1024,3072) ch_and | [3072,5120) maj_and
//   [5120,18757) round aux | [18757,23173) schedule aux | [23173,24197) E_NEW
//   [24197,25221) A_NEW | [25221,25469) output carries | 25469 the constant one.
// The matrix builder follows walk_rows_cfg (sha2.rs:544-707); the witness follows
// build_group_batch_major (sha2.rs:1743-1850) for a single lane.
#pragma once
#include "r1cs_common.h"
#include "hashes.h"

namespace flock {
namespace s2r1cs {

constexpr int K_LOG = 15;
constexpr uint32_t K = 1u << K_LOG;
constexpr int N_ROUNDS = 64, N_SCHED = 48, WORD_BITS = 32, CARRIES = 31, RIPPLE = 30, EA_PERIOD = 2;

constexpr uint32_t H_BASE = 0, H_OUT_BASE = 256, M_BASE = 512, CH_AND_BASE = 1024, MAJ_AND_BASE = 3072,
                   ROUND_CARRY_BASE = 5120;
constexpr uint32_t RC_MAJ1 = 0, RC_MAJ2 = 31, RC_RIP = 62, RC_AMAJ = 92, RC_ARIP = 123, RC_ENEW = 153, RC_ADDK = 184;
constexpr uint32_t SCHED_ADD_BITS = 92, SC_MAJ1 = 0, SC_MAJ2 = 31, SC_RIP = 62;

constexpr int k_seed_t(int r) { return __builtin_ctz(Sha256::K[r]) + 1; }
constexpr int k_add_rows(int r) { return CARRIES - k_seed_t(r); }
constexpr uint32_t round_add_bits(int r) { return RC_ADDK + (uint32_t)k_add_rows(r); }

struct RoundBase {
  uint32_t v[N_ROUNDS + 1];
  constexpr RoundBase() : v() {
    uint32_t acc = ROUND_CARRY_BASE;
    for (int r = 0; r < N_ROUNDS; ++r) { v[r] = acc; acc += round_add_bits(r); }
    v[N_ROUNDS] = acc;
  }
};
constexpr RoundBase ROUND_BASE{};
constexpr uint32_t SCHED_CARRY_BASE = ROUND_BASE.v[N_ROUNDS];
constexpr uint32_t E_NEW_BASE = SCHED_CARRY_BASE + N_SCHED * SCHED_ADD_BITS;
constexpr uint32_t A_NEW_BASE = E_NEW_BASE + 32 * 32;
constexpr uint32_t OUT_CARRY_BASE = A_NEW_BASE + 32 * 32;
constexpr uint32_t Z_CONST_POS = OUT_CARRY_BASE + 8 * CARRIES;
constexpr uint32_t USEFUL_BITS = Z_CONST_POS + 1;
static_assert(SCHED_CARRY_BASE == 18757, "SHA-256 schedule aux base");
static_assert(Z_CONST_POS == 25469, "SHA-256 constant wire position");

inline uint32_t h_bit(int w, int b) { return H_BASE + 32 * w + b; }
inline uint32_t m_bit(int i, int b) { return M_BASE + 32 * i + b; }
inline uint32_t round_bit(int r, uint32_t off) { return ROUND_BASE.v[r] + off; }
inline uint32_t sched_bit(int t, uint32_t off) { return SCHED_CARRY_BASE + (t - 16) * SCHED_ADD_BITS + off; }
inline uint32_t e_new_bit(int r, int b) { return E_NEW_BASE + 32 * (r / EA_PERIOD) + b; }
inline uint32_t a_new_bit(int r, int b) { return A_NEW_BASE + 32 * (r / EA_PERIOD) + b; }
inline uint32_t out_carry_bit(int w, int b) { return OUT_CARRY_BASE + w * CARRIES + b; }
inline uint32_t h_out_bit(int w, int b) { return H_OUT_BASE + 32 * w + b; }

inline uint32_t big_sigma0(uint32_t x) { return rotr32(x, 2) ^ rotr32(x, 13) ^ rotr32(x, 22); }
inline uint32_t big_sigma1(uint32_t x) { return rotr32(x, 6) ^ rotr32(x, 11) ^ rotr32(x, 25); }
inline uint32_t small_sigma0(uint32_t x) { return rotr32(x, 7) ^ rotr32(x, 18) ^ (x >> 3); }
inline uint32_t small_sigma1(uint32_t x) { return rotr32(x, 17) ^ rotr32(x, 19) ^ (x >> 10); }

// ---- symbolic walk -----------------------------------------------------------------
using Sup = std::vector<uint32_t>;
using SWord = std::array<Sup, 32>;

inline Sup xs(const Sup& a, const Sup& b) {  // symmetric difference of sorted supports
  Sup o;
  o.reserve(a.size() + b.size());
  size_t i = 0, j = 0;
  while (i < a.size() && j < b.size()) {
    if (a[i] < b[j]) o.push_back(a[i++]);
    else if (a[i] > b[j]) o.push_back(b[j++]);
    else { ++i; ++j; }
  }
  o.insert(o.end(), a.begin() + i, a.end());
  o.insert(o.end(), b.begin() + j, b.end());
  return o;
}
inline Sup xs3(const Sup& a, const Sup& b, const Sup& c) { return xs(xs(a, b), c); }
inline SWord wire(uint32_t base) { SWord w; for (int b = 0; b < 32; ++b) w[b] = {base + (uint32_t)b}; return w; }
inline SWord xw(const SWord& x, const SWord& y) { SWord w; for (int i = 0; i < 32; ++i) w[i] = xs(x[i], y[i]); return w; }
inline SWord rotw(const SWord& x, int n) { SWord w; for (int i = 0; i < 32; ++i) w[i] = x[(i + n) % 32]; return w; }
inline SWord shrw(const SWord& x, int n) { SWord w; for (int i = 0; i < 32; ++i) if (i + n < 32) w[i] = x[i + n]; return w; }
inline SWord rx3(const SWord& x, int a, int b, int c) {
  SWord p = rotw(x, a), q = rotw(x, b), r = rotw(x, c), o;
  for (int i = 0; i < 32; ++i) o[i] = xs3(p[i], q[i], r[i]);
  return o;
}
inline SWord sx3(const SWord& x, int a, int b, int sh) {
  SWord p = rotw(x, a), q = rotw(x, b), r = shrw(x, sh), o;
  for (int i = 0; i < 32; ++i) o[i] = xs3(p[i], q[i], r[i]);
  return o;
}

struct MatSink {
  SparseRows& A; SparseRows& B;
  void row(uint32_t slot, const Sup& a, const Sup& b) { A.rows[slot] = a; B.rows[slot] = b; }
};

template <class S> SWord add32(const SWord& x, const SWord& y, uint32_t carry_base, S& s) {
  SWord sum; Sup cin;
  for (int i = 0; i < 32; ++i) {
    sum[i] = xs3(x[i], y[i], cin);
    if (i < CARRIES) {
      uint32_t slot = carry_base + i;
      s.row(slot, xs(x[i], cin), xs(y[i], cin));
      cin = xs(cin, Sup{slot});
    }
  }
  return sum;
}
template <class S> SWord add_const(uint32_t k, const SWord& y, uint32_t base, S& s) {
  int t = __builtin_ctz(k) + 1;
  auto ks = [&](int i) { return ((k >> i) & 1) ? Sup{Z_CONST_POS} : Sup{}; };
  SWord sum; Sup carry;
  for (int i = 0; i < 32; ++i) {
    if (i == t) carry = y[t - 1];
    sum[i] = xs3(ks(i), y[i], carry);
    if (i >= t && i < CARRIES) {
      uint32_t slot = base + (i - t);
      s.row(slot, xs(ks(i), carry), xs(y[i], carry));
      carry = xs(carry, Sup{slot});
    }
  }
  return sum;
}
template <class S> void csa_layer(const SWord& x, const SWord& y, const SWord& z, uint32_t maj, S& s, SWord& p, SWord& bw) {
  for (int i = 0; i < 32; ++i) { p[i] = xs3(x[i], y[i], z[i]); bw[i].clear(); }
  for (int i = 0; i < CARRIES; ++i) {
    uint32_t slot = maj + i;
    s.row(slot, xs(x[i], z[i]), xs(y[i], z[i]));
    bw[i + 1] = xs(Sup{slot}, z[i]);
  }
}
template <class S> SWord csa_ripple(const SWord& p, const SWord& bw, uint32_t rip, S& s) {
  SWord sum; Sup g;
  for (int i = 0; i < 32; ++i) {
    sum[i] = xs3(p[i], bw[i], g);
    if (i >= 1 && i <= RIPPLE) {
      uint32_t slot = rip + (i - 1);
      s.row(slot, xs(p[i], g), xs(bw[i], g));
      g = xs(g, Sup{slot});
    }
  }
  return sum;
}
template <class S> SWord fadd3(const SWord& x, const SWord& y, const SWord& z, uint32_t maj, uint32_t rip, S& s) {
  SWord p, bw;
  csa_layer(x, y, z, maj, s, p, bw);
  return csa_ripple(p, bw, rip, s);
}
template <class S> SWord fadd4(const SWord& x, const SWord& y, const SWord& z, const SWord& w, uint32_t m1, uint32_t m2,
                               uint32_t rip, S& s) {
  SWord p1, b1, p2, b2;
  csa_layer(x, y, z, m1, s, p1, b1);
  csa_layer(p1, b1, w, m2, s, p2, b2);
  return csa_ripple(p2, b2, rip, s);
}
template <class S> SWord materialize(const SWord& raw, uint32_t base, S& s) {
  SWord o;
  for (int b = 0; b < 32; ++b) { s.row(base + b, raw[b], Sup{Z_CONST_POS}); o[b] = {base + (uint32_t)b}; }
  return o;
}

template <class S> void walk_rows(S& s) {
  s.row(Z_CONST_POS, Sup{Z_CONST_POS}, Sup{Z_CONST_POS});
  for (int w = 0; w < 8; ++w) for (int b = 0; b < 32; ++b) s.row(h_bit(w, b), Sup{h_bit(w, b)}, Sup{Z_CONST_POS});
  for (int i = 0; i < 16; ++i) for (int b = 0; b < 32; ++b) s.row(m_bit(i, b), Sup{m_bit(i, b)}, Sup{Z_CONST_POS});
  std::vector<SWord> h_in(8), w_arr;
  for (int w = 0; w < 8; ++w) h_in[w] = wire(h_bit(w, 0));
  for (int i = 0; i < 16; ++i) w_arr.push_back(wire(m_bit(i, 0)));
  for (int t = 16; t < 64; ++t) {
    SWord s1 = sx3(w_arr[t - 2], 17, 19, 10), s0 = sx3(w_arr[t - 15], 7, 18, 3);
    w_arr.push_back(fadd4(s1, s0, w_arr[t - 7], w_arr[t - 16], sched_bit(t, SC_MAJ1), sched_bit(t, SC_MAJ2),
                          sched_bit(t, SC_RIP), s));
  }
  std::array<SWord, 8> st;
  for (int i = 0; i < 8; ++i) st[i] = h_in[i];
  for (int r = 0; r < N_ROUNDS; ++r) {
    SWord a = st[0], bb = st[1], c = st[2], d = st[3], e = st[4], f = st[5], g = st[6], h = st[7];
    SWord ch_and, maj_and;
    for (int b = 0; b < 32; ++b) {
      uint32_t sl = CH_AND_BASE + 32 * r + b;
      s.row(sl, e[b], xs(f[b], g[b]));
      ch_and[b] = {sl};
    }
    for (int b = 0; b < 32; ++b) {
      uint32_t sl = MAJ_AND_BASE + 32 * r + b;
      s.row(sl, xs(a[b], bb[b]), xs(a[b], c[b]));
      maj_and[b] = {sl};
    }
    SWord ch_out = xw(ch_and, g), maj_out = xw(maj_and, a);
    SWord hk = add_const(Sha256::K[r], h, round_bit(r, RC_ADDK), s);
    SWord t1 = fadd4(hk, rx3(e, 6, 11, 25), ch_out, w_arr[r], round_bit(r, RC_MAJ1), round_bit(r, RC_MAJ2),
                     round_bit(r, RC_RIP), s);
    SWord a_raw = fadd3(t1, rx3(a, 2, 13, 22), maj_out, round_bit(r, RC_AMAJ), round_bit(r, RC_ARIP), s);
    bool mat = (r % EA_PERIOD) == EA_PERIOD - 1;
    SWord a_new = mat ? materialize(a_raw, a_new_bit(r, 0), s) : a_raw;
    SWord e_raw = add32(d, t1, round_bit(r, RC_ENEW), s);
    SWord e_new = mat ? materialize(e_raw, e_new_bit(r, 0), s) : e_raw;
    st = {a_new, a, bb, c, e_new, e, f, g};
  }
  for (int w = 0; w < 8; ++w) {
    SWord raw = add32(st[w], h_in[w], out_carry_bit(w, 0), s);
    materialize(raw, h_out_bit(w, 0), s);
  }
}

inline void build_matrices(SparseRows& A, SparseRows& B) {
  A.num_rows = A.num_cols = B.num_rows = B.num_cols = K;
  A.rows.assign(K, {});
  B.rows.assign(K, {});
  MatSink s{A, B};
  walk_rows(s);
}

struct Compression {
  uint32_t h[8];
  uint32_t w[16];
};

// Witness bits z, a = A_0 z, b = B_0 z of one block (caller-zeroed K-bit buffers).
inline void witness_block(const Compression& in, uint64_t* z, uint64_t* a, uint64_t* b) {
  auto lin = [&](uint32_t bit, uint32_t v) { or_u32_at(z, bit, v); or_u32_at(a, bit, v); or_u32_at(b, bit, 0xFFFFFFFFu); };
  auto put3 = [&](uint32_t bit, uint32_t zv, uint32_t av, uint32_t bv) { or_u32_at(z, bit, zv); or_u32_at(a, bit, av); or_u32_at(b, bit, bv); };
  or_bit_at(z, Z_CONST_POS); or_bit_at(a, Z_CONST_POS); or_bit_at(b, Z_CONST_POS);
  for (int w = 0; w < 8; ++w) lin(h_bit(w, 0), in.h[w]);
  for (int i = 0; i < 16; ++i) lin(m_bit(i, 0), in.w[i]);
  uint32_t W[64];
  for (int i = 0; i < 16; ++i) W[i] = in.w[i];
  for (int t = 16; t < 64; ++t) {
    Add4Parts p = fused_add4_parts(small_sigma1(W[t - 2]), small_sigma0(W[t - 15]), W[t - 7], W[t - 16]);
    put3(sched_bit(t, SC_MAJ1), p.maj1[2], p.maj1[0], p.maj1[1]);
    put3(sched_bit(t, SC_MAJ2), p.maj2[2], p.maj2[0], p.maj2[1]);
    put3(sched_bit(t, SC_RIP), p.rip[2], p.rip[0], p.rip[1]);
    W[t] = p.sum;
  }
  uint32_t aa = in.h[0], bb = in.h[1], cc = in.h[2], dd = in.h[3], ee = in.h[4], ff = in.h[5], gg = in.h[6], hh = in.h[7];
  for (int r = 0; r < N_ROUNDS; ++r) {
    uint32_t fxg = ff ^ gg, ch_and = ee & fxg;
    put3(CH_AND_BASE + 32 * r, ch_and, ee, fxg);
    uint32_t bxa = bb ^ aa, cxa = cc ^ aa, maj_and = bxa & cxa;
    put3(MAJ_AND_BASE + 32 * r, maj_and, bxa, cxa);
    uint32_t ch_out = ch_and ^ gg, maj_out = maj_and ^ aa;
    AddParts kp = const_add_parts(Sha256::K[r], hh);
    put3(round_bit(r, RC_ADDK), kp.carry, kp.left, kp.right);
    Add4Parts t1 = fused_add4_parts(kp.sum, big_sigma1(ee), ch_out, W[r]);
    put3(round_bit(r, RC_MAJ1), t1.maj1[2], t1.maj1[0], t1.maj1[1]);
    put3(round_bit(r, RC_MAJ2), t1.maj2[2], t1.maj2[0], t1.maj2[1]);
    put3(round_bit(r, RC_RIP), t1.rip[2], t1.rip[0], t1.rip[1]);
    Add3Parts an = fused_add3_parts(t1.sum, big_sigma0(aa), maj_out);
    put3(round_bit(r, RC_AMAJ), an.maj[2], an.maj[0], an.maj[1]);
    put3(round_bit(r, RC_ARIP), an.rip[2], an.rip[0], an.rip[1]);
    AddParts en = add_carry_parts(dd, t1.sum);
    put3(round_bit(r, RC_ENEW), en.carry, en.left, en.right);
    if (r % EA_PERIOD == EA_PERIOD - 1) {
      lin(a_new_bit(r, 0), an.sum);
      lin(e_new_bit(r, 0), en.sum);
    }
    hh = gg; gg = ff; ff = ee; ee = en.sum; dd = cc; cc = bb; bb = aa; aa = an.sum;
  }
  uint32_t fs[8] = {aa, bb, cc, dd, ee, ff, gg, hh};
  for (int w = 0; w < 8; ++w) {
    AddParts o = add_carry_parts(fs[w], in.h[w]);
    put3(out_carry_bit(w, 0), o.carry, o.left, o.right);
    lin(h_out_bit(w, 0), o.sum);
  }
}

}  // namespace s2r1cs
}  // namespace flock
