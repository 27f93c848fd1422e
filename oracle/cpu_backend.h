// ORACLE — test infrastructure only. A plain CPU restatement of every bulk step of
// the prove_fast path, used by the tests and the benchmark's CPU baseline as the
// checker for the CUDA backend. It is never linked into the product library.
//
// Each method restates the reference's definition of the step directly:
//   witness layout       crates/flock-prover/src/r1cs_hashes/common.rs:456-600 (batch-major words, byte stripe)
//   L0 commit            crates/flock-core/src/pcs/commit.rs:474-530, ntt/additive_ntt_f128.rs:67-158,627-648,
//                        merkle.rs:593-661
//   zerocheck round 1    crates/flock-core/src/zerocheck/univariate_skip.rs:50-140, :380-470 (naive
//                        definition, extract-c and s_hat_v_c forms), ntt.rs:18-117 (GF(2^8) NTT)
//   zerocheck folds      zerocheck/multilinear.rs:250-330, :1148-1200
//   lincheck             lincheck.rs:238-281 (column folds; Keccak-f from the forward rows,
//                        keccak_columns.h), :930-990 (row fold), :1479-1630 (sumcheck)
//   merged open          pcs/jagged.rs:1521-1650, :4693-4760
//   Ligerito             pcs/ligerito/extension.rs:17-80, :210-260, :1507-1600, pcs/ligerito.rs:3086-3150
#pragma once
#include "../flock_gb300/csrc/host/prover.h"
#include "keccak_columns.h"

namespace flock {
namespace oracle {

// ---- host parallelism for the checker's bulk loops ------------------------------------
// Contiguous chunks of [0, n) over the host thread pool. Every sum below is over GF(2^k)
// (XOR), so per-chunk partial sums combine to the same bits in any split or order.
inline size_t par_parts(size_t n, size_t grain = 1024) {
  if (n < 2 * grain) return 1;
  return std::min<size_t>(n / grain, 8 * (ThreadPool::instance().workers() + 1));
}
template <class Fn>
inline void par_chunks(size_t n, Fn&& fn, size_t grain = 1024) {
  const size_t parts = par_parts(n, grain);
  if (parts <= 1) { if (n) fn(size_t(0), n); return; }
  parallel_for(parts, [&](size_t p) { fn(n * p / parts, n * (p + 1) / parts); });
}
// Sum of per-chunk partials: fn(begin, end, acc) adds its chunk's terms into acc.
template <class T, class Fn>
inline T par_sum(size_t n, Fn&& fn) {
  const size_t parts = par_parts(n);
  std::vector<T> part(std::max<size_t>(parts, 1));
  if (parts <= 1) { if (n) fn(size_t(0), n, part[0]); return part[0]; }
  parallel_for(parts, [&](size_t p) { fn(n * p / parts, n * (p + 1) / parts, part[p]); });
  T acc = part[0];
  for (size_t p = 1; p < parts; ++p) acc = acc + part[p];
  return acc;
}
struct Two128 {
  F128 x, y;
  Two128 operator+(const Two128& o) const { return {x + o.x, y + o.y}; }
};
struct Two256 {
  F256 x, y;
  Two256 operator+(const Two256& o) const { return {x + o.x, y + o.y}; }
};
// eq table of build_eq (field.h) with the widest layers expanded in parallel.
inline std::vector<F128> par_build_eq(const std::vector<F128>& point, F128 scale = F128::one()) {
  std::vector<F128> out(size_t(1) << point.size());
  out[0] = scale;
  for (size_t j = 0; j < point.size(); ++j) {
    const size_t len = size_t(1) << j;
    const F128 r = point[j], r1 = r + F128::one();
    par_chunks(len, [&](size_t b, size_t e) {
      for (size_t i = b; i < e; ++i) {
        F128 v = out[i];
        out[i + len] = v * r;
        out[i] = v * r1;
      }
    });
  }
  return out;
}
// GF(2^8) product table (from gf8_mul) for the round-1 extension products.
inline const std::vector<uint8_t>& gf8_mul_table() {
  static const std::vector<uint8_t> t = [] {
    std::vector<uint8_t> v(65536);
    for (int a = 0; a < 256; ++a)
      for (int b = 0; b < 256; ++b) v[a * 256 + b] = gf8_mul((uint8_t)a, (uint8_t)b);
    return v;
  }();
  return t;
}

// ---- GF(2^8) additive NTT (ntt.rs:18-117) --------------------------------------------
inline std::vector<uint8_t> gf8_twiddles(int k, uint8_t beta) {
  int n = 1 << k;
  std::vector<uint8_t> tw(n - 1, 0);
  int len = 1 << (k - 1);
  std::vector<uint8_t> layer(len);
  for (int i = 0; i < len; ++i) layer[i] = beta ^ (uint8_t)(2 * i);
  uint8_t s_at_root = 1;
  int write_at = len;
  for (int i = 0; i < len; ++i) tw[write_at - 1 + i] = layer[i];
  auto next_s = [](uint8_t s, uint8_t root) { return (uint8_t)(gf8_mul(s, s) ^ gf8_mul(root, s)); };
  for (int it = 1; it < k; ++it) {
    write_at >>= 1;
    uint8_t next_root = next_s(layer[1] ^ layer[0], s_at_root);
    int new_len = write_at;
    for (int i = 0; i < new_len; ++i) layer[i] = next_s(layer[2 * i], s_at_root);
    len = new_len;
    s_at_root = next_root;
    uint8_t sinv = gf8_inv(s_at_root);
    for (int j = 0; j < len; ++j) tw[write_at - 1 + j] = gf8_mul(sinv, layer[j]);
  }
  return tw;
}
inline void gf8_fft(uint8_t* v, int n, const std::vector<uint8_t>& tw, int idx) {
  if (n == 1) return;
  int half = n >> 1;
  uint8_t lam = tw[idx - 1];
  for (int i = 0; i < half; ++i) { uint8_t w = v[half + i]; v[i] ^= gf8_mul(lam, w); v[half + i] = w ^ v[i]; }
  gf8_fft(v, half, tw, 2 * idx);
  gf8_fft(v + half, half, tw, 2 * idx + 1);
}
inline void gf8_ifft(uint8_t* v, int n, const std::vector<uint8_t>& tw, int idx) {
  if (n == 1) return;
  int half = n >> 1;
  gf8_ifft(v, half, tw, 2 * idx);
  gf8_ifft(v + half, half, tw, 2 * idx + 1);
  uint8_t lam = tw[idx - 1];
  for (int i = 0; i < half; ++i) { v[half + i] ^= v[i]; v[i] ^= gf8_mul(lam, v[half + i]); }
}
// Extension S -> Lambda of a 64-point bit row, as 8 byte-chunk tables of 64 outputs.
struct SkipExtension {
  uint8_t tab[8][256][64];
  uint8_t unit[64][64];  // extension of each unit vector e_s
  SkipExtension() {
    auto tws = gf8_twiddles(6, 0), twl = gf8_twiddles(6, 64);
    for (int s = 0; s < 64; ++s) {
      uint8_t v[64] = {0};
      v[s] = 1;
      gf8_ifft(v, 64, tws, 1);
      gf8_fft(v, 64, twl, 1);
      memcpy(unit[s], v, 64);
    }
    for (int c = 0; c < 8; ++c)
      for (int x = 0; x < 256; ++x) {
        uint8_t o[64] = {0};
        for (int b = 0; b < 8; ++b)
          if ((x >> b) & 1) for (int i = 0; i < 64; ++i) o[i] ^= unit[8 * c + b][i];
        memcpy(tab[c][x], o, 64);
      }
  }
  void extend(uint64_t bits, uint8_t out[64]) const {
    memset(out, 0, 64);
    for (int c = 0; c < 8; ++c) {
      const uint8_t* t = tab[c][(bits >> (8 * c)) & 255];
      for (int i = 0; i < 64; ++i) out[i] ^= t[i];
    }
  }
};
inline const SkipExtension& skip_extension() { static SkipExtension e; return e; }

// ---- additive NTT over F128 (additive_ntt_f128.rs:67-158, 627-648) -------------------
struct Ntt128 {
  uint32_t log_d = 0;
  std::vector<F128> tw;  // tw[(1 << layer) - 1 + block]
  explicit Ntt128(uint32_t ld) : log_d(ld) {
    // normalised subspace-polynomial table evals[i] = [W_i(b_i) .. W_i(b_{l-1})] / W_i(b_i)
    std::vector<std::vector<F128>> ev(ld);
    std::vector<F128> basis(ld);
    for (uint32_t i = 0; i < ld; ++i) basis[i] = F128(1ull << i, 0);
    if (ld) ev[0] = basis;
    for (uint32_t i = 1; i < ld; ++i)
      for (size_t k = 1; k < ev[i - 1].size(); ++k) ev[i].push_back(ev[i - 1][k] * (ev[i - 1][k] + ev[i - 1][0]));
    for (auto& row : ev) { F128 iv = inv(row[0]); for (auto& v : row) v = v * iv; }
    tw.assign(ld ? (size_t(1) << ld) - 1 : 0, F128());
    for (uint32_t layer = 0; layer < ld; ++layer) {
      const auto& v = ev[ld - layer - 1];
      for (size_t block = 0; block < (size_t(1) << layer); ++block) {
        F128 acc;
        for (size_t j = 0; j + 1 < v.size(); ++j) if ((block >> j) & 1) acc += v[j + 1];
        tw[(size_t(1) << layer) - 1 + block] = acc;
      }
    }
  }
  // Interleaved SoA transform of `lanes` independent NTTs (data[pos * lanes + lane]),
  // layers [start, log_d).
  void forward_interleaved(F128* data, size_t lanes, uint32_t start) const {
    if (log_d == 0) return;
    for (uint32_t layer = start; layer < log_d; ++layer) {
      const uint32_t hl = log_d - layer - 1;
      const size_t half = size_t(1) << hl;
      // butterfly j: block j >> hl, offset j & (half - 1)
      par_chunks(size_t(1) << (log_d - 1), [&](size_t jb, size_t je) {
        for (size_t j = jb; j < je; ++j) {
          const size_t block = j >> hl;
          const F128 t = tw[(size_t(1) << layer) - 1 + block];
          const size_t i0 = (block << (hl + 1)) + (j & (half - 1));
          F128* u = data + i0 * lanes;
          F128* v = data + (i0 | half) * lanes;
          for (size_t l = 0; l < lanes; ++l) {
            F128 nu = u[l] + v[l] * t;
            u[l] = nu;
            v[l] = v[l] + nu;
          }
        }
      });
    }
  }
};

inline std::vector<Hash> merkle_tree(const F128* data, size_t n_leaves, size_t leaf_words) {
  std::vector<Hash> tree(2 * n_leaves - 1);
  par_chunks(n_leaves, [&](size_t b, size_t e) {
    for (size_t i = b; i < e; ++i) tree[i] = Sha256::hash(data + i * leaf_words, leaf_words * 16);
  });
  size_t rs = 0, rl = n_leaves;
  while (rl > 1) {
    par_chunks(rl / 2, [&](size_t b, size_t e) {
      for (size_t i = b; i < e; ++i) {
        Sha256 h;
        h.update(tree[rs + 2 * i].data(), 32);
        h.update(tree[rs + 2 * i + 1].data(), 32);
        tree[rs + rl + i] = h.digest();
      }
    });
    rs += rl;
    rl >>= 1;
  }
  return tree;
}
inline std::vector<Hash> cap_layer(const std::vector<Hash>& tree, size_t n_leaves, uint32_t c) {
  size_t l = size_t(1) << c;
  return std::vector<Hash>(tree.begin() + (2 * n_leaves - 2 * l), tree.begin() + (2 * n_leaves - l));
}
inline void merkle_path_capped(const std::vector<Hash>& tree, size_t n_leaves, size_t idx, uint32_t c,
                               std::vector<Hash>& out) {
  size_t start = 0, len = n_leaves;
  while (len > (size_t(1) << c)) {
    out.push_back(tree[start + (idx ^ 1)]);
    start += len;
    len >>= 1;
    idx >>= 1;
  }
}

inline Msg256 round_msg(const std::vector<F256>& f, const std::vector<F256>& b, size_t d) {
  size_t n = f.size();
  if (d == 1 || n == d) d = 1;
  // pair j: block j / d, offset j % d
  Two256 s = par_sum<Two256>(n / 2, [&](size_t jb, size_t je, Two256& acc) {
    for (size_t j = jb; j < je; ++j) {
      size_t lo = 2 * (j / d) * d + j % d, hi = lo + d;
      acc.x += f[lo] * b[lo];
      acc.y += (f[lo] + f[hi]) * (b[lo] + b[hi]);
    }
  });
  Msg256 m;
  m.u0 = s.x;
  m.u2 = s.y;
  return m;
}
inline std::vector<F256> fold_ext(const std::vector<F256>& v, F256 r, size_t d) {
  size_t half = v.size() / 2;
  std::vector<F256> o(half);
  par_chunks(half, [&](size_t ib, size_t ie) {
    for (size_t i = ib; i < ie; ++i) {
      size_t blk = i / d, w = i % d, lo = 2 * blk * d + w, hi = lo + d;
      o[i] = v[lo] + r * (v[hi] + v[lo]);
    }
  });
  return o;
}

// Column folds of one slot's matrices by the row weight eq_inner = skip_w (x) eq(xir)
// (lincheck.rs:238-281, lincheck/union.rs:255-275): comb_a = eq_inner^T A_0,
// comb_b = eq_inner^T B_0 (CSC for BLAKE3 / SHA-256; Keccak-f from the forward rows).
inline void lincheck_combs(const SlotInfo& T, const std::vector<F128>& skip_w, const std::vector<F128>& xir,
                           std::vector<F128>& comb_a, std::vector<F128>& comb_b) {
  const uint32_t K = 1u << T.k_log;
  auto er = par_build_eq(xir);
  std::vector<F128> eqi(K);
  par_chunks(K, [&](size_t b, size_t e) {
    for (size_t i = b; i < e; ++i) eqi[i] = skip_w[i & 63] * er[i >> 6];
  });
  if (T.hash == HASH_KECCAK) {
    keccak_columns_forward(eqi.data(), comb_a, comb_b);
    return;
  }
  comb_a.assign(K, F128()); comb_b.assign(K, F128());
  par_chunks(K, [&](size_t cb, size_t ce) {
    for (size_t c = cb; c < ce; ++c) {
      for (uint32_t p = T.csc_a->col_ptr[c]; p < T.csc_a->col_ptr[c + 1]; ++p) comb_a[c] += eqi[T.csc_a->rows_flat[p]];
      for (uint32_t p = T.csc_b->col_ptr[c]; p < T.csc_b->col_ptr[c + 1]; ++p) comb_b[c] += eqi[T.csc_b->rows_flat[p]];
    }
  });
}
// Slot t's share of x_inner_rest: its own k_log_t - 6 column coordinates.
inline std::vector<F128> slot_inner(const SlotInfo& T, const std::vector<F128>& x_inner_rest) {
  return std::vector<F128>(x_inner_rest.begin(), x_inner_rest.begin() + (T.k_log - 6));
}

class CpuBackend : public ProverBackend {
 public:
  explicit CpuBackend(const Statement& s) : S(s) {}

  const Statement& S;
  std::vector<F128> z, a, b;        // 2^(m-7) words, batch-major union buffers
  std::vector<F128> q;              // the committed stack (the compaction of z)
  std::vector<F128> cw0;            // L0 codeword, SoA (pos * lanes + lane)
  std::vector<std::vector<F128>> slot_ca, slot_cb;  // per-slot column folds
  std::vector<Hash> tree0;
  std::vector<F128> amlv, bmlv;
  std::vector<F128> comb_a, comb_b, comb, zv, zv_cap;
  std::vector<F128> mq, mw;
  std::vector<F256> lf, lb, pending;
  struct Level { std::vector<F128> mat; std::vector<Hash> tree; size_t block_len = 0, lanes = 0; };
  std::vector<Level> levels;

  size_t words() const { return size_t(1) << (S.m - 7); }

  // Union witness (union.rs:674-760): slot t's block is the aligned word range starting
  // at its offset / 128; instance o of the slot writes word ((c << nu) + o) of that block;
  // rows [count, 2^nu), unused columns and gaps stay zero.
  void witness(const std::vector<const uint8_t*>& slot_inputs) override {
    const uint32_t nu = S.nu;
    z.assign(words(), F128()); a.assign(words(), F128()); b.assign(words(), F128());
    for (size_t si = 0; si < S.slots.size(); ++si) {
      const SlotInfo& T = S.slots[si];
      const uint32_t K = 1u << T.k_log;
      const size_t rec = input_record_bytes(T.hash), base = T.offset >> 7;
      const uint8_t* inputs = slot_inputs[si];
      par_chunks(T.count, [&](size_t ob, size_t oe) {
        std::vector<uint64_t> bz(K / 64), ba(K / 64), bb(K / 64);
        for (size_t o = ob; o < oe; ++o) {
          std::fill(bz.begin(), bz.end(), 0); std::fill(ba.begin(), ba.end(), 0); std::fill(bb.begin(), bb.end(), 0);
          const uint8_t* in = inputs + o * rec;
          if (T.hash == HASH_BLAKE3) {
            b3r1cs::Compression c; memcpy(&c, in, sizeof(c));
            b3r1cs::witness_block(c, bz.data(), ba.data(), bb.data());
          } else if (T.hash == HASH_SHA256) {
            s2r1cs::Compression c; memcpy(&c, in, sizeof(c));
            s2r1cs::witness_block(c, bz.data(), ba.data(), bb.data());
          } else {
            uint64_t w[25]; memcpy(w, in, sizeof(w));
            kr1cs::witness_block(w, bz.data(), ba.data(), bb.data());
          }
          for (uint32_t c = 0; c < K / 128; ++c) {
            size_t wi = base + (size_t(c) << nu) + o;
            z[wi] = F128(bz[2 * c], bz[2 * c + 1]);
            a[wi] = F128(ba[2 * c], ba[2 * c + 1]);
            b[wi] = F128(bb[2 * c], bb[2 * c + 1]);
          }
        }
      }, 4);
    }
  }

  // q = the declared n_t-row prefix of every used chunk-column, slot by slot, zero-padded
  // to the committed length (union.rs:436-495, compact_witness).
  void compact() {
    if (S.identity) { q = z; return; }
    q.assign(S.committed_words, F128());
    const uint32_t nu = S.nu;
    size_t cursor = 0;
    for (const SlotInfo& T : S.slots) {
      const size_t start = T.offset >> 7;
      for (uint64_t c = 0; c < T.used_cols; ++c)
        for (uint64_t r = 0; r < T.count; ++r) q[cursor++] = z[start + (c << nu) + r];
    }
  }

  void commit_l0(uint32_t cap_depth, std::vector<Hash>& cap) override {
    const size_t t = S.lanes, D = size_t(1) << S.log_dim, npos = size_t(1) << S.k_code;
    compact();
    cw0.assign(npos * t, F128());
    par_chunks(npos, [&](size_t pb, size_t pe) {
      for (size_t p = pb; p < pe; ++p)
        for (size_t l = 0; l < t; ++l) cw0[p * t + l] = q[l * D + (p % D)];
    });
    Ntt128 ntt(S.k_code);
    ntt.forward_interleaved(cw0.data(), t, 1);
    tree0 = merkle_tree(cw0.data(), npos, t);
    cap = cap_layer(tree0, npos, cap_depth);
  }

  // ---- zerocheck
  static uint64_t row_bits(const std::vector<F128>& v, size_t x) { return (x & 1) ? v[x >> 1].hi : v[x >> 1].lo; }

  void zc_round1(const std::vector<F128>& r, std::vector<F128>& ab, std::vector<F128>& c,
                 std::vector<F128>& svc) override {
    const uint32_t m = S.m;
    const size_t nrows = size_t(1) << (m - 6);
    std::vector<F128> rr(r.begin() + 6, r.end());
    auto eq = par_build_eq(rr);
    const SkipExtension& E = skip_extension();
    const uint8_t* gm = gf8_mul_table().data();
    // acc[i * 256 + v] = sum of eq over rows whose extended product at point i is v;
    // cs[s] = sum of eq over rows with bit s of c set
    struct Round1Acc {
      std::vector<F128> acc, cs;
      Round1Acc operator+(const Round1Acc& o) const {
        Round1Acc r = *this;
        if (r.acc.empty()) return o;
        if (!o.acc.empty()) {
          for (size_t i = 0; i < r.acc.size(); ++i) r.acc[i] += o.acc[i];
          for (size_t i = 0; i < r.cs.size(); ++i) r.cs[i] += o.cs[i];
        }
        return r;
      }
    };
    Round1Acc tot = par_sum<Round1Acc>(nrows, [&](size_t xb, size_t xe, Round1Acc& R) {
      R.acc.assign(64 * 256, F128());
      R.cs.assign(64, F128());
      uint8_t ea[64], eb[64];
      for (size_t x = xb; x < xe; ++x) {
        uint64_t abits = row_bits(a, x), bbits = row_bits(b, x), cbits = row_bits(z, x);
        F128 e = eq[x];
        if (abits && bbits) {
          E.extend(abits, ea);
          E.extend(bbits, eb);
          for (int i = 0; i < 64; ++i) {
            uint8_t p = gm[ea[i] * 256 + eb[i]];
            if (p) R.acc[i * 256 + p] += e;
          }
        }
        while (cbits) { int s = __builtin_ctzll(cbits); R.cs[s] += e; cbits &= cbits - 1; }
      }
    });
    std::vector<F128>& acc = tot.acc;
    std::vector<F128>& cs = tot.cs;
    ab.assign(64, F128()); c.assign(64, F128());
    for (int i = 0; i < 64; ++i)
      for (int v = 1; v < 256; ++v) if (!acc[i * 256 + v].is_zero()) ab[i] += phi8((uint8_t)v) * acc[i * 256 + v];
    for (int i = 0; i < 64; ++i)
      for (int s = 0; s < 64; ++s) if (E.unit[s][i]) c[i] += phi8(E.unit[s][i]) * cs[s];
    // s_hat_v_c[t] = sum_w eq(r[7..m], w) * bit_t(z[w])
    std::vector<F128> r7(r.begin() + 7, r.end());
    auto eq7 = par_build_eq(r7);
    struct Vec128 {
      std::vector<F128> v;
      Vec128 operator+(const Vec128& o) const {
        Vec128 r = *this;
        for (size_t i = 0; i < r.v.size(); ++i) r.v[i] += o.v[i];
        return r;
      }
    };
    svc = par_sum<Vec128>(words(), [&](size_t wb, size_t we, Vec128& R) {
      R.v.assign(128, F128());
      for (size_t w = wb; w < we; ++w) {
        uint64_t lo = z[w].lo, hi = z[w].hi;
        while (lo) { int t = __builtin_ctzll(lo); R.v[t] += eq7[w]; lo &= lo - 1; }
        while (hi) { int t = __builtin_ctzll(hi); R.v[64 + t] += eq7[w]; hi &= hi - 1; }
      }
    }).v;
  }

  static void pair_message(const std::vector<F128>& A, const std::vector<F128>& Bv, const std::vector<F128>& eqp,
                           F128& g1, F128& gi) {
    auto eq = par_build_eq(eqp);
    Two128 s = par_sum<Two128>(A.size() / 2, [&](size_t xb, size_t xe, Two128& acc) {
      for (size_t x = xb; x < xe; ++x) {
        F128 a0 = A[2 * x], a1 = A[2 * x + 1], b0 = Bv[2 * x], b1 = Bv[2 * x + 1];
        acc.x += eq[x] * (a1 * b1);
        acc.y += eq[x] * ((a0 + a1) * (b0 + b1));
      }
    });
    g1 = s.x;
    gi = s.y;
  }
  void zc_fold_skip(const std::vector<F128>& w, const std::vector<F128>& eq_point, F128& g1, F128& gi) override {
    const size_t nrows = size_t(1) << (S.m - 6);
    amlv.assign(nrows, F128()); bmlv.assign(nrows, F128());
    par_chunks(nrows, [&](size_t xb, size_t xe) {
      for (size_t x = xb; x < xe; ++x) {
        uint64_t ab_ = row_bits(a, x), bb_ = row_bits(b, x);
        F128 sa, sb;
        while (ab_) { int s = __builtin_ctzll(ab_); sa += w[s]; ab_ &= ab_ - 1; }
        while (bb_) { int s = __builtin_ctzll(bb_); sb += w[s]; bb_ &= bb_ - 1; }
        amlv[x] = sa; bmlv[x] = sb;
      }
    });
    pair_message(amlv, bmlv, eq_point, g1, gi);
  }
  static void fold_low(std::vector<F128>& v, F128 r) {
    size_t h = v.size() / 2;
    std::vector<F128> o(h);
    par_chunks(h, [&](size_t xb, size_t xe) {
      for (size_t x = xb; x < xe; ++x) o[x] = v[2 * x] + r * (v[2 * x + 1] + v[2 * x]);
    });
    v.swap(o);
  }
  void zc_fold(F128 rho, const std::vector<F128>& eq_point, F128& g1, F128& gi) override {
    fold_low(amlv, rho); fold_low(bmlv, rho);
    pair_message(amlv, bmlv, eq_point, g1, gi);
  }
  void zc_final(F128 rho, F128& ae, F128& be) override {
    fold_low(amlv, rho); fold_low(bmlv, rho);
    ae = amlv[0]; be = bmlv[0];
  }

  // ---- lincheck
  void lc_comb(const std::vector<F128>& skip_w, const std::vector<F128>& xir) override {
    slot_ca.assign(S.slots.size(), {});
    slot_cb.assign(S.slots.size(), {});
    for (size_t t = 0; t < S.slots.size(); ++t)
      lincheck_combs(S.slots[t], skip_w, slot_inner(S.slots[t], xir), slot_ca[t], slot_cb[t]);
  }
  void lc_zvec(const std::vector<F128>& x_outer) override {
    const uint32_t K = 1u << S.k_log, nu = S.nu;
    auto eo = par_build_eq(x_outer);
    zv.assign(K, F128());
    parallel_for(K / 128, [&](size_t cc) {
      for (size_t row = 0; row < (size_t(1) << nu); ++row) {
        F128 w = z[(size_t(cc) << nu) + row];
        uint64_t lo = w.lo, hi = w.hi;
        while (lo) { int t = __builtin_ctzll(lo); zv[cc * 128 + t] += eo[row]; lo &= lo - 1; }
        while (hi) { int t = __builtin_ctzll(hi); zv[cc * 128 + 64 + t] += eo[row]; hi &= hi - 1; }
      }
    });
    zv_cap = zv;
  }
  static void top_message(const std::vector<F128>& c, const std::vector<F128>& v, F128& e1, F128& ei) {
    size_t h = c.size() / 2;
    e1 = F128(); ei = F128();
    for (size_t i = 0; i < h; ++i) {
      e1 += c[h + i] * v[h + i];
      ei += (c[h + i] + c[i]) * (v[h + i] + v[i]);
    }
  }
  void lc_start(F128 alpha, const std::vector<SlotComb>& sc, F128& e1, F128& ei) override {
    comb.assign(size_t(1) << S.k_log, F128());
    for (size_t t = 0; t < S.slots.size(); ++t) {
      const auto& ca = slot_ca[t];
      const auto& cb = slot_cb[t];
      par_chunks(ca.size(), [&](size_t b0, size_t e0) {
        for (size_t i = b0; i < e0; ++i) comb[sc[t].offset + i] = sc[t].weight * (alpha * ca[i] + cb[i]);
      });
    }
    for (size_t t = 0; t < S.slots.size(); ++t) comb[sc[t].offset + sc[t].pin] += sc[t].beta;
    top_message(comb, zv, e1, ei);
  }
  static void bind_top(std::vector<F128>& v, F128 r) {
    size_t h = v.size() / 2;
    for (size_t i = 0; i < h; ++i) v[i] = v[i] + r * (v[i + h] + v[i]);
    v.resize(h);
  }
  void lc_round(F128 r, bool last, F128& e1, F128& ei) override {
    bind_top(comb, r); bind_top(zv, r);
    if (!last) top_message(comb, zv, e1, ei);
  }
  void lc_partial(std::vector<F128>& zp) override { zp = zv; }
  void lc_matrix_evals(const std::vector<F128>& rest, const std::vector<F128>& zp, std::vector<Pair128>& evals) override {
    for (size_t t = 0; t < S.slots.size(); ++t) {
      auto er = build_eq(slot_inner(S.slots[t], rest));
      F128 ea, eb;
      for (size_t c = 0; c < slot_ca[t].size(); ++c) {
        F128 w = er[c >> 6] * zp[c & 63];
        ea += w * slot_ca[t][c];
        eb += w * slot_cb[t][c];
      }
      evals.push_back({ea, eb});
    }
  }
  void lc_s_hat_v(const std::vector<F128>& tail, std::vector<F128>& out) override {
    auto et = par_build_eq(tail);
    out.assign(128, F128());
    parallel_for(128, [&](size_t bb) {
      for (size_t k = 0; k < et.size(); ++k) out[bb] += et[k] * zv_cap[bb + 128 * k];
    });
  }

  // ---- merged open
  void mo_build_w(const std::vector<WeightClaim>& cl, uint32_t nu, uint64_t area, F128& u0, F128& u2) override {
    const size_t n = q.size();
    mw.assign(n, F128());
    std::vector<std::vector<F128>> er(cl.size()), ec(cl.size());
    for (size_t i = 0; i < cl.size(); ++i) { er[i] = par_build_eq(cl[i].z_row); ec[i] = par_build_eq(cl[i].z_col); }
    // jagged unrank (jagged.rs:132-140): column y holds dense [pfx[y], pfx[y+1])
    const auto& pfx = S.col_prefix;
    parallel_for(pfx.size() - 1, [&](size_t col) {
      for (uint64_t d = pfx[col]; d < pfx[col + 1] && d < area; ++d) {
        const size_t row = d - pfx[col];
        F128 acc;
        for (size_t i = 0; i < cl.size(); ++i) acc += fold_one_slot(er[i][row] * ec[i][col], cl[i].table.data());
        mw[d] = acc;
      }
    });
    (void)nu;
    mq = q;
    Two128 s = par_sum<Two128>(n / 2, [&](size_t ib, size_t ie, Two128& acc) {
      for (size_t i = ib; i < ie; ++i) {
        acc.x += mq[2 * i] * mw[2 * i];
        acc.y += (mq[2 * i] + mq[2 * i + 1]) * (mw[2 * i] + mw[2 * i + 1]);
      }
    });
    u0 = s.x;
    u2 = s.y;
  }
  void mo_round(F128 r, bool last, F128& g1, F128& gi) override {
    fold_low(mq, r); fold_low(mw, r);
    if (!last) {
      Two128 s = par_sum<Two128>(mq.size() / 2, [&](size_t ib, size_t ie, Two128& acc) {
        for (size_t i = ib; i < ie; ++i) {
          acc.x += mq[2 * i + 1] * mw[2 * i + 1];
          acc.y += (mq[2 * i] + mq[2 * i + 1]) * (mw[2 * i] + mw[2 * i + 1]);
        }
      });
      g1 = s.x;
      gi = s.y;
    }
  }
  F128 mo_q_eval() override { return mq[0]; }

  // ---- Ligerito
  void lg_basis_eq(F128 gamma, const std::vector<F128>& rho) override {
    auto e = par_build_eq(rho, gamma);
    lb.resize(e.size());
    par_chunks(e.size(), [&](size_t b, size_t en) { for (size_t i = b; i < en; ++i) lb[i] = F256(e[i]); });
    lf.resize(q.size());
    par_chunks(q.size(), [&](size_t b, size_t en) { for (size_t i = b; i < en; ++i) lf[i] = F256(q[i]); });
  }
  F128 lg_eval_eq(const std::vector<F128>& zp) override {
    auto e = par_build_eq(zp);
    return par_sum<F128>(lf.size(), [&](size_t b, size_t en, F128& acc) {
      for (size_t i = b; i < en; ++i) acc += lf[i].c0 * e[i];
    });
  }
  void lg_add_eq(F128 beta, const std::vector<F128>& zp) override {
    auto e = par_build_eq(zp, beta);
    par_chunks(lb.size(), [&](size_t b, size_t en) { for (size_t i = b; i < en; ++i) lb[i] += F256(e[i]); });
  }
  Msg256 lg_message(size_t d) override { return round_msg(lf, lb, d); }
  void lg_fold(F256 r, size_t d) override { lf = fold_ext(lf, r, d); lb = fold_ext(lb, r, d); }
  void lg_code_switch() override {
    std::vector<F256> nf(2 * lf.size()), nb(2 * lb.size());
    par_chunks(lf.size(), [&](size_t b, size_t e) {
      for (size_t i = b; i < e; ++i) { nf[2 * i] = F256(lf[i].c0); nf[2 * i + 1] = F256(lf[i].c1); }
    });
    par_chunks(lb.size(), [&](size_t b, size_t e) {
      for (size_t i = b; i < e; ++i) { nb[2 * i] = lb[i]; nb[2 * i + 1] = F256::u() * lb[i]; }
    });
    lf.swap(nf); lb.swap(nb);
  }
  void lg_commit(uint32_t level, uint32_t log_cols, uint32_t log_lanes, uint32_t log_rate, uint32_t cap_depth,
                 std::vector<Hash>& cap) override {
    Level L;
    L.lanes = size_t(1) << log_lanes;
    L.block_len = size_t(1) << (log_cols + log_rate);
    size_t msg = lf.size();
    L.mat.resize(L.block_len * L.lanes);
    par_chunks(L.mat.size(), [&](size_t b, size_t e) { for (size_t i = b; i < e; ++i) L.mat[i] = lf[i % msg].c0; });
    Ntt128 ntt(log_cols + log_rate);
    ntt.forward_interleaved(L.mat.data(), L.lanes, log_rate);
    L.tree = merkle_tree(L.mat.data(), L.block_len, L.lanes);
    cap = cap_layer(L.tree, L.block_len, cap_depth);
    if (levels.size() < level + 1) levels.resize(level + 1);
    levels[level] = std::move(L);
  }
  Msg256 lg_introduce_eq(const std::vector<F128>& zp, F128& answer) override {
    auto e = par_build_eq(zp);
    pending.resize(e.size());
    answer = par_sum<F128>(e.size(), [&](size_t b, size_t en, F128& acc) {
      for (size_t i = b; i < en; ++i) { acc += lf[i].c0 * e[i]; pending[i] = F256(e[i]); }
    });
    return round_msg(lf, pending, 1);
  }
  Msg256 lg_introduce_induced(uint32_t ln, uint32_t, const std::vector<uint64_t>&, const std::vector<F128>& w,
                              const std::vector<std::vector<F128>>& what) override {
    size_t n = size_t(1) << ln;
    // queries split into a few groups, each summing its own basis vector
    const size_t groups = std::min<size_t>(w.size(), ThreadPool::instance().workers() + 1);
    std::vector<std::vector<F128>> part(groups, std::vector<F128>(n));
    parallel_for(groups, [&](size_t g) {
      std::vector<F128> tmp(n);
      for (size_t q = w.size() * g / groups; q < w.size() * (g + 1) / groups; ++q) {
        tmp[0] = w[q];
        for (uint32_t k = 0; k < ln; ++k) {
          size_t cur = size_t(1) << k;
          for (size_t i = 0; i < cur; ++i) tmp[i + cur] = what[q][k] * tmp[i];
        }
        for (size_t i = 0; i < n; ++i) part[g][i] += tmp[i];
      }
    });
    std::vector<F128> basis(n);
    for (auto& pv : part)
      for (size_t i = 0; i < n; ++i) basis[i] += pv[i];
    pending.resize(2 * n);
    for (size_t i = 0; i < n; ++i) { pending[2 * i] = F256(basis[i]); pending[2 * i + 1] = F256::u() * F256(basis[i]); }
    return round_msg(lf, pending, 1);
  }
  void lg_glue(F128 beta) override {
    par_chunks(lb.size(), [&](size_t b, size_t e) { for (size_t i = b; i < e; ++i) lb[i] += pending[i] * beta; });
  }
  void lg_open(uint32_t level, const std::vector<uint64_t>& pos, uint32_t cap_depth,
               std::vector<std::vector<F128>>& rows, std::vector<Hash>& paths) override {
    const F128* mat; size_t lanes, bl; const std::vector<Hash>* tree;
    if (level == 0) { mat = cw0.data(); lanes = S.lanes; bl = size_t(1) << S.k_code; tree = &tree0; }
    else { mat = levels[level].mat.data(); lanes = levels[level].lanes; bl = levels[level].block_len; tree = &levels[level].tree; }
    for (uint64_t q : pos) {
      rows.emplace_back(mat + q * lanes, mat + (q + 1) * lanes);
      merkle_path_capped(*tree, bl, q, cap_depth, paths);
    }
  }
  std::vector<F256> lg_residual() override { return lf; }
};

}  // namespace oracle
}  // namespace flock
