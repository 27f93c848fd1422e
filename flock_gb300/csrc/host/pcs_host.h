// Host-side algebra of the prove_fast path: the pieces that act on O(128)- to
// O(m * 2^col_log)-sized objects and therefore never touch the committed data.
//
//  * Lagrange weights on the phi8 node sets S = phi8{0..63} and Lambda = phi8{64..127}
//    (crates/flock-core/src/zerocheck/multilinear.rs:150-240).
//  * The ring-switch reduction of one claim (crates/flock-core/src/pcs/ring_switch.rs:
//    1406-1450, 1587-1603, 2724-2760) and the linearised form of its fold map
//    (ring_switch.rs:1686-1775).
//  * The multipoint twisted assist and its untwisted anchor
//    (crates/flock-core/src/pcs/jagged.rs:146-260, 556-720, 1660-2020, 2790-3300),
//    restated in closed form for the aligned full-height column layout every
//    full-utilisation single-slot statement has (columns c < used_cols hold rows
//    [0, 2^nu), dense index d = c * 2^nu + row).
//  * The Ligerito induced-basis point weights (crates/flock-core/src/pcs/ligerito.rs:
//    2396-2460) and the queried-row enforced sum (pcs/ligerito/extension.rs:2893-2916).
#pragma once
#include "field.h"
#include "transcript.h"
#include "parallel.h"
#include "proof.h"
#include "setup.h"
#include <thread>

namespace flock {

// ---------------------------------------------------------------- Lagrange on phi8 sets
inline const std::pair<F128, F128>& subspace_den6() {
  static std::pair<F128, F128> d = [] {
    F128 den = F128::one();
    for (int i = 1; i < 64; ++i) den = den * phi8((uint8_t)i);
    return std::make_pair(den, inv(den));
  }();
  return d;
}
inline const std::pair<F128, F128>& subspace_den7() {
  static std::pair<F128, F128> d = [] {
    F128 den = F128::one();
    for (int i = 1; i < 128; ++i) den = den * phi8((uint8_t)i);
    return std::make_pair(den, inv(den));
  }();
  return d;
}
// Weights L_i(z) on the 64 nodes phi8(offset + i), offset in {0, 64}.
inline std::vector<F128> lagrange_weights64(F128 z, int offset) {
  std::vector<F128> w(64);
  F128 zn = F128::one();
  for (int i = 0; i < 64; ++i) zn = zn * (z + phi8((uint8_t)(offset + i)));
  if (zn.is_zero()) {
    for (int i = 0; i < 64; ++i) w[i] = (z == phi8((uint8_t)(offset + i))) ? F128::one() : F128();
    return w;
  }
  F128 scale = zn * subspace_den6().second;
  // batched inversion of the 64 differences: one field inversion and 3 * 63 products
  F128 d[64], pre[64];
  F128 run = F128::one();
  for (int i = 0; i < 64; ++i) {
    d[i] = z + phi8((uint8_t)(offset + i));
    pre[i] = run;
    run = run * d[i];
  }
  F128 inv_run = inv(run) * scale;
  for (int i = 63; i >= 0; --i) {
    w[i] = inv_run * pre[i];
    inv_run = inv_run * d[i];
  }
  return w;
}
inline F128 interpolate_on_lambda(const std::vector<F128>& vals, F128 z) {
  auto w = lagrange_weights64(z, 64);
  F128 acc;
  for (int i = 0; i < 64; ++i) acc += w[i] * vals[i];
  return acc;
}

// ---------------------------------------------------------------- ring switch
inline std::vector<F128> tensor_transpose128(const std::vector<F128>& v) {
  std::vector<F128> u(128);
  for (int i = 0; i < 128; ++i) {
    for (int b = 0; b < 128; ++b) {
      uint64_t bit = b < 64 ? (v[i].lo >> b) & 1 : (v[i].hi >> (b - 64)) & 1;
      if (bit) { if (i < 64) u[b].lo |= 1ull << i; else u[b].hi |= 1ull << (i - 64); }
    }
  }
  return u;
}
// 16 x 256 byte tables: tab[k*256 + v] = sum of eq[8k + bit] over set bits of v (each
// entry one XOR from the entry without v's lowest set bit).
inline std::vector<F128> fold_byte_table(const std::vector<F128>& eq128) {
  std::vector<F128> t(16 * 256);
  for (int k = 0; k < 16; ++k)
    for (int v = 1; v < 256; ++v)
      t[k * 256 + v] = t[k * 256 + (v & (v - 1))] + eq128[8 * k + __builtin_ctz((unsigned)v)];
  return t;
}
inline F128 fold_one_slot(const F128& x, const F128* tab) {
  F128 acc;
  for (int k = 0; k < 8; ++k) acc += tab[k * 256 + ((x.lo >> (8 * k)) & 255)];
  for (int k = 0; k < 8; ++k) acc += tab[(8 + k) * 256 + ((x.hi >> (8 * k)) & 255)];
  return acc;
}
inline F128 bit_basis(int t) { return t < 64 ? F128(1ull << t, 0) : F128(0, 1ull << (t - 64)); }

// Inverse of the Moore matrix M[t][j] = e_t^(2^j), row-major inv[j*128 + t].
inline const std::vector<F128>& moore_inverse() {
  static std::vector<F128> inv_m = [] {
    const int N = 128;
    std::vector<F128> m(N * N), iv(N * N);
    for (int t = 0; t < N; ++t) {
      F128 x = bit_basis(t);
      for (int j = 0; j < N; ++j) { m[t * N + j] = x; x = x * x; }
    }
    for (int i = 0; i < N; ++i) iv[i * N + i] = F128::one();
    for (int col = 0; col < N; ++col) {
      int piv = col;
      while (m[piv * N + col].is_zero()) ++piv;
      if (piv != col)
        for (int k = 0; k < N; ++k) { std::swap(m[col * N + k], m[piv * N + k]); std::swap(iv[col * N + k], iv[piv * N + k]); }
      F128 p = inv(m[col * N + col]);
      for (int k = 0; k < N; ++k) { m[col * N + k] = m[col * N + k] * p; iv[col * N + k] = iv[col * N + k] * p; }
      for (int r = 0; r < N; ++r) {
        if (r == col || m[r * N + col].is_zero()) continue;
        F128 f = m[r * N + col];
        for (int k = 0; k < N; ++k) { m[r * N + k] += f * m[col * N + k]; iv[r * N + k] += f * iv[col * N + k]; }
      }
    }
    return iv;
  }();
  return inv_m;
}
inline std::vector<F128> linearized_coefficients(const std::vector<F128>& tab) {
  const auto& mi = moore_inverse();
  std::vector<F128> phi(128), c(128);
  for (int t = 0; t < 128; ++t) phi[t] = fold_one_slot(bit_basis(t), tab.data());
  parallel_for(16, [&](size_t blk) {
    for (int j = 8 * (int)blk; j < 8 * (int)blk + 8; ++j) {
      F128 acc;
      for (int t = 0; t < 128; ++t) acc += mi[j * 128 + t] * phi[t];
      c[j] = acc;
    }
  });
  return c;
}

// One claim of the batched ring switch: absorb s_hat_v, sample r'' under PoW, return
// the sumcheck claim <transpose(s_hat_v), eq(r'')> and the (unscaled) fold table.
struct RingSwitchOut {
  RingSwitchProof proof;
  F128 sumcheck_claim;
  std::vector<F128> eq;     // eq(r'') over the 128 packing positions
  std::vector<F128> table;  // fold_byte_table(eq)
  // The table of gamma * eq: the table is linear in eq, so this is gamma times every
  // entry, built from 128 products instead of 4096.
  void scale(F128 gamma) {
    for (auto& e : eq) e = e * gamma;
    table = fold_byte_table(eq);
  }
};
inline RingSwitchOut ring_switch_claim(Transcript& T, const std::vector<F128>& s_hat_v, uint32_t bits) {
  RingSwitchOut o;
  T.observe_label("flock-ring-switch-v0");
  T.observe_f128_slice(s_hat_v);
  std::vector<F128> rdp;
  if (bits) { auto pr = T.grind_pow_and_sample_f128_vec(bits, 7); o.proof.grinding_nonce = pr.first; rdp = pr.second; }
  else rdp = T.sample_f128_vec(7);
  auto eq = build_eq(rdp);
  auto u = tensor_transpose128(s_hat_v);
  F128 acc;
  for (int i = 0; i < 128; ++i) acc += u[i] * eq[i];
  o.sumcheck_claim = acc;
  o.table = fold_byte_table(eq);
  o.eq = std::move(eq);
  o.proof.s_hat_v = s_hat_v;
  return o;
}

// ---------------------------------------------------------------- aligned jagged layout
// General jagged layout (jagged.rs:87-140): column y of 2^k occupies dense indices
// [pfx[y], pfx[y+1]); rows n, dense variables m.
struct JaggedLayout {
  uint32_t n = 0, k = 0, m = 0;
  std::vector<uint64_t> pfx;
  uint64_t area() const { return pfx.empty() ? 0 : pfx.back(); }
};

struct AlignedJagged {
  uint32_t n = 0;       // row variables (nu)
  uint32_t k = 0;       // column variables (col_log)
  uint32_t m = 0;       // dense variables = n + k
  uint64_t used = 0;    // full-height columns [0, used)
  uint64_t area() const { return used << n; }
};

// sum over boolean c < used of prod_b f_b(c_b), with f_b given as (f_b(0), f_b(1)).
inline F128 prefix_product_sum(const std::pair<F128, F128>* f, int k, uint64_t used) {
  if (used >= (uint64_t(1) << k)) {
    F128 p = F128::one();
    for (int b = 0; b < k; ++b) p = p * (f[b].first + f[b].second);
    return p;
  }
  // suffix totals of the free low bits
  F128 low_total[65];
  low_total[0] = F128::one();
  for (int b = 0; b < k; ++b) low_total[b + 1] = low_total[b] * (f[b].first + f[b].second);
  F128 acc, high = F128::one();
  for (int j = k - 1; j >= 0; --j) {
    if ((used >> j) & 1) {
      acc += high * f[j].first * low_total[j];
      high = high * f[j].second;
    } else {
      high = high * f[j].first;
    }
  }
  return acc;
}
inline F128 prefix_product_sum(const std::vector<std::pair<F128, F128>>& f, uint64_t used) {
  return prefix_product_sum(f.data(), (int)f.size(), used);
}
// eq(a, b) for boolean b as field value: (1 + a) or a.
inline std::pair<F128, F128> eq_pair(F128 a) { return {a + F128::one(), a}; }

// ---------------------------------------------------------------- the anchor assist
// Width-4 branching program for g(a, b, c, d) = [b < d and b = a + c] read LSB-first
// (jagged.rs:164-192). state = carry + 2 * comparison.
inline int bp_transition(int row, int index, int curr, int next, int state) {
  int carry = state & 1, cmp = (state >> 1) & 1;
  int sum = row + carry + curr;
  if (index != (sum & 1)) return -1;
  int nc = sum >> 1;
  int ncmp = index == next ? cmp : next;
  return nc + (ncmp << 1);
}
constexpr int BP_INITIAL = 0, BP_SUCCESS = 2;

// Layer matrix M(a, b; c, d)[s][s'] for boolean c, d, given eq4[row + 2 index] = eq((a,b), (row,index)).
inline void bp_layer_matrix(const F128 eq4[4], int c, int d, F128 M[4][4]) {
  for (int s = 0; s < 4; ++s) for (int t = 0; t < 4; ++t) M[s][t] = F128();
  for (int s = 0; s < 4; ++s)
    for (int row = 0; row < 2; ++row)
      for (int idx = 0; idx < 2; ++idx) {
        int o = bp_transition(row, idx, c, d, s);
        if (o >= 0) M[s][o] += eq4[row + 2 * idx];
      }
}

struct AssistStatement {
  std::vector<F128> z_row;                    // length n (zero-padded beyond)
  std::vector<F128> w;                        // per boundary-run weight
  std::vector<std::pair<uint64_t, uint64_t>> t;  // (t_{y-1}, t_y) per run
};

// Prover of the batched (untwisted) assist over `sts` at `point` (length m): proves
// V = sum_st sum_runs w * g_hat(z_row, point, t_c, t_next) with 2(m+1) degree-2 rounds.
inline FrobeniusAssistProof prove_anchor_assist(Transcript& T, const std::vector<AssistStatement>& sts,
                                                const std::vector<F128>& point, uint32_t m, uint32_t round_bits) {
  const int L = (int)m + 1;  // layers 0..m
  auto pbit = [](const std::vector<F128>& z, int l) { return l < (int)z.size() ? z[l] : F128(); };
  struct St {
    std::vector<std::array<F128, 4>> eq4;                // per layer
    std::vector<std::vector<std::array<F128, 4>>> sfx;   // sfx[l][run] = S_l (state vector), l in 0..L
    std::vector<F128> part;                              // per-run partial weights
    std::array<F128, 4> prefix;
    // Layers [0, uniform) read the same (c, d) bits for every run (for the aligned layout:
    // the row bits, all zero). There part[r] = w_r * common and the per-run bucket sum is
    // common * ws[l], ws[l] = sum_r w_r S_{l+1}(r), precomputed in parallel.
    int uniform = 0;
    int ucd = 0;
    F128 common = F128::one();
    std::vector<std::array<F128, 4>> ws;
  };
  std::vector<St> S(sts.size());
  for (size_t si = 0; si < sts.size(); ++si) {
    const AssistStatement& a = sts[si];
    St& s = S[si];
    s.eq4.resize(L);
    for (int l = 0; l < L; ++l) {
      auto e = build_eq({pbit(a.z_row, l), pbit(point, l)});
      s.eq4[l] = {e[0], e[1], e[2], e[3]};
    }
    size_t R = a.w.size();
    s.sfx.assign(L + 1, std::vector<std::array<F128, 4>>(R));
    for (size_t r = 0; r < R; ++r) { s.sfx[L][r] = {F128(), F128(), F128(), F128()}; s.sfx[L][r][BP_SUCCESS] = F128::one(); }
    std::vector<std::array<std::array<std::array<F128, 4>, 4>, 4>> Mc(L);
    for (int l = 0; l < L; ++l)
      for (int cd = 0; cd < 4; ++cd) {
        F128 M[4][4];
        bp_layer_matrix(s.eq4[l].data(), cd & 1, (cd >> 1) & 1, M);
        for (int st = 0; st < 4; ++st)
          for (int o = 0; o < 4; ++o) Mc[l][cd][st][o] = M[st][o];
      }
    parallel_for(R, [&](size_t r) {
      for (int l = L - 1; l >= 0; --l) {
        int c = (int)((a.t[r].first >> l) & 1), d = (int)((a.t[r].second >> l) & 1);
        const auto& nx = s.sfx[l + 1][r];
        const auto& M = Mc[l][c + 2 * d];
        std::array<F128, 4> out{};
        for (int st = 0; st < 4; ++st) {
          F128 acc;
          for (int o = 0; o < 4; ++o) acc += M[st][o] * nx[o];
          out[st] = acc;
        }
        s.sfx[l][r] = out;
      }
    });
    s.part = a.w;
    s.prefix = {F128(), F128(), F128(), F128()};
    s.prefix[BP_INITIAL] = F128::one();
    // longest prefix of layers with one (c, d) for every run
    auto cd_of = [&](size_t r, int l) { return (int)((a.t[r].first >> l) & 1) + 2 * (int)((a.t[r].second >> l) & 1); };
    while (s.uniform < L && R > 0) {
      int cd0 = cd_of(0, s.uniform);
      bool same = true;
      for (size_t r = 1; r < R && same; ++r) same = cd_of(r, s.uniform) == cd0;
      if (!same || (s.uniform > 0 && cd0 != s.ucd)) break;
      s.ucd = cd0;
      s.uniform++;
    }
    s.ws.assign(s.uniform, {F128(), F128(), F128(), F128()});
    parallel_for((size_t)s.uniform, [&](size_t l) {
      std::array<F128, 4> acc{};
      for (size_t r = 0; r < R; ++r)
        for (int o = 0; o < 4; ++o) acc[o] += a.w[r] * s.sfx[l + 1][r][o];
      s.ws[l] = acc;
    });
  }
  FrobeniusAssistProof pf;
  F128 v;
  for (size_t si = 0; si < sts.size(); ++si)
    for (size_t r = 0; r < sts[si].w.size(); ++r) v += S[si].part[r] * S[si].sfx[0][r][BP_INITIAL];
  pf.v = v;
  T.observe_label("flock-frobenius-assist-v0");
  T.observe_f128(v);
  auto dot4 = [](const std::array<F128, 4>& a, const std::array<F128, 4>& b) {
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2] + a[3] * b[3];
  };
  auto add4 = [](const std::array<F128, 4>& a, const std::array<F128, 4>& b) {
    return std::array<F128, 4>{a[0] + b[0], a[1] + b[1], a[2] + b[2], a[3] + b[3]};
  };
  auto comb4 = [](F128 x, const std::array<F128, 4>& a, F128 y, const std::array<F128, 4>& b) {
    return std::array<F128, 4>{x * a[0] + y * b[0], x * a[1] + y * b[1], x * a[2] + y * b[2], x * a[3] + y * b[3]};
  };
  // Per-run work of layer l in one parallel pass over (statement, run chunk): first fold
  // the run partials by layer l - 1's bits and challenges (rc_prev, rd_prev), then add
  // part * S_{l+1} into the chunk's (c, d) buckets for layer l. Chunk buckets are summed
  // (XOR) afterwards, so the result does not depend on the split.
  constexpr size_t NCH = 32;
  using Bucket = std::array<std::array<F128, 4>, 4>;
  std::vector<Bucket> chunk_b(S.size() * NCH);
  std::vector<Bucket> B(S.size());
  auto run_pass = [&](int l, F128 rc_prev, F128 rd_prev) {
    parallel_for(S.size() * NCH, [&](size_t task) {
      const size_t si = task / NCH, ch = task % NCH;
      const AssistStatement& a = sts[si];
      St& s = S[si];
      const size_t R = a.w.size(), r0 = R * ch / NCH, r1 = R * (ch + 1) / NCH;
      Bucket bk{};
      const bool fold = l > 0 && l - 1 >= s.uniform, seed = l > 0 && l == s.uniform;
      const bool bucket = l < L && l >= s.uniform;
      const F128 rc1 = rc_prev + F128::one(), rd1 = rd_prev + F128::one();
      for (size_t r = r0; r < r1; ++r) {
        if (seed) s.part[r] = a.w[r] * s.common;
        if (fold) {
          int c = (int)((a.t[r].first >> (l - 1)) & 1), d = (int)((a.t[r].second >> (l - 1)) & 1);
          s.part[r] = s.part[r] * (c ? rc_prev : rc1) * (d ? rd_prev : rd1);
        }
        if (bucket) {
          int c = (int)((a.t[r].first >> l) & 1), d = (int)((a.t[r].second >> l) & 1);
          const auto& nx = s.sfx[l + 1][r];
          for (int o = 0; o < 4; ++o) bk[c + 2 * d][o] += s.part[r] * nx[o];
        }
      }
      chunk_b[task] = bk;
    });
    for (size_t si = 0; si < S.size(); ++si) {
      Bucket acc{};
      for (size_t ch = 0; ch < NCH; ++ch)
        for (int cd = 0; cd < 4; ++cd)
          for (int o = 0; o < 4; ++o) acc[cd][o] += chunk_b[si * NCH + ch][cd][o];
      B[si] = acc;
    }
  };
  run_pass(0, F128(), F128());
  for (int l = 0; l < L; ++l) {
    // per statement: u[cd] = prefix * M_l(c, d); bucket[cd] = sum over runs with bits (c,d) of part * S_{l+1}
    std::vector<std::array<std::array<F128, 4>, 4>> U(S.size());
    for (size_t si = 0; si < S.size(); ++si) {
      St& s = S[si];
      for (int cd = 0; cd < 4; ++cd) {
        F128 M[4][4];
        bp_layer_matrix(s.eq4[l].data(), cd & 1, (cd >> 1) & 1, M);
        for (int o = 0; o < 4; ++o) {
          F128 acc;
          for (int st = 0; st < 4; ++st) acc += s.prefix[st] * M[st][o];
          U[si][cd][o] = acc;
        }
      }
      if (l < s.uniform) {  // every run has the bits ucd here: one bucket, from the precomputed sums
        for (int cd = 0; cd < 4; ++cd) B[si][cd] = {F128(), F128(), F128(), F128()};
        for (int o = 0; o < 4; ++o) B[si][s.ucd][o] = s.common * s.ws[l][o];
      }
    }
    F128 g1, gi;
    for (size_t si = 0; si < S.size(); ++si) {
      g1 += dot4(U[si][1], B[si][1]) + dot4(U[si][3], B[si][3]);
      gi += dot4(add4(U[si][0], U[si][1]), add4(B[si][0], B[si][1])) + dot4(add4(U[si][2], U[si][3]), add4(B[si][2], B[si][3]));
    }
    T.observe_f128(g1); T.observe_f128(gi);
    F128 rc;
    if (round_bits) { auto pr = T.grind_pow_and_sample_f128(round_bits); pf.grinding_nonces.push_back(pr.first); rc = pr.second; }
    else rc = T.sample_f128();
    pf.rounds.push_back({g1, gi});
    F128 rc1 = rc + F128::one();
    g1 = F128(); gi = F128();
    std::vector<std::pair<std::array<F128, 4>, std::array<F128, 4>>> folded(S.size());
    for (size_t si = 0; si < S.size(); ++si) {
      auto ud0 = comb4(rc1, U[si][0], rc, U[si][1]);
      auto ud1 = comb4(rc1, U[si][2], rc, U[si][3]);
      auto d0 = comb4(rc1, B[si][0], rc, B[si][1]);
      auto d1 = comb4(rc1, B[si][2], rc, B[si][3]);
      g1 += dot4(ud1, d1);
      gi += dot4(add4(ud0, ud1), add4(d0, d1));
      folded[si] = {ud0, ud1};
    }
    T.observe_f128(g1); T.observe_f128(gi);
    F128 rd;
    if (round_bits) { auto pr = T.grind_pow_and_sample_f128(round_bits); pf.grinding_nonces.push_back(pr.first); rd = pr.second; }
    else rd = T.sample_f128();
    pf.rounds.push_back({g1, gi});
    F128 rd1 = rd + F128::one();
    for (size_t si = 0; si < S.size(); ++si) {
      S[si].prefix = comb4(rd1, folded[si].first, rd, folded[si].second);
      St& s = S[si];
      if (l < s.uniform) s.common = s.common * ((s.ucd & 1) ? rc : rc1) * ((s.ucd & 2) ? rd : rd1);
    }
    // the run partials fold by this layer's bits in the next layer's pass (not needed after
    // the last layer)
    if (l + 1 < L) run_pass(l + 1, rc, rd);
  }
  return pf;
}

// Runs of equal boundary pairs for the aligned layout and their column-weight sums.
inline AssistStatement aligned_statement(const AlignedJagged& J, const std::vector<F128>& z_row,
                                         const std::vector<F128>& z_col, F128 coeff) {
  AssistStatement a;
  a.z_row = z_row;
  auto eqc = build_eq(z_col);
  uint64_t H = uint64_t(1) << J.n;
  for (uint64_t y = 0; y < J.used; ++y) { a.w.push_back(eqc[y] * coeff); a.t.push_back({y * H, (y + 1) * H}); }
  uint64_t ncol = uint64_t(1) << J.k;
  if (J.used < ncol) {
    F128 s;
    for (uint64_t y = J.used; y < ncol; ++y) s += eqc[y];
    a.w.push_back(s * coeff);
    a.t.push_back({J.area(), J.area()});
  }
  return a;
}

// ---------------------------------------------------------------- multipoint twisted assist
struct RsClaimPoint {
  std::vector<F128> z_row, z_col;   // (n, k)
  std::vector<F128> coeffs;         // 128 linearised coefficients (gamma baked)
};

// x^(2^-j) for j = 0..127 of every coordinate (x^(2^128) = x).
inline std::vector<std::vector<F128>> rho_inverse_powers(const std::vector<F128>& rho) {
  std::vector<std::vector<F128>> sq(128, std::vector<F128>(rho.size()));
  for (size_t i = 0; i < rho.size(); ++i) {
    F128 x = rho[i];
    sq[0][i] = x;
    for (int e = 1; e < 128; ++e) { x = x * x; sq[e][i] = x; }
  }
  std::vector<std::vector<F128>> out(128);
  for (int j = 0; j < 128; ++j) out[j] = sq[(128 - j) % 128];
  return out;
}

// Prover of the multipoint twisted evaluation for ring-switched claims over the aligned
// layout (jagged.rs:2884-3290): 128 dual values per claim, one m-round two-product
// sumcheck of sum_d abar(d) g(d) with abar = sum_i gamma^(128 i) a_i and
// g = sum_j gamma^j eq(rho^(2^-j), .), then the untwisted anchor at the endpoint.
// Every message is evaluated in closed form over the tensor structure of a_i and g.
inline MultipointTwistedProof prove_multipoint(Transcript& T, const AlignedJagged& J,
                                               const std::vector<RsClaimPoint>& claims,
                                               const std::vector<F128>& rho, uint32_t round_bits,
                                               uint32_t anchor_round_bits) {
  const uint32_t n = J.n, k = J.k, m = J.m;
  const size_t R = claims.size();
  auto rp = rho_inverse_powers(rho);  // rp[j][t]
  MultipointTwistedProof pf;
  // ---- dual values A_{i,j}
  auto col_pps = [&](const std::vector<F128>& zc, const std::vector<F128>& rj, uint32_t off) {
    std::vector<std::pair<F128, F128>> f(k);
    for (uint32_t b = 0; b < k; ++b) {
      auto ez = eq_pair(zc[b]), er = eq_pair(rj[off + b]);
      f[b] = {ez.first * er.first, ez.second * er.second};
    }
    return prefix_product_sum(f, J.used);
  };
  pf.values.assign(R, std::vector<F128>(128));
  parallel_for(R * 128, [&](size_t ij) {
    size_t i = ij / 128, j = ij % 128;
    F128 rowp = F128::one();
    for (uint32_t t = 0; t < n; ++t) rowp = rowp * (F128::one() + claims[i].z_row[t] + rp[j][t]);
    pf.values[i][j] = rowp * col_pps(claims[i].z_col, rp[j], n);
  });
  T.observe_label("flock-multipoint-twisted-v1");
  for (auto& vs : pf.values) for (auto& v : vs) T.observe_f128(v);
  uint32_t gamma_bits = std::max<uint32_t>(1, grinding_bits_for_degree(128 * R - 1));
  auto gp = T.grind_pow_and_sample_f128(gamma_bits);
  pf.gamma_grinding_nonce = gp.first;
  F128 gamma = gp.second;
  std::vector<F128> gpow(128 * R);
  F128 p = F128::one();
  for (auto& g : gpow) { g = p; p = p * gamma; }
  // ---- closed-form two-product sumcheck
  // coef_ij = gamma^(128 i + j); prefix products over bound bits; row suffix products.
  std::vector<std::vector<F128>> P(R, std::vector<F128>(128)), rowsuf(R, std::vector<F128>(128 * (n + 1)));
  std::vector<std::vector<F128>> Ccol(R, std::vector<F128>(128));
  parallel_for(R * 128, [&](size_t ij) {
    size_t i = ij / 128, j = ij % 128;
    P[i][j] = gpow[128 * i + j];
    F128* sf = &rowsuf[i][j * (n + 1)];
    sf[n] = F128::one();
    for (int t = (int)n - 1; t >= 0; --t) sf[t] = sf[t + 1] * (F128::one() + claims[i].z_row[t] + rp[j][t]);
    Ccol[i][j] = col_pps(claims[i].z_col, rp[j], n);
  });
  std::vector<F128> s;  // bound challenges
  std::vector<F128> c1v(R * 128), civ(R * 128);
  // absorb the variable bound in round t (challenge r) into the prefix products
  auto absorb = [&](size_t ij, uint32_t t, F128 r) {
    size_t i = ij / 128, j = ij % 128;
    F128 f = F128::one() + rp[j][t] + r;  // eq(rho_j[t], r)
    if (t < n) f = f * (F128::one() + claims[i].z_row[t] + r);
    P[i][j] = P[i][j] * f;
  };
  // message of round t; with bind_prev, each item first absorbs round t - 1's challenge
  // (one parallel pass per round instead of two)
  auto message = [&](uint32_t t, F128& g1, F128& gi, bool bind_prev, F128 r_prev) {
    g1 = F128(); gi = F128();
    if (t < n) {
      parallel_for(R * 128, [&](size_t ij) {
        if (bind_prev) absorb(ij, t - 1, r_prev);
        size_t i = ij / 128, j = ij % 128;
        F128 c = P[i][j] * rowsuf[i][j * (n + 1) + t + 1] * Ccol[i][j];
        c1v[ij] = c * claims[i].z_row[t] * rp[j][t];
        civ[ij] = c;
      });
      for (size_t ij = 0; ij < R * 128; ++ij) { g1 += c1v[ij]; gi += civ[ij]; }
    } else {
      uint32_t b = t - n;
      parallel_for(R * 128, [&](size_t ij) {
        if (bind_prev) absorb(ij, t - 1, r_prev);
        size_t i = ij / 128, j = ij % 128;
        {
          // column weights: u < b bound to s, u = b the round variable, u > b summed against rho_j
          std::pair<F128, F128> f0[64], f1[64];
          for (uint32_t u = 0; u < k; ++u) {
            auto ez = eq_pair(claims[i].z_col[u]);
            std::pair<F128, F128> w;
            if (u < b) w = eq_pair(s[n + u]);
            else if (u > b) w = eq_pair(rp[j][n + u]);
            if (u == b) { f0[u] = {ez.first, F128()}; f1[u] = {F128(), ez.second}; }
            else { f0[u] = f1[u] = {ez.first * w.first, ez.second * w.second}; }
          }
          F128 l20 = prefix_product_sum(f0, (int)k, J.used), l21 = prefix_product_sum(f1, (int)k, J.used);
          F128 c = P[i][j];  // row factors and bound column factors of g already folded in
          c1v[ij] = c * rp[j][n + b] * l21;
          civ[ij] = c * (l20 + l21);
        }
      });
      for (size_t ij = 0; ij < R * 128; ++ij) { g1 += c1v[ij]; gi += civ[ij]; }
    }
  };
  F128 g1, gi;
  message(0, g1, gi, false, F128());
  for (uint32_t t = 0; t < m; ++t) {
    T.observe_f128(g1); T.observe_f128(gi);
    F128 r;
    if (round_bits) { auto pr = T.grind_pow_and_sample_f128(round_bits); pf.round_grinding_nonces.push_back(pr.first); r = pr.second; }
    else r = T.sample_f128();
    pf.rounds.push_back({g1, gi});
    s.push_back(r);
    if (t + 1 == m) break;
    message(t + 1, g1, gi, true, r);
  }
  // ---- anchor at the endpoint rho'' = s
  F128 g_at;
  std::vector<F128> gj(128);
  parallel_for(128, [&](size_t j) {
    F128 prod = gpow[j];
    for (uint32_t t = 0; t < m; ++t) prod = prod * (s[t] * rp[j][t] + (F128::one() + s[t]) * (F128::one() + rp[j][t]));
    gj[j] = prod;
  });
  for (int j = 0; j < 128; ++j) g_at += gj[j];
  std::vector<AssistStatement> sts;
  for (size_t i = 0; i < R; ++i) sts.push_back(aligned_statement(J, claims[i].z_row, claims[i].z_col, gpow[128 * i] * g_at));
  pf.anchor = prove_anchor_assist(T, sts, s, m, anchor_round_bits);
  return pf;
}

// Runs of equal boundary pairs (t_y, t_{y+1}) of a general layout, each with its summed
// column weight coeff * eq(z_col, y) (jagged.rs:564-620; grouping identical summands
// does not change any transcript value).
inline AssistStatement jagged_statement(const JaggedLayout& L, const std::vector<F128>& z_row,
                                        const std::vector<F128>& z_col, F128 coeff) {
  AssistStatement a;
  a.z_row = z_row;
  auto eqc = build_eq(z_col);
  for (size_t y = 0; y + 1 < L.pfx.size(); ++y) {
    std::pair<uint64_t, uint64_t> b{L.pfx[y], L.pfx[y + 1]};
    F128 w = eqc[y] * coeff;
    if (!a.t.empty() && a.t.back() == b) a.w.back() += w;
    else { a.w.push_back(w); a.t.push_back(b); }
  }
  return a;
}

// sum over runs of w * g_hat(z_row, point, t_c, t_next): the jagged weight's multilinear
// extension at `point` by the branching-program DP (jagged.rs:2547-2580, assist_g_values).
inline F128 jagged_weight_eval(const AssistStatement& a, const std::vector<F128>& point, uint32_t m) {
  const int L = (int)m + 1;
  auto pbit = [](const std::vector<F128>& z, int l) { return l < (int)z.size() ? z[l] : F128(); };
  std::vector<std::array<std::array<std::array<F128, 4>, 4>, 4>> Mc(L);
  for (int l = 0; l < L; ++l) {
    auto e = build_eq({pbit(a.z_row, l), pbit(point, l)});
    F128 eq4[4] = {e[0], e[1], e[2], e[3]};
    for (int cd = 0; cd < 4; ++cd) {
      F128 M[4][4];
      bp_layer_matrix(eq4, cd & 1, (cd >> 1) & 1, M);
      for (int st = 0; st < 4; ++st)
        for (int o = 0; o < 4; ++o) Mc[l][cd][st][o] = M[st][o];
    }
  }
  F128 acc;
  for (size_t r = 0; r < a.w.size(); ++r) {
    std::array<F128, 4> v{};
    v[BP_SUCCESS] = F128::one();
    for (int l = L - 1; l >= 0; --l) {
      const int c = (int)((a.t[r].first >> l) & 1), d = (int)((a.t[r].second >> l) & 1);
      const auto& M = Mc[l][c + 2 * d];
      std::array<F128, 4> out{};
      for (int st = 0; st < 4; ++st) {
        F128 x;
        for (int o = 0; o < 4; ++o) x += M[st][o] * v[o];
        out[st] = x;
      }
      v = out;
    }
    acc += a.w[r] * v[BP_INITIAL];
  }
  return acc;
}

// The multipoint twisted evaluation over a general jagged layout (jagged.rs:2884-3380,
// the materialised path): dual values A_ij = sum_d a_i(d) eq(rho^(2^-j), d) from the
// branching-program DP, then the m-round two-product sumcheck of sum_d abar(d) g(d) with
// abar = sum_i gamma^(128 i) a_i and g = sum_j gamma^j eq(rho^(2^-j), .) both
// materialised (g(d) is the F2-linear map x -> sum_j gamma^j x^(2^-j) of eq(rho, d)),
// then the untwisted anchor. The same field values as prove_multipoint on an aligned layout.
inline MultipointTwistedProof prove_multipoint_jagged(Transcript& T, const JaggedLayout& L,
                                                      const std::vector<RsClaimPoint>& claims,
                                                      const std::vector<F128>& rho, uint32_t round_bits,
                                                      uint32_t anchor_round_bits) {
  const uint32_t n = L.n, m = L.m;
  const size_t R = claims.size();
  auto rp = rho_inverse_powers(rho);
  MultipointTwistedProof pf;
  std::vector<AssistStatement> unit(R);
  for (size_t i = 0; i < R; ++i) unit[i] = jagged_statement(L, claims[i].z_row, claims[i].z_col, F128::one());
  pf.values.assign(R, std::vector<F128>(128));
  parallel_for(R * 128, [&](size_t ij) {
    const size_t i = ij / 128, j = ij % 128;
    pf.values[i][j] = jagged_weight_eval(unit[i], rp[j], m);
  });
  T.observe_label("flock-multipoint-twisted-v1");
  for (auto& vs : pf.values) for (auto& v : vs) T.observe_f128(v);
  uint32_t gamma_bits = std::max<uint32_t>(1, grinding_bits_for_degree(128 * R - 1));
  auto gp = T.grind_pow_and_sample_f128(gamma_bits);
  pf.gamma_grinding_nonce = gp.first;
  F128 gamma = gp.second;
  std::vector<F128> gpow(128 * R);
  F128 p = F128::one();
  for (auto& g : gpow) { g = p; p = p * gamma; }
  // ---- materialised abar (zero past the area) and g
  const size_t N = size_t(1) << m;
  std::vector<F128> abar(N), g(N);
  {
    std::vector<std::vector<F128>> er(R), ec(R);
    for (size_t i = 0; i < R; ++i) { er[i] = build_eq(claims[i].z_row); ec[i] = build_eq(claims[i].z_col); }
    const size_t ncol = L.pfx.size() - 1;
    parallel_for(ncol, [&](size_t y) {
      for (uint64_t d = L.pfx[y]; d < L.pfx[y + 1]; ++d) {
        F128 acc;
        for (size_t i = 0; i < R; ++i) acc += gpow[128 * i] * er[i][d - L.pfx[y]] * ec[i][y];
        abar[d] = acc;
      }
    });
    // images of the basis under x -> sum_j gamma^j x^(2^(128-j)), byte tables
    std::vector<F128> img(128);
    parallel_for(128, [&](size_t b) {
      std::vector<F128> sq(128);
      F128 x = bit_basis((int)b);
      for (int e = 0; e < 128; ++e) { sq[e] = x; x = x * x; }
      F128 acc;
      for (int j = 0; j < 128; ++j) acc += gpow[j] * sq[(128 - j) % 128];
      img[b] = acc;
    });
    std::vector<F128> tab(16 * 256);
    for (int kb = 0; kb < 16; ++kb)
      for (int v = 0; v < 256; ++v) {
        F128 acc;
        for (int i = 0; i < 8; ++i) if ((v >> i) & 1) acc += img[8 * kb + i];
        tab[kb * 256 + v] = acc;
      }
    auto e = build_eq(rho);
    parallel_for((N + 4095) / 4096, [&](size_t c) {
      for (size_t d = c * 4096; d < std::min(N, (c + 1) * 4096); ++d) g[d] = fold_one_slot(e[d], tab.data());
    });
  }
  auto message = [&](size_t len, F128& g1, F128& gi) {
    const size_t half = len / 2, nch = std::max<size_t>(1, std::min<size_t>(64, half / 1024));
    std::vector<F128> p1(nch), pi(nch);
    parallel_for(nch, [&](size_t c) {
      F128 a1, ai;
      for (size_t i = half * c / nch; i < half * (c + 1) / nch; ++i) {
        a1 += abar[2 * i + 1] * g[2 * i + 1];
        ai += (abar[2 * i] + abar[2 * i + 1]) * (g[2 * i] + g[2 * i + 1]);
      }
      p1[c] = a1;
      pi[c] = ai;
    });
    g1 = F128(); gi = F128();
    for (size_t c = 0; c < nch; ++c) { g1 += p1[c]; gi += pi[c]; }
  };
  auto fold = [&](size_t len, F128 r) {
    const size_t half = len / 2;
    std::vector<F128> na(half), ng(half);
    parallel_for((half + 4095) / 4096, [&](size_t c) {
      for (size_t i = c * 4096; i < std::min(half, (c + 1) * 4096); ++i) {
        na[i] = abar[2 * i] + r * (abar[2 * i + 1] + abar[2 * i]);
        ng[i] = g[2 * i] + r * (g[2 * i + 1] + g[2 * i]);
      }
    });
    abar.swap(na);
    g.swap(ng);
  };
  std::vector<F128> s;
  F128 g1, gi;
  size_t len = N;
  message(len, g1, gi);
  for (uint32_t t = 0; t < m; ++t) {
    T.observe_f128(g1); T.observe_f128(gi);
    F128 r;
    if (round_bits) { auto pr = T.grind_pow_and_sample_f128(round_bits); pf.round_grinding_nonces.push_back(pr.first); r = pr.second; }
    else r = T.sample_f128();
    pf.rounds.push_back({g1, gi});
    s.push_back(r);
    if (t + 1 == m) break;
    fold(len, r);
    len /= 2;
    message(len, g1, gi);
  }
  (void)n;
  // ---- anchor at the endpoint rho'' = s
  F128 g_at;
  std::vector<F128> gj(128);
  parallel_for(128, [&](size_t j) {
    F128 prod = gpow[j];
    for (uint32_t t = 0; t < m; ++t) prod = prod * (s[t] * rp[j][t] + (F128::one() + s[t]) * (F128::one() + rp[j][t]));
    gj[j] = prod;
  });
  for (int j = 0; j < 128; ++j) g_at += gj[j];
  std::vector<AssistStatement> sts;
  for (size_t i = 0; i < R; ++i) sts.push_back(jagged_statement(L, claims[i].z_row, claims[i].z_col, gpow[128 * i] * g_at));
  pf.anchor = prove_anchor_assist(T, sts, s, m, anchor_round_bits);
  return pf;
}

}  // namespace flock
