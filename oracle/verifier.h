// ORACLE — test infrastructure only. A verifier for prove_fast bundles: it replays the
// Fiat-Shamir transcript from the statement and the proof alone and checks every
// relation the reference verifier checks for a single-slot boolean union proof over the
// merged Ligerito transport. The tests use it as the acceptance check of proofs made by
// the CUDA path (the reference's own verifier cannot run here); it is never linked into
// the product library.
//
// Reference verifier, in call order (crates/flock-core/src/...):
//   statement binding      union.rs:619-628 (bind_statement)
//   zerocheck              zerocheck.rs:1032-1200 (verify_with_grinding),
//                          zerocheck/multilinear.rs:215-265 (Lambda / Lambda u S interpolation)
//   lincheck               lincheck/union.rs:711-945 (verify_union_deferred_with_grinding),
//                          :579-626 (MatrixAssertion::check), :538-572 (check_reported)
//   claim points           union.rs:541-599 (x_ab_from_mlv, ab_claim_point, c_claim_point)
//   merged opening         pcs.rs:2039-2300 (verify_batch_merged_core),
//                          pcs/ring_switch.rs:2966-3001 (verify_succinct_with_grinding)
//   multipoint assist      pcs/jagged.rs:4418-4590, :2068-2210 (anchor assist)
//   inner opening          pcs.rs:1129-1335 (verify_opening_batch_ligerito_mixed_with_grinding)
//   Ligerito F256 ladder   pcs/ligerito/extension.rs:2409-2796, :2290-2406 (residual bases),
//                          pcs/ligerito.rs:4564-4574, :5152-5214 (queries, capped openings),
//                          merkle.rs:698-735
// Grinding policies are the ones the prover applies (prover.h).
#pragma once
#include "cpu_backend.h"
#include <stdexcept>
#include <string>

namespace flock {
namespace oracle {

struct Reject : std::runtime_error {
  explicit Reject(const std::string& what) : std::runtime_error(what) {}
};
inline void require(bool ok, const char* what) {
  if (!ok) throw Reject(what);
}

// ---------------------------------------------------------------- bincode reader
class BincodeReader {
 public:
  BincodeReader(const uint8_t* p, size_t n) : p_(p), n_(n) {}
  size_t remaining() const { return n_ - o_; }
  uint64_t u64() {
    require(remaining() >= 8, "bundle: truncated");
    uint64_t v = 0;
    for (int i = 0; i < 8; ++i) v |= (uint64_t)p_[o_ + i] << (8 * i);
    o_ += 8;
    return v;
  }
  F128 f128() {
    uint64_t lo = u64();
    return F128(lo, u64());
  }
  F256 f256() {
    F128 a = f128();
    return F256(a, f128());
  }
  Hash hash() {
    require(remaining() >= 32, "bundle: truncated");
    Hash h;
    memcpy(h.data(), p_ + o_, 32);
    o_ += 32;
    return h;
  }
  // a length prefix whose items (each at least `item` bytes) fit in what is left
  size_t len(size_t item) {
    uint64_t n = u64();
    require(n <= remaining() / item, "bundle: vector length past the end");
    return (size_t)n;
  }
  std::vector<F128> vf() { std::vector<F128> v(len(16)); for (auto& x : v) x = f128(); return v; }
  std::vector<uint64_t> vu() { std::vector<uint64_t> v(len(8)); for (auto& x : v) x = u64(); return v; }
  std::vector<Pair128> vp() {
    std::vector<Pair128> v(len(32));
    for (auto& x : v) { x.first = f128(); x.second = f128(); }
    return v;
  }
  std::vector<Hash> vh() { std::vector<Hash> v(len(32)); for (auto& x : v) x = hash(); return v; }
  std::vector<std::vector<F128>> vvf() { std::vector<std::vector<F128>> v(len(8)); for (auto& x : v) x = vf(); return v; }
  RecursiveProof rec() { RecursiveProof r; r.opened_rows = vvf(); r.merkle_proof = vh(); return r; }

  MergedProof merged() {
    MergedProof p;
    ZerocheckProof& z = p.zerocheck;
    z.round1_ab = vf(); z.round1_c = vf(); z.multilinear_rounds = vp();
    z.final_a_eval = f128(); z.final_b_eval = f128(); z.final_c_eval = f128(); z.grinding_nonces = vu();
    LincheckProof& l = p.lincheck;
    l.rounds = vp(); l.z_partial = vf(); l.matrix_evals = vp(); l.grinding_nonces = vu();
    MergedOpenProof& o = p.pcs_open;
    o.ring_switches = rs(); o.batching_nonces = vu(); o.merged_rounds = vp(); o.merged_round_nonces = vu();
    o.q_eval = f128();
    MultipointTwistedProof& mp = o.frobenius;
    mp.values = vvf(); mp.group_values = vf(); mp.gamma_grinding_nonce = u64(); mp.rounds = vp();
    mp.round_grinding_nonces = vu();
    mp.anchor.v = f128(); mp.anchor.rounds = vp(); mp.anchor.grinding_nonces = vu();
    o.inner.ring_switches = rs(); o.inner.batching_nonces = vu();
    LigeritoProof& g = o.inner.ligerito;
    g.initial_cap = vh();
    g.initial_proof = rec();
    g.recursive_caps.resize(len(8));
    for (auto& c : g.recursive_caps) c = vh();
    g.recursive_proofs.resize(len(16));
    for (auto& r : g.recursive_proofs) r = rec();
    g.final_proof.yr = vf(); g.final_proof.opened_rows = vvf(); g.final_proof.merkle_proof = vh();
    g.sumcheck_transcript = vp();
    g.sumcheck_transcript_f256.resize(len(64));
    for (auto& m : g.sumcheck_transcript_f256) { m.u0 = f256(); m.u2 = f256(); }
    g.grinding_nonces = vu(); g.ood_values = vf(); g.fold_grinding_nonces = vu();
    g.claim_batch_grinding_nonces = vu(); g.consistency_batch_grinding_nonces = vu();
    return p;
  }

 private:
  std::vector<RingSwitchProof> rs() {
    std::vector<RingSwitchProof> v(len(16));
    for (auto& r : v) { r.s_hat_v = vf(); r.grinding_nonce = u64(); }
    return v;
  }
  const uint8_t* p_;
  size_t n_, o_ = 0;
};

// Bundle: u64 proof_len | bincode proof | u64 cap_len | cap x 32 | ab_value | c_value.
struct Bundle {
  MergedProof proof;
  std::vector<Hash> cap;
  ProofClaims claims;
};
inline Bundle parse_bundle(const uint8_t* p, size_t n) {
  BincodeReader outer(p, n);
  uint64_t plen = outer.u64();
  require(plen <= outer.remaining(), "bundle: proof length past the end");
  Bundle b;
  BincodeReader in(p + 8, (size_t)plen);
  b.proof = in.merged();
  require(in.remaining() == 0, "bundle: trailing bytes after the proof");
  BincodeReader tail(p + 8 + plen, n - 8 - (size_t)plen);
  b.cap = tail.vh();
  b.claims.ab_value = tail.f128();
  b.claims.c_value = tail.f128();
  require(tail.remaining() == 0, "bundle: trailing bytes");
  return b;
}

// ---------------------------------------------------------------- small algebra
// Interpolation at z of the degree < 128 polynomial that is zero on S = phi8{0..63} and
// takes `vals` on Lambda = phi8{64..127} (Lagrange over the 7-dimensional subspace
// S u Lambda: L_v(z) = Z(z) / (C (z + v)), C = product of its non-zero elements).
inline F128 interpolate_combined(const std::vector<F128>& vals, F128 z) {
  F128 zz = F128::one();
  for (int i = 0; i < 128; ++i) zz = zz * (z + phi8((uint8_t)i));
  if (zz.is_zero()) {
    for (int i = 0; i < 64; ++i)
      if (z == phi8((uint8_t)(64 + i))) return vals[i];
    return F128();
  }
  F128 scale = zz * subspace_den7().second, acc;
  for (int i = 0; i < 64; ++i) acc += scale * inv(z + phi8((uint8_t)(64 + i))) * vals[i];
  return acc;
}
inline F128 fold_round_claim(F128 claim, F128 g1, F128 gi, F128 r) {
  F128 g0 = claim + g1;
  return g0 + (g1 + g0 + gi) * r + gi * (r * r);
}
inline F128 pow_2j(F128 x, int j) {
  for (int i = 0; i < j; ++i) x = x * x;
  return x;
}

struct Quad256 {  // c + b X + a X^2 from a message (u0, u2) and the running claim
  F256 c, b, a;
  static Quad256 from(const Msg256& m, F256 claim) { return {m.u0, claim + m.u2, m.u2}; }
  F256 eval(F256 r) const { return c + r * b + (r * r) * a; }
  Quad256 fold(const Quad256& o, F128 al) const { return {c + o.c * al, b + o.b * al, a + o.a * al}; }
};

// ---------------------------------------------------------------- anchor + multipoint
// Anchor assist: replay 2 (m + 1) rounds, then the expected endpoint value
// sum_st (sum_runs w_r eq(t_r, sigma)) * g_hat(z_row, point, sigma) (jagged.rs:2068-2210).
// prod_j eq(coords[j], bit_j(bits)) (lincheck/union.rs:90-101).
inline F128 eq_prefix_weight(const std::vector<F128>& coords, uint64_t bits) {
  F128 acc = F128::one();
  for (size_t j = 0; j < coords.size(); ++j) acc = acc * (((bits >> j) & 1) ? coords[j] : F128::one() + coords[j]);
  return acc;
}
// sum_{i < n} eq(point, i) in O(|point|) (lincheck/union.rs:107-128); exactly one at n = 2^|point|.
inline F128 eq_prefix_sum(const std::vector<F128>& point, uint64_t n) {
  const size_t d = point.size();
  if (n == (uint64_t(1) << d)) return F128::one();
  F128 acc, high = F128::one();
  for (size_t j = d; j-- > 0;) {
    if ((n >> j) & 1) {
      acc += high * (F128::one() + point[j]);
      high = high * point[j];
    } else {
      high = high * (F128::one() + point[j]);
    }
  }
  return acc;
}

inline F128 verify_anchor(Transcript& T, const std::vector<AssistStatement>& sts, const std::vector<F128>& point,
                          uint32_t m, const FrobeniusAssistProof& pf, uint32_t bits) {
  require(pf.rounds.size() == 2 * (size_t(m) + 1), "anchor: round count");
  require(pf.grinding_nonces.size() == (bits ? pf.rounds.size() : 0), "anchor: nonce count");
  T.observe_label("flock-frobenius-assist-v0");
  T.observe_f128(pf.v);
  F128 claim = pf.v;
  std::vector<F128> sigma;
  for (size_t i = 0; i < pf.rounds.size(); ++i) {
    T.observe_f128(pf.rounds[i].first);
    T.observe_f128(pf.rounds[i].second);
    if (bits) require(T.verify_pow(pf.grinding_nonces[i], bits), "anchor: round grinding");
    F128 r = T.sample_f128();
    claim = fold_round_claim(claim, pf.rounds[i].first, pf.rounds[i].second, r);
    sigma.push_back(r);
  }
  const int L = (int)m + 1;
  auto coord = [](const std::vector<F128>& v, int l) { return l < (int)v.size() ? v[l] : F128(); };
  F128 expect;
  for (const AssistStatement& st : sts) {
    F128 w;
    for (size_t r = 0; r < st.w.size(); ++r) {
      F128 e = st.w[r];
      for (int l = 0; l < L; ++l) {
        int c = (int)((st.t[r].first >> l) & 1), d = (int)((st.t[r].second >> l) & 1);
        e = e * (c ? sigma[2 * l] : F128::one() + sigma[2 * l]) * (d ? sigma[2 * l + 1] : F128::one() + sigma[2 * l + 1]);
      }
      w += e;
    }
    F128 g[4] = {F128(), F128(), F128(), F128()};
    g[BP_SUCCESS] = F128::one();
    for (int l = L - 1; l >= 0; --l) {
      auto e4 = build_eq({coord(st.z_row, l), coord(point, l)});
      F128 eq4[4] = {e4[0], e4[1], e4[2], e4[3]};
      F128 rc = sigma[2 * l], rd = sigma[2 * l + 1];
      F128 prev[4] = {F128(), F128(), F128(), F128()};
      for (int cd = 0; cd < 4; ++cd) {
        int c = cd & 1, d = cd >> 1;
        F128 ecd = (c ? rc : F128::one() + rc) * (d ? rd : F128::one() + rd);
        F128 M[4][4];
        bp_layer_matrix(eq4, c, d, M);
        for (int s = 0; s < 4; ++s) {
          F128 acc;
          for (int o = 0; o < 4; ++o) acc += M[s][o] * g[o];
          prev[s] += ecd * acc;
        }
      }
      for (int s = 0; s < 4; ++s) g[s] = prev[s];
    }
    expect += w * g[BP_INITIAL];
  }
  require(claim == expect, "anchor: endpoint check");
  return pf.v;
}

// Multipoint twisted evaluation of the ring-switched claims at rho (jagged.rs:4418-4590):
// returns V = sum_{i,j} c_ij A_ij^(2^j) once the dual values A are proven.
// make_stmt(z_row, z_col, coeff) builds a claim's anchor statement over the statement's
// jagged layout (aligned or general).
template <class MakeStmt>
inline F128 verify_multipoint(Transcript& T, uint32_t m, const MakeStmt& make_stmt,
                              const std::vector<RsClaimPoint>& claims, const std::vector<F128>& rho,
                              const MultipointTwistedProof& pf, uint32_t round_bits, uint32_t anchor_bits) {
  const size_t R = claims.size();
  require(pf.values.size() == R && pf.group_values.empty() && pf.rounds.size() == m, "multipoint: shape");
  for (auto& vs : pf.values) require(vs.size() == 128, "multipoint: dual value count");
  require(pf.round_grinding_nonces.size() == (round_bits ? m : 0), "multipoint: nonce count");
  T.observe_label("flock-multipoint-twisted-v1");
  for (auto& vs : pf.values) for (auto& v : vs) T.observe_f128(v);
  uint32_t gamma_bits = std::max<uint32_t>(1, grinding_bits_for_degree(128 * R - 1));
  require(T.verify_pow(pf.gamma_grinding_nonce, gamma_bits), "multipoint: gamma grinding");
  F128 gamma = T.sample_f128();
  std::vector<F128> gpow(128 * R);
  F128 p = F128::one();
  for (auto& g : gpow) { g = p; p = p * gamma; }
  F128 running;
  for (size_t i = 0; i < R; ++i)
    for (int j = 0; j < 128; ++j) running += gpow[128 * i + j] * pf.values[i][j];
  std::vector<F128> point;
  for (uint32_t t = 0; t < m; ++t) {
    T.observe_f128(pf.rounds[t].first);
    T.observe_f128(pf.rounds[t].second);
    if (round_bits) require(T.verify_pow(pf.round_grinding_nonces[t], round_bits), "multipoint: round grinding");
    F128 r = T.sample_f128();
    running = fold_round_claim(running, pf.rounds[t].first, pf.rounds[t].second, r);
    point.push_back(r);
  }
  // twisted eq at the endpoint: sum_j gamma^j eq(rho^(2^-j), point)
  auto rp = rho_inverse_powers(rho);
  F128 g_at;
  for (int j = 0; j < 128; ++j) {
    F128 prod = gpow[j];
    for (uint32_t t = 0; t < m; ++t)
      prod = prod * (point[t] * rp[j][t] + (F128::one() + point[t]) * (F128::one() + rp[j][t]));
    g_at += prod;
  }
  std::vector<AssistStatement> sts;
  for (size_t i = 0; i < R; ++i) sts.push_back(make_stmt(claims[i].z_row, claims[i].z_col, gpow[128 * i] * g_at));
  F128 s_at = verify_anchor(T, sts, point, m, pf.anchor, anchor_bits);
  require(running == s_at, "multipoint: sumcheck endpoint");
  F128 total;
  for (size_t i = 0; i < R; ++i)
    for (int j = 0; j < 128; ++j)
      if (!claims[i].coeffs[j].is_zero()) total += claims[i].coeffs[j] * pow_2j(pf.values[i][j], j);
  return total;
}

// ---------------------------------------------------------------- Ligerito ladder
inline std::vector<uint64_t> sample_level_queries(Transcript& T, uint64_t nonce, uint32_t bits, uint32_t count,
                                                  const LevelSchedule& sc) {
  require(T.verify_pow(nonce, bits), "ligerito: query grinding");
  auto words = T.sample_f128_vec(count);
  std::vector<uint64_t> q;
  size_t w = 0;
  for (uint32_t c : sc.depths)
    for (uint64_t stratum = 0; stratum < (uint64_t(1) << c); ++stratum) {
      uint32_t lo_bits = sc.log_block_len - c;
      uint64_t mask = lo_bits >= 64 ? ~0ull : ((uint64_t(1) << lo_bits) - 1);
      q.push_back((stratum << lo_bits) | (words[w++].lo & mask));
    }
  return q;
}
inline bool verify_capped_path(const std::vector<Hash>& cap, uint64_t n_leaves, const Hash& leaf, uint64_t idx,
                               const Hash* path, size_t path_len) {
  Hash acc = leaf;
  for (size_t i = 0; i < path_len; ++i) {
    Sha256 h;
    if ((idx & 1) == 0) { h.update(acc.data(), 32); h.update(path[i].data(), 32); }
    else { h.update(path[i].data(), 32); h.update(acc.data(), 32); }
    acc = h.digest();
    idx >>= 1;
  }
  (void)n_leaves;
  return idx < cap.size() && acc == cap[idx];
}
inline void verify_level_opens(const std::vector<Hash>& cap, uint64_t block_len, const std::vector<uint64_t>& q,
                               const std::vector<std::vector<F128>>& rows, size_t lanes,
                               const std::vector<Hash>& paths, const LevelSchedule& sc) {
  require(rows.size() == q.size(), "ligerito: opened row count");
  uint32_t d = 0;
  while ((uint64_t(1) << d) < block_len) ++d;
  require((uint64_t(1) << d) == block_len && sc.log_block_len == d && sc.queries() == q.size(),
          "ligerito: opening schedule");
  const uint32_t c1 = sc.cap_depth();
  require(cap.size() == (size_t(1) << c1), "ligerito: cap size");
  const size_t path_len = d - c1;
  require(paths.size() == q.size() * path_len, "ligerito: path sibling count");
  for (size_t i = 0; i < q.size(); ++i) {
    require(rows[i].size() == lanes, "ligerito: opened row width");
    Hash leaf = Sha256::hash(rows[i].data(), rows[i].size() * sizeof(F128));
    require(q[i] < block_len && verify_capped_path(cap, block_len, leaf, q[i], paths.data() + i * path_len, path_len),
            "ligerito: Merkle path");
  }
}
inline F256 induce_enforced_sum(const std::vector<std::vector<F128>>& rows, const std::vector<F256>& lane_ch,
                                const std::vector<F128>& alpha) {
  auto lw = build_eq256(lane_ch);
  auto rw = build_eq(alpha);
  F256 acc;
  for (size_t i = 0; i < rows.size(); ++i) {
    require(rows[i].size() <= lw.size(), "ligerito: row wider than the lane weights");
    F256 s;
    for (size_t l = 0; l < rows[i].size(); ++l) s += lw[l] * rows[i][l];
    acc += s * rw[i];
  }
  return acc;
}
inline F256 coordinate_factor_product(const std::vector<std::vector<F256>>& levels, size_t start) {
  F256 acc = F256::one();
  for (size_t i = start; i < levels.size(); ++i) acc = acc * (F256::one() + levels[i][0] * (F256::one() + F256::u()));
  return acc;
}
inline std::vector<F256> residual_original_challenges(const std::vector<F256>& initial,
                                                      const std::vector<std::vector<F256>>& levels, size_t start) {
  std::vector<F256> out;
  if (start == 0) out = initial;
  for (size_t i = start; i < levels.size(); ++i) out.insert(out.end(), levels[i].begin() + 1, levels[i].end());
  return out;
}
inline std::vector<F256> eq_residual(const std::vector<F128>& point, const std::vector<F256>& fixed, uint32_t res_log,
                                     F256 scale) {
  require(fixed.size() + res_log == point.size(), "ligerito: residual point length");
  F256 prefix = scale;
  for (size_t i = 0; i < fixed.size(); ++i) prefix = prefix * (F256::one() + F256(point[i]) + fixed[i]);
  std::vector<F256> out(size_t(1) << res_log);
  for (size_t y = 0; y < out.size(); ++y) {
    F256 acc = prefix;
    for (uint32_t j = 0; j < res_log; ++j) {
      F128 z = point[fixed.size() + j];
      acc = acc * (((y >> j) & 1) ? z : F128::one() + z);
    }
    out[y] = acc;
  }
  return out;
}
inline std::vector<F256> induced_basis_at_residual(uint32_t log_cols, const std::vector<uint64_t>& q,
                                                   const std::vector<F128>& alpha, const std::vector<F256>& fixed,
                                                   uint32_t res_log) {
  require(fixed.size() + res_log == log_cols, "ligerito: induced basis split");
  LchSks sk = lch_sks(log_cols);
  auto wts = build_eq(alpha);
  std::vector<F256> out(size_t(1) << res_log);
  for (size_t i = 0; i < q.size(); ++i) {
    auto w = lch_basis_factors(q[i], log_cols, sk);
    F256 prefix = F256::one();
    for (size_t k = 0; k < fixed.size(); ++k) prefix = prefix * (F256::one() + fixed[k] * (F128::one() + w[k]));
    for (size_t y = 0; y < out.size(); ++y) {
      F256 t = prefix * wts[i];
      for (uint32_t j = 0; j < res_log; ++j)
        if ((y >> j) & 1) t = t * w[fixed.size() + j];
      out[y] += t;
    }
  }
  return out;
}

// The F256 ladder over the lane-major L0 commitment with one packed-direct claim
// (point `rho`, batching coefficient `g`) of value target / g (extension.rs:2409-2796).
inline void verify_ligerito(Transcript& T, const LigeritoParams& P, const LigeritoProof& pf, uint32_t log_n, F128 target,
                            const std::vector<Hash>& commit_cap, uint32_t l0_lanes, const std::vector<F128>& rho,
                            F128 g) {
  const uint32_t initial_k = P.initial_k, rounds = P.r;
  require(rounds >= 1 && pf.initial_cap == commit_cap && pf.sumcheck_transcript.empty() &&
              !pf.sumcheck_transcript_f256.empty() && pf.fold_grinding_nonces.empty(),
          "ligerito: proof shape");
  for (uint32_t k : P.recursive_ks) require(k >= 2, "ligerito: recursive k");
  const bool lane_major = l0_lanes < (1u << initial_k);
  T.observe_label("flock-ligerito-basis-f256-split-v0");
  T.observe_f128(target);
  {
    std::vector<uint8_t> capb;
    for (auto& h : pf.initial_cap) capb.insert(capb.end(), h.begin(), h.end());
    T.observe_bytes(capb);
  }
  const uint32_t log_cols_0 = log_n - initial_k;
  const uint64_t block_len_0 = uint64_t(1) << (log_cols_0 + P.log_inv_rates[0]);
  size_t tx = 0, ood_index = 0, claim_nonce = 0, consistency_nonce = 0, query_nonce = 0;
  F256 claim(target);
  struct Ood { std::vector<F128> point; F128 beta; int split_level; };
  struct Cons { uint32_t log_cols; std::vector<uint64_t> q; std::vector<F128> alpha; F128 beta; size_t start; };
  std::vector<Ood> oods;
  std::vector<Cons> cons;
  auto next_msg = [&]() -> const Msg256& {
    require(tx < pf.sumcheck_transcript_f256.size(), "ligerito: missing sumcheck message");
    const Msg256& m = pf.sumcheck_transcript_f256[tx++];
    T.observe_f256(m.u0);
    T.observe_f256(m.u2);
    return m;
  };
  auto next_ood = [&]() {
    require(ood_index < pf.ood_values.size(), "ligerito: missing OOD value");
    return pf.ood_values[ood_index++];
  };
  auto claim_beta = [&](uint32_t bits) {
    require(claim_nonce < pf.claim_batch_grinding_nonces.size(), "ligerito: missing claim nonce");
    require(T.verify_pow(pf.claim_batch_grinding_nonces[claim_nonce++], bits), "ligerito: claim grinding");
    return T.sample_f128();
  };
  auto consistency_alpha = [&](uint32_t bits, uint32_t n) {
    require(consistency_nonce < pf.consistency_batch_grinding_nonces.size(), "ligerito: missing consistency nonce");
    require(T.verify_pow(pf.consistency_batch_grinding_nonces[consistency_nonce++], bits),
            "ligerito: consistency grinding");
    return T.sample_f128_vec(n);
  };
  auto queries = [&](uint32_t level, uint64_t block_len) {
    require(query_nonce < pf.grinding_nonces.size(), "ligerito: missing query nonce");
    require(P.sched[level].log_block_len < 64 && (uint64_t(1) << P.sched[level].log_block_len) == block_len,
            "ligerito: query block");
    return sample_level_queries(T, pf.grinding_nonces[query_nonce++], P.grinding_bits[level], P.queries[level],
                                P.sched[level]);
  };
  for (uint32_t o = 0; o < P.ood_samples[0]; ++o) {
    auto point = T.sample_f128_vec(log_n);
    if (lane_major) std::rotate(point.begin(), point.begin() + (log_n - initial_k), point.end());
    F128 y = next_ood();
    T.observe_f128(y);
    F128 beta = claim_beta(P.claim_bits[0]);
    claim += F256(beta * y);
    oods.push_back({point, beta, -1});
  }
  Quad256 quad = Quad256::from(next_msg(), claim);
  std::vector<F256> initial_ch;
  for (uint32_t j = 0; j < initial_k; ++j) {
    F256 ch = T.sample_f256();
    claim = quad.eval(ch);
    initial_ch.push_back(ch);
    quad = Quad256::from(next_msg(), claim);
  }
  uint32_t split_dim = log_n - initial_k + 1;
  require(!pf.recursive_caps.empty(), "ligerito: missing level-1 cap");
  auto observe_cap = [&](const std::vector<Hash>& c) {
    std::vector<uint8_t> capb;
    for (auto& h : c) capb.insert(capb.end(), h.begin(), h.end());
    T.observe_bytes(capb);
  };
  observe_cap(pf.recursive_caps[0]);
  for (uint32_t o = 0; o < P.ood_samples[1]; ++o) {
    auto point = T.sample_f128_vec(split_dim);
    F128 y = next_ood();
    T.observe_f128(y);
    Quad256 intro = Quad256::from(next_msg(), F256(y));
    F128 beta = claim_beta(P.claim_bits[1]);
    quad = quad.fold(intro, beta);
    claim += F256(beta * y);
    oods.push_back({point, beta, 0});
  }
  {
    auto q0 = queries(0, block_len_0);
    auto a0 = consistency_alpha(P.consistency_bits[0], ceil_log2(P.queries[0]));
    verify_level_opens(pf.initial_cap, block_len_0, q0, pf.initial_proof.opened_rows, l0_lanes,
                       pf.initial_proof.merkle_proof, P.sched[0]);
    F256 enforced = induce_enforced_sum(pf.initial_proof.opened_rows, initial_ch, a0);
    Quad256 intro = Quad256::from(next_msg(), enforced);
    F128 beta = claim_beta(P.claim_bits[1]);
    quad = quad.fold(intro, beta);
    claim += enforced * beta;
    cons.push_back({log_cols_0, q0, a0, beta, 0});
  }
  std::vector<std::vector<F256>> level_ch;
  const std::vector<Hash>* prev_cap = &pf.recursive_caps[0];
  uint32_t prev_log_lanes = P.recursive_ks[0];
  require(split_dim >= prev_log_lanes, "ligerito: level width");
  uint32_t prev_log_cols = split_dim - prev_log_lanes, prev_rate = P.log_inv_rates[1];
  size_t cap_index = 1, proof_index = 0;
  for (uint32_t i = 0; i < rounds; ++i) {
    const uint32_t k = P.recursive_ks[i];
    require(split_dim >= k, "ligerito: fold depth");
    std::vector<F256> chs;
    for (uint32_t j = 0; j < k; ++j) {
      F256 ch = T.sample_f256();
      claim = quad.eval(ch);
      chs.push_back(ch);
      quad = Quad256::from(next_msg(), claim);
    }
    level_ch.push_back(chs);
    const uint32_t ext_dim = split_dim - k, level = i + 1;
    const uint64_t block_len = uint64_t(1) << (prev_log_cols + prev_rate);
    if (i + 1 == rounds) {
      require(tx == pf.sumcheck_transcript_f256.size() && pf.final_proof.yr.size() == (size_t(2) << ext_dim),
              "ligerito: final shape");
      for (auto& v : pf.final_proof.yr) T.observe_f128(v);
      auto q = queries(level, block_len);
      auto al = consistency_alpha(P.consistency_bits[level], ceil_log2(P.queries[level]));
      verify_level_opens(*prev_cap, block_len, q, pf.final_proof.opened_rows, size_t(1) << prev_log_lanes,
                         pf.final_proof.merkle_proof, P.sched[level]);
      F256 enforced = induce_enforced_sum(pf.final_proof.opened_rows, level_ch[i], al);
      F128 beta = claim_beta(P.claim_bits[level]);
      claim += enforced * beta;
      cons.push_back({ext_dim, q, al, beta, rounds});

      // residual basis at the bound challenges
      auto orig = residual_original_challenges(initial_ch, level_ch, 0);
      require(orig.size() + ext_dim == log_n, "ligerito: residual split");
      std::vector<F128> pt(rho.begin(), rho.end());
      if (lane_major) std::rotate(pt.begin(), pt.begin() + (pt.size() - initial_k), pt.end());
      F256 pre = F256::one();
      for (size_t t = 0; t < orig.size(); ++t) pre = pre * (F256::one() + F256(pt[t]) + orig[t]);
      std::vector<F256> residual(size_t(1) << ext_dim);
      F256 s0 = coordinate_factor_product(level_ch, 0);
      for (size_t y = 0; y < residual.size(); ++y) {
        F128 suffix = F128::one();
        for (uint32_t j = 0; j < ext_dim; ++j) {
          F128 p = pt[orig.size() + j];
          suffix = suffix * (((y >> j) & 1) ? p : F128::one() + p);
        }
        residual[y] = pre * (g * suffix) * s0;
      }
      for (const Ood& o : oods) {
        std::vector<F256> fixed;
        F256 scale;
        if (o.split_level < 0) {
          fixed = orig;
          scale = coordinate_factor_product(level_ch, 0);
        } else {
          size_t s = (size_t)o.split_level;
          fixed = level_ch[s];
          for (size_t l = s + 1; l < level_ch.size(); ++l) fixed.insert(fixed.end(), level_ch[l].begin() + 1, level_ch[l].end());
          scale = coordinate_factor_product(level_ch, s + 1);
        }
        auto vals = eq_residual(o.point, fixed, ext_dim, scale * o.beta);
        for (size_t y = 0; y < residual.size(); ++y) residual[y] += vals[y];
      }
      for (const Cons& c : cons) {
        auto fixed = residual_original_challenges({}, level_ch, c.start);
        auto vals = induced_basis_at_residual(c.log_cols, c.q, c.alpha, fixed, ext_dim);
        F256 scale = coordinate_factor_product(level_ch, c.start) * c.beta;
        for (size_t y = 0; y < residual.size(); ++y) residual[y] += vals[y] * scale;
      }
      F256 rc;
      for (size_t y = 0; y < residual.size(); ++y) {
        rc += residual[y] * pf.final_proof.yr[2 * y];
        rc += (F256::u() * residual[y]) * pf.final_proof.yr[2 * y + 1];
      }
      require(rc == claim, "ligerito: residual check");
      require(ood_index == pf.ood_values.size() && query_nonce == pf.grinding_nonces.size() &&
                  claim_nonce == pf.claim_batch_grinding_nonces.size() &&
                  consistency_nonce == pf.consistency_batch_grinding_nonces.size() &&
                  cap_index == pf.recursive_caps.size() && proof_index == pf.recursive_proofs.size(),
              "ligerito: unconsumed proof items");
      return;
    }
    split_dim = ext_dim + 1;
    require(cap_index < pf.recursive_caps.size(), "ligerito: missing cap");
    const std::vector<Hash>& cap = pf.recursive_caps[cap_index++];
    observe_cap(cap);
    for (uint32_t o = 0; o < P.ood_samples[level + 1]; ++o) {
      auto point = T.sample_f128_vec(split_dim);
      F128 y = next_ood();
      T.observe_f128(y);
      Quad256 intro = Quad256::from(next_msg(), F256(y));
      F128 beta = claim_beta(P.claim_bits[level + 1]);
      quad = quad.fold(intro, beta);
      claim += F256(beta * y);
      oods.push_back({point, beta, (int)(i + 1)});
    }
    auto q = queries(level, block_len);
    auto al = consistency_alpha(P.consistency_bits[level], ceil_log2(P.queries[level]));
    require(proof_index < pf.recursive_proofs.size(), "ligerito: missing level opening");
    const RecursiveProof& op = pf.recursive_proofs[proof_index++];
    verify_level_opens(*prev_cap, block_len, q, op.opened_rows, size_t(1) << prev_log_lanes, op.merkle_proof,
                       P.sched[level]);
    F256 enforced = induce_enforced_sum(op.opened_rows, level_ch[i], al);
    Quad256 intro = Quad256::from(next_msg(), enforced);
    F128 beta = claim_beta(P.claim_bits[level + 1]);
    quad = quad.fold(intro, beta);
    claim += enforced * beta;
    cons.push_back({ext_dim, q, al, beta, (size_t)(i + 1)});
    prev_cap = &cap;
    prev_log_lanes = P.recursive_ks[i + 1];
    require(split_dim >= prev_log_lanes, "ligerito: level width");
    prev_log_cols = split_dim - prev_log_lanes;
    prev_rate = P.log_inv_rates[i + 2];
  }
  throw Reject("ligerito: no final level");
}

// ---------------------------------------------------------------- the whole proof
// Throws Reject with the first failed check.
inline void verify_bundle(const Statement& S, const Bundle& B, const uint8_t* domain, size_t domain_len) {
  const MergedProof& P = B.proof;
  const uint32_t m = S.m, nu = S.nu, k_log = S.k_log, n_mlv = m - 6;
  require(B.cap.size() == (size_t(1) << S.lig.sched[0].cap_depth()), "statement: cap size");
  Transcript T(domain, domain_len);
  T.observe_label("flock-mixed-v1");
  T.observe_bytes(S.registry_digest.data(), 32);
  {
    // the counts vector, one u64 LE per slot (union.rs:619-628)
    std::vector<uint8_t> counts;
    for (const SlotInfo& t : S.slots)
      for (int i = 0; i < 8; ++i) counts.push_back((uint8_t)(t.count >> (8 * i)));
    T.observe_bytes(counts);
    std::vector<uint8_t> capb;
    for (auto& h : B.cap) capb.insert(capb.end(), h.begin(), h.end());
    T.observe_bytes(capb);
  }

  // ---- zerocheck
  const ZerocheckProof& zc = P.zerocheck;
  require(zc.round1_ab.size() == 64 && zc.round1_c.size() == 64 && zc.multilinear_rounds.size() == n_mlv &&
              zc.grinding_nonces.size() == 2 + n_mlv,
          "zerocheck: shape");
  T.observe_label("flock-zerocheck-v0");
  std::vector<F128> r(m);
  {
    require(T.verify_pow(zc.grinding_nonces[0], bits_for(m)), "zerocheck: initial grinding");
    auto rs = T.sample_f128_vec(6);
    for (int i = 0; i < 6; ++i) r[i] = rs[i];
    const auto& fixed = zc_fixed_challenges();
    for (int i = 0; i < 7; ++i) r[6 + i] = fixed[i];
    auto ro = T.sample_f128_vec(m - 13);
    for (uint32_t i = 0; i < m - 13; ++i) r[13 + i] = ro[i];
  }
  T.observe_f128_slice(zc.round1_ab);
  T.observe_f128_slice(zc.round1_c);
  require(T.verify_pow(zc.grinding_nonces[1], bits_for(127)), "zerocheck: skip grinding");
  const F128 zskip = T.sample_f128();
  const F128 c_eval = interpolate_on_lambda(zc.round1_c, zskip);
  require(c_eval == zc.final_c_eval, "zerocheck: c evaluation");
  std::vector<F128> combined(64);
  for (int i = 0; i < 64; ++i) combined[i] = zc.round1_ab[i] + zc.round1_c[i];
  F128 running = interpolate_combined(combined, zskip) + c_eval;
  std::vector<F128> mlv;
  for (uint32_t i = 0; i < n_mlv; ++i) {
    const F128 r_eq = r[6 + i], g1 = zc.multilinear_rounds[i].first, gi = zc.multilinear_rounds[i].second;
    const F128 g0 = (running + r_eq * g1) * inv(F128::one() + r_eq);
    T.observe_f128(g1);
    T.observe_f128(gi);
    require(T.verify_pow(zc.grinding_nonces[2 + i], 2), "zerocheck: round grinding");
    const F128 rho = T.sample_f128();
    mlv.push_back(rho);
    const F128 rho1 = F128::one() + rho;
    running = g0 * rho1 + g1 * rho + gi * rho * rho1;
  }
  require(running == zc.final_a_eval * zc.final_b_eval, "zerocheck: final product");
  T.observe_f128(zc.final_a_eval);
  T.observe_f128(zc.final_b_eval);

  // ---- lincheck
  std::vector<F128> x_inner_rest, x_outer(mlv.begin() + 1, mlv.begin() + 1 + nu);
  x_inner_rest.push_back(mlv[0]);
  x_inner_rest.insert(x_inner_rest.end(), mlv.begin() + 1 + nu, mlv.end());
  const LincheckProof& lc = P.lincheck;
  const uint32_t inner_rest_len = k_log - 6;
  const size_t n_slots = S.slots.size();
  require(lc.rounds.size() == inner_rest_len && lc.z_partial.size() == 64 && lc.matrix_evals.size() == n_slots &&
              lc.grinding_nonces.size() == inner_rest_len + 2 + n_slots,
          "lincheck: shape");
  T.observe_label("flock-lincheck-v0");
  require(T.verify_pow(lc.grinding_nonces[0], 1), "lincheck: alpha grinding");
  const F128 alpha = T.sample_f128();
  // one const-pin challenge per slot; the target gains beta_t * sum_{row < n_t}
  // eq(x_outer, row), exactly beta_t at full utilisation (lincheck/union.rs:800-830)
  F128 lrun = alpha * zc.final_a_eval + zc.final_b_eval;
  std::vector<F128> betas;
  for (size_t t = 0; t < n_slots; ++t) {
    require(T.verify_pow(lc.grinding_nonces[1 + t], 1), "lincheck: beta grinding");
    betas.push_back(T.sample_f128());
    lrun += betas[t] * eq_prefix_sum(x_outer, S.slots[t].count);
  }
  std::vector<F128> r_rounds;
  for (uint32_t t = 0; t < inner_rest_len; ++t) {
    const F128 e1 = lc.rounds[t].first, ei = lc.rounds[t].second;
    T.observe_f128(e1);
    T.observe_f128(ei);
    require(T.verify_pow(lc.grinding_nonces[1 + n_slots + t], 2), "lincheck: round grinding");
    const F128 rt = T.sample_f128();
    const F128 e0 = lrun + e1, c1 = e0 + e1 + ei;
    lrun = ei * rt * rt + c1 * rt + e0;
    r_rounds.push_back(rt);
  }
  T.observe_f128_slice(lc.z_partial);
  require(T.verify_pow(lc.grinding_nonces[1 + n_slots + inner_rest_len], 6), "lincheck: skip grinding");
  const F128 r_inner_skip = T.sample_f128();
  const std::vector<F128> rr(r_rounds.rbegin(), r_rounds.rend());
  {
    // matrix discharge: the union comb collapse at the bound column point
    // (lincheck/union.rs:540-625): per slot t with inner_t = k_log_t - 6 own column
    // coordinates, w_t = eq weight of its prefix at the row point, P_t at the bound point
    F128 acc, reported;
    for (size_t t = 0; t < n_slots; ++t) {
      const SlotInfo& T_ = S.slots[t];
      const size_t inner = T_.k_log - 6;
      std::vector<F128> ca, cb;
      lincheck_combs(T_, lagrange_weights64(zskip, 0), slot_inner(T_, x_inner_rest), ca, cb);
      const F128 w_t = eq_prefix_weight(std::vector<F128>(x_inner_rest.begin() + inner, x_inner_rest.end()), T_.prefix);
      const F128 p_t = eq_prefix_weight(std::vector<F128>(rr.begin() + inner, rr.end()), T_.prefix);
      auto er = build_eq(std::vector<F128>(rr.begin(), rr.begin() + inner));
      F128 slot_acc;
      for (size_t c = 0; c < ca.size(); ++c) {
        F128 comb = w_t * (alpha * ca[c] + cb[c]);
        if (c == T_.const_pin) comb += betas[t];
        slot_acc += er[c >> 6] * comb * lc.z_partial[c & 63];
      }
      acc += p_t * slot_acc;
      const F128 w_pin = er[T_.const_pin >> 6] * lc.z_partial[T_.const_pin & 63];
      reported += p_t * (w_t * (alpha * lc.matrix_evals[t].first + lc.matrix_evals[t].second) + betas[t] * w_pin);
    }
    require(acc == lrun, "lincheck: matrix consistency");
    require(reported == lrun, "lincheck: reported matrix evaluations");
  }
  F128 w_ab;
  {
    auto lw = lagrange_weights64(r_inner_skip, 0);
    for (int i = 0; i < 64; ++i) w_ab += lw[i] * lc.z_partial[i];
  }
  require(w_ab == B.claims.ab_value && zc.final_c_eval == B.claims.c_value, "claims: bundle values");

  // ---- merged opening
  std::vector<F128> x_ab;  // [dim6 | rows | columns]
  x_ab.push_back(rr[0]);
  x_ab.insert(x_ab.end(), x_outer.begin(), x_outer.end());
  x_ab.insert(x_ab.end(), rr.begin() + 1, rr.end());
  std::vector<F128> x_c(r.begin() + 6, r.end());
  const MergedOpenProof& mo = P.pcs_open;
  require(mo.ring_switches.size() == 2 && mo.batching_nonces.size() == 1, "merged open: shape");
  T.observe_label("flock-merged-open-v1");
  const F128 claim_vals[2] = {w_ab, zc.final_c_eval};
  const F128 skips[2] = {r_inner_skip, zskip};
  const std::vector<F128>* xs[2] = {&x_ab, &x_c};
  F128 rs_claim[2];
  std::vector<F128> eq_rdp[2];
  for (int i = 0; i < 2; ++i) {
    const RingSwitchProof& rp = mo.ring_switches[i];
    require(rp.s_hat_v.size() == 128, "ring switch: s_hat_v length");
    T.observe_label("flock-ring-switch-v0");
    T.observe_f128_slice(rp.s_hat_v);
    auto sw = lagrange_weights64(skips[i], 0);
    const F128 x0 = (*xs[i])[0];
    F128 chk;
    for (int t = 0; t < 128; ++t) chk += sw[t & 63] * (t < 64 ? F128::one() + x0 : x0) * rp.s_hat_v[t];
    require(chk == claim_vals[i], "ring switch: claim");
    require(T.verify_pow(rp.grinding_nonce, 3), "ring switch: grinding");
    eq_rdp[i] = build_eq(T.sample_f128_vec(7));
    auto u = tensor_transpose128(rp.s_hat_v);
    F128 acc;
    for (int t = 0; t < 128; ++t) acc += u[t] * eq_rdp[i][t];
    rs_claim[i] = acc;
  }
  require(T.verify_pow(mo.batching_nonces[0], 6), "merged open: batching grinding");
  auto gam = T.sample_f128_vec(2);
  F128 mrun = gam[0] * rs_claim[0] + gam[1] * rs_claim[1];
  const uint32_t dense_log = S.geo.dense_m - 7;
  require(mo.merged_rounds.size() == dense_log && mo.merged_round_nonces.size() == dense_log, "merged open: rounds");
  std::vector<F128> rho;
  for (uint32_t rd = 0; rd < dense_log; ++rd) {
    T.observe_f128(mo.merged_rounds[rd].first);
    T.observe_f128(mo.merged_rounds[rd].second);
    require(T.verify_pow(mo.merged_round_nonces[rd], 2), "merged open: round grinding");
    const F128 rt = T.sample_f128();
    mrun = fold_round_claim(mrun, mo.merged_rounds[rd].first, mo.merged_rounds[rd].second, rt);
    rho.push_back(rt);
  }
  const bool aligned = S.slots.size() == 1 && S.identity;
  AlignedJagged J{nu, S.geo.col_log, dense_log, aligned ? S.slots[0].used_cols : 0};
  JaggedLayout JL{nu, S.geo.col_log, dense_log, S.col_prefix};
  require(aligned ? J.n + J.k == J.m : J.n + J.k >= J.m, "merged open: jagged split");
  std::vector<RsClaimPoint> fcl(2);
  for (int i = 0; i < 2; ++i) {
    const std::vector<F128>& x = *xs[i];
    require(x.size() == 1 + size_t(nu) + J.k, "merged open: claim point length");
    fcl[i].z_row.assign(x.begin() + 1, x.begin() + 1 + nu);
    fcl[i].z_col.assign(x.begin() + 1 + nu, x.end());
    std::vector<F128> scaled(128);
    for (int t = 0; t < 128; ++t) scaled[t] = gam[i] * eq_rdp[i][t];
    fcl[i].coeffs = linearized_coefficients(fold_byte_table(scaled));
  }
  Transcript ch_a = T.fork("flock-par-assist-v1");
  auto stmt = [&](const std::vector<F128>& zr, const std::vector<F128>& zc, F128 coeff) {
    return aligned ? aligned_statement(J, zr, zc, coeff) : jagged_statement(JL, zr, zc, coeff);
  };
  const F128 v = verify_multipoint(ch_a, dense_log, stmt, fcl, rho, mo.frobenius, 2, 2);

  // ---- inner opening of q_hat(rho) = q_eval
  const BatchOpeningProofLigerito& in = mo.inner;
  require(in.ring_switches.empty() && in.batching_nonces.empty(), "inner open: shape");
  T.observe_label("flock-pcs-open-batch-v0");
  T.observe_label("flock-pcs-packed-direct-v0");
  T.observe_f128(mo.q_eval);
  const F128 gamma = T.sample_f128_vec(1)[0];
  verify_ligerito(T, S.lig, in.ligerito, dense_log, gamma * mo.q_eval, B.cap, S.lanes, rho, gamma);
  T.merge_child(ch_a);
  require(mrun == mo.q_eval * v, "merged open: final check");
}

}  // namespace oracle
}  // namespace flock
