// prove_fast: the transcript-ordered protocol of
//   Blake3Setup / Sha256HybridSetup / KeccakSetup ::prove_fast
//   -> prover::prove_fast_ligerito_union -> prove_union_with_binding_zc
// (crates/flock-prover/src/prover.rs:587-620, 831-1468) for a single-slot,
// full-utilisation union, written against an abstract backend that owns the
// committed data and runs every operation whose cost grows with the witness.
//
// Section references:
//   commit + statement binding     prover.rs:975-1003, union.rs:619-628, pcs/commit.rs:474-530
//   zerocheck                      zerocheck.rs:618-1019
//   union lincheck                 lincheck/union.rs:203-430, lincheck.rs:1907-2031
//   s_hat_v of the AB claim        prover.rs:1190-1210, pcs/ring_switch.rs:1278-1320
//   merged open                    pcs.rs:1433-1850
//   inner eq-basis open            pcs.rs:214-560
//   Ligerito F256 ladder           pcs/ligerito/extension.rs:1636-2290
#pragma once
#include <future>
#include "pcs_host.h"
#include <chrono>
#include <cstdio>

namespace flock {

// The backend owns z/a/b/stripe, the L0 codeword and tree, the zerocheck and
// lincheck tables, the merged-open weight and every Ligerito level. All vectors
// passed here are O(128) or O(m) long.
class ProverBackend {
 public:
  virtual ~ProverBackend() = default;
  // Witness of every slot: slot_inputs[t] holds slots[t].count records of
  // input_record_bytes(slots[t].hash); rows [count, 2^nu) of a slot are zero.
  virtual void witness(const std::vector<const uint8_t*>& slot_inputs) = 0;
  // L0 commit of the committed stack q (the height-n_t compaction of z; z itself under
  // identity compaction): lane-major fill, NTT from layer 1, Merkle.
  virtual void commit_l0(uint32_t cap_depth, std::vector<Hash>& cap) = 0;

  // ---- zerocheck (r has m coordinates; all values in wire convention)
  virtual void zc_round1(const std::vector<F128>& r, std::vector<F128>& ab, std::vector<F128>& c,
                         std::vector<F128>& s_hat_v_c) = 0;
  // Fold a, b at the skip point z (Lagrange weights `w` on S), then the first
  // multilinear message with eq over `eq_point` (= r[7..m]).
  virtual void zc_fold_skip(const std::vector<F128>& w, const std::vector<F128>& eq_point, F128& g1, F128& ginf) = 0;
  // Fold the low variable at rho, then the next message with eq over eq_point.
  virtual void zc_fold(F128 rho, const std::vector<F128>& eq_point, F128& g1, F128& ginf) = 0;
  virtual void zc_final(F128 rho, F128& a_eval, F128& b_eval) = 0;

  // ---- lincheck
  // Per slot t: eq_inner_t = skip_w (64) tensor eq(x_inner_rest[.. k_log_t - 6]);
  // comb_a_t, comb_b_t = eq_inner_t^T (A_0, B_0) of the slot's type.
  virtual void lc_comb(const std::vector<F128>& skip_w, const std::vector<F128>& x_inner_rest) = 0;
  // z_vec[c] = sum_row eq(x_outer, row) * z(row, c) over the union columns, also kept as
  // the captured copy.
  virtual void lc_zvec(const std::vector<F128>& x_outer) = 0;
  // The union comb: per slot t, comb[off_t + c] = w_t (alpha comb_a_t[c] + comb_b_t[c]),
  // then comb[off_t + pin_t] += beta_t; first product-sumcheck message.
  struct SlotComb {
    F128 weight, beta;
    uint64_t offset = 0;  // off_t = prefix_t << k_log_t
    uint32_t pin = 0;
  };
  virtual void lc_start(F128 alpha, const std::vector<SlotComb>& slots, F128& e1, F128& einf) = 0;
  // Bind the top variable of comb and z_vec at r; next message unless `last`.
  virtual void lc_round(F128 r, bool last, F128& e1, F128& einf) = 0;
  virtual void lc_partial(std::vector<F128>& z_partial64) = 0;
  // Per slot t: (<w_col_t, comb_a_t>, <w_col_t, comb_b_t>) with
  // w_col_t = eq(rest_point[.. k_log_t - 6]) tensor z_partial.
  virtual void lc_matrix_evals(const std::vector<F128>& rest_point, const std::vector<F128>& z_partial64,
                               std::vector<Pair128>& evals) = 0;
  // s_hat_v[b] = sum_k eq(tail, k) * z_vec_captured[b + 128 k].
  virtual void lc_s_hat_v(const std::vector<F128>& tail, std::vector<F128>& out128) = 0;

  // ---- merged open
  struct WeightClaim {
    std::vector<F128> z_row, z_col;
    std::vector<F128> table;  // 16 x 256, gamma baked
  };
  // W[d] = sum_i fold_one_slot(eq(z_row_i)[row(d)] * eq(z_col_i)[col(d)], table_i) for
  // d < area, 0 beyond, with (row, col) the jagged unrank of d (the statement's column
  // prefix sums; col = d >> nu, row = d mod 2^nu under identity compaction); returns the
  // round-0 prime (u0, u2) of sum_d q[d] W[d].
  virtual void mo_build_w(const std::vector<WeightClaim>& claims, uint32_t nu, uint64_t area, F128& u0, F128& u2) = 0;
  // Fold q and W at r (low bit); next (g1, ginf) unless `last`.
  virtual void mo_round(F128 r, bool last, F128& g1, F128& ginf) = 0;
  virtual F128 mo_q_eval() = 0;

  // ---- Ligerito (f starts as the committed stack q, length 2^log_n)
  virtual void lg_basis_eq(F128 gamma, const std::vector<F128>& rho) = 0;   // b = gamma * eq(rho)
  virtual F128 lg_eval_eq(const std::vector<F128>& z) = 0;                  // sum f * eq(z) (f base)
  virtual void lg_add_eq(F128 beta, const std::vector<F128>& z) = 0;        // b += beta * eq(z)
  virtual Msg256 lg_message(size_t d) = 0;                                  // (u0, u2) with block pairing d
  virtual void lg_fold(F256 r, size_t d) = 0;                               // fold f and b at r, block d
  virtual void lg_code_switch() = 0;                                        // split f and b
  // Commit the current (base-valued) f: lanes = 2^log_lanes, LSB-lane layout.
  virtual void lg_commit(uint32_t level, uint32_t log_cols, uint32_t log_lanes, uint32_t log_rate,
                         uint32_t cap_depth, std::vector<Hash>& cap) = 0;
  // Introduce a pending basis (eq(z), base values) : returns (message, answer).
  virtual Msg256 lg_introduce_eq(const std::vector<F128>& z, F128& answer) = 0;
  // Introduce the induced basis of the queried positions (weights w_i) split:
  //   basis[i] = sum_q w_q prod_{k in bits(i)} W_k(pos_q),
  // what[q][k] = W_k(pos_q) (normalised LCH basis factors). The codeword of that level is
  // the NTT (from layer log_rate) of the replicated message, so basis = NTT^T(sum_q w_q e_pos_q)
  // folded over the replicas: a backend may use the positions instead of `what`, in which
  // case induced_from_positions() is true and `what` is passed empty.
  virtual Msg256 lg_introduce_induced(uint32_t log_msg_cols, uint32_t log_rate, const std::vector<uint64_t>& positions,
                                      const std::vector<F128>& w, const std::vector<std::vector<F128>>& what) = 0;
  virtual bool induced_from_positions() const { return false; }
  virtual void lg_glue(F128 beta) = 0;
  // Rows of level `level` (0 = the L0 commit) at positions, and capped paths.
  virtual void lg_open(uint32_t level, const std::vector<uint64_t>& positions, uint32_t cap_depth,
                       std::vector<std::vector<F128>>& rows, std::vector<Hash>& paths) = 0;
  virtual std::vector<F256> lg_residual() = 0;

  // Device proof-of-work search (optional): smallest nonce with the PoW property.
  virtual PowSearchFn pow_search() { return {}; }

};

struct ProveTimings {
  double witness = 0, commit = 0, zerocheck = 0, lincheck = 0, open = 0, total = 0;
  double assist = 0, assist_wait = 0;  // multipoint assist thread, and the open phase's wait for it
};

inline double now_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

// Small constants of the zerocheck (univariate_skip_optimized.rs:70-125).
inline const std::vector<F128>& zc_fixed_challenges() {
  static const std::vector<F128> v = [] {
    std::vector<F128> c;
    const uint8_t small[3] = {0xF7, 0x53, 0xB5};
    for (int i = 0; i < 3; ++i) c.push_back(phi8(small[i]));
    for (int e : {1, 2, 4, 8}) {
      F128 g(1ull << e, 0);
      c.push_back(g * inv(F128::one() + g));
    }
    return c;
  }();
  return v;
}

inline uint32_t ceil_log2(uint64_t n) { uint32_t l = 0; while ((uint64_t(1) << l) < n) ++l; return l; }
inline uint32_t bits_for(uint64_t x) { uint32_t b = 0; while (x) { ++b; x >>= 1; } return b; }

// s_k(v_k) for k = 0..ln and their inverses (eval_sk_at_vks, ligerito.rs:2402-2425).
struct LchSks {
  std::vector<F128> sks, inv_sks;
};
inline LchSks lch_sks(uint32_t ln) {
  LchSks r;
  r.sks.assign(ln + 1, F128());
  r.sks[0] = F128::one();
  std::vector<F128> layer(ln);
  for (uint32_t i = 1; i <= ln; ++i) layer[i - 1] = F128(1ull << i, 0);
  uint32_t cur = ln;
  for (uint32_t i = 0; i < ln; ++i) {
    for (uint32_t j = 0; j < cur; ++j) {
      F128 v = layer[j] * layer[j] + r.sks[i] * layer[j];
      if (j == 0) r.sks[i + 1] = v; else layer[j - 1] = v;
    }
    cur--;
  }
  r.inv_sks.resize(ln + 1);
  for (uint32_t i = 0; i <= ln; ++i) r.inv_sks[i] = r.sks[i].is_zero() ? F128() : inv(r.sks[i]);
  return r;
}
// Normalised LCH basis factors W_k(q) = s_k(q) / s_k(v_k), k < ln
// (ligerito.rs:2431-2460, evaluate_scaled_basis_inplace).
inline std::vector<F128> lch_basis_factors(uint64_t q, uint32_t ln, const LchSks& t) {
  std::vector<F128> s(ln);
  if (ln > 0) {
    s[0] = F128(q, 0);
    for (uint32_t i = 1; i < ln; ++i) s[i] = s[i - 1] * s[i - 1] + t.sks[i - 1] * s[i - 1];
    for (uint32_t i = 0; i < ln; ++i) s[i] = s[i] * t.inv_sks[i];
  }
  return s;
}

struct ProveResult {
  MergedProof proof;
  std::vector<Hash> cap;
  ProofClaims claims;
  ProveTimings t;
};

// prove_fast_ligerito_union over the statement's registry and declared counts
// (prover.rs:587-620, 831-1468); slot_inputs[t] holds the records of slot t (slot order).
// A single-hash statement is the one-slot union: Blake3Setup / Sha256HybridSetup /
// KeccakSetup ::prove_fast.
inline ProveResult prove_fast(const Statement& S, ProverBackend& B, const std::vector<const uint8_t*>& slot_inputs,
                              const uint8_t* domain, size_t domain_len) {
  ProveResult R;
  double t0 = now_ms();
  Transcript T(domain, domain_len);
  T.set_pow_search(B.pow_search());
  const uint32_t m = S.m, nu = S.nu, k_log = S.k_log;
  const uint32_t n_mlv = m - 6;
  if (slot_inputs.size() != S.slots.size()) throw std::runtime_error("one input pointer per registry slot");

  // ---- witness + commit + bind (union.rs:619-628: label, registry digest, the counts
  // vector as one u64 LE per slot, the cap)
  B.witness(slot_inputs);
  double t1 = now_ms();
  B.commit_l0(S.lig.sched[0].cap_depth(), R.cap);
  double t2 = now_ms();
  T.observe_label("flock-mixed-v1");
  T.observe_bytes(S.registry_digest.data(), 32);
  std::vector<uint8_t> counts;
  for (const SlotInfo& t : S.slots)
    for (int i = 0; i < 8; ++i) counts.push_back((uint8_t)(t.count >> (8 * i)));
  T.observe_bytes(counts.data(), counts.size());
  {
    std::vector<uint8_t> capb;
    for (auto& h : R.cap) capb.insert(capb.end(), h.begin(), h.end());
    T.observe_bytes(capb);
  }

  // ---- zerocheck
  ZerocheckProof& zc = R.proof.zerocheck;
  T.observe_label("flock-zerocheck-v0");
  std::vector<F128> r(m);
  {
    auto pr = T.grind_pow_and_sample_f128_vec(bits_for(m), 6);
    zc.grinding_nonces.push_back(pr.first);
    for (int i = 0; i < 6; ++i) r[i] = pr.second[i];
    const auto& fixed = zc_fixed_challenges();
    for (int i = 0; i < 7; ++i) r[6 + i] = fixed[i];
    auto ro = T.sample_f128_vec(m - 13);
    for (uint32_t i = 0; i < m - 13; ++i) r[13 + i] = ro[i];
  }
  std::vector<F128> s_hat_v_c;
  B.zc_round1(r, zc.round1_ab, zc.round1_c, s_hat_v_c);
  T.observe_f128_slice(zc.round1_ab);
  T.observe_f128_slice(zc.round1_c);
  F128 zskip;
  {
    auto pr = T.grind_pow_and_sample_f128(bits_for(127));
    zc.grinding_nonces.push_back(pr.first);
    zskip = pr.second;
  }
  zc.final_c_eval = interpolate_on_lambda(zc.round1_c, zskip);
  std::vector<F128> mlv;
  const std::vector<F128> skip_w = lagrange_weights64(zskip, 0);
  {
    std::vector<F128> eqp(r.begin() + 7, r.end());
    F128 g1, gi;
    B.zc_fold_skip(skip_w, eqp, g1, gi);
    zc.multilinear_rounds.push_back({g1, gi});
    T.observe_f128(g1); T.observe_f128(gi);
    auto pr = T.grind_pow_and_sample_f128(2);
    zc.grinding_nonces.push_back(pr.first);
    mlv.push_back(pr.second);
    for (uint32_t i = 0; i + 1 < n_mlv; ++i) {
      std::vector<F128> eqn(r.begin() + 6 + i + 2, r.end());
      B.zc_fold(mlv[i], eqn, g1, gi);
      zc.multilinear_rounds.push_back({g1, gi});
      T.observe_f128(g1); T.observe_f128(gi);
      auto p2 = T.grind_pow_and_sample_f128(2);
      zc.grinding_nonces.push_back(p2.first);
      mlv.push_back(p2.second);
    }
    B.zc_final(mlv.back(), zc.final_a_eval, zc.final_b_eval);
    T.observe_f128(zc.final_a_eval);
    T.observe_f128(zc.final_b_eval);
  }
  double t3 = now_ms();

  // ---- lincheck (x_ab: inner_rest = [mlv0] ++ mlv[1+nu..], outer = mlv[1..1+nu])
  std::vector<F128> x_inner_rest, x_outer(mlv.begin() + 1, mlv.begin() + 1 + nu);
  x_inner_rest.push_back(mlv[0]);
  x_inner_rest.insert(x_inner_rest.end(), mlv.begin() + 1 + nu, mlv.end());
  LincheckProof& lc = R.proof.lincheck;
  T.observe_label("flock-lincheck-v0");
  auto pa = T.grind_pow_and_sample_f128(1);
  lc.grinding_nonces.push_back(pa.first);
  F128 alpha = pa.second;
  B.lc_comb(skip_w, x_inner_rest);
  // one const-pin challenge per slot, in slot order; a slot's comb is scaled by the eq
  // weight of its prefix over the remaining column coordinates (lincheck/union.rs:270-330)
  std::vector<ProverBackend::SlotComb> slot_comb;
  for (const SlotInfo& t : S.slots) {
    auto pb = T.grind_pow_and_sample_f128(1);
    lc.grinding_nonces.push_back(pb.first);
    ProverBackend::SlotComb c;
    c.beta = pb.second;
    c.offset = t.prefix << t.k_log;
    c.pin = t.const_pin;
    c.weight = F128::one();
    for (size_t j = t.k_log - 6; j < x_inner_rest.size(); ++j) {
      const uint64_t bit = (t.prefix >> (j - (t.k_log - 6))) & 1;
      c.weight = c.weight * (bit ? x_inner_rest[j] : F128::one() + x_inner_rest[j]);
    }
    slot_comb.push_back(c);
  }
  B.lc_zvec(x_outer);
  const uint32_t inner_rest_len = k_log - 6;
  std::vector<F128> r_rounds;
  {
    F128 e1, ei;
    B.lc_start(alpha, slot_comb, e1, ei);
    for (uint32_t t = 0; t < inner_rest_len; ++t) {
      T.observe_f128(e1); T.observe_f128(ei);
      auto pr = T.grind_pow_and_sample_f128(2);
      lc.grinding_nonces.push_back(pr.first);
      lc.rounds.push_back({e1, ei});
      r_rounds.push_back(pr.second);
      B.lc_round(pr.second, t + 1 == inner_rest_len, e1, ei);
    }
  }
  B.lc_partial(lc.z_partial);
  T.observe_f128_slice(lc.z_partial);
  auto ps = T.grind_pow_and_sample_f128(6);
  lc.grinding_nonces.push_back(ps.first);
  F128 r_inner_skip = ps.second;
  F128 w_ab;
  {
    auto lw = lagrange_weights64(r_inner_skip, 0);
    for (int i = 0; i < 64; ++i) w_ab += lw[i] * lc.z_partial[i];
  }
  std::vector<F128> r_inner_rest(r_rounds.rbegin(), r_rounds.rend());
  B.lc_matrix_evals(r_inner_rest, lc.z_partial, lc.matrix_evals);
  std::vector<F128> s_hat_v_ab;
  B.lc_s_hat_v(std::vector<F128>(r_inner_rest.begin() + 1, r_inner_rest.end()), s_hat_v_ab);
  R.claims.ab_value = w_ab;
  R.claims.c_value = zc.final_c_eval;
  double t4 = now_ms();

  // ---- merged open: claim points (address-ordered, dim6 first)
  std::vector<F128> x_ab;
  x_ab.push_back(r_inner_rest[0]);
  x_ab.insert(x_ab.end(), x_outer.begin(), x_outer.end());
  x_ab.insert(x_ab.end(), r_inner_rest.begin() + 1, r_inner_rest.end());
  std::vector<F128> x_c(r.begin() + 6, r.end());
  MergedOpenProof& mo = R.proof.pcs_open;
  T.observe_label("flock-merged-open-v1");
  const uint32_t rs_bits = 3, batch_bits = 6, merged_bits = 2;
  RingSwitchOut rs_ab = ring_switch_claim(T, s_hat_v_ab, rs_bits);
  RingSwitchOut rs_c = ring_switch_claim(T, s_hat_v_c, rs_bits);
  auto pg = T.grind_pow_and_sample_f128_vec(batch_bits, 2);
  mo.batching_nonces.push_back(pg.first);
  F128 g_ab = pg.second[0], g_c = pg.second[1];
  rs_ab.scale(g_ab);
  rs_c.scale(g_c);
  // The assist's linearised fold coefficients depend only on the scaled tables: compute
  // them on another host thread while the merged sumcheck runs on the backend.
  auto coeffs = std::async(std::launch::async, [&rs_ab, &rs_c] {
    return std::make_pair(linearized_coefficients(rs_ab.table), linearized_coefficients(rs_c.table));
  });
  F128 target = g_ab * rs_ab.sumcheck_claim + g_c * rs_c.sumcheck_claim;
  mo.ring_switches = {rs_ab.proof, rs_c.proof};
  const uint32_t dense_log = S.geo.dense_m - 7;
  // the jagged layout of the committed stack: one slot at full height with its used
  // columns first is the aligned shape with closed-form assist sums; any other layout
  // takes the general (materialised) path
  const bool aligned = S.slots.size() == 1 && S.identity;
  AlignedJagged J{nu, S.geo.col_log, dense_log, aligned ? S.slots[0].used_cols : 0};
  JaggedLayout JL{nu, S.geo.col_log, dense_log, S.col_prefix};
  std::vector<ProverBackend::WeightClaim> wc(2);
  wc[0].z_row.assign(x_ab.begin() + 1, x_ab.begin() + 1 + nu);
  wc[0].z_col.assign(x_ab.begin() + 1 + nu, x_ab.end());
  wc[0].table = rs_ab.table;
  wc[1].z_row.assign(x_c.begin() + 1, x_c.begin() + 1 + nu);
  wc[1].z_col.assign(x_c.begin() + 1 + nu, x_c.end());
  wc[1].table = rs_c.table;
  std::vector<F128> rho;
  {
    F128 u0, u2;
    B.mo_build_w(wc, nu, S.area(), u0, u2);
    F128 g1 = target + u0, gi = u2;
    for (uint32_t rd = 0; rd < dense_log; ++rd) {
      T.observe_f128(g1); T.observe_f128(gi);
      auto pr = T.grind_pow_and_sample_f128(merged_bits);
      mo.merged_round_nonces.push_back(pr.first);
      mo.merged_rounds.push_back({g1, gi});
      rho.push_back(pr.second);
      B.mo_round(pr.second, rd + 1 == dense_log, g1, gi);
    }
    mo.q_eval = B.mo_q_eval();
  }
  // Frobenius multipoint assist on a forked chain, concurrent with the inner open.
  std::vector<RsClaimPoint> fcl(2);
  {
    auto cf = coeffs.get();
    fcl[0].coeffs = std::move(cf.first);
    fcl[1].coeffs = std::move(cf.second);
  }
  fcl[0].z_row = wc[0].z_row; fcl[0].z_col = wc[0].z_col;
  fcl[1].z_row = wc[1].z_row; fcl[1].z_col = wc[1].z_col;
  Transcript ch_a = T.fork("flock-par-assist-v1");
  double assist_ms = 0;
  std::thread assist([&] {
    double a0 = now_ms();
    mo.frobenius = aligned ? prove_multipoint(ch_a, J, fcl, rho, 2, 2) : prove_multipoint_jagged(ch_a, JL, fcl, rho, 2, 2);
    assist_ms = now_ms() - a0;
  });

  // ---- inner open of q_hat(rho) = q_eval (packed-direct EqPoint claim)
  BatchOpeningProofLigerito& in = mo.inner;
  T.observe_label("flock-pcs-open-batch-v0");
  T.observe_label("flock-pcs-packed-direct-v0");
  T.observe_f128(mo.q_eval);
  F128 gamma = T.sample_f128_vec(1)[0];
  F128 lig_target = gamma * mo.q_eval;
  B.lg_basis_eq(gamma, rho);

  // ---- Ligerito F256 ladder
  const LigeritoParams& P = S.lig;
  LigeritoProof& lp = in.ligerito;
  const uint32_t log_n = dense_log, initial_k = P.initial_k, n1 = log_n - initial_k;
  const size_t fold_block = size_t(1) << n1;  // lane-major L0: lane bits are the high bits
  T.observe_label("flock-ligerito-basis-f256-split-v0");
  T.observe_f128(lig_target);
  lp.initial_cap = R.cap;  // cap depth of level 0 is the commitment's
  {
    std::vector<uint8_t> capb;
    for (auto& h : lp.initial_cap) capb.insert(capb.end(), h.begin(), h.end());
    T.observe_bytes(capb);
  }
  auto observe_msg = [&](const Msg256& msg) { T.observe_f256(msg.u0); T.observe_f256(msg.u2); lp.sumcheck_transcript_f256.push_back(msg); };
  for (uint32_t o = 0; o < P.ood_samples[0]; ++o) {
    auto z = T.sample_f128_vec(log_n);
    F128 y = B.lg_eval_eq(z);
    T.observe_f128(y);
    lp.ood_values.push_back(y);
    auto pr = T.grind_pow_and_sample_f128(P.claim_bits[0]);
    lp.claim_batch_grinding_nonces.push_back(pr.first);
    lig_target += pr.second * y;
    B.lg_add_eq(pr.second, z);
  }
  observe_msg(B.lg_message(fold_block));
  for (uint32_t j = 0; j < initial_k; ++j) {
    F256 ch = T.sample_f256();
    B.lg_fold(ch, fold_block);
    if (j + 1 < initial_k) observe_msg(B.lg_message(fold_block));
    else { B.lg_code_switch(); observe_msg(B.lg_message(1)); }
  }
  uint32_t split_dim = n1 + 1;
  auto level_cap_depth = [&](uint32_t level) { return P.sched[level].cap_depth(); };
  std::vector<Hash> cap1;
  {
    uint32_t log_lanes = P.recursive_ks[0];
    B.lg_commit(1, split_dim - log_lanes, log_lanes, P.log_inv_rates[1], level_cap_depth(1), cap1);
    lp.recursive_caps.push_back(cap1);
    std::vector<uint8_t> capb;
    for (auto& h : cap1) capb.insert(capb.end(), h.begin(), h.end());
    T.observe_bytes(capb);
  }
  auto do_oods = [&](uint32_t level) {
    for (uint32_t o = 0; o < P.ood_samples[level]; ++o) {
      auto z = T.sample_f128_vec(split_dim);
      F128 y;
      Msg256 msg = B.lg_introduce_eq(z, y);
      T.observe_f128(y);
      lp.ood_values.push_back(y);
      observe_msg(msg);
      auto pr = T.grind_pow_and_sample_f128(P.claim_bits[level]);
      lp.claim_batch_grinding_nonces.push_back(pr.first);
      B.lg_glue(pr.second);
    }
  };
  do_oods(1);
  auto sample_queries = [&](uint32_t level, uint64_t& nonce) {
    const LevelSchedule& sc = P.sched[level];
    auto pr = T.grind_pow_and_sample_f128_vec(P.grinding_bits[level], P.queries[level]);
    nonce = pr.first;
    std::vector<uint64_t> q;
    size_t w = 0;
    for (uint32_t c : sc.depths)
      for (uint64_t stratum = 0; stratum < (uint64_t(1) << c); ++stratum) {
        uint32_t lo_bits = sc.log_block_len - c;
        uint64_t mask = lo_bits >= 64 ? ~0ull : ((uint64_t(1) << lo_bits) - 1);
        q.push_back((stratum << lo_bits) | (pr.second[w++].lo & mask));
      }
    return q;
  };
  auto induce = [&](uint32_t log_msg_cols, uint32_t log_rate, const std::vector<uint64_t>& q,
                    const std::vector<F128>& alpha) {
    auto rw = build_eq(alpha);
    std::vector<F128> w(rw.begin(), rw.begin() + q.size());
    std::vector<std::vector<F128>> what;
    if (!B.induced_from_positions()) {
      what.resize(q.size());
      LchSks sk = lch_sks(log_msg_cols);
      for (size_t i = 0; i < q.size(); ++i) what[i] = lch_basis_factors(q[i], log_msg_cols, sk);
    }
    return B.lg_introduce_induced(log_msg_cols, log_rate, q, w, what);
  };
  {
    uint64_t nonce;
    auto q0 = sample_queries(0, nonce);
    lp.grinding_nonces.push_back(nonce);
    auto pr = T.grind_pow_and_sample_f128_vec(P.consistency_bits[0], ceil_log2(P.queries[0]));
    lp.consistency_batch_grinding_nonces.push_back(pr.first);
    B.lg_open(0, q0, level_cap_depth(0), lp.initial_proof.opened_rows, lp.initial_proof.merkle_proof);
    observe_msg(induce(n1, P.log_inv_rates[0], q0, pr.second));
    auto pb2 = T.grind_pow_and_sample_f128(P.claim_bits[1]);
    lp.claim_batch_grinding_nonces.push_back(pb2.first);
    B.lg_glue(pb2.second);
  }
  for (uint32_t i = 0; i < P.r; ++i) {
    uint32_t k = P.recursive_ks[i];
    for (uint32_t j = 0; j < k; ++j) {
      F256 ch = T.sample_f256();
      bool switching = (j + 1 == k) && (i + 1 != P.r);
      B.lg_fold(ch, 1);
      if (switching) { B.lg_code_switch(); observe_msg(B.lg_message(1)); }
      else observe_msg(B.lg_message(1));
    }
    uint32_t ext_dim = split_dim - k;
    uint32_t level = i + 1;
    if (i + 1 == P.r) {
      auto res = B.lg_residual();
      for (auto& v : res) { lp.final_proof.yr.push_back(v.c0); lp.final_proof.yr.push_back(v.c1); }
      for (auto& v : lp.final_proof.yr) T.observe_f128(v);
      uint64_t nonce;
      auto q = sample_queries(level, nonce);
      lp.grinding_nonces.push_back(nonce);
      auto pc = T.grind_pow_and_sample_f128_vec(P.consistency_bits[level], ceil_log2(P.queries[level]));
      lp.consistency_batch_grinding_nonces.push_back(pc.first);
      auto pcb = T.grind_pow_and_sample_f128(P.claim_bits[level]);
      lp.claim_batch_grinding_nonces.push_back(pcb.first);
      B.lg_open(level, q, level_cap_depth(level), lp.final_proof.opened_rows, lp.final_proof.merkle_proof);
      break;
    }
    split_dim = ext_dim + 1;
    uint32_t next_level = i + 2;
    std::vector<Hash> capn;
    uint32_t log_lanes = P.recursive_ks[next_level - 1];
    B.lg_commit(next_level, split_dim - log_lanes, log_lanes, P.log_inv_rates[next_level], level_cap_depth(next_level), capn);
    lp.recursive_caps.push_back(capn);
    {
      std::vector<uint8_t> capb;
      for (auto& h : capn) capb.insert(capb.end(), h.begin(), h.end());
      T.observe_bytes(capb);
    }
    do_oods(next_level);
    uint64_t nonce;
    auto q = sample_queries(level, nonce);
    lp.grinding_nonces.push_back(nonce);
    auto pc = T.grind_pow_and_sample_f128_vec(P.consistency_bits[level], ceil_log2(P.queries[level]));
    lp.consistency_batch_grinding_nonces.push_back(pc.first);
    RecursiveProof rp;
    B.lg_open(level, q, level_cap_depth(level), rp.opened_rows, rp.merkle_proof);
    lp.recursive_proofs.push_back(rp);
    observe_msg(induce(ext_dim, P.log_inv_rates[level], q, pc.second));
    auto pb3 = T.grind_pow_and_sample_f128(P.claim_bits[next_level]);
    lp.claim_batch_grinding_nonces.push_back(pb3.first);
    B.lg_glue(pb3.second);
  }
  double w0 = now_ms();
  assist.join();
  R.t.assist_wait = now_ms() - w0;
  R.t.assist = assist_ms;
  T.merge_child(ch_a);
  double t5 = now_ms();
  R.t.witness = t1 - t0; R.t.commit = t2 - t1; R.t.zerocheck = t3 - t2; R.t.lincheck = t4 - t3;
  R.t.open = t5 - t4; R.t.total = t5 - t0;
  return R;
}

inline ProveResult prove_fast(const Statement& S, ProverBackend& B, const uint8_t* inputs, const uint8_t* domain,
                              size_t domain_len) {
  return prove_fast(S, B, std::vector<const uint8_t*>{inputs}, domain, domain_len);
}

// SHA-256 over bincode(proof) || cap || claim values (the byte-identity digest of
// crates/flock-prover/tests/union_m6_fixtures.rs:166-180).
inline std::vector<uint8_t> proof_bytes(const MergedProof& p) {
  Bincode bc;
  bc.merged(p);
  return std::move(bc.out);
}
inline Hash bundle_digest(const std::vector<uint8_t>& proof_bytes, const std::vector<Hash>& cap, const ProofClaims& c) {
  Sha256 h;
  h.update(proof_bytes.data(), proof_bytes.size());
  for (auto& x : cap) h.update(x.data(), 32);
  uint8_t b[16];
  for (F128 v : {c.ab_value, c.c_value}) {
    for (int i = 0; i < 8; ++i) { b[i] = (uint8_t)(v.lo >> (8 * i)); b[8 + i] = (uint8_t)(v.hi >> (8 * i)); }
    h.update(b, 16);
  }
  return h.digest();
}

}  // namespace flock
