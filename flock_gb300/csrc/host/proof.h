// Proof objects of the prove_fast path and their bincode 1.x encoding
// (little-endian fixed-width integers, Vec = u64 length + items, struct fields in
// declaration order, [u8; 32] as 32 raw bytes, tuples as their fields in order).
//
// Field order follows the reference types exactly:
//   R1csProofMergedLigerito   crates/flock-core/src/proof.rs:43-48
//   ZerocheckProof            crates/flock-core/src/zerocheck.rs:428-445
//   LincheckProof             crates/flock-core/src/lincheck.rs:520-560
//   MergedOpenProof           crates/flock-core/src/pcs.rs:1362-1377
//   RingSwitchProof           crates/flock-core/src/pcs/ring_switch.rs:2193-2199
//   MultipointTwistedProof    crates/flock-core/src/pcs/jagged.rs:2790-2802
//   FrobeniusAssistProof      crates/flock-core/src/pcs/jagged.rs:1679-1687
//   BatchOpeningProofLigerito crates/flock-core/src/pcs.rs:46-55
//   LigeritoProof, RecursiveProof, FinalProof  crates/flock-core/src/pcs/ligerito.rs:2156-2218
#pragma once
#include "field.h"
#include <array>
#include <cstring>
#include <vector>

namespace flock {

using Hash = std::array<uint8_t, 32>;
using Pair128 = std::pair<F128, F128>;

struct Msg256 { F256 u0, u2; };

struct ZerocheckProof {
  std::vector<F128> round1_ab, round1_c;
  std::vector<Pair128> multilinear_rounds;
  F128 final_a_eval, final_b_eval, final_c_eval;
  std::vector<uint64_t> grinding_nonces;
};
struct LincheckProof {
  std::vector<Pair128> rounds;
  std::vector<F128> z_partial;
  std::vector<Pair128> matrix_evals;
  std::vector<uint64_t> grinding_nonces;
};
struct RingSwitchProof {
  std::vector<F128> s_hat_v;
  uint64_t grinding_nonce = 0;
};
struct FrobeniusAssistProof {
  F128 v;
  std::vector<Pair128> rounds;
  std::vector<uint64_t> grinding_nonces;
};
struct MultipointTwistedProof {
  std::vector<std::vector<F128>> values;
  std::vector<F128> group_values;
  uint64_t gamma_grinding_nonce = 0;
  std::vector<Pair128> rounds;
  std::vector<uint64_t> round_grinding_nonces;
  FrobeniusAssistProof anchor;
};
struct RecursiveProof {
  std::vector<std::vector<F128>> opened_rows;
  std::vector<Hash> merkle_proof;
};
struct FinalProof {
  std::vector<F128> yr;
  std::vector<std::vector<F128>> opened_rows;
  std::vector<Hash> merkle_proof;
};
struct LigeritoProof {
  std::vector<Hash> initial_cap;
  RecursiveProof initial_proof;
  std::vector<std::vector<Hash>> recursive_caps;
  std::vector<RecursiveProof> recursive_proofs;
  FinalProof final_proof;
  std::vector<Pair128> sumcheck_transcript;  // base-field messages (empty on this path)
  std::vector<Msg256> sumcheck_transcript_f256;
  std::vector<uint64_t> grinding_nonces;
  std::vector<F128> ood_values;
  std::vector<uint64_t> fold_grinding_nonces;
  std::vector<uint64_t> claim_batch_grinding_nonces;
  std::vector<uint64_t> consistency_batch_grinding_nonces;
};
struct BatchOpeningProofLigerito {
  std::vector<RingSwitchProof> ring_switches;
  std::vector<uint64_t> batching_nonces;
  LigeritoProof ligerito;
};
struct MergedOpenProof {
  std::vector<RingSwitchProof> ring_switches;
  std::vector<uint64_t> batching_nonces;
  std::vector<Pair128> merged_rounds;
  std::vector<uint64_t> merged_round_nonces;
  F128 q_eval;
  MultipointTwistedProof frobenius;
  BatchOpeningProofLigerito inner;
};
struct MergedProof {  // R1csProofMergedLigerito
  ZerocheckProof zerocheck;
  LincheckProof lincheck;
  MergedOpenProof pcs_open;
};
// The claims a proof establishes (R1csClaim): the values the digest binds.
struct ProofClaims {
  F128 ab_value, c_value;
};

// ---- bincode writer --------------------------------------------------------------
// Writes grow the buffer once per value or per vector (a proof is hundreds of KB; a
// byte-at-a-time writer spent about a millisecond of host time per proof here).
struct Bincode {
  std::vector<uint8_t> out;
  Bincode() { out.reserve(size_t(1) << 20); }
  uint8_t* grow(size_t n) {
    const size_t at = out.size();
    out.resize(at + n);
    return out.data() + at;
  }
  static void put64(uint8_t* p, uint64_t v) {
    for (int i = 0; i < 8; ++i) p[i] = (uint8_t)(v >> (8 * i));
  }
  static uint8_t* put128(uint8_t* p, const F128& v) {
    put64(p, v.lo);
    put64(p + 8, v.hi);
    return p + 16;
  }
  void u64(uint64_t v) { put64(grow(8), v); }
  void f128(const F128& v) { put128(grow(16), v); }
  void f256(const F256& v) { put128(put128(grow(32), v.c0), v.c1); }
  void hash(const Hash& h) { memcpy(grow(32), h.data(), 32); }
  void vf(const std::vector<F128>& v) {
    u64(v.size());
    uint8_t* p = grow(16 * v.size());
    for (auto& x : v) p = put128(p, x);
  }
  void vu(const std::vector<uint64_t>& v) {
    u64(v.size());
    uint8_t* p = grow(8 * v.size());
    for (auto x : v) { put64(p, x); p += 8; }
  }
  void vp(const std::vector<Pair128>& v) {
    u64(v.size());
    uint8_t* p = grow(32 * v.size());
    for (auto& q : v) p = put128(put128(p, q.first), q.second);
  }
  void vh(const std::vector<Hash>& v) {
    u64(v.size());
    uint8_t* p = grow(32 * v.size());
    for (auto& h : v) { memcpy(p, h.data(), 32); p += 32; }
  }
  void vvf(const std::vector<std::vector<F128>>& v) { u64(v.size()); for (auto& x : v) vf(x); }

  void zc(const ZerocheckProof& p) {
    vf(p.round1_ab); vf(p.round1_c); vp(p.multilinear_rounds);
    f128(p.final_a_eval); f128(p.final_b_eval); f128(p.final_c_eval); vu(p.grinding_nonces);
  }
  void lc(const LincheckProof& p) { vp(p.rounds); vf(p.z_partial); vp(p.matrix_evals); vu(p.grinding_nonces); }
  void rs(const std::vector<RingSwitchProof>& v) { u64(v.size()); for (auto& r : v) { vf(r.s_hat_v); u64(r.grinding_nonce); } }
  void rec(const RecursiveProof& p) { vvf(p.opened_rows); vh(p.merkle_proof); }
  void lig(const LigeritoProof& p) {
    vh(p.initial_cap);
    rec(p.initial_proof);
    u64(p.recursive_caps.size()); for (auto& c : p.recursive_caps) vh(c);
    u64(p.recursive_proofs.size()); for (auto& r : p.recursive_proofs) rec(r);
    vf(p.final_proof.yr); vvf(p.final_proof.opened_rows); vh(p.final_proof.merkle_proof);
    vp(p.sumcheck_transcript);
    u64(p.sumcheck_transcript_f256.size()); for (auto& m : p.sumcheck_transcript_f256) { f256(m.u0); f256(m.u2); }
    vu(p.grinding_nonces); vf(p.ood_values); vu(p.fold_grinding_nonces);
    vu(p.claim_batch_grinding_nonces); vu(p.consistency_batch_grinding_nonces);
  }
  void mp(const MultipointTwistedProof& p) {
    vvf(p.values); vf(p.group_values); u64(p.gamma_grinding_nonce); vp(p.rounds); vu(p.round_grinding_nonces);
    f128(p.anchor.v); vp(p.anchor.rounds); vu(p.anchor.grinding_nonces);
  }
  void merged(const MergedProof& p) {
    zc(p.zerocheck);
    lc(p.lincheck);
    const MergedOpenProof& o = p.pcs_open;
    rs(o.ring_switches); vu(o.batching_nonces); vp(o.merged_rounds); vu(o.merged_round_nonces);
    f128(o.q_eval); mp(o.frobenius);
    rs(o.inner.ring_switches); vu(o.inner.batching_nonces); lig(o.inner.ligerito);
  }
};

}  // namespace flock
