// The reference's proof file / wire format (crates/flock-prover/src/proof_io.rs:8-15,
// 238-282, 309-313):
//   "FLOCK" | VERSION 21 | flavor 2 (R1cs) | bincode(R1csProofBundleLigerito)
//   "FLOCK" | VERSION 21 | flavor 4 (Mixed) | bincode(MixedProofBundleLigerito)
// with R1csProofBundleLigerito = { commitment: Commitment { cap, params: PcsParams }, proof }
// (pcs/commit.rs:306-309, :32-70). PcsParams in bincode 1.x: m, log_inv_rate,
// log_batch_size as u64; profile as a u32 variant index (Fast = 0,
// pcs/ligerito.rs:71-73); num_lanes as Option<u64> (u8 tag, then the value); merkle_hash as
// a u32 variant index (Sha256 = 0, hash.rs:23-27). The setups build these params in
// r1cs_hashes/sha2.rs:1248-1259 (same for BLAKE3 and Keccak): m = dense_m, rate 1,
// log_batch_size = the Ligerito initial_k, num_lanes = Some(t) only when t < 2^initial_k
// (union.rs:386-390).
#pragma once
#include "proof.h"
#include "setup.h"
#include <stdexcept>

namespace flock {

constexpr uint8_t PROOF_IO_VERSION = 21;
constexpr uint8_t PROOF_IO_FLAVOR_R1CS = 2;
constexpr uint8_t PROOF_IO_FLAVOR_MIXED = 4;

// A proof bundle (u64 proof_len | bincode proof | u64 cap_len | cap | ab | c), split.
struct BundleParts {
  const uint8_t* proof = nullptr;
  uint64_t proof_len = 0;
  const uint8_t* cap = nullptr;
  uint64_t n_cap = 0;
};
inline BundleParts split_bundle(const uint8_t* b, size_t n) {
  auto rd = [&](size_t off) {
    if (off + 8 > n) throw std::invalid_argument("bundle truncated");
    uint64_t v = 0;
    for (int i = 0; i < 8; ++i) v |= (uint64_t)b[off + i] << (8 * i);
    return v;
  };
  BundleParts p;
  p.proof_len = rd(0);
  if (p.proof_len > n - 8) throw std::invalid_argument("bundle proof length past the end");
  p.n_cap = rd(8 + p.proof_len);
  if (p.n_cap > (n - 16 - p.proof_len) / 32 || 16 + p.proof_len + 32 * p.n_cap + 32 != n)
    throw std::invalid_argument("bundle cap length");
  p.proof = b + 8;
  p.cap = b + 16 + p.proof_len;
  return p;
}

inline void write_header(Bincode& out, uint8_t flavor) {
  const char magic[5] = {'F', 'L', 'O', 'C', 'K'};
  out.out.insert(out.out.end(), magic, magic + 5);
  out.out.push_back(PROOF_IO_VERSION);
  out.out.push_back(flavor);
}
// Commitment { cap, params: PcsParams } of a statement's L0 commit.
inline void write_commitment(Bincode& out, const Statement& S, const BundleParts& p) {
  out.u64(p.n_cap);
  out.out.insert(out.out.end(), p.cap, p.cap + 32 * p.n_cap);
  const uint32_t initial_k = S.lig.initial_k;
  out.u64(S.geo.dense_m);
  out.u64(1);  // log_inv_rate
  out.u64(initial_k);
  for (int i = 0; i < 4; ++i) out.out.push_back(0);  // profile: Fast
  if (S.lanes < (1u << initial_k)) {
    out.out.push_back(1);
    out.u64(S.lanes);
  } else {
    out.out.push_back(0);
  }
  for (int i = 0; i < 4; ++i) out.out.push_back(0);  // merkle_hash: Sha256
}

// bundle -> proof-io bytes of R1csProofBundleLigerito (flavor 2)
inline std::vector<uint8_t> proof_io_from_bundle(const Statement& S, const uint8_t* b, size_t n) {
  BundleParts p = split_bundle(b, n);
  Bincode out;
  write_header(out, PROOF_IO_FLAVOR_R1CS);
  write_commitment(out, S, p);
  out.out.insert(out.out.end(), p.proof, p.proof + p.proof_len);  // proof (already bincode)
  return std::move(out.out);
}

// The built-in mixed registry tiers the wire format names (crates/flock-prover/src/
// mixed.rs:55-97): the stable one-byte code of a BLAKE3 + SHA-256 registry at nu 7 or 10;
// 0 when the statement's registry is no such tier.
inline uint8_t mixed_registry_code(const Statement& S) {
  if (S.slots.size() != 2 || S.slots[0].hash != HASH_SHA256 || S.slots[1].hash != HASH_BLAKE3) return 0;
  if (S.nu == 7) return 1;   // Blake3Sha2Nu7
  if (S.nu == 10) return 2;  // Blake3Sha2Nu10
  return 0;
}

// bundle -> proof-io bytes of MixedProofBundleLigerito (flavor 4, proof_io.rs:254-282):
// header | registry id (u8 code) | counts (Vec<u64>, slot order) | Commitment | proof.
inline std::vector<uint8_t> mixed_proof_io_from_bundle(const Statement& S, const uint8_t* b, size_t n) {
  const uint8_t code = mixed_registry_code(S);
  if (!code) throw std::invalid_argument("the registry is not a built-in mixed tier (BLAKE3 + SHA-256 at nu 7 or 10)");
  BundleParts p = split_bundle(b, n);
  Bincode out;
  write_header(out, PROOF_IO_FLAVOR_MIXED);
  out.out.push_back(code);
  out.u64(S.slots.size());
  for (const SlotInfo& t : S.slots) out.u64(t.count);
  write_commitment(out, S, p);
  out.out.insert(out.out.end(), p.proof, p.proof + p.proof_len);
  return std::move(out.out);
}

}  // namespace flock
