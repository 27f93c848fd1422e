// The reference's proof file / wire format for a standalone hash proof
// (crates/flock-prover/src/proof_io.rs:8-15, 238-252, 309-313):
//   "FLOCK" | VERSION 21 | flavor 2 (R1cs) | bincode(R1csProofBundleLigerito)
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

// bundle (u64 proof_len | bincode proof | u64 cap_len | cap | ab | c) -> proof-io bytes
inline std::vector<uint8_t> proof_io_from_bundle(const Statement& S, const uint8_t* b, size_t n) {
  auto rd = [&](size_t off) {
    if (off + 8 > n) throw std::invalid_argument("bundle truncated");
    uint64_t v = 0;
    for (int i = 0; i < 8; ++i) v |= (uint64_t)b[off + i] << (8 * i);
    return v;
  };
  uint64_t plen = rd(0);
  if (plen > n - 8) throw std::invalid_argument("bundle proof length past the end");
  uint64_t ncap = rd(8 + plen);
  if (ncap > (n - 16 - plen) / 32 || 16 + plen + 32 * ncap + 32 != n) throw std::invalid_argument("bundle cap length");
  Bincode out;
  const char magic[5] = {'F', 'L', 'O', 'C', 'K'};
  out.out.insert(out.out.end(), magic, magic + 5);
  out.out.push_back(PROOF_IO_VERSION);
  out.out.push_back(PROOF_IO_FLAVOR_R1CS);
  // Commitment { cap, params }
  out.u64(ncap);
  out.out.insert(out.out.end(), b + 16 + plen, b + 16 + plen + 32 * ncap);
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
  out.out.insert(out.out.end(), b + 8, b + 8 + plen);  // proof (already bincode)
  return std::move(out.out);
}

}  // namespace flock
