// Keccak-f[1600] as a block R1CS over GF(2) with C = I and the constraint
// definition held by a lincheck walker instead of materialised matrices
// (crates/flock-prover/src/r1cs_hashes/keccak.rs:1-70, :430-560, :678-836). The walker's
// column folds run on the device (sumcheck.cu, keccak_lincheck_columns_kernel).
//
// Layout of one 2^16-bit block: state_0 at [0,1600) (lane-contiguous, slot of 2048),
// state_24 at [2048,3648), the constant one at 4096, t_0..t_23 (the 24 chi
// AND outputs) at 4160 + 1600 r. Useful bits 42,560.
//
// Input convention: a permutation input is 25 u64 words where bit j of word i is
// state bit 64 i + j, state bit index x + 5y + 25z (keccak.rs:136-140, and the
// benchmark's random_keccak_state, benches/hash_throughput.rs:53-62).
#pragma once
#include "field.h"
#include "r1cs_common.h"

namespace flock {
namespace kr1cs {

constexpr int K_LOG = 16;
constexpr uint32_t K = 1u << K_LOG;
constexpr int STATE_BITS = 1600, N_LANES = 25, N_T = 24, N_ROUNDS = 24;
constexpr uint32_t STATE0_BIT_BASE = 0, STATE24_BIT_BASE = 2048, Z_CONST = 4096, T_PACKED_BIT_BASE = 4160;
constexpr uint32_t USEFUL_BITS = T_PACKED_BIT_BASE + N_T * STATE_BITS;  // 42,560
constexpr uint32_t U64_PER_BLOCK = K / 64;

constexpr uint32_t RHO[5][5] = {{0, 36, 3, 41, 18}, {1, 44, 10, 45, 2}, {62, 6, 43, 15, 61},
                                {28, 55, 25, 21, 56}, {27, 20, 39, 8, 14}};
constexpr uint64_t RC[24] = {
    0x0000000000000001ull, 0x0000000000008082ull, 0x800000000000808Aull, 0x8000000080008000ull,
    0x000000000000808Bull, 0x0000000080000001ull, 0x8000000080008081ull, 0x8000000000008009ull,
    0x000000000000008Aull, 0x0000000000000088ull, 0x0000000080008009ull, 0x000000008000000Aull,
    0x000000008000808Bull, 0x800000000000008Bull, 0x8000000000008089ull, 0x8000000000008003ull,
    0x8000000000008002ull, 0x8000000000000080ull, 0x000000000000800Aull, 0x800000008000000Aull,
    0x8000000080008081ull, 0x8000000000008080ull, 0x0000000080000001ull, 0x8000000080008008ull};

inline int state_idx(int x, int y, int z) { return x + 5 * y + 25 * z; }
inline uint64_t rotl64(uint64_t v, uint32_t r) { r &= 63; return r ? (v << r) | (v >> (64 - r)) : v; }

// Bit-packed state words (bit j of word i = state bit 64 i + j) -> Keccak lanes (x + 5y).
inline void words_to_lanes(const uint64_t words[25], uint64_t lanes[25]) {
  for (int i = 0; i < 25; ++i) lanes[i] = 0;
  for (int j = 0; j < STATE_BITS; ++j) {
    if ((words[j >> 6] >> (j & 63)) & 1) {
      int xy = j % 25, z = j / 25;
      lanes[xy] |= 1ull << z;
    }
  }
}

inline void theta(uint64_t s[25]) {
  uint64_t c[5], d[5];
  for (int x = 0; x < 5; ++x) c[x] = s[x] ^ s[x + 5] ^ s[x + 10] ^ s[x + 15] ^ s[x + 20];
  for (int x = 0; x < 5; ++x) d[x] = c[(x + 4) % 5] ^ rotl64(c[(x + 1) % 5], 1);
  for (int i = 0; i < 25; ++i) s[i] ^= d[i % 5];
}
inline void rho_pi(const uint64_t in[25], uint64_t out[25]) {
  for (int y = 0; y < 5; ++y)
    for (int x = 0; x < 5; ++x) {
      int a = (x + 3 * y) % 5, b = x;
      out[x + 5 * y] = rotl64(in[a + 5 * b], RHO[a][b] % 64);
    }
}

// Witness bits z, a, b of one block (caller-zeroed, K bits each as u64 words).
inline void witness_block(const uint64_t words[25], uint64_t* z, uint64_t* a, uint64_t* b) {
  z[Z_CONST / 64] = 1; a[Z_CONST / 64] = 1; b[Z_CONST / 64] = 1;
  uint64_t st[25];
  words_to_lanes(words, st);
  for (int l = 0; l < 25; ++l) { z[l] = st[l]; a[l] = st[l]; b[l] = ~0ull; }
  for (int r = 0; r < N_ROUNDS; ++r) {
    uint64_t th[25], bs[25], t[25];
    for (int i = 0; i < 25; ++i) th[i] = st[i];
    theta(th);
    rho_pi(th, bs);
    for (int y = 0; y < 5; ++y)
      for (int x = 0; x < 5; ++x) t[x + 5 * y] = (~bs[(x + 1) % 5 + 5 * y]) & bs[(x + 2) % 5 + 5 * y];
    uint32_t tb = T_PACKED_BIT_BASE / 64 + r * 25;
    for (int y = 0; y < 5; ++y)
      for (int x = 0; x < 5; ++x) {
        int l = x + 5 * y;
        z[tb + l] = t[l];
        a[tb + l] = ~bs[(x + 1) % 5 + 5 * y];
        b[tb + l] = bs[(x + 2) % 5 + 5 * y];
      }
    for (int i = 0; i < 25; ++i) st[i] = bs[i] ^ t[i];
    st[0] ^= RC[r];
  }
  for (int l = 0; l < 25; ++l) { z[STATE24_BIT_BASE / 64 + l] = st[l]; a[STATE24_BIT_BASE / 64 + l] = st[l]; b[STATE24_BIT_BASE / 64 + l] = ~0ull; }
}

// Column position of state bit s of a lane-contiguous 1600-bit vector starting at u64 `base`.
inline uint32_t lane_pos(uint32_t base_u64, int s) { return (base_u64 + s % 25) * 64 + s / 25; }

// Empty K x K stub used for the registry digest of the walker-based type.
inline const SparseRows& empty_stub() {
  static SparseRows m = [] { SparseRows s; s.num_rows = s.num_cols = K; s.rows.assign(K, {}); return s; }();
  return m;
}

}  // namespace kr1cs
}  // namespace flock
