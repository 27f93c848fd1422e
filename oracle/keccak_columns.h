// ORACLE — test infrastructure only.
//
// The column folds of the Keccak-f block R1CS, ca = eq^T A_0 and cb = eq^T B_0, computed
// from the FORWARD definition of the constraint rows rather than from a transposed walker:
// the rows A_0 z and B_0 z are the linear (affine in z_Z, the constant-one column) maps the
// witness relation defines (crates/flock-prover/src/r1cs_hashes/keccak.rs:430-560, the
// encoder restated in r1cs_keccak.h: a = state_in / ~B[x+1] / state_out, b = 1 / B[x+2] /
// 1, with B = (pi o rho o theta)(state) and state_{r+1} = B ^ t_r ^ RC_r). Every column j
// that any row reads (z_Z, the 1600 input-state bits and the 24 x 1600 chi outputs t_r) is
// pushed through that map as a unit vector, 64 columns at a time in bit-sliced u64 words
// (bit l of a word = column l of the batch), and ca[j] = sum of eq over the rows whose
// image has bit l set. This is what KeccakLincheckCircuit::fold_alpha_batched
// (keccak.rs:692-829) computes by walking the map backwards; the two meet only in the
// result, so a GPU proof that equals this oracle's proof checks the device walker.
#pragma once
#include "../flock_gb300/csrc/host/r1cs_keccak.h"
#include "../flock_gb300/csrc/host/parallel.h"

namespace flock {
namespace oracle {

inline void keccak_columns_forward(const F128* eq, std::vector<F128>& ca, std::vector<F128>& cb) {
  using namespace kr1cs;
  ca.assign(K, F128());
  cb.assign(K, F128());
  // the columns the rows read, in a fixed order: z_Z, state_0 bits, then t_r bits
  std::vector<uint32_t> cols;
  cols.push_back(Z_CONST);
  for (int s = 0; s < STATE_BITS; ++s) cols.push_back(lane_pos(STATE0_BIT_BASE / 64, s));
  for (int r = 0; r < N_T; ++r)
    for (int s = 0; s < STATE_BITS; ++s) cols.push_back(lane_pos(T_PACKED_BIT_BASE / 64 + 25 * r, s));
  const size_t n_batches = (cols.size() + 63) / 64;
  parallel_for(n_batches, [&](size_t bt) {
    // unit-vector words of this batch: column index i = 64 bt + l
    auto unit = [&](size_t i) -> uint64_t {
      return (i >= 64 * bt && i < 64 * bt + 64) ? (uint64_t(1) << (i - 64 * bt)) : 0;
    };
    const uint64_t c1 = unit(0);
    // bit-sliced state: st[lane x + 5 y][z]
    uint64_t st[25][64], th[25][64], bs[25][64];
    for (int s = 0; s < STATE_BITS; ++s) st[s % 25][s / 25] = unit(1 + s);
    // rows: (eq row index, image word)
    auto add_row = [&](std::vector<F128>& out, uint32_t row, uint64_t img) {
      const F128 e = eq[row];
      while (img) {
        const int l = __builtin_ctzll(img);
        out[cols[64 * bt + l]] += e;
        img &= img - 1;
      }
    };
    add_row(ca, Z_CONST, c1);
    add_row(cb, Z_CONST, c1);
    for (int s = 0; s < STATE_BITS; ++s) {
      add_row(ca, lane_pos(STATE0_BIT_BASE / 64, s), st[s % 25][s / 25]);
      add_row(cb, lane_pos(STATE0_BIT_BASE / 64, s), c1);
    }
    for (int r = 0; r < N_ROUNDS; ++r) {
      // theta: column parities C[x][z], D[x][z] = C[x-1][z] ^ C[x+1][z-1]
      uint64_t C[5][64];
      for (int x = 0; x < 5; ++x)
        for (int z = 0; z < 64; ++z) C[x][z] = st[x][z] ^ st[x + 5][z] ^ st[x + 10][z] ^ st[x + 15][z] ^ st[x + 20][z];
      for (int l = 0; l < 25; ++l)
        for (int z = 0; z < 64; ++z) th[l][z] = st[l][z] ^ C[(l % 5 + 4) % 5][z] ^ C[(l % 5 + 1) % 5][(z + 63) % 64];
      // rho and pi: lane x + 5 y of the output is lane a + 5 b rotated left by rho(a, b),
      // (a, b) = ((x + 3 y) mod 5, x)
      for (int y = 0; y < 5; ++y)
        for (int x = 0; x < 5; ++x) {
          const int a = (x + 3 * y) % 5, b = x, rot = (int)(RHO[a][b] % 64);
          for (int z = 0; z < 64; ++z) bs[x + 5 * y][z] = th[a + 5 * b][(z + 64 - rot) % 64];
        }
      const uint32_t tb = T_PACKED_BIT_BASE / 64 + 25 * r;
      for (int y = 0; y < 5; ++y)
        for (int x = 0; x < 5; ++x)
          for (int z = 0; z < 64; ++z) {
            const int s = state_idx(x, y, z);
            add_row(ca, lane_pos(tb, s), bs[(x + 1) % 5 + 5 * y][z] ^ c1);
            add_row(cb, lane_pos(tb, s), bs[(x + 2) % 5 + 5 * y][z]);
          }
      for (int s = 0; s < STATE_BITS; ++s) st[s % 25][s / 25] = bs[s % 25][s / 25] ^ unit(1 + STATE_BITS * (r + 1) + s);
      for (int z = 0; z < 64; ++z)
        if ((RC[r] >> z) & 1) st[0][z] ^= c1;
    }
    for (int s = 0; s < STATE_BITS; ++s) {
      add_row(ca, lane_pos(STATE24_BIT_BASE / 64, s), st[s % 25][s / 25]);
      add_row(cb, lane_pos(STATE24_BIT_BASE / 64, s), c1);
    }
  });
}

}  // namespace oracle
}  // namespace flock
