// Constant tables the device kernels read, built once per process on the host.
//
//  * NTT twiddles of the additive LCH transform over GF(2^128) with the standard
//    basis {1, x, x^2, ...} (crates/flock-core/src/ntt/additive_ntt_f128.rs:67-158):
//    W_i are the normalised subspace polynomials, evals[i] = [W_i(b_i) .. W_i(b_{l-1})] /
//    W_i(b_i), and the twiddle of (layer, block) is the XOR of evals[l - layer - 1][j + 1]
//    over the set bits j of `block`; stored flat as tw[(1 << layer) - 1 + block].
//  * The univariate-skip extension S -> Lambda of a 64-point GF(2) row: the GF(2^8)
//    additive NTT of crates/flock-core/src/ntt.rs:18-117 with cosets beta = 0 (S) and
//    beta = 64 (Lambda), inverse on S then forward on Lambda, tabulated per input byte
//    (ext[c][v][i] = sum over set bits b of v of unit(8c + b)[i]).
#pragma once
#include "field.h"

namespace flock {

// Flat twiddle table of a transform of size 2^log_d (all layers).
inline std::vector<F128> ntt_twiddles(uint32_t log_d) {
  std::vector<std::vector<F128>> ev(log_d);
  for (uint32_t i = 0; i < log_d; ++i) {
    if (i == 0) {
      for (uint32_t k = 0; k < log_d; ++k) ev[0].push_back(k < 64 ? F128(1ull << k, 0) : F128(0, 1ull << (k - 64)));
    } else {
      const auto& p = ev[i - 1];
      for (size_t k = 1; k < p.size(); ++k) ev[i].push_back(p[k] * (p[k] + p[0]));
    }
  }
  for (auto& row : ev) {
    F128 s = inv(row[0]);
    for (auto& v : row) v = v * s;
  }
  std::vector<F128> tw(log_d ? (size_t(1) << log_d) - 1 : 0);
  for (uint32_t layer = 0; layer < log_d; ++layer) {
    const auto& v = ev[log_d - layer - 1];
    F128* t = tw.data() + (size_t(1) << layer) - 1;
    t[0] = F128();
    // block b = (b without its top bit) + one more term: O(1) per entry
    for (size_t b = 1; b < (size_t(1) << layer); ++b) {
      uint32_t top = 63 - __builtin_clzll((unsigned long long)b);
      t[b] = t[b ^ (size_t(1) << top)] + v[top + 1];
    }
  }
  return tw;
}

// GF(2^8) additive NTT of size 64 on the coset beta + span{1, 2, 4, ..., 32}.
struct Gf8Ntt64 {
  uint8_t tw[63];
  explicit Gf8Ntt64(uint8_t beta) {
    const int k = 6;
    int len = 32;
    uint8_t layer[32];
    for (int i = 0; i < len; ++i) layer[i] = (uint8_t)(beta ^ (2 * i));
    int at = len;
    for (int i = 0; i < len; ++i) tw[at - 1 + i] = layer[i];
    uint8_t s_root = 1;
    auto next_s = [](uint8_t s, uint8_t root) { return (uint8_t)(gf8_mul(s, s) ^ gf8_mul(root, s)); };
    for (int it = 1; it < k; ++it) {
      at >>= 1;
      uint8_t nroot = next_s((uint8_t)(layer[1] ^ layer[0]), s_root);
      for (int i = 0; i < at; ++i) layer[i] = next_s(layer[2 * i], s_root);
      s_root = nroot;
      uint8_t si = gf8_inv(s_root);
      for (int j = 0; j < at; ++j) tw[at - 1 + j] = gf8_mul(si, layer[j]);
    }
  }
  void forward(uint8_t* v, int n, int idx) const {
    if (n == 1) return;
    int h = n / 2;
    uint8_t lam = tw[idx - 1];
    for (int i = 0; i < h; ++i) {
      uint8_t w = v[h + i];
      v[i] ^= gf8_mul(lam, w);
      v[h + i] = w ^ v[i];
    }
    forward(v, h, 2 * idx);
    forward(v + h, h, 2 * idx + 1);
  }
  void inverse(uint8_t* v, int n, int idx) const {
    if (n == 1) return;
    int h = n / 2;
    inverse(v, h, 2 * idx);
    inverse(v + h, h, 2 * idx + 1);
    uint8_t lam = tw[idx - 1];
    for (int i = 0; i < h; ++i) {
      v[h + i] ^= v[i];
      v[i] ^= gf8_mul(lam, v[h + i]);
    }
  }
};

// ext[c * 256 * 64 + v * 64 + i]: extension on Lambda of the bits v placed at S[8c..8c+8).
struct SkipTables {
  std::vector<uint8_t> ext;   // 8 x 256 x 64
  uint8_t unit[64][64];       // extension of each unit vector
};
inline const SkipTables& skip_tables() {
  static SkipTables t = [] {
    SkipTables s;
    Gf8Ntt64 on_s(0), on_l(64);
    for (int b = 0; b < 64; ++b) {
      uint8_t v[64] = {0};
      v[b] = 1;
      on_s.inverse(v, 64, 1);
      on_l.forward(v, 64, 1);
      memcpy(s.unit[b], v, 64);
    }
    s.ext.assign(8 * 256 * 64, 0);
    for (int c = 0; c < 8; ++c)
      for (int v = 0; v < 256; ++v)
        for (int b = 0; b < 8; ++b)
          if ((v >> b) & 1)
            for (int i = 0; i < 64; ++i) s.ext[(c * 256 + v) * 64 + i] ^= s.unit[8 * c + b][i];
    return s;
  }();
  return t;
}

}  // namespace flock
