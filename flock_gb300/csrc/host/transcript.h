// Fiat-Shamir transcript over SHA-256 — the FsChallenger discipline of
// crates/flock-core/src/challenger.rs:609-1095, SHA-256 variant (the default,
// `FsChallenger::new`):
//   * every operation absorbs a 16-byte header [op, kind, 0 x 6, len u64 LE]
//     (challenger.rs:700-715) and byte payloads are zero-padded to 16 bytes;
//   * a squeeze absorbs its OP_SQUEEZE header, then derives the output stream as
//     SHA256(state || ctr_le64) for ctr = 0, 1, ... (challenger.rs:735-760) without
//     mutating the state;
//   * proof-of-work: digest = SHA256(state); nonce = the smallest u64 with
//     SHA256(digest || nonce_le) having `bits` leading zero bits (MSB-first),
//     then the nonce is absorbed as observe_bytes (challenger.rs:884-990).
// fork / merge_child follow challenger.rs:187-205 and :975-987.
#pragma once
#include "field.h"
#include "hashes.h"
#include <functional>

namespace flock {

enum : uint8_t { OP_DOMAIN = 1, OP_LABEL = 2, OP_OBSERVE = 3, OP_SQUEEZE = 4, OP_BYTES = 5 };
enum : uint8_t { KIND_NONE = 0, KIND_SCALAR = 1, KIND_SLICE = 2 };

// Number of leading-zero PoW bits that make a degree-`d` Schwartz-Zippel event
// strictly below 2^-128 (challenger.rs:45-52).
inline uint32_t grinding_bits_for_degree(uint64_t degree) {
  if (degree == 0) return 0;
  uint32_t b = 0;
  while (degree) { b++; degree >>= 1; }
  return b;
}

inline bool has_leading_zero_bits(const uint8_t* h, uint32_t bits) {
  uint32_t full = bits / 8, extra = bits % 8;
  for (uint32_t i = 0; i < full; ++i) if (h[i]) return false;
  if (extra && (h[full] >> (8 - extra))) return false;
  return true;
}

// The nonce search can be delegated (the GPU backend searches on the device); the
// default is a sequential host scan. The contract is the SMALLEST satisfying nonce.
using PowSearchFn = std::function<uint64_t(const std::array<uint8_t, 32>& digest, uint32_t bits)>;

// SHA256(digest || nonce_le) is one padded 64-byte block: build it once, then per nonce
// rewrite the 8 nonce bytes and run a single compression.
struct PowBlock {
  uint8_t blk[64];
  explicit PowBlock(const std::array<uint8_t, 32>& digest) {
    memcpy(blk, digest.data(), 32);
    memset(blk + 32, 0, 32);
    blk[40] = 0x80;
    blk[62] = 0x01;  // 320 bits, big-endian
    blk[63] = 0x40;
  }
  // leading-zero test of SHA256(digest || nonce) on the big-endian state words
  bool meets(uint64_t nonce, uint32_t bits) {
    for (int i = 0; i < 8; ++i) blk[32 + i] = (uint8_t)(nonce >> (8 * i));
    uint32_t st[8];
    memcpy(st, Sha256::IV, sizeof(st));
    Sha256::compress(st, blk);
    for (uint32_t w = 0; bits; ++w) {
      const uint32_t take = bits < 32 ? bits : 32;
      if (st[w] >> (32 - take)) return false;
      bits -= take;
    }
    return true;
  }
};

inline uint64_t pow_search_host(const std::array<uint8_t, 32>& digest, uint32_t bits) {
  PowBlock pb(digest);
  for (uint64_t nonce = 0;; ++nonce)
    if (pb.meets(nonce, bits)) return nonce;
}

class Transcript {
 public:
  explicit Transcript(const uint8_t* domain, size_t len) {
    header(OP_DOMAIN, KIND_NONE, len);
    padded(domain, len);
  }
  explicit Transcript(const std::string& domain) : Transcript((const uint8_t*)domain.data(), domain.size()) {}

  void set_pow_search(PowSearchFn f) { pow_ = std::move(f); }

  void observe_label(const std::string& label) {
    header(OP_LABEL, KIND_NONE, label.size());
    padded((const uint8_t*)label.data(), label.size());
  }
  void observe_f128(F128 v) {
    header(OP_OBSERVE, KIND_SCALAR, 1);
    absorb_f128(v);
  }
  void observe_f128_slice(const F128* v, size_t n) {
    header(OP_OBSERVE, KIND_SLICE, n);
    for (size_t i = 0; i < n; ++i) absorb_f128(v[i]);
  }
  void observe_f128_slice(const std::vector<F128>& v) { observe_f128_slice(v.data(), v.size()); }
  void observe_f256(F256 v) {
    F128 c[2] = {v.c0, v.c1};
    observe_f128_slice(c, 2);
  }
  void observe_bytes(const uint8_t* p, size_t n) {
    header(OP_BYTES, KIND_NONE, n);
    padded(p, n);
  }
  void observe_bytes(const std::vector<uint8_t>& v) { observe_bytes(v.data(), v.size()); }

  F128 sample_f128() {
    header(OP_SQUEEZE, KIND_SCALAR, 1);
    uint8_t buf[16];
    squeeze(buf, 16);
    return load_f128(buf);
  }
  std::vector<F128> sample_f128_vec(size_t n) {
    header(OP_SQUEEZE, KIND_SLICE, n);
    std::vector<uint8_t> buf(n * 16);
    squeeze(buf.data(), buf.size());
    std::vector<F128> out(n);
    for (size_t i = 0; i < n; ++i) out[i] = load_f128(buf.data() + 16 * i);
    return out;
  }
  F256 sample_f256() {
    auto w = sample_f128_vec(2);
    return F256(w[0], w[1]);
  }

  uint64_t grind_pow(uint32_t bits) {
    auto digest = state_.digest();
    uint64_t nonce = 0;
    if (bits != 0) nonce = pow_ ? pow_(digest, bits) : pow_search_host(digest, bits);
    uint8_t le[8];
    for (int i = 0; i < 8; ++i) le[i] = (uint8_t)(nonce >> (8 * i));
    observe_bytes(le, 8);
    return nonce;
  }
  std::pair<uint64_t, F128> grind_pow_and_sample_f128(uint32_t bits) {
    uint64_t n = grind_pow(bits);
    return {n, sample_f128()};
  }
  std::pair<uint64_t, std::vector<F128>> grind_pow_and_sample_f128_vec(uint32_t bits, size_t n) {
    uint64_t nonce = grind_pow(bits);
    return {nonce, sample_f128_vec(n)};
  }
  // Verifier mirror of grind_pow: check the nonce against the current state, then absorb it.
  bool verify_pow(uint64_t nonce, uint32_t bits) {
    auto digest = state_.digest();
    bool ok;
    if (bits == 0) {
      ok = nonce == 0;
    } else {
      ok = bits <= 256 && PowBlock(digest).meets(nonce, bits);
    }
    uint8_t le[8];
    for (int i = 0; i < 8; ++i) le[i] = (uint8_t)(nonce >> (8 * i));
    observe_bytes(le, 8);
    return ok;
  }

  Transcript fork(const std::string& label) {
    F128 s0 = sample_f128();
    F128 s1 = sample_f128();
    Transcript child(label);
    child.pow_ = pow_;
    child.observe_f128(s0);
    child.observe_f128(s1);
    return child;
  }
  void merge_child(Transcript& child) {
    F128 d0 = child.sample_f128();
    F128 d1 = child.sample_f128();
    observe_f128(d0);
    observe_f128(d1);
  }

  std::array<uint8_t, 32> state_digest() const { return state_.digest(); }

 private:
  Sha256 state_;
  PowSearchFn pow_;

  static F128 load_f128(const uint8_t* b) {
    uint64_t lo = 0, hi = 0;
    for (int i = 0; i < 8; ++i) { lo |= (uint64_t)b[i] << (8 * i); hi |= (uint64_t)b[8 + i] << (8 * i); }
    return F128(lo, hi);
  }
  void header(uint8_t op, uint8_t kind, uint64_t len) {
    uint8_t h[16] = {0};
    h[0] = op; h[1] = kind;
    for (int i = 0; i < 8; ++i) h[8 + i] = (uint8_t)(len >> (8 * i));
    state_.update(h, 16);
  }
  void padded(const uint8_t* p, size_t n) {
    state_.update(p, n);
    size_t rem = n % 16;
    if (rem) {
      uint8_t z[16] = {0};
      state_.update(z, 16 - rem);
    }
  }
  void absorb_f128(F128 v) {
    uint8_t b[16];
    for (int i = 0; i < 8; ++i) { b[i] = (uint8_t)(v.lo >> (8 * i)); b[8 + i] = (uint8_t)(v.hi >> (8 * i)); }
    state_.update(b, 16);
  }
  void squeeze(uint8_t* out, size_t n) {
    size_t off = 0;
    uint64_t ctr = 0;
    while (off < n) {
      Sha256 c = state_;
      uint8_t le[8];
      for (int i = 0; i < 8; ++i) le[i] = (uint8_t)(ctr >> (8 * i));
      c.update(le, 8);
      auto blk = c.digest();
      size_t take = n - off < 32 ? n - off : 32;
      memcpy(out + off, blk.data(), take);
      off += take;
      ctr++;
    }
  }
};

}  // namespace flock
