// Host hash primitives used by the transcript, the Merkle commitments and the
// statement digests of the prove_fast path.
//
//  * SHA-256 (FIPS 180-4) with a copyable streaming state — the Fiat-Shamir
//    transcript squeezes by cloning it (crates/flock-core/src/challenger.rs:735-760),
//    and Merkle leaves / nodes are plain SHA-256 digests
//    (crates/flock-core/src/merkle.rs:205-232).
//  * BLAKE3: the compression function (crates/flock-core/src/hash.rs:74-140) and the
//    standard chunked tree hasher with 32-byte output, which the registry digest
//    (crates/flock-core/src/schedule.rs:542-578) runs over the R1CS matrices.
//
// On aarch64 hosts built with the SHA-2 extension (-march=armv8-a+crypto), host-compiler
// translation units run the SHA-256 block function on the ACLE SHA-256 intrinsics;
// elsewhere (and under nvcc) it is the plain C++ form.
#pragma once
#include <cstdint>
#include <cstring>
#include <vector>
#include <array>
#include <string>
#if defined(__aarch64__) && defined(__ARM_FEATURE_SHA2) && !defined(__CUDACC__)
#include <arm_neon.h>
#define FLOCK_HOST_SHA2 1
#endif

namespace flock {

#if defined(__CUDACC__)
// One SHA-256 compression for host code that nvcc compiles, in host_accel.cc (built by the
// host compiler with the SHA-2 instructions where the target has them).
void sha256_compress_host_accel(uint32_t st[8], const uint8_t* p);
#endif

// ------------------------------------------------------------------ SHA-256
struct Sha256 {
  uint32_t h[8];
  uint8_t buf[64];
  uint64_t total = 0;  // bytes absorbed
  uint32_t blen = 0;

  static constexpr uint32_t K[64] = {
      0x428a2f98, 0x71374491, 0xb5c0fbcf, 0xe9b5dba5, 0x3956c25b, 0x59f111f1, 0x923f82a4, 0xab1c5ed5,
      0xd807aa98, 0x12835b01, 0x243185be, 0x550c7dc3, 0x72be5d74, 0x80deb1fe, 0x9bdc06a7, 0xc19bf174,
      0xe49b69c1, 0xefbe4786, 0x0fc19dc6, 0x240ca1cc, 0x2de92c6f, 0x4a7484aa, 0x5cb0a9dc, 0x76f988da,
      0x983e5152, 0xa831c66d, 0xb00327c8, 0xbf597fc7, 0xc6e00bf3, 0xd5a79147, 0x06ca6351, 0x14292967,
      0x27b70a85, 0x2e1b2138, 0x4d2c6dfc, 0x53380d13, 0x650a7354, 0x766a0abb, 0x81c2c92e, 0x92722c85,
      0xa2bfe8a1, 0xa81a664b, 0xc24b8b70, 0xc76c51a3, 0xd192e819, 0xd6990624, 0xf40e3585, 0x106aa070,
      0x19a4c116, 0x1e376c08, 0x2748774c, 0x34b0bcb5, 0x391c0cb3, 0x4ed8aa4a, 0x5b9cca4f, 0x682e6ff3,
      0x748f82ee, 0x78a5636f, 0x84c87814, 0x8cc70208, 0x90befffa, 0xa4506ceb, 0xbef9a3f7, 0xc67178f2};
  static constexpr uint32_t IV[8] = {0x6a09e667, 0xbb67ae85, 0x3c6ef372, 0xa54ff53a,
                                     0x510e527f, 0x9b05688c, 0x1f83d9ab, 0x5be0cd19};

  Sha256() { memcpy(h, IV, sizeof(h)); }

  static inline uint32_t rotr(uint32_t x, int n) { return (x >> n) | (x << (32 - n)); }

  // One compression over a 64-byte block (big-endian words).
  static void compress(uint32_t st[8], const uint8_t* p) {
#if defined(__CUDACC__)
    sha256_compress_host_accel(st, p);
#else
    compress_impl(st, p);
#endif
  }
  static void compress_impl(uint32_t st[8], const uint8_t* p) {
#ifdef FLOCK_HOST_SHA2
    // four rounds per step: SHA256H / SHA256H2 on (abcd, efgh), the schedule by SHA256SU0/SU1
    uint32x4_t abcd = vld1q_u32(st), efgh = vld1q_u32(st + 4);
    const uint32x4_t abcd0 = abcd, efgh0 = efgh;
    uint32x4_t m[4];
    for (int i = 0; i < 4; ++i) m[i] = vreinterpretq_u32_u8(vrev32q_u8(vld1q_u8(p + 16 * i)));
    for (int i = 0; i < 16; ++i) {
      const uint32x4_t wk = vaddq_u32(m[0], vld1q_u32(K + 4 * i));
      const uint32x4_t prev = abcd;
      abcd = vsha256hq_u32(abcd, efgh, wk);
      efgh = vsha256h2q_u32(efgh, prev, wk);
      const uint32x4_t next = vsha256su1q_u32(vsha256su0q_u32(m[0], m[1]), m[2], m[3]);
      m[0] = m[1]; m[1] = m[2]; m[2] = m[3]; m[3] = next;
    }
    vst1q_u32(st, vaddq_u32(abcd, abcd0));
    vst1q_u32(st + 4, vaddq_u32(efgh, efgh0));
#else
    uint32_t w[64];
    for (int i = 0; i < 16; ++i)
      w[i] = (uint32_t)p[4 * i] << 24 | (uint32_t)p[4 * i + 1] << 16 | (uint32_t)p[4 * i + 2] << 8 | p[4 * i + 3];
    for (int i = 16; i < 64; ++i) {
      uint32_t s0 = rotr(w[i - 15], 7) ^ rotr(w[i - 15], 18) ^ (w[i - 15] >> 3);
      uint32_t s1 = rotr(w[i - 2], 17) ^ rotr(w[i - 2], 19) ^ (w[i - 2] >> 10);
      w[i] = w[i - 16] + s0 + w[i - 7] + s1;
    }
    uint32_t a = st[0], b = st[1], c = st[2], d = st[3], e = st[4], f = st[5], g = st[6], hh = st[7];
    for (int i = 0; i < 64; ++i) {
      uint32_t S1 = rotr(e, 6) ^ rotr(e, 11) ^ rotr(e, 25);
      uint32_t ch = (e & f) ^ (~e & g);
      uint32_t t1 = hh + S1 + ch + K[i] + w[i];
      uint32_t S0 = rotr(a, 2) ^ rotr(a, 13) ^ rotr(a, 22);
      uint32_t mj = (a & b) ^ (a & c) ^ (b & c);
      uint32_t t2 = S0 + mj;
      hh = g; g = f; f = e; e = d + t1; d = c; c = b; b = a; a = t1 + t2;
    }
    st[0] += a; st[1] += b; st[2] += c; st[3] += d; st[4] += e; st[5] += f; st[6] += g; st[7] += hh;
#endif
  }

  void update(const void* data, size_t n) {
    const uint8_t* p = (const uint8_t*)data;
    total += n;
    if (blen) {
      size_t take = 64 - blen < n ? 64 - blen : n;
      memcpy(buf + blen, p, take);
      blen += (uint32_t)take; p += take; n -= take;
      if (blen == 64) { compress(h, buf); blen = 0; }
    }
    while (n >= 64) { compress(h, p); p += 64; n -= 64; }
    if (n) { memcpy(buf, p, n); blen = (uint32_t)n; }
  }

  // Finalize a COPY (the state stays usable): 0x80, zeros to 56 mod 64, the bit length.
  std::array<uint8_t, 32> digest() const {
    uint32_t st[8];
    memcpy(st, h, sizeof(st));
    uint8_t blk[128];
    memcpy(blk, buf, blen);
    const uint32_t end = blen < 56 ? 64 : 128;
    memset(blk + blen, 0, end - blen);
    blk[blen] = 0x80;
    const uint64_t bits = total * 8;
    for (int i = 0; i < 8; ++i) blk[end - 8 + i] = (uint8_t)(bits >> (56 - 8 * i));
    compress(st, blk);
    if (end == 128) compress(st, blk + 64);
    std::array<uint8_t, 32> out;
    for (int i = 0; i < 8; ++i) {
      out[4 * i] = (uint8_t)(st[i] >> 24); out[4 * i + 1] = (uint8_t)(st[i] >> 16);
      out[4 * i + 2] = (uint8_t)(st[i] >> 8); out[4 * i + 3] = (uint8_t)st[i];
    }
    return out;
  }

  static std::array<uint8_t, 32> hash(const void* data, size_t n) {
    Sha256 s; s.update(data, n); return s.digest();
  }
};

// ------------------------------------------------------------------ BLAKE3
constexpr uint32_t BLAKE3_IV[8] = {0x6a09e667, 0xbb67ae85, 0x3c6ef372, 0xa54ff53a,
                                   0x510e527f, 0x9b05688c, 0x1f83d9ab, 0x5be0cd19};
constexpr int B3_MSG_PERM[16] = {2, 6, 3, 10, 7, 0, 4, 13, 1, 11, 12, 5, 9, 14, 15, 8};

inline uint32_t rotr32(uint32_t x, int n) { return (x >> n) | (x << (32 - n)); }

inline void b3_g(uint32_t* s, int a, int b, int c, int d, uint32_t mx, uint32_t my) {
  s[a] = s[a] + s[b] + mx; s[d] = rotr32(s[d] ^ s[a], 16);
  s[c] = s[c] + s[d];      s[b] = rotr32(s[b] ^ s[c], 12);
  s[a] = s[a] + s[b] + my; s[d] = rotr32(s[d] ^ s[a], 8);
  s[c] = s[c] + s[d];      s[b] = rotr32(s[b] ^ s[c], 7);
}

// Full 16-word output state of one BLAKE3 compression (the chaining value is out[0..8]).
inline void blake3_compress(const uint32_t cv[8], const uint32_t block[16], uint64_t counter,
                            uint32_t block_len, uint32_t flags, uint32_t out[16]) {
  uint32_t s[16] = {cv[0], cv[1], cv[2], cv[3], cv[4], cv[5], cv[6], cv[7],
                    BLAKE3_IV[0], BLAKE3_IV[1], BLAKE3_IV[2], BLAKE3_IV[3],
                    (uint32_t)counter, (uint32_t)(counter >> 32), block_len, flags};
  uint32_t m[16];
  memcpy(m, block, sizeof(m));
  for (int r = 0; r < 7; ++r) {
    b3_g(s, 0, 4, 8, 12, m[0], m[1]);
    b3_g(s, 1, 5, 9, 13, m[2], m[3]);
    b3_g(s, 2, 6, 10, 14, m[4], m[5]);
    b3_g(s, 3, 7, 11, 15, m[6], m[7]);
    b3_g(s, 0, 5, 10, 15, m[8], m[9]);
    b3_g(s, 1, 6, 11, 12, m[10], m[11]);
    b3_g(s, 2, 7, 8, 13, m[12], m[13]);
    b3_g(s, 3, 4, 9, 14, m[14], m[15]);
    if (r < 6) {
      uint32_t p[16];
      for (int i = 0; i < 16; ++i) p[i] = m[B3_MSG_PERM[i]];
      memcpy(m, p, sizeof(m));
    }
  }
  for (int i = 0; i < 8; ++i) { out[i] = s[i] ^ s[i + 8]; out[i + 8] = s[i + 8] ^ cv[i]; }
}

// Standard BLAKE3 hash (default mode, 32-byte output): 1024-byte chunks of 64-byte
// blocks, CHUNK_START/CHUNK_END/PARENT/ROOT flags, a merge stack for the binary tree.
class Blake3Hasher {
 public:
  enum : uint32_t { CHUNK_START = 1, CHUNK_END = 2, PARENT = 4, ROOT = 8 };

  Blake3Hasher() { reset_chunk(0); }

  void update(const void* data, size_t n) {
    const uint8_t* p = (const uint8_t*)data;
    while (n) {
      if (chunk_bytes_ == 1024) {
        // chunk complete and more input follows: finalize it as a non-root chaining value
        uint32_t cv[8];
        chunk_output_cv(cv);
        push_chunk_cv(cv, chunk_counter_);
        reset_chunk(chunk_counter_ + 1);
      }
      if (blen_ == 64) {
        compress_block_into_cv();
      }
      size_t take = 64 - blen_;
      size_t room = 1024 - chunk_bytes_;
      if (take > n) take = n;
      if (take > room) take = room;
      memcpy(block_ + blen_, p, take);
      blen_ += (uint32_t)take; chunk_bytes_ += (uint32_t)take;
      p += take; n -= take;
    }
  }

  std::array<uint8_t, 32> finalize() const {
    // Output of the current (last) chunk.
    uint32_t cv_in[8], words[16], flags;
    memcpy(cv_in, cv_, sizeof(cv_in));
    load_block(block_, blen_, words);
    flags = (blocks_compressed_ == 0 ? CHUNK_START : 0) | CHUNK_END;
    uint64_t counter = chunk_counter_;
    uint32_t blen = blen_;
    // Fold the stack from the top.
    size_t depth = stack_.size();
    uint32_t out[16];
    if (depth == 0) {
      blake3_compress(cv_in, words, counter, blen, flags | ROOT, out);
      return to_bytes(out);
    }
    uint32_t cv[8];
    blake3_compress(cv_in, words, counter, blen, flags, out);
    memcpy(cv, out, sizeof(cv));
    for (size_t i = depth; i-- > 0;) {
      uint32_t pw[16];
      memcpy(pw, stack_[i].data(), 32);
      memcpy(pw + 8, cv, 32);
      uint32_t f = PARENT | (i == 0 ? ROOT : 0);
      blake3_compress(BLAKE3_IV, pw, 0, 64, f, out);
      memcpy(cv, out, sizeof(cv));
    }
    return to_bytes(out);
  }

  static std::array<uint8_t, 32> hash(const void* data, size_t n) {
    Blake3Hasher h; h.update(data, n); return h.finalize();
  }

 private:
  uint32_t cv_[8];
  uint8_t block_[64];
  uint32_t blen_ = 0;
  uint32_t chunk_bytes_ = 0;
  uint32_t blocks_compressed_ = 0;
  uint64_t chunk_counter_ = 0;
  std::vector<std::array<uint32_t, 8>> stack_;

  static void load_block(const uint8_t* b, uint32_t len, uint32_t w[16]) {
    uint8_t tmp[64] = {0};
    memcpy(tmp, b, len);
    for (int i = 0; i < 16; ++i)
      w[i] = (uint32_t)tmp[4 * i] | (uint32_t)tmp[4 * i + 1] << 8 | (uint32_t)tmp[4 * i + 2] << 16 |
             (uint32_t)tmp[4 * i + 3] << 24;
  }
  static std::array<uint8_t, 32> to_bytes(const uint32_t out[16]) {
    std::array<uint8_t, 32> r;
    for (int i = 0; i < 8; ++i)
      for (int j = 0; j < 4; ++j) r[4 * i + j] = (uint8_t)(out[i] >> (8 * j));
    return r;
  }
  void reset_chunk(uint64_t counter) {
    memcpy(cv_, BLAKE3_IV, sizeof(cv_));
    blen_ = 0; chunk_bytes_ = 0; blocks_compressed_ = 0; chunk_counter_ = counter;
  }
  void compress_block_into_cv() {
    uint32_t w[16], out[16];
    load_block(block_, 64, w);
    uint32_t flags = blocks_compressed_ == 0 ? CHUNK_START : 0;
    blake3_compress(cv_, w, chunk_counter_, 64, flags, out);
    memcpy(cv_, out, 32);
    blocks_compressed_++;
    blen_ = 0;
  }
  void chunk_output_cv(uint32_t cv[8]) const {
    uint32_t w[16], out[16];
    load_block(block_, blen_, w);
    uint32_t flags = (blocks_compressed_ == 0 ? CHUNK_START : 0) | CHUNK_END;
    blake3_compress(cv_, w, chunk_counter_, blen_, flags, out);
    memcpy(cv, out, 32);
  }
  void push_chunk_cv(const uint32_t cv[8], uint64_t chunk_index) {
    // merge completed subtrees: number of merges = trailing zeros of (chunk_index + 1)
    std::array<uint32_t, 8> cur;
    memcpy(cur.data(), cv, 32);
    uint64_t total = chunk_index + 1;
    while ((total & 1) == 0) {
      uint32_t pw[16], out[16];
      memcpy(pw, stack_.back().data(), 32);
      memcpy(pw + 8, cur.data(), 32);
      stack_.pop_back();
      blake3_compress(BLAKE3_IV, pw, 0, 64, PARENT, out);
      memcpy(cur.data(), out, 32);
      total >>= 1;
    }
    stack_.push_back(cur);
  }
};

inline std::string to_hex(const uint8_t* p, size_t n) {
  static const char* d = "0123456789abcdef";
  std::string s;
  for (size_t i = 0; i < n; ++i) { s += d[p[i] >> 4]; s += d[p[i] & 15]; }
  return s;
}

}  // namespace flock
