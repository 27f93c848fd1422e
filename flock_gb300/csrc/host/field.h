// Host-side finite-field arithmetic for the prove_fast path.
//
// F128  : GF(2^128), polynomial basis modulo x^128 + x^7 + x^2 + x + 1,
//         `lo` = coefficients of x^0..x^63, `hi` = x^64..x^127
//         (crates/flock-core/src/field/gf2_128.rs:1-30).
// F256  : F128[u] / (u^2 + u + x^-1)   (crates/flock-core/src/field/gf2_256.rs:1-120).
// GF8   : GF(2^8) with the AES polynomial 0x11B (crates/flock-core/src/field/gf2_8.rs).
// phi8  : the field embedding GF(2^8) -> F128. A homomorphism of fields is fixed by the
//         image of the generator x = 0x02; the image used by the reference table
//         (crates/flock-core/src/field/phi8.rs:19-30, entry 2) is PHI8_OF_X below and
//         every other entry is generated here as a sum of its powers.
//
// Portable C++: the same code builds on x86_64 and aarch64 hosts and gives the same bits.
// On aarch64 hosts built with the AES extension (the build passes -march=armv8-a+crypto
// there) host-compiler translation units take the 64x64 carry-less product from the PMULL
// instruction through the ACLE intrinsic vmull_p64; everywhere else (and in nvcc
// translation units, whose front end does not parse arm_neon.h) it is the
// integer-multiply form below.
#pragma once
#include <cstdint>
#include <cstring>
#include <vector>
#include <array>
#if defined(__aarch64__) && defined(__ARM_FEATURE_AES) && !defined(__CUDACC__)
#include <arm_neon.h>
#define FLOCK_HOST_PMULL 1
#endif

namespace flock {

struct F128 {
  uint64_t lo = 0, hi = 0;
  constexpr F128() = default;
  constexpr F128(uint64_t l, uint64_t h) : lo(l), hi(h) {}
  static constexpr F128 zero() { return F128(0, 0); }
  static constexpr F128 one() { return F128(1, 0); }
  bool is_zero() const { return (lo | hi) == 0; }
  bool operator==(const F128& o) const { return lo == o.lo && hi == o.hi; }
  bool operator!=(const F128& o) const { return !(*this == o); }
  F128 operator+(const F128& o) const { return F128(lo ^ o.lo, hi ^ o.hi); }
  F128& operator+=(const F128& o) { lo ^= o.lo; hi ^= o.hi; return *this; }
};
static_assert(sizeof(F128) == 16, "F128 is two little-endian u64 words");

// 32x32 -> 64 carry-less product from sixteen 64-bit integer products of operands thinned
// to every fourth bit: within one residue class mod 4 a product column collects at most 8
// partial products, so no carry reaches the next bit of the same class, and the class bits
// of the integer products are the GF(2) sums. Portable (plain 64-bit multiplies).
inline uint64_t clmul32(uint32_t x, uint32_t y) {
  const uint32_t m0 = 0x11111111u, m1 = 0x22222222u, m2 = 0x44444444u, m3 = 0x88888888u;
  const uint64_t x0 = x & m0, x1 = x & m1, x2 = x & m2, x3 = x & m3;
  const uint64_t y0 = y & m0, y1 = y & m1, y2 = y & m2, y3 = y & m3;
  const uint64_t z0 = (x0 * y0) ^ (x1 * y3) ^ (x2 * y2) ^ (x3 * y1);
  const uint64_t z1 = (x0 * y1) ^ (x1 * y0) ^ (x2 * y3) ^ (x3 * y2);
  const uint64_t z2 = (x0 * y2) ^ (x1 * y1) ^ (x2 * y0) ^ (x3 * y3);
  const uint64_t z3 = (x0 * y3) ^ (x1 * y2) ^ (x2 * y1) ^ (x3 * y0);
  return (z0 & 0x1111111111111111ull) | (z1 & 0x2222222222222222ull) | (z2 & 0x4444444444444444ull) |
         (z3 & 0x8888888888888888ull);
}
// 64x64 -> 128 carry-less product (Karatsuba over 32-bit halves, or PMULL).
inline void clmul64(uint64_t a, uint64_t b, uint64_t& rlo, uint64_t& rhi) {
#ifdef FLOCK_HOST_PMULL
  const uint64x2_t v = vreinterpretq_u64_p128(vmull_p64((poly64_t)a, (poly64_t)b));
  rlo = vgetq_lane_u64(v, 0);
  rhi = vgetq_lane_u64(v, 1);
#else
  const uint32_t a0 = (uint32_t)a, a1 = (uint32_t)(a >> 32), b0 = (uint32_t)b, b1 = (uint32_t)(b >> 32);
  const uint64_t l = clmul32(a0, b0), h = clmul32(a1, b1), m = clmul32(a0 ^ a1, b0 ^ b1) ^ l ^ h;
  rlo = l ^ (m << 32);
  rhi = h ^ (m >> 32);
#endif
}

// Reduce a 256-bit product (r0 lowest) modulo x^128 + x^7 + x^2 + x + 1.
// x^128 = x^7 + x^2 + x + 1, so the upper half U folds as U ^ U<<1 ^ U<<2 ^ U<<7
// and the bits pushed past x^127 by those shifts fold once more.
inline F128 ghash_reduce(uint64_t r0, uint64_t r1, uint64_t r2, uint64_t r3) {
  uint64_t t_lo = r2 ^ (r2 << 1) ^ (r2 << 2) ^ (r2 << 7);
  uint64_t t_hi = r3 ^ ((r3 << 1) | (r2 >> 63)) ^ ((r3 << 2) | (r2 >> 62)) ^ ((r3 << 7) | (r2 >> 57));
  uint64_t ov = (r3 >> 63) ^ (r3 >> 62) ^ (r3 >> 57);
  uint64_t corr = ov ^ (ov << 1) ^ (ov << 2) ^ (ov << 7);
  return F128(r0 ^ t_lo ^ corr, r1 ^ t_hi);
}

static inline F128 mul_impl(const F128& a, const F128& b) {
  uint64_t l0, l1, h0, h1, m0, m1;
  clmul64(a.lo, b.lo, l0, l1);
  clmul64(a.hi, b.hi, h0, h1);
  clmul64(a.lo ^ a.hi, b.lo ^ b.hi, m0, m1);
  m0 ^= l0 ^ h0;
  m1 ^= l1 ^ h1;
  return ghash_reduce(l0, l1 ^ m0, h0 ^ m1, h1);
}
#if defined(__CUDACC__)
// Host code that nvcc compiles cannot use the crypto intrinsics (the arm_neon.h route is
// closed to it): its products go to host_accel.cc, which the host compiler builds with the
// target's crypto extensions (PMULL on aarch64).
F128 mul_host_accel(const F128& a, const F128& b);
inline F128 mul(const F128& a, const F128& b) { return mul_host_accel(a, b); }
#else
inline F128 mul(const F128& a, const F128& b) { return mul_impl(a, b); }
#endif
inline F128 operator*(const F128& a, const F128& b) { return mul(a, b); }
inline F128& operator*=(F128& a, const F128& b) { a = mul(a, b); return a; }
inline F128 sqr(const F128& a) { return mul(a, a); }

// Multiplicative inverse by Fermat: a^(2^128 - 2).
inline F128 inv(const F128& a) {
  F128 r = F128::one();
  F128 cur = a * a;
  for (int i = 1; i < 128; ++i) { r = r * cur; cur = cur * cur; }
  return r;
}

inline F128 mul_by_x(const F128& z) {
  uint64_t mask = 0ull - (z.hi >> 63);
  return F128((z.lo << 1) ^ (0x87ull & mask), (z.hi << 1) | (z.lo >> 63));
}
inline F128 mul_by_x_inv(const F128& z) {
  uint64_t mask = 0ull - (z.lo & 1);
  return F128(((z.lo >> 1) | (z.hi << 63)) ^ (0x43ull & mask), (z.hi >> 1) ^ ((1ull << 63) & mask));
}

// ---- F256 = F128[u]/(u^2 + u + x^-1) ----------------------------------------------
struct F256 {
  F128 c0, c1;
  constexpr F256() = default;
  constexpr F256(F128 a, F128 b) : c0(a), c1(b) {}
  explicit constexpr F256(F128 a) : c0(a), c1() {}
  static constexpr F256 zero() { return F256(); }
  static constexpr F256 one() { return F256(F128::one(), F128()); }
  static constexpr F256 u() { return F256(F128(), F128::one()); }
  bool is_zero() const { return c0.is_zero() && c1.is_zero(); }
  bool operator==(const F256& o) const { return c0 == o.c0 && c1 == o.c1; }
  F256 operator+(const F256& o) const { return F256(c0 + o.c0, c1 + o.c1); }
  F256& operator+=(const F256& o) { c0 += o.c0; c1 += o.c1; return *this; }
};
inline F256 operator*(const F256& a, const F256& b) {
  F128 p0 = a.c0 * b.c0, p1 = a.c1 * b.c1, p2 = (a.c0 + a.c1) * (b.c0 + b.c1);
  return F256(p0 + mul_by_x_inv(p1), p2 + p0);
}
inline F256 operator*(const F256& a, const F128& b) { return F256(a.c0 * b, a.c1 * b); }
inline F256 operator*(const F128& b, const F256& a) { return F256(a.c0 * b, a.c1 * b); }

// ---- GF(2^8), AES polynomial ---------------------------------------------------------
inline uint8_t gf8_mul(uint8_t a, uint8_t b) {
  uint16_t p = 0;
  for (int i = 0; i < 8; ++i)
    if ((b >> i) & 1) p ^= (uint16_t)a << i;
  for (int i = 15; i >= 8; --i)
    if ((p >> i) & 1) p ^= (uint16_t)0x11B << (i - 8);
  return (uint8_t)p;
}
inline uint8_t gf8_inv(uint8_t a) {
  // a^254
  uint8_t r = 1, base = a;
  unsigned e = 254;
  while (e) { if (e & 1) r = gf8_mul(r, base); base = gf8_mul(base, base); e >>= 1; }
  return r;
}

// Image of the GF(2^8) element x (0x02) under the embedding (phi8.rs:27-30).
constexpr F128 PHI8_OF_X = F128(0x6b8330483c2e9849ull, 0x0dcb364640a222feull);

// phi8[v] = sum over set bits i of v of PHI8_OF_X^i (a ring homomorphism is additive).
inline const std::array<F128, 256>& phi8_table() {
  static const std::array<F128, 256> t = [] {
    std::array<F128, 256> tab{};
    F128 pw[8];
    pw[0] = F128::one();
    for (int i = 1; i < 8; ++i) pw[i] = pw[i - 1] * PHI8_OF_X;
    for (int v = 0; v < 256; ++v) {
      F128 acc;
      for (int i = 0; i < 8; ++i) if ((v >> i) & 1) acc += pw[i];
      tab[v] = acc;
    }
    return tab;
  }();
  return t;
}
inline F128 phi8(uint8_t v) { return phi8_table()[v]; }

// ---- eq tables -------------------------------------------------------------------
// out[i] = prod_j eq(point[j], bit_j(i)), eq(r, 0) = 1 + r, eq(r, 1) = r.
inline std::vector<F128> build_eq(const std::vector<F128>& point, F128 scale = F128::one()) {
  std::vector<F128> out(size_t(1) << point.size());
  out[0] = scale;
  for (size_t j = 0; j < point.size(); ++j) {
    size_t len = size_t(1) << j;
    F128 r = point[j], r1 = r + F128::one();
    for (size_t i = 0; i < len; ++i) {
      F128 v = out[i];
      out[i + len] = v * r;
      out[i] = v * r1;
    }
  }
  return out;
}
inline std::vector<F256> build_eq256(const std::vector<F256>& point) {
  std::vector<F256> out(size_t(1) << point.size());
  out[0] = F256::one();
  for (size_t j = 0; j < point.size(); ++j) {
    size_t len = size_t(1) << j;
    F256 r = point[j], r1 = r + F256::one();
    for (size_t i = 0; i < len; ++i) {
      F256 v = out[i];
      out[i + len] = v * r;
      out[i] = v * r1;
    }
  }
  return out;
}
inline F128 eq_eval(const std::vector<F128>& a, const std::vector<F128>& b) {
  F128 acc = F128::one();
  for (size_t i = 0; i < a.size(); ++i) acc = acc * (F128::one() + a[i] + b[i]);
  return acc;
}

}  // namespace flock
