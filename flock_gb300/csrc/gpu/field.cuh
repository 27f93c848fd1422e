// Device arithmetic in GF(2^128) (x^128 + x^7 + x^2 + x + 1, lo = x^0..x^63) and
// GF(2^256) = F128[u]/(u^2 + u + x^-1), the fields of the prove_fast path
// (crates/flock-core/src/field/gf2_128.rs, gf2_256.rs).
//
// sm_103a has no carry-less multiply instruction. A 32x32 -> 64 carry-less product is
// formed from sixteen 32x32 -> 64 integer multiplies of operands thinned to every
// fourth bit ("holes"): within one residue class mod 4 each product column receives at
// most 8 partial products, so no carry reaches the next bit of the same class and the
// class bits of the integer product are the GF(2) sums (pairs of products whose columns
// stay below 16 are summed as integers, clmul32_classes). The four classes are masked
// and merged. Two Karatsuba levels build the 128 x 128 product from nine such products,
// followed by the shift-and-fold reduction.
//
// The thinned-operand ("holes") carry-less multiply is a published constant-time
// technique: Thomas Pornin's BearSSL uses it for GHASH on CPUs without a carry-less
// multiply instruction (ghash_ctmul32.c / ghash_ctmul64.c, with a write-up in BearSSL's
// "Constant-Time Mul" notes). The form here — 32x32 -> 64 products from mul.wide/mad.wide,
// same-class pairs summed in the multiply's addend, two Karatsuba levels — is this
// library's own arrangement of it for the GPU's integer multiply pipe.
#pragma once
#include <cstdint>

namespace flock {
namespace gpu {

struct __align__(16) F128d {
  uint64_t lo, hi;
};
struct __align__(16) F256d {
  F128d c0, c1;
};

__host__ __device__ __forceinline__ F128d f128(uint64_t lo, uint64_t hi) { F128d r; r.lo = lo; r.hi = hi; return r; }
__host__ __device__ __forceinline__ F128d f128_zero() { return f128(0, 0); }
__host__ __device__ __forceinline__ F128d f128_one() { return f128(1, 0); }
__host__ __device__ __forceinline__ F128d operator+(F128d a, F128d b) { return f128(a.lo ^ b.lo, a.hi ^ b.hi); }
__host__ __device__ __forceinline__ F128d& operator+=(F128d& a, F128d b) { a.lo ^= b.lo; a.hi ^= b.hi; return a; }
__host__ __device__ __forceinline__ bool is_zero(F128d a) { return (a.lo | a.hi) == 0; }

// 32 x 32 -> 64 integer product, and the same plus a 64-bit addend. Written as PTX
// mul.wide / mad.wide: the C++ form (uint64_t)a * (uint64_t)b compiles to a wide multiply
// plus an extra add on the same multiply pipe, which costs the GF(2^128) product ~14%.
__device__ __forceinline__ uint64_t mulw(uint32_t a, uint32_t b) {
  uint64_t r;
  asm("mul.wide.u32 %0, %1, %2;" : "=l"(r) : "r"(a), "r"(b));
  return r;
}
__device__ __forceinline__ uint64_t madw(uint32_t a, uint32_t b, uint64_t c) {
  uint64_t r;
  asm("mad.wide.u32 %0, %1, %2, %3;" : "=l"(r) : "r"(a), "r"(b), "l"(c));
  return r;
}

// The carry-less product from the operands' residue classes: class c of the result
// collects the four products x_i y_j with i + j = c (mod 4). A product's column p holds
// g(u) = #{s + t = u : 0 <= s, t <= 7} partial products, u = (p - i - j) / 4, at most 8.
// Two products of one class whose index sums differ by 4 peak one column apart, so their
// integer sum holds at most g(u) + g(u - 1) <= 15 per column: still no carry into the
// next column of the class. Such pairs are added (in the multiply's addend) instead of
// XORed, which moves work from the logic pipe to the multiply pipe.
__device__ __forceinline__ uint64_t clmul32_classes(uint32_t x0, uint32_t x1, uint32_t x2, uint32_t x3, uint32_t y0,
                                                    uint32_t y1, uint32_t y2, uint32_t y3) {
  const uint64_t z0 = madw(x0, y0, mulw(x1, y3)) ^ mulw(x2, y2) ^ mulw(x3, y1);
  const uint64_t z1 = madw(x0, y1, mulw(x2, y3)) ^ madw(x1, y0, mulw(x3, y2));
  const uint64_t z2 = madw(x0, y2, mulw(x3, y3)) ^ mulw(x1, y1) ^ mulw(x2, y0);
  const uint64_t z3 = mulw(x0, y3) ^ mulw(x1, y2) ^ mulw(x2, y1) ^ mulw(x3, y0);
  const uint64_t M0 = 0x1111111111111111ull, M1 = 0x2222222222222222ull, M2 = 0x4444444444444444ull,
                 M3 = 0x8888888888888888ull;
  return (z0 & M0) | (z1 & M1) | (z2 & M2) | (z3 & M3);
}

// 32 x 32 -> 64 carry-less product.
__device__ __forceinline__ uint64_t clmul32(uint32_t x, uint32_t y) {
  const uint32_t m0 = 0x11111111u, m1 = 0x22222222u, m2 = 0x44444444u, m3 = 0x88888888u;
  uint32_t x0 = x & m0, x1 = x & m1, x2 = x & m2, x3 = x & m3;
  uint32_t y0 = y & m0, y1 = y & m1, y2 = y & m2, y3 = y & m3;
  return clmul32_classes(x0, x1, x2, x3, y0, y1, y2, y3);
}

// 64 x 64 -> 128 carry-less product (Karatsuba over 32-bit halves).
__device__ __forceinline__ void clmul64(uint64_t a, uint64_t b, uint64_t& lo, uint64_t& hi) {
  uint32_t a0 = (uint32_t)a, a1 = (uint32_t)(a >> 32), b0 = (uint32_t)b, b1 = (uint32_t)(b >> 32);
  uint64_t l = clmul32(a0, b0), h = clmul32(a1, b1), m = clmul32(a0 ^ a1, b0 ^ b1) ^ l ^ h;
  lo = l ^ (m << 32);
  hi = h ^ (m >> 32);
}

__device__ __forceinline__ F128d ghash_reduce(uint64_t r0, uint64_t r1, uint64_t r2, uint64_t r3) {
  uint64_t t_lo = r2 ^ (r2 << 1) ^ (r2 << 2) ^ (r2 << 7);
  uint64_t t_hi = r3 ^ ((r3 << 1) | (r2 >> 63)) ^ ((r3 << 2) | (r2 >> 62)) ^ ((r3 << 7) | (r2 >> 57));
  uint64_t ov = (r3 >> 63) ^ (r3 >> 62) ^ (r3 >> 57);
  uint64_t corr = ov ^ (ov << 1) ^ (ov << 2) ^ (ov << 7);
  return f128(r0 ^ t_lo ^ corr, r1 ^ t_hi);
}

__device__ __forceinline__ F128d mul(F128d a, F128d b) {
  uint64_t l0, l1, h0, h1, m0, m1;
  clmul64(a.lo, b.lo, l0, l1);
  clmul64(a.hi, b.hi, h0, h1);
  clmul64(a.lo ^ a.hi, b.lo ^ b.hi, m0, m1);
  m0 ^= l0 ^ h0;
  m1 ^= l1 ^ h1;
  return ghash_reduce(l0, l1 ^ m0, h0 ^ m1, h1);
}
__device__ __forceinline__ F128d operator*(F128d a, F128d b) { return mul(a, b); }
// The same product out of line: kernels that hold several products in flight per
// iteration (the sumcheck folds) spill or lose occupancy when every product is inlined;
// a call keeps one product's temporaries live at a time.
__device__ __noinline__ static F128d mul_call(F128d a, F128d b) { return mul(a, b); }

// One factor of mul() in the form clmul32 consumes it: the nine Karatsuba words (for each
// of b.lo, b.hi and b.lo ^ b.hi: its low half, its high half and their sum), each thinned
// to its four residue classes. Multiplying many values by one constant (an NTT twiddle, a
// fold challenge) from this form skips the constant's 41 splitting and pre-add operations
// per product; the products are bit-identical to mul().
struct __align__(16) F128split {
  uint32_t w[9][4];
};
__device__ __forceinline__ void split_classes(uint32_t y, uint32_t* o) {
  o[0] = y & 0x11111111u;
  o[1] = y & 0x22222222u;
  o[2] = y & 0x44444444u;
  o[3] = y & 0x88888888u;
}
__device__ __forceinline__ F128split split_factor(F128d b) {
  F128split s;
  const uint64_t hl[3] = {b.lo, b.hi, b.lo ^ b.hi};
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    const uint32_t y0 = (uint32_t)hl[q], y1 = (uint32_t)(hl[q] >> 32);
    split_classes(y0, s.w[3 * q]);
    split_classes(y1, s.w[3 * q + 1]);
    split_classes(y0 ^ y1, s.w[3 * q + 2]);
  }
  return s;
}
__device__ __forceinline__ uint64_t clmul32_split(uint32_t x, const uint32_t* y) {
  const uint32_t x0 = x & 0x11111111u, x1 = x & 0x22222222u, x2 = x & 0x44444444u, x3 = x & 0x88888888u;
  return clmul32_classes(x0, x1, x2, x3, y[0], y[1], y[2], y[3]);
}
__device__ __forceinline__ void clmul64_split(uint64_t a, const uint32_t (*y)[4], uint64_t& lo, uint64_t& hi) {
  const uint32_t a0 = (uint32_t)a, a1 = (uint32_t)(a >> 32);
  uint64_t l = clmul32_split(a0, y[0]), h = clmul32_split(a1, y[1]), m = clmul32_split(a0 ^ a1, y[2]) ^ l ^ h;
  lo = l ^ (m << 32);
  hi = h ^ (m >> 32);
}
// a * b with b given as split_factor(b).
__device__ __forceinline__ F128d mul_split(F128d a, const F128split& b) {
  uint64_t l0, l1, h0, h1, m0, m1;
  clmul64_split(a.lo, b.w, l0, l1);
  clmul64_split(a.hi, b.w + 3, h0, h1);
  clmul64_split(a.lo ^ a.hi, b.w + 6, m0, m1);
  m0 ^= l0 ^ h0;
  m1 ^= l1 ^ h1;
  return ghash_reduce(l0, l1 ^ m0, h0 ^ m1, h1);
}

// Out-of-line mul_split (see mul_call); b is typically staged once per block in shared
// memory.
__device__ __noinline__ static F128d mul_split_call(F128d a, const F128split* b) { return mul_split(a, *b); }

__device__ __forceinline__ F128d mul_by_x(F128d z) {
  uint64_t mask = 0ull - (z.hi >> 63);
  return f128((z.lo << 1) ^ (0x87ull & mask), (z.hi << 1) | (z.lo >> 63));
}

// ---- products by one constant from byte tables in shared memory
// T[256 k + v] = c * (v x^(8k)) for the 16 byte positions k of the other factor (k < 8:
// bytes of lo, k >= 8: bytes of hi). By linearity c * a is the XOR of T[256 k + a_k] over
// the bytes a_k of a: 16 table lookups and XORs, no multiply and no reduction. The lookups
// run on the load/store pipe while integer-multiply products run on the FMA pipe, so a
// kernel that forms its products by a round constant this way and its products of two
// variables by mul() keeps both pipes busy (measured on GB300: 5.9e10 table products/s
// alone, 8.1e10 products/s for an even mix, against 4.8e10 for mul_split alone).
constexpr uint32_t BYTE_TABLE_ENTRIES = 16 * 256;
// Shared-memory F128 entries build_byte_table needs: the table, then 512 nibble-table and
// 128 power entries of scratch.
constexpr uint32_t BYTE_TABLE_SMEM_ENTRIES = BYTE_TABLE_ENTRIES + 512 + 128;

// The same tables serve any GF(2)-linear map f of GF(2^128): T[256 k + v] = f(v x^(8k)),
// built from the 128 images E[i] = f(x^i).
__device__ __forceinline__ F128d unit_power(uint32_t i) { return i < 64 ? f128(1ull << i, 0) : f128(0, 1ull << (i - 64)); }
// Every thread of the block calls this; T has BYTE_TABLE_SMEM_ENTRIES entries and its
// scratch already holds the images (byte_table_images(T)[i] = f(x^i), written before a
// block barrier). The table is complete when it returns. Nibble tables N[4-bit position
// j][u] = sum of u's bits times E[4j + bit], then each byte entry as the XOR of its two
// nibble entries.
__device__ __forceinline__ F128d* byte_table_images(F128d* T) { return T + BYTE_TABLE_ENTRIES + 512; }
__device__ __forceinline__ void byte_table_from_images(F128d* T) {
  F128d* N = T + BYTE_TABLE_ENTRIES;
  const F128d* E = byte_table_images(T);
  for (uint32_t e = threadIdx.x; e < 512; e += blockDim.x) {
    const uint32_t j = e >> 4, u = e & 15;
    F128d acc = f128_zero();
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const uint64_t m = 0ull - (uint64_t)((u >> b) & 1);
      const F128d p = E[4 * j + b];
      acc.lo ^= p.lo & m;
      acc.hi ^= p.hi & m;
    }
    N[e] = acc;
  }
  __syncthreads();
  for (uint32_t e = threadIdx.x; e < BYTE_TABLE_ENTRIES; e += blockDim.x) {
    const uint32_t k = e >> 8, v = e & 255;
    T[e] = N[32 * k + (v & 15)] + N[32 * k + 16 + (v >> 4)];
  }
  __syncthreads();
}
// The tables of the product by c: E[i] = c x^i (128 products), then as above.
__device__ __forceinline__ void build_byte_table(F128d c, F128d* T) {
  F128d* E = byte_table_images(T);
  for (uint32_t i = threadIdx.x; i < 128; i += blockDim.x) E[i] = mul_call(c, unit_power(i));
  __syncthreads();
  byte_table_from_images(T);
}
__device__ __forceinline__ F128d mul_table(F128d a, const F128d* __restrict__ T) {
  F128d acc = f128_zero();
#pragma unroll
  for (int k = 0; k < 8; ++k) acc += T[256 * k + ((a.lo >> (8 * k)) & 255)];
#pragma unroll
  for (int k = 0; k < 8; ++k) acc += T[256 * (8 + k) + ((a.hi >> (8 * k)) & 255)];
  return acc;
}
__device__ __forceinline__ F128d mul_by_x_inv(F128d z) {
  uint64_t mask = 0ull - (z.lo & 1);
  return f128(((z.lo >> 1) | (z.hi << 63)) ^ (0x43ull & mask), (z.hi >> 1) ^ ((1ull << 63) & mask));
}

// ---- F256
__host__ __device__ __forceinline__ F256d f256(F128d a, F128d b) { F256d r; r.c0 = a; r.c1 = b; return r; }
__host__ __device__ __forceinline__ F256d f256_base(F128d a) { return f256(a, f128_zero()); }
__host__ __device__ __forceinline__ F256d operator+(F256d a, F256d b) { return f256(a.c0 + b.c0, a.c1 + b.c1); }
__host__ __device__ __forceinline__ F256d& operator+=(F256d& a, F256d b) { a.c0 += b.c0; a.c1 += b.c1; return a; }
__device__ __forceinline__ F256d operator*(F256d a, F256d b) {
  F128d p0 = a.c0 * b.c0, p1 = a.c1 * b.c1, p2 = (a.c0 + a.c1) * (b.c0 + b.c1);
  return f256(p0 + mul_by_x_inv(p1), p2 + p0);
}
__device__ __forceinline__ F256d operator*(F256d a, F128d b) { return f256(a.c0 * b, a.c1 * b); }
// Out-of-line F256 product (see mul_call).
__device__ __noinline__ static F256d f256_mul_call(F256d a, F256d b) { return a * b; }

// ---- warp / block XOR reductions
__device__ __forceinline__ F128d warp_xor(F128d v) {
  for (int o = 16; o > 0; o >>= 1) {
    v.lo ^= __shfl_xor_sync(0xffffffffu, v.lo, o);
    v.hi ^= __shfl_xor_sync(0xffffffffu, v.hi, o);
  }
  return v;
}

}  // namespace gpu
}  // namespace flock
