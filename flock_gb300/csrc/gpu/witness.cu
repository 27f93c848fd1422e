// Witness generation on the device: one thread per hash instance writes its block's
// z, a = A_0 z and b = B_0 z bits straight into the batch-major layout
// (word (c << nu) + instance holds bits [128 c, 128 c + 128) of the instance's block;
// crates/flock-prover/src/r1cs_hashes/common.rs:456-585). Threads of a warp are
// consecutive instances, so every 16-byte chunk store of a warp is one coalesced
// 512-byte line. Fields are emitted in increasing bit position per region and each
// region streams through a 128-bit accumulator, so every word is written exactly once
// (gaps between fields are written as zeros).
//
// Per-hash field semantics follow build_group_batch_major:
//   BLAKE3   blake3.rs:1929-2040      SHA-256  sha2.rs:1743-1850      Keccak  keccak.rs:565-640
#include "kernels.h"
#include <mutex>
#include "../host/r1cs_blake3.h"
#include "../host/r1cs_sha2.h"
#include "../host/r1cs_keccak.h"

namespace flock {
namespace gpu {

// Streams fields of one region (increasing bit positions) for z, a and b.
struct ChunkWriter {
  uint4* z; uint4* a; uint4* b;     // arrays as 128-bit words
  uint32_t nu, inst;                // word index = (chunk << nu) + inst
  int32_t cur;                      // current chunk, -1 = none
  uint64_t z0, z1, a0, a1, b0, b1;

  __device__ void init(uint4* zz, uint4* aa, uint4* bb, uint32_t nu_, uint32_t inst_, uint32_t first_chunk) {
    z = zz; a = aa; b = bb; nu = nu_; inst = inst_;
    cur = (int32_t)first_chunk;
    z0 = z1 = a0 = a1 = b0 = b1 = 0;
  }
  __device__ __forceinline__ void store(uint32_t chunk, uint64_t zl, uint64_t zh, uint64_t al, uint64_t ah,
                                        uint64_t bl, uint64_t bh) {
    size_t wi = ((size_t)chunk << nu) + inst;
    z[wi] = make_uint4((uint32_t)zl, (uint32_t)(zl >> 32), (uint32_t)zh, (uint32_t)(zh >> 32));
    a[wi] = make_uint4((uint32_t)al, (uint32_t)(al >> 32), (uint32_t)ah, (uint32_t)(ah >> 32));
    b[wi] = make_uint4((uint32_t)bl, (uint32_t)(bl >> 32), (uint32_t)bh, (uint32_t)(bh >> 32));
  }
  __device__ __forceinline__ void advance_to(uint32_t chunk) {
    while ((uint32_t)cur < chunk) {
      store((uint32_t)cur, z0, z1, a0, a1, b0, b1);
      z0 = z1 = a0 = a1 = b0 = b1 = 0;
      cur++;
    }
  }
  // OR `n`-bit (n <= 32) values into bit position `pos`.
  __device__ __forceinline__ void put(uint32_t pos, uint32_t zv, uint32_t av, uint32_t bv) {
    uint32_t chunk = pos >> 7, off = pos & 127;
    advance_to(chunk);
    uint64_t zz = zv, aa = av, bb = bv;
    if (off < 64) {
      z0 |= zz << off; a0 |= aa << off; b0 |= bb << off;
      if (off > 32) {
        uint32_t sh = 64 - off;
        z1 |= zz >> sh; a1 |= aa >> sh; b1 |= bb >> sh;
      }
    } else {
      uint32_t o = off - 64;
      z1 |= zz << o; a1 |= aa << o; b1 |= bb << o;
      if (o > 32) {
        // Bits past the chunk go to the next one. A field narrower than 32 bits may
        // leave nothing to spill; the chunk then stays open for the fields after it.
        uint32_t sh = 64 - o;
        uint64_t sz = zz >> sh, sa = aa >> sh, sb = bb >> sh;
        if (sz | sa | sb) {
          advance_to(chunk + 1);
          z0 |= sz; a0 |= sa; b0 |= sb;
        }
      }
    }
  }
  // Flush through `end_chunk` (exclusive).
  __device__ __forceinline__ void finish(uint32_t end_chunk) { advance_to(end_chunk); }
};

__device__ __forceinline__ uint32_t rotr32d(uint32_t x, int n) { return __funnelshift_r(x, x, n); }

struct Add3 { uint32_t sum, m0, m1, m2, r0, r1, r2; };
__device__ __forceinline__ Add3 fadd3(uint32_t x, uint32_t y, uint32_t m) {
  uint32_t xm = x ^ m, ym = y ^ m, w = xm & ym, p = x ^ y ^ m, bw = (w ^ m) << 1;
  uint32_t sum = p + bw, cin = sum ^ p ^ bw, rl = p ^ cin, rr = bw ^ cin;
  Add3 o;
  o.sum = sum;
  o.m0 = xm & 0x7FFFFFFFu; o.m1 = ym & 0x7FFFFFFFu; o.m2 = w & 0x7FFFFFFFu;
  o.r0 = (rl >> 1) & 0x3FFFFFFFu; o.r1 = (rr >> 1) & 0x3FFFFFFFu; o.r2 = ((rl & rr) >> 1) & 0x3FFFFFFFu;
  return o;
}
struct Add2 { uint32_t sum, l, r, c; };
__device__ __forceinline__ Add2 add2(uint32_t x, uint32_t y) {
  uint32_t s = x + y, cin = s ^ x ^ y, l = (x ^ cin) & 0x7FFFFFFFu, r = (y ^ cin) & 0x7FFFFFFFu;
  Add2 o; o.sum = s; o.l = l; o.r = r; o.c = l & r;
  return o;
}

// ------------------------------------------------------------------------ BLAKE3
__constant__ uint32_t B3_IV_C[8] = {0x6a09e667, 0xbb67ae85, 0x3c6ef372, 0xa54ff53a,
                                    0x510e527f, 0x9b05688c, 0x1f83d9ab, 0x5be0cd19};
__constant__ uint8_t B3_MSG_IDX[7][16];   // per round, the permuted message index of slot i
__constant__ uint32_t B3_GBASE[57];
__constant__ int8_t B3_LANES[8][4] = {{0, 4, 8, 12}, {1, 5, 9, 13}, {2, 6, 10, 14}, {3, 7, 11, 15},
                                      {0, 5, 10, 15}, {1, 6, 11, 12}, {2, 7, 8, 13}, {3, 4, 9, 14}};

__global__ void witness_blake3_kernel(const b3r1cs::Compression* __restrict__ in, uint32_t n_inst, uint32_t nu,
                                      uint4* z, uint4* a, uint4* b, uint32_t used_chunks) {
  uint32_t o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= n_inst) return;
  b3r1cs::Compression c = in[o];
  // Final state first (the output words sit before the G blocks).
  uint32_t s[16];
  for (int i = 0; i < 8; ++i) s[i] = c.cv[i];
  for (int i = 0; i < 4; ++i) s[8 + i] = B3_IV_C[i];
  uint32_t tlo = (uint32_t)c.counter, thi = (uint32_t)(c.counter >> 32);
  s[12] = tlo; s[13] = thi; s[14] = c.block_len; s[15] = c.flags;
  for (int r = 0; r < 7; ++r)
    for (int gi = 0; gi < 8; ++gi) {
      int la = B3_LANES[gi][0], lb = B3_LANES[gi][1], lc = B3_LANES[gi][2], ld = B3_LANES[gi][3];
      uint32_t mx = c.m[B3_MSG_IDX[r][2 * gi]], my = c.m[B3_MSG_IDX[r][2 * gi + 1]];
      s[la] = s[la] + s[lb] + mx; s[ld] = rotr32d(s[ld] ^ s[la], 16);
      s[lc] = s[lc] + s[ld];      s[lb] = rotr32d(s[lb] ^ s[lc], 12);
      s[la] = s[la] + s[lb] + my; s[ld] = rotr32d(s[ld] ^ s[la], 8);
      s[lc] = s[lc] + s[ld];      s[lb] = rotr32d(s[lb] ^ s[lc], 7);
    }
  ChunkWriter W;
  W.init(z, a, b, nu, o, 0);
  const uint32_t ONES = 0xFFFFFFFFu;
  for (int w = 0; w < 8; ++w) W.put(b3r1cs::CV_BASE + 32 * w, c.cv[w], c.cv[w], ONES);
  for (int w = 0; w < 8; ++w) { uint32_t v = s[w] ^ s[w + 8]; W.put(b3r1cs::OUT_LO_BASE + 32 * w, v, v, ONES); }
  for (int i = 0; i < 16; ++i) W.put(b3r1cs::M_BASE + 32 * i, c.m[i], c.m[i], ONES);
  W.put(b3r1cs::T_LO_BASE, tlo, tlo, ONES);
  W.put(b3r1cs::T_HI_BASE, thi, thi, ONES);
  W.put(b3r1cs::BLEN_BASE, c.block_len, c.block_len, ONES);
  W.put(b3r1cs::FLAGS_BASE, c.flags, c.flags, ONES);
  for (int w = 0; w < 8; ++w) { uint32_t v = s[w + 8] ^ c.cv[w]; W.put(b3r1cs::OUT_HI_BASE + 32 * w, v, v, ONES); }
  // G blocks with the witness products.
  for (int i = 0; i < 8; ++i) s[i] = c.cv[i];
  for (int i = 0; i < 4; ++i) s[8 + i] = B3_IV_C[i];
  s[12] = tlo; s[13] = thi; s[14] = c.block_len; s[15] = c.flags;
  for (int r = 0; r < 7; ++r)
    for (int gi = 0; gi < 8; ++gi) {
      int g = r * 8 + gi;
      int la = B3_LANES[gi][0], lb = B3_LANES[gi][1], lc = B3_LANES[gi][2], ld = B3_LANES[gi][3];
      uint32_t mx = c.m[B3_MSG_IDX[r][2 * gi]], my = c.m[B3_MSG_IDX[r][2 * gi + 1]];
      uint32_t gb = B3_GBASE[g];
      Add3 f1 = fadd3(s[la], s[lb], mx);
      W.put(gb, f1.m2, f1.m0, f1.m1);
      W.put(gb + 31, f1.r2, f1.r0, f1.r1);
      uint32_t d1 = rotr32d(s[ld] ^ f1.sum, 16);
      uint32_t c1;
      int c1rows;
      if (g < 4) {
        c1rows = g < 2 ? 30 : 29;
        int t = 31 - c1rows;
        uint32_t mask = (1u << c1rows) - 1;
        Add2 p = add2(B3_IV_C[g], d1);
        W.put(gb + 61, (p.c >> t) & mask, (p.l >> t) & mask, (p.r >> t) & mask);
        c1 = p.sum;
      } else {
        c1rows = 31;
        Add2 p = add2(s[lc], d1);
        W.put(gb + 61, p.c, p.l, p.r);
        c1 = p.sum;
      }
      uint32_t b1 = rotr32d(s[lb] ^ c1, 12);
      uint32_t om2 = 61 + c1rows;
      Add3 f2 = fadd3(f1.sum, b1, my);
      W.put(gb + om2, f2.m2, f2.m0, f2.m1);
      W.put(gb + om2 + 31, f2.r2, f2.r0, f2.r1);
      uint32_t d2 = rotr32d(d1 ^ f2.sum, 8);
      Add2 p2 = add2(c1, d2);
      W.put(gb + om2 + 61, p2.c, p2.l, p2.r);
      uint32_t bn = rotr32d(b1 ^ p2.sum, 7);
      s[la] = f2.sum; s[lb] = bn; s[lc] = p2.sum; s[ld] = d2;
    }
  W.put(b3r1cs::Z_CONST_POS, 1, 1, 1);
  W.finish(used_chunks);
}

// ------------------------------------------------------------------------ SHA-256
__constant__ uint32_t S2_K[64];
__constant__ uint32_t S2_ROUND_BASE[65];

__device__ __forceinline__ uint32_t bs0(uint32_t x) { return rotr32d(x, 2) ^ rotr32d(x, 13) ^ rotr32d(x, 22); }
__device__ __forceinline__ uint32_t bs1(uint32_t x) { return rotr32d(x, 6) ^ rotr32d(x, 11) ^ rotr32d(x, 25); }
__device__ __forceinline__ uint32_t ss0(uint32_t x) { return rotr32d(x, 7) ^ rotr32d(x, 18) ^ (x >> 3); }
__device__ __forceinline__ uint32_t ss1(uint32_t x) { return rotr32d(x, 17) ^ rotr32d(x, 19) ^ (x >> 10); }

struct Add4 { uint32_t sum, m1[3], m2[3], r[3]; };
__device__ __forceinline__ Add4 fadd4(uint32_t x, uint32_t y, uint32_t z, uint32_t w) {
  uint32_t xz = x ^ z, yz = y ^ z, w1 = xz & yz, p1 = x ^ y ^ z, b1 = (w1 ^ z) << 1;
  uint32_t pw = p1 ^ w, bw = b1 ^ w, w2 = pw & bw, p2 = p1 ^ b1 ^ w, b2 = (w2 ^ w) << 1;
  uint32_t sum = p2 + b2, cin = sum ^ p2 ^ b2, rl = p2 ^ cin, rr = b2 ^ cin;
  Add4 o;
  o.sum = sum;
  o.m1[0] = xz & 0x7FFFFFFFu; o.m1[1] = yz & 0x7FFFFFFFu; o.m1[2] = w1 & 0x7FFFFFFFu;
  o.m2[0] = pw & 0x7FFFFFFFu; o.m2[1] = bw & 0x7FFFFFFFu; o.m2[2] = w2 & 0x7FFFFFFFu;
  o.r[0] = (rl >> 1) & 0x3FFFFFFFu; o.r[1] = (rr >> 1) & 0x3FFFFFFFu; o.r[2] = ((rl & rr) >> 1) & 0x3FFFFFFFu;
  return o;
}

__global__ void witness_sha2_kernel(const s2r1cs::Compression* __restrict__ in, uint32_t n_inst, uint32_t nu,
                                    uint4* z, uint4* a, uint4* b, uint32_t used_chunks) {
  uint32_t o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= n_inst) return;
  s2r1cs::Compression c = in[o];
  const uint32_t ONES = 0xFFFFFFFFu;
  // Schedule, final state and output (the I/O region precedes everything else).
  uint32_t W[64];
  for (int i = 0; i < 16; ++i) W[i] = c.w[i];
  for (int t = 16; t < 64; ++t) W[t] = ss1(W[t - 2]) + W[t - 7] + ss0(W[t - 15]) + W[t - 16];
  uint32_t st[8];
  {
    uint32_t A = c.h[0], B = c.h[1], C = c.h[2], D = c.h[3], E = c.h[4], F = c.h[5], G = c.h[6], H = c.h[7];
    for (int r = 0; r < 64; ++r) {
      uint32_t t1 = H + bs1(E) + ((E & F) ^ (~E & G)) + S2_K[r] + W[r];
      uint32_t t2 = bs0(A) + ((A & B) ^ (A & C) ^ (B & C));
      H = G; G = F; F = E; E = D + t1; D = C; C = B; B = A; A = t1 + t2;
    }
    st[0] = A; st[1] = B; st[2] = C; st[3] = D; st[4] = E; st[5] = F; st[6] = G; st[7] = H;
  }
  // Region 1: [0, 1024) H_in, H_out, M.
  {
    ChunkWriter R;
    R.init(z, a, b, nu, o, 0);
    for (int w = 0; w < 8; ++w) R.put(32 * w, c.h[w], c.h[w], ONES);
    for (int w = 0; w < 8; ++w) { uint32_t v = st[w] + c.h[w]; R.put(256 + 32 * w, v, v, ONES); }
    for (int i = 0; i < 16; ++i) R.put(512 + 32 * i, c.w[i], c.w[i], ONES);
    R.finish(1024 / 128);
  }
  // Region 2: schedule aux [18757, 23173) then E_NEW, A_NEW, output carries and Z_CONST;
  // region 3: ch_and + maj_and [1024, 5120); region 4: round aux [5120, 18757).
  ChunkWriter RS, RCM, RR;
  RS.init(z, a, b, nu, o, s2r1cs::SCHED_CARRY_BASE >> 7);
  for (int t = 16; t < 64; ++t) {
    Add4 p = fadd4(ss1(W[t - 2]), ss0(W[t - 15]), W[t - 7], W[t - 16]);
    uint32_t base = s2r1cs::SCHED_CARRY_BASE + (t - 16) * s2r1cs::SCHED_ADD_BITS;
    RS.put(base, p.m1[2], p.m1[0], p.m1[1]);
    RS.put(base + 31, p.m2[2], p.m2[0], p.m2[1]);
    RS.put(base + 62, p.r[2], p.r[0], p.r[1]);
  }
  RCM.init(z, a, b, nu, o, 1024 >> 7);
  RR.init(z, a, b, nu, o, s2r1cs::ROUND_CARRY_BASE >> 7);
  // ch_and and maj_and are two sub-regions of RCM: collect maj_and values to emit after ch_and.
  uint32_t maj_z[64], maj_a[64], maj_b[64];
  uint32_t AA = c.h[0], BB = c.h[1], CC = c.h[2], DD = c.h[3], EE = c.h[4], FF = c.h[5], GG = c.h[6], HH = c.h[7];
  uint32_t enew_v[32], anew_v[32];
  for (int r = 0; r < 64; ++r) {
    uint32_t fxg = FF ^ GG, ch_and = EE & fxg;
    RCM.put(1024 + 32 * r, ch_and, EE, fxg);
    uint32_t bxa = BB ^ AA, cxa = CC ^ AA, maj_and = bxa & cxa;
    maj_z[r] = maj_and; maj_a[r] = bxa; maj_b[r] = cxa;
    uint32_t ch_out = ch_and ^ GG, maj_out = maj_and ^ AA;
    uint32_t rb = S2_ROUND_BASE[r];
    uint32_t k = S2_K[r];
    int t = __ffs(k);  // trailing_zeros(k) + 1
    int nrows = 31 - t;
    Add2 kp = add2(k, HH);
    uint32_t kmask = (1u << nrows) - 1;
    Add4 t1 = fadd4(kp.sum, bs1(EE), ch_out, W[r]);
    RR.put(rb + 0, t1.m1[2], t1.m1[0], t1.m1[1]);
    RR.put(rb + 31, t1.m2[2], t1.m2[0], t1.m2[1]);
    RR.put(rb + 62, t1.r[2], t1.r[0], t1.r[1]);
    Add3 an = fadd3(t1.sum, bs0(AA), maj_out);
    RR.put(rb + 92, an.m2, an.m0, an.m1);
    RR.put(rb + 123, an.r2, an.r0, an.r1);
    Add2 en = add2(DD, t1.sum);
    RR.put(rb + 153, en.c, en.l, en.r);
    RR.put(rb + 184, (kp.c >> t) & kmask, (kp.l >> t) & kmask, (kp.r >> t) & kmask);
    if (r & 1) { anew_v[r >> 1] = an.sum; enew_v[r >> 1] = en.sum; }
    HH = GG; GG = FF; FF = EE; EE = en.sum; DD = CC; CC = BB; BB = AA; AA = an.sum;
  }
  for (int r = 0; r < 64; ++r) RCM.put(3072 + 32 * r, maj_z[r], maj_a[r], maj_b[r]);
  RCM.finish(5120 >> 7);  // chunk 40 = [5120, 5248) begins RR's region
  // The round-aux region ends inside the chunk where the schedule region starts. The
  // schedule writer has already stored that chunk (its region spans 35 chunks), so
  // RR's partial accumulator is OR-ed into the stored word.
  RR.advance_to(s2r1cs::SCHED_CARRY_BASE >> 7);
  {
    uint32_t ch = s2r1cs::SCHED_CARRY_BASE >> 7;
    size_t wi = ((size_t)ch << nu) + o;
    uint4 vz = z[wi], va = a[wi], vb = b[wi];
    vz.x |= (uint32_t)RR.z0; vz.y |= (uint32_t)(RR.z0 >> 32); vz.z |= (uint32_t)RR.z1; vz.w |= (uint32_t)(RR.z1 >> 32);
    va.x |= (uint32_t)RR.a0; va.y |= (uint32_t)(RR.a0 >> 32); va.z |= (uint32_t)RR.a1; va.w |= (uint32_t)(RR.a1 >> 32);
    vb.x |= (uint32_t)RR.b0; vb.y |= (uint32_t)(RR.b0 >> 32); vb.z |= (uint32_t)RR.b1; vb.w |= (uint32_t)(RR.b1 >> 32);
    z[wi] = vz; a[wi] = va; b[wi] = vb;
  }
  for (int i = 0; i < 32; ++i) RS.put(s2r1cs::E_NEW_BASE + 32 * i, enew_v[i], enew_v[i], ONES);
  for (int i = 0; i < 32; ++i) RS.put(s2r1cs::A_NEW_BASE + 32 * i, anew_v[i], anew_v[i], ONES);
  uint32_t fs[8] = {AA, BB, CC, DD, EE, FF, GG, HH};
  for (int w = 0; w < 8; ++w) {
    Add2 oc = add2(fs[w], c.h[w]);
    RS.put(s2r1cs::OUT_CARRY_BASE + 31 * w, oc.c, oc.l, oc.r);
  }
  RS.put(s2r1cs::Z_CONST_POS, 1, 1, 1);
  RS.finish(used_chunks);
}

// ------------------------------------------------------------------------ Keccak-f[1600]
__constant__ uint64_t KC_RC[24];
__constant__ uint8_t KC_RHO[25];   // rotation for source lane a + 5b

__device__ __forceinline__ uint64_t rotl64d(uint64_t v, uint32_t r) { return r ? (v << r) | (v >> (64 - r)) : v; }

__global__ void witness_keccak_kernel(const uint64_t* __restrict__ in, uint32_t n_inst, uint32_t nu,
                                      uint64_t* z, uint64_t* a, uint64_t* b, uint32_t used_words) {
  uint32_t o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= n_inst) return;
  // input words -> Keccak lanes: input bit j is bit j / 25 of lane j % 25. The input words
  // are loaded once and every index below is a compile-time constant (fully unrolled), so
  // the lanes stay in registers.
  uint64_t iw[25];
#pragma unroll
  for (int i = 0; i < 25; ++i) iw[i] = in[(size_t)o * 25 + i];
  uint64_t st[25];
#pragma unroll
  for (int l = 0; l < 25; ++l) {
    uint64_t v = 0;
#pragma unroll
    for (int k = 0; k < 64; ++k) {
      const int j = 25 * k + l;
      v |= ((iw[j >> 6] >> (j & 63)) & 1ull) << k;
    }
    st[l] = v;
  }
  // u64 word w of the block sits at z[(((w >> 1) << nu) + o) * 2 + (w & 1)]
  auto put = [&](uint32_t w, uint64_t zv, uint64_t av, uint64_t bv) {
    size_t idx = ((((size_t)(w >> 1)) << nu) + o) * 2 + (w & 1);
    z[idx] = zv; a[idx] = av; b[idx] = bv;
  };
  for (int l = 0; l < 25; ++l) put(l, st[l], st[l], ~0ull);
  for (uint32_t w = 25; w < 32; ++w) put(w, 0, 0, 0);
  for (int r = 0; r < 24; ++r) {
    uint64_t th[25], bs[25];
    uint64_t cc[5];
    for (int x = 0; x < 5; ++x) cc[x] = st[x] ^ st[x + 5] ^ st[x + 10] ^ st[x + 15] ^ st[x + 20];
    for (int i = 0; i < 25; ++i) { int x = i % 5; th[i] = st[i] ^ cc[(x + 4) % 5] ^ rotl64d(cc[(x + 1) % 5], 1); }
    for (int y = 0; y < 5; ++y)
      for (int x = 0; x < 5; ++x) {
        int aa = (x + 3 * y) % 5, bb = x;
        bs[x + 5 * y] = rotl64d(th[aa + 5 * bb], KC_RHO[aa + 5 * bb]);
      }
    uint32_t tb = kr1cs::T_PACKED_BIT_BASE / 64 + r * 25;
    for (int y = 0; y < 5; ++y)
      for (int x = 0; x < 5; ++x) {
        uint64_t b1 = bs[(x + 1) % 5 + 5 * y], b2 = bs[(x + 2) % 5 + 5 * y];
        uint64_t t = (~b1) & b2;
        put(tb + x + 5 * y, t, ~b1, b2);
        st[x + 5 * y] = bs[x + 5 * y] ^ t;
      }
    st[0] ^= KC_RC[r];
  }
  for (int l = 0; l < 25; ++l) put(32 + l, st[l], st[l], ~0ull);
  for (uint32_t w = 57; w < 64; ++w) put(w, 0, 0, 0);
  put(64, 1, 1, 1);
  for (uint32_t w = kr1cs::T_PACKED_BIT_BASE / 64 + 24 * 25; w < used_words; ++w) put(w, 0, 0, 0);
}

// ------------------------------------------------------------------------ launchers
void upload_witness_constants() {
  // module constants are per device
  static std::mutex mu;
  static bool done[MAX_DEVICES] = {};
  int dev = 0;
  CUDA_OK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= MAX_DEVICES) throw std::runtime_error("device index out of range");
  std::lock_guard<std::mutex> g(mu);
  if (done[dev]) return;
  auto mi = b3r1cs::msg_idx();
  uint8_t idx[7][16];
  for (int r = 0; r < 7; ++r)
    for (int g = 0; g < 8; ++g) { idx[r][2 * g] = (uint8_t)mi[r][g][0]; idx[r][2 * g + 1] = (uint8_t)mi[r][g][1]; }
  CUDA_OK(cudaMemcpyToSymbol(B3_MSG_IDX, idx, sizeof(idx)));
  CUDA_OK(cudaMemcpyToSymbol(B3_GBASE, b3r1cs::G_BASE.v, sizeof(uint32_t) * 57));
  CUDA_OK(cudaMemcpyToSymbol(S2_K, Sha256::K, sizeof(uint32_t) * 64));
  CUDA_OK(cudaMemcpyToSymbol(S2_ROUND_BASE, s2r1cs::ROUND_BASE.v, sizeof(uint32_t) * 65));
  CUDA_OK(cudaMemcpyToSymbol(KC_RC, kr1cs::RC, sizeof(uint64_t) * 24));
  uint8_t rho[25];
  for (int a = 0; a < 5; ++a)
    for (int b = 0; b < 5; ++b) rho[a + 5 * b] = (uint8_t)(kr1cs::RHO[a][b] % 64);
  CUDA_OK(cudaMemcpyToSymbol(KC_RHO, rho, sizeof(rho)));
  // the copies above may still be in flight when they return; kernels of non-blocking
  // streams are not ordered after them
  CUDA_OK(cudaDeviceSynchronize());
  done[dev] = true;
}

void launch_witness(int hash, const void* d_inputs, uint32_t n_inst, uint32_t nu, F128d* z, F128d* a, F128d* b,
                    uint32_t used_chunks, cudaStream_t s) {
  upload_witness_constants();
  uint32_t threads = 64, blocks = (n_inst + threads - 1) / threads;
  if (hash == 0)
    witness_blake3_kernel<<<blocks, threads, 0, s>>>((const b3r1cs::Compression*)d_inputs, n_inst, nu, (uint4*)z,
                                                     (uint4*)a, (uint4*)b, used_chunks);
  else if (hash == 1)
    witness_sha2_kernel<<<blocks, threads, 0, s>>>((const s2r1cs::Compression*)d_inputs, n_inst, nu, (uint4*)z,
                                                   (uint4*)a, (uint4*)b, used_chunks);
  else
    witness_keccak_kernel<<<blocks, threads, 0, s>>>((const uint64_t*)d_inputs, n_inst, nu, (uint64_t*)z,
                                                     (uint64_t*)a, (uint64_t*)b, used_chunks * 2);
  LAUNCH_OK();
}

}  // namespace gpu
}  // namespace flock
