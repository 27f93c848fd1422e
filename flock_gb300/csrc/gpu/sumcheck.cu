// Sumcheck-side kernels of prove_fast: the zerocheck round 1 on the skip domain and
// its folds, the lincheck column folds / row fold / product sumcheck, the merged-open
// weight build and folds, and the Ligerito F256 ladder (basis tables, folds, messages,
// code switch, induced basis).
//
// Reductions: every message kernel writes per-block XOR partials to `part`
// (part[block * width + j]); reduce_parts XORs them into `width` values.
// Eq tables over many variables are never materialised: eq(i) = lo[i & (2^lo_bits - 1)]
// * hi[i >> lo_bits], and kernels that sum eq-weighted terms walk chunks of 2^lo_bits
// consecutive indices, summing lo-weighted terms and multiplying by hi once per chunk.
#include "kernels.h"
#include <atomic>
#include <mutex>
#include <set>
#include <tuple>

namespace flock {
namespace gpu {

__device__ __forceinline__ F128d block_xor(F128d v, F128d* sh) {
  v = warp_xor(v);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = (blockDim.x + 31) >> 5;
  __syncthreads();
  if (l == 0) sh[w] = v;
  __syncthreads();
  F128d r = f128_zero();
  if (w == 0) {
    r = l < nw ? sh[l] : f128_zero();
    r = warp_xor(r);
  }
  return r;  // valid in thread 0
}

__device__ __forceinline__ F128d eq_at(const F128d* lo, uint32_t lo_bits, const F128d* hi, uint64_t i) {
  F128d l = lo[i & ((1ull << lo_bits) - 1)];
  return hi ? l * hi[i >> lo_bits] : l;
}

// ------------------------------------------------------------------ generic pieces
__global__ void eq_table_kernel(const F128d* __restrict__ p, uint32_t n, F128d scale, F128d* __restrict__ out) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (1ull << n)) return;
  F128d v = scale;
  for (uint32_t j = 0; j < n; ++j) {
    F128d r = p[j];
    if (!((i >> j) & 1)) r.lo ^= 1;
    v = v * r;
  }
  out[i] = v;
}
void launch_eq_table(const F128d* d_point, uint32_t n, F128d scale, F128d* out, cudaStream_t s) {
  uint64_t len = 1ull << n;
  eq_table_kernel<<<(unsigned)((len + 255) / 256), 256, 0, s>>>(d_point, n, scale, out);
  LAUNCH_OK();
}
// Both tables of an eq split in one launch: lo = eq(p[0 .. lo_bits)) and
// hi = scale * eq(p[lo_bits .. lo_bits + hi_bits)); entry e < 2^lo_bits is a lo entry.
__global__ void eq_split_kernel(const F128d* __restrict__ p, uint32_t lo_bits, uint32_t hi_bits, F128d scale,
                                F128d* __restrict__ lo, F128d* __restrict__ hi) {
  const uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  const uint64_t n_lo = 1ull << lo_bits;
  if (e >= n_lo + (1ull << hi_bits)) return;
  const bool is_lo = e < n_lo;
  const uint64_t i = is_lo ? e : e - n_lo;
  const uint32_t n = is_lo ? lo_bits : hi_bits;
  const F128d* q = is_lo ? p : p + lo_bits;
  F128d v = is_lo ? f128_one() : scale;
  for (uint32_t j = 0; j < n; ++j) {
    F128d r = q[j];
    if (!((i >> j) & 1)) r.lo ^= 1;
    v = v * r;
  }
  (is_lo ? lo : hi)[i] = v;
}
void launch_eq_split(const F128d* d_point, uint32_t lo_bits, uint32_t hi_bits, F128d scale, F128d* lo, F128d* hi,
                     cudaStream_t s) {
  const uint64_t len = (1ull << lo_bits) + (1ull << hi_bits);
  eq_split_kernel<<<(unsigned)((len + 255) / 256), 256, 0, s>>>(d_point, lo_bits, hi_bits, scale, lo, hi);
  LAUNCH_OK();
}

__global__ void reduce_parts_kernel(const F128d* __restrict__ part, uint32_t n_blocks, uint32_t width,
                                    F128d* __restrict__ out) {
  __shared__ F128d sh[32];
  uint32_t col = blockIdx.x;
  F128d acc = f128_zero();
  for (uint32_t b = threadIdx.x; b < n_blocks; b += blockDim.x) acc += part[(uint64_t)b * width + col];
  acc = block_xor(acc, sh);
  if (threadIdx.x == 0) out[col] = acc;
}
void launch_reduce_parts(const F128d* part, uint32_t n_blocks, uint32_t width, F128d* out, cudaStream_t s) {
  reduce_parts_kernel<<<width, 256, 0, s>>>(part, n_blocks, width, out);
  LAUNCH_OK();
}

static std::atomic<uint64_t> g_launches{0};
uint64_t launch_count() { return g_launches.load(std::memory_order_relaxed); }
void note_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

static int current_device() {
  int dev = 0;
  CUDA_OK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= MAX_DEVICES) throw std::runtime_error("device index out of range");
  return dev;
}
int sm_count() {
  static std::atomic<int> cache[MAX_DEVICES];
  const int dev = current_device();
  int n = cache[dev].load(std::memory_order_relaxed);
  if (!n) {
    CUDA_OK(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
    cache[dev].store(n, std::memory_order_relaxed);
  }
  return n;
}
void set_dynamic_smem(const void* kernel, int bytes) {
  static std::mutex mu;
  static std::set<std::tuple<const void*, int, int>> done;
  const auto key = std::make_tuple(kernel, current_device(), bytes);
  std::lock_guard<std::mutex> g(mu);
  if (done.count(key)) return;
  CUDA_OK(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  done.insert(key);
}

// ------------------------------------------------------------------ zerocheck round 1
// With the fixed challenges r[6..13) the row eq factorises. For a row x (m - 6 bits)
// = (K: 3 bits, M: 4 bits, xo):
//   eq(r[6..m], x) = phi8(e_K) * D * x^M * eq(r[13..m], xo),
// e_K = prod_j (K_j ? c_j : 1 + c_j) over the three GF(2^8) constants c_j (phi8 is a
// ring embedding), and D = prod_i (1 + g_i)^-1 over the medium constants g_i = x^(2^i)
// (the bit-1 factor g/(1+g) and the bit-0 factor 1/(1+g)). Hence per Lambda point i
//   P_ab(i) = D * sum_xo eq_o(xo) * sum_M x^M * phi8( sum_K e_K * ext(a_x)(i) * ext(b_x)(i) )
// where the inner sums are GF(2^8) byte arithmetic and each xo costs one F128 multiply
// per output. The same factorisation over words w = (K2: 2 bits, M, xo) with e2 over
// r[7], r[8] gives s_hat_v_c[t] from bit t of z_w. P_c needs no pass of its own: it is
// linear in the z bits and the host derives it from s_hat_v_c. D is applied by the host.
struct ZcConsts {
  uint8_t ext[8 * 256 * 64];   // ext[c][v][i]: extension of byte v at S[8c..8c+8)
  F128d phi8[256];
  uint8_t mulk[8][256];        // e_K * v
  F128d wconst[64];            // word weights within an xo: x^M * phi8(e2[K2]) for word 4M + K2
  uint8_t gmul[256 * 256];     // GF(2^8) products: gmul[256 a + b] = a * b
};
constexpr size_t ZC_CONST_BYTES = (sizeof(ZcConsts) + 15) & ~size_t(15);

// Byte b of a word, zero-extended: one byte-permute.
__device__ __forceinline__ uint32_t byte_of(uint32_t v, int b) { return __byte_perm(v, 0, 0x4440 | b); }
// Every byte of v set to 0xFF where its bit 7 is set (prmt with the sign-replicate bit
// set in each selector nibble, which __byte_perm does not expose).
__device__ __forceinline__ uint32_t msb_spread(uint32_t v) {
  uint32_t r;
  asm("prmt.b32 %0, %1, %2, 0xBA98;" : "=r"(r) : "r"(v), "r"(0u));
  return r;
}
// Four GF(2^8) products (AES polynomial) of packed bytes, shift-and-add in registers.
__device__ __forceinline__ uint32_t gf8_mul4(uint32_t a, uint32_t b) {
  uint32_t r = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    r ^= a & msb_spread(b << (7 - k));  // bit k of each byte of b selects a * x^k
    if (k < 7) a = ((a << 1) & 0xFEFEFEFEu) ^ (msb_spread(a) & 0x1B1B1B1Bu);
  }
  return r;
}

// P_ab: one team of 16 threads per xo, thread = four Lambda points; no block barriers
// after the constants are staged. Per row x = 8M + K the team extends the a and b rows
// (8 byte-table lookups each), multiplies pointwise in GF(2^8) (the 64 KB product table is
// symmetric, so its index may put either factor high) and accumulates e_K * p into g_M;
// then F = sum_M x^M phi8(g_M) (Horner) and acc += eq_o(xo) * F. Tables: about 199 KB of
// shared memory, one block per SM.
constexpr int ZC_TEAMS = 32;  // teams per block (512 threads)
__global__ void __launch_bounds__(16 * ZC_TEAMS, 1)
zc_round1_ab_kernel(const F128d* __restrict__ a, const F128d* __restrict__ b, uint64_t n_xo,
                    const ZcConsts* __restrict__ gconst, const F128d* __restrict__ eq_lo, uint32_t lo_bits,
                    const F128d* __restrict__ eq_hi, F128d* __restrict__ part) {
  extern __shared__ __align__(16) uint8_t smem[];
  ZcConsts& C = *reinterpret_cast<ZcConsts*>(smem);
  {
    const uint4* src = reinterpret_cast<const uint4*>(gconst);
    uint4* dst = reinterpret_cast<uint4*>(smem);
    for (uint32_t i = threadIdx.x; i < ZC_CONST_BYTES / 16; i += blockDim.x) dst[i] = src[i];
  }
  __syncthreads();
  const uint32_t team = threadIdx.x >> 4, lane = threadIdx.x & 15;
  // ext as bytes: table c, value v, this lane's four points at c * 16384 + v * 64 + 4 * lane
  const uint8_t* extb = C.ext + 4 * lane;
  F128d acc[4] = {f128_zero(), f128_zero(), f128_zero(), f128_zero()};
  const uint64_t stride = (uint64_t)gridDim.x * ZC_TEAMS;
  for (uint64_t xo = (uint64_t)blockIdx.x * ZC_TEAMS + team; xo < n_xo; xo += stride) {
    const uint4* wa = reinterpret_cast<const uint4*>(a + xo * 64);
    const uint4* wb = reinterpret_cast<const uint4*>(b + xo * 64);
    uint32_t G[16];
#pragma unroll 1
    for (int M = 0; M < 16; ++M) {
      uint32_t g = 0;
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) {
        uint4 A = wa[4 * M + kk], B = wb[4 * M + kk];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          uint32_t a0 = h ? A.z : A.x, a1 = h ? A.w : A.y;  // the 64-bit row as two words
          uint32_t b0 = h ? B.z : B.x, b1 = h ? B.w : B.y;
          uint32_t ea = 0, eb = 0;
#pragma unroll
          for (int c = 0; c < 4; ++c) {
            ea ^= *reinterpret_cast<const uint32_t*>(extb + c * 16384 + (byte_of(a0, c) << 6)) ^
                  *reinterpret_cast<const uint32_t*>(extb + (c + 4) * 16384 + (byte_of(a1, c) << 6));
            eb ^= *reinterpret_cast<const uint32_t*>(extb + c * 16384 + (byte_of(b0, c) << 6)) ^
                  *reinterpret_cast<const uint32_t*>(extb + (c + 4) * 16384 + (byte_of(b1, c) << 6));
          }
          // the four GF(2^8) products, then e_K times each (mulk table): half of the rows take
          // the products from the 64 KB product table (shared-memory pipe), half compute them
          // in registers (logic pipe), which balances the two pipes
          const uint8_t* mk = C.mulk[2 * kk + h];
          if (h == 0) {
            const uint32_t i01 = __byte_perm(ea, eb, 0x5140), i23 = __byte_perm(ea, eb, 0x7362);
            g ^= (uint32_t)mk[C.gmul[i01 & 0xFFFF]] | ((uint32_t)mk[C.gmul[i01 >> 16]] << 8) |
                 ((uint32_t)mk[C.gmul[i23 & 0xFFFF]] << 16) | ((uint32_t)mk[C.gmul[i23 >> 16]] << 24);
          } else {
            const uint32_t p = gf8_mul4(ea, eb);
            g ^= (uint32_t)mk[byte_of(p, 0)] | ((uint32_t)mk[byte_of(p, 1)] << 8) | ((uint32_t)mk[byte_of(p, 2)] << 16) |
                 ((uint32_t)mk[byte_of(p, 3)] << 24);
          }
        }
      }
      G[M] = g;
    }
    F128d e = eq_at(eq_lo, lo_bits, eq_hi, xo);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      F128d F = f128_zero();
#pragma unroll
      for (int M = 15; M >= 0; --M) F = mul_by_x(F) + C.phi8[(G[M] >> (8 * k)) & 255];
      acc[k] += mul_call(e, F);
    }
  }
  uint64_t row = (uint64_t)blockIdx.x * ZC_TEAMS + team;
#pragma unroll
  for (int k = 0; k < 4; ++k) part[row * 64 + 4 * lane + k] = acc[k];
}

// Warp-wide 32 x 32 bit transpose: lane r holds word x_r; afterwards lane c holds the word
// whose bit r is bit c of x_r (five exchange stages of halving block size).
__device__ __forceinline__ uint32_t warp_transpose32(uint32_t x) {
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t masks[5] = {0x0000FFFFu, 0x00FF00FFu, 0x0F0F0F0Fu, 0x33333333u, 0x55555555u};
#pragma unroll
  for (int s = 0; s < 5; ++s) {
    const uint32_t j = 16u >> s, m = masks[s];
    const uint32_t y = __shfl_xor_sync(0xffffffffu, x, j);
    x = (lane & j) ? ((x & ~m) | ((y & ~m) >> j)) : ((x & m) | ((y & m) << j));
  }
  return x;
}

// s_hat_v_c[t] = sum_xo eq_o(xo) sum_w wconst[w] bit_t(z[64 xo + w]). The word constants
// and the eq_hi factor are applied once per eq_hi chunk, not per xo:
//   part[t] = sum_chunks eq_hi(chunk) * sum_{w in group} wconst[w] * U[w][t],
//   U[w][t] = sum_{xo in chunk} eq_lo(xo) bit_t(z[64 xo + w]),
// so the inner loop has no multiply. Block = 128 threads (one per bit t; warp = 32-bit
// limb) x one group of 8 words (blockIdx.y) x a run of xo_per_block consecutive xo
// (blockIdx.x); runs and chunks are powers of two. Per tile of 32 xo and word w, the warp
// transposes the 32 xo's limb words (lane r loads xo r), so thread t holds bit t of all 32
// xo in one register; each byte of it indexes the 256 subset sums of eight xo's eq weights.
constexpr uint32_t SVC_WORDS = 8;
constexpr uint32_t SVC_TILE = 32;  // xo staged in shared memory per step (one warp's lanes)
constexpr uint32_t SVC_ZS_STRIDE = SVC_WORDS * 4 + 1;  // 32-bit words per staged xo, padded
__global__ void __launch_bounds__(128)
zc_svc_kernel(const F128d* __restrict__ z, uint64_t xo_per_block, uint64_t xo_live, const ZcConsts* __restrict__ gconst,
              const F128d* __restrict__ eq_lo, uint32_t lo_bits, const F128d* __restrict__ eq_hi,
              F128d* __restrict__ part) {
  __shared__ uint32_t zs[SVC_TILE * SVC_ZS_STRIDE];  // zs[xo * stride + 4 w + limb]
  __shared__ F128d et[SVC_TILE];
  __shared__ F128d et4[SVC_TILE / 4][16];   // et4[q][v] = sum of et[4 q + k] over the bits k of v
  __shared__ F128d et8[SVC_TILE / 8][256];  // et8[q][v] = sum of et[8 q + k] over the bits k of v
  const uint32_t t = threadIdx.x, limb = t >> 5, lane = t & 31;
  const uint32_t g = blockIdx.y;
  const uint64_t xo0 = (uint64_t)blockIdx.x * xo_per_block;
  const uint64_t chunk = 1ull << lo_bits;
  const uint64_t seg = xo_per_block < chunk ? xo_per_block : chunk;
  const uint32_t tile = seg < SVC_TILE ? (uint32_t)seg : SVC_TILE;
  const F128d* wc = gconst->wconst + g * SVC_WORDS;
  const uint32_t* z32 = reinterpret_cast<const uint32_t*>(z);
  // xo from xo_live on hold zero words: the block stops there (a block wholly past it
  // writes a zero partial)
  const uint64_t xo_end = xo0 + xo_per_block < xo_live ? xo0 + xo_per_block : xo_live;
  F128d acc = f128_zero();
  for (uint64_t s0 = xo0; s0 < xo_end; s0 += seg) {
    F128d U[SVC_WORDS];
#pragma unroll
    for (uint32_t w = 0; w < SVC_WORDS; ++w) U[w] = f128_zero();
    const uint64_t s_end = s0 + seg < xo_end ? s0 + seg : xo_end;
    for (uint64_t xt = s0; xt < s_end; xt += tile) {
      const uint32_t cur = xt + tile <= s_end ? tile : (uint32_t)(s_end - xt);
      __syncthreads();
      // xo past a short tile are staged as zero words with zero weight: they add nothing
      for (uint32_t i = t; i < SVC_TILE * SVC_WORDS * 4; i += blockDim.x) {
        const uint32_t xl = i / (SVC_WORDS * 4), rem = i % (SVC_WORDS * 4);
        zs[xl * SVC_ZS_STRIDE + rem] = xl < cur ? z32[((xt + xl) * 64 + g * SVC_WORDS) * 4 + rem] : 0u;
      }
      if (t < SVC_TILE) et[t] = t < cur ? eq_lo[(xt + t) & (chunk - 1)] : f128_zero();
      __syncthreads();
      {
        const uint32_t q = t >> 4, v = t & 15;  // 128 threads: one nibble-table entry each
        F128d a = f128_zero();
#pragma unroll
        for (uint32_t k = 0; k < 4; ++k)
          if ((v >> k) & 1) a += et[4 * q + k];
        et4[q][v] = a;
      }
      __syncthreads();
      for (uint32_t i = t; i < (SVC_TILE / 8) * 256; i += blockDim.x) {
        const uint32_t q = i >> 8, v = i & 255;
        et8[q][v] = et4[2 * q][v & 15] + et4[2 * q + 1][v >> 4];
      }
      __syncthreads();
#pragma unroll
      for (uint32_t w = 0; w < SVC_WORDS; ++w) {
        const uint32_t bits = warp_transpose32(zs[lane * SVC_ZS_STRIDE + 4 * w + limb]);  // bit r: xo r
#pragma unroll
        for (uint32_t q = 0; q < SVC_TILE / 8; ++q) U[w] += et8[q][(bits >> (8 * q)) & 255];
      }
    }
    F128d v = f128_zero();
#pragma unroll
    for (uint32_t w = 0; w < SVC_WORDS; ++w) v += mul_call(wc[w], U[w]);
    acc += eq_hi ? mul_call(eq_hi[s0 >> lo_bits], v) : v;
  }
  part[((uint64_t)blockIdx.y * gridDim.x + blockIdx.x) * 128 + t] = acc;
}

static ZcConsts* g_zc_consts_dev[MAX_DEVICES] = {};  // written under the caller's lock, before any prover launches
static ZcConsts* zc_consts() { return g_zc_consts_dev[current_device()]; }
void upload_zc_consts(const uint8_t* ext, const F128d* phi8, const uint8_t mulk[8][256], const F128d* wconst) {
  const int dev = current_device();
  if (g_zc_consts_dev[dev]) return;
  ZcConsts* h = new ZcConsts();
  memcpy(h->ext, ext, sizeof(h->ext));
  memcpy(h->phi8, phi8, sizeof(h->phi8));
  memcpy(h->mulk, mulk, sizeof(h->mulk));
  memcpy(h->wconst, wconst, sizeof(h->wconst));
  for (uint32_t a = 0; a < 256; ++a)
    for (uint32_t b = 0; b < 256; ++b) {
      uint32_t p = 0, x = a;  // shift-and-add modulo the AES polynomial x^8 + x^4 + x^3 + x + 1
      for (int k = 0; k < 8; ++k) {
        if ((b >> k) & 1) p ^= x;
        x = (x << 1) ^ ((x & 0x80) ? 0x11B : 0);
      }
      h->gmul[256 * a + b] = (uint8_t)p;
    }
  ZcConsts* d = nullptr;
  CUDA_OK(cudaMalloc(&d, ZC_CONST_BYTES));
  CUDA_OK(cudaMemset(d, 0, ZC_CONST_BYTES));
  CUDA_OK(cudaMemcpy(d, h, sizeof(ZcConsts), cudaMemcpyHostToDevice));
  CUDA_OK(cudaDeviceSynchronize());  // complete before any kernel of a non-blocking stream reads it
  delete h;
  g_zc_consts_dev[dev] = d;
}

void launch_zc_round1(const F128d* a, const F128d* b, const F128d* z, uint32_t m, uint64_t live_words,
                      const F128d* eq_lo, uint32_t lo_bits, const F128d* eq_hi, F128d* part_ab, uint32_t* nrows_ab,
                      F128d* part_svc, uint32_t* nrows_svc, cudaStream_t s) {
  ZcConsts* g_zc_consts = zc_consts();
  if (!g_zc_consts) throw std::runtime_error("zerocheck constants not uploaded");
  uint64_t n_xo = 1ull << (m - 13);
  // xo past the live words hold zero rows of z, a and b and add nothing to any sum
  const uint64_t xo_live = std::min<uint64_t>(n_xo, (live_words + 63) / 64);
  size_t smem = ZC_CONST_BYTES;
  set_dynamic_smem((const void*)zc_round1_ab_kernel, (int)smem);
  uint32_t blocks = (uint32_t)std::max<uint64_t>(
      1, std::min<uint64_t>((xo_live + ZC_TEAMS - 1) / ZC_TEAMS, (uint64_t)sm_count()));
  zc_round1_ab_kernel<<<blocks, 16 * ZC_TEAMS, smem, s>>>(a, b, xo_live, g_zc_consts, eq_lo, lo_bits, eq_hi, part_ab);
  LAUNCH_OK();
  *nrows_ab = blocks * ZC_TEAMS;
  // at most 256 runs of xo per word group (n_xo and the chunks are powers of two)
  const uint64_t runs = std::min<uint64_t>(n_xo, 256);
  const uint64_t run = n_xo / runs;
  zc_svc_kernel<<<dim3((uint32_t)runs, 64 / SVC_WORDS), 128, 0, s>>>(z, run, xo_live, g_zc_consts, eq_lo, lo_bits,
                                                                   eq_hi, part_svc);
  LAUNCH_OK();
  *nrows_svc = (uint32_t)(runs * (64 / SVC_WORDS));
}

// ------------------------------------------------------------------ zerocheck skip fold
// a_mlv[x] = sum_{s in bits(a_x)} w[s] via 8 byte tables of the 64 Lagrange weights;
// word w holds rows 2w (lo) and 2w+1 (hi), which is exactly the first multilinear pair.
// Message: g1 = sum_w eq(w) a1 b1, ginf = sum_w eq(w) (a0 + a1)(b0 + b1). The folded
// vectors are not stored: the next round recomputes them from the bits (below).
__global__ void __launch_bounds__(256)
zc_fold_skip_kernel(const F128d* __restrict__ a, const F128d* __restrict__ b, const F128d* __restrict__ w64,
                    uint64_t n_words, const F128d* __restrict__ eq_lo, uint32_t lo_bits,
                    const F128d* __restrict__ eq_hi, F128d* __restrict__ part) {
  __shared__ F128d T[8][256];
  __shared__ F128d sh[32];
  for (uint32_t e = threadIdx.x; e < 2048; e += blockDim.x) {
    uint32_t c = e >> 8, v = e & 255;
    F128d acc = f128_zero();
    for (int k = 0; k < 8; ++k)
      if ((v >> k) & 1) acc += w64[8 * c + k];
    T[c][v] = acc;
  }
  __syncthreads();
  const uint64_t chunk = 1ull << lo_bits;
  const uint64_t n_chunks = (n_words + chunk - 1) / chunk;
  F128d G1 = f128_zero(), GI = f128_zero();
  for (uint64_t ch = blockIdx.x; ch < n_chunks; ch += gridDim.x) {
    F128d g1 = f128_zero(), gi = f128_zero();
    uint64_t end = min(n_words, (ch + 1) * chunk);
    for (uint64_t wi = ch * chunk + threadIdx.x; wi < end; wi += blockDim.x) {
      F128d av = a[wi], bv = b[wi];
      F128d a0 = f128_zero(), a1 = f128_zero(), b0 = f128_zero(), b1 = f128_zero();
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        a0 += T[c][(av.lo >> (8 * c)) & 255];
        a1 += T[c][(av.hi >> (8 * c)) & 255];
        b0 += T[c][(bv.lo >> (8 * c)) & 255];
        b1 += T[c][(bv.hi >> (8 * c)) & 255];
      }
      F128d e = eq_lo[wi & (chunk - 1)];
      g1 += mul_call(e, mul_call(a1, b1));
      gi += mul_call(e, mul_call(a0 + a1, b0 + b1));
    }
    g1 = block_xor(g1, sh);
    gi = block_xor(gi, sh);
    if (threadIdx.x == 0) {
      F128d h = eq_hi ? eq_hi[ch] : f128_one();
      G1 += h * g1;
      GI += h * gi;
    }
  }
  if (threadIdx.x == 0) { part[blockIdx.x * 2] = G1; part[blockIdx.x * 2 + 1] = GI; }
}
// The same message with the eq factors applied in the other order, for chunks of 1024
// words (lo_bits = 10) and 256 threads: thread t sees the four low indices l = t + 256 k of
// every chunk, so
//   g1 = sum_k eq_lo[l_k] S1_k,  S1_k = sum_chunks eq_hi[chunk] (a1 b1)[chunk 1024 + l_k]
// (ginf alike), and each per-word product by eq_lo becomes a product by the chunk's eq_hi,
// taken from the chunk's byte tables on the load/store pipe; eq_lo enters in eight
// products per thread at the end. Per word two products of variables stay on the multiply
// pipe instead of four.
constexpr uint32_t ZC_SKIP_DEFER_LO_BITS = 10;
__global__ void __launch_bounds__(256, 2)
zc_fold_skip_defer_kernel(const F128d* __restrict__ a, const F128d* __restrict__ b, const F128d* __restrict__ w64,
                          uint64_t n_chunks, const F128d* __restrict__ eq_lo, const F128d* __restrict__ eq_hi,
                          F128d* __restrict__ part) {
  __shared__ F128d T[8][256];
  __shared__ F128d sh[32];
  extern __shared__ __align__(16) F128d htab[];  // build_byte_table's BYTE_TABLE_SMEM_ENTRIES
  for (uint32_t e = threadIdx.x; e < 2048; e += blockDim.x) {
    uint32_t c = e >> 8, v = e & 255;
    F128d acc = f128_zero();
    for (int k = 0; k < 8; ++k)
      if ((v >> k) & 1) acc += w64[8 * c + k];
    T[c][v] = acc;
  }
  F128d S1[4], SI[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) S1[k] = SI[k] = f128_zero();
  for (uint64_t ch = blockIdx.x; ch < n_chunks; ch += gridDim.x) {
    __syncthreads();  // T is complete; the previous chunk's table is no longer read
    build_byte_table(eq_hi[ch], htab);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const uint64_t wi = (ch << ZC_SKIP_DEFER_LO_BITS) + threadIdx.x + 256 * k;
      const F128d av = a[wi], bv = b[wi];
      F128d a0 = f128_zero(), a1 = f128_zero(), b0 = f128_zero(), b1 = f128_zero();
#pragma unroll
      for (int c = 0; c < 8; ++c) {
        a0 += T[c][(av.lo >> (8 * c)) & 255];
        a1 += T[c][(av.hi >> (8 * c)) & 255];
        b0 += T[c][(bv.lo >> (8 * c)) & 255];
        b1 += T[c][(bv.hi >> (8 * c)) & 255];
      }
      S1[k] += mul_table(mul_call(a1, b1), htab);
      SI[k] += mul_table(mul_call(a0 + a1, b0 + b1), htab);
    }
  }
  F128d G1 = f128_zero(), GI = f128_zero();
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const F128d e = eq_lo[threadIdx.x + 256 * k];
    G1 += mul_call(e, S1[k]);
    GI += mul_call(e, SI[k]);
  }
  G1 = block_xor(G1, sh);
  GI = block_xor(GI, sh);
  if (threadIdx.x == 0) { part[blockIdx.x * 2] = G1; part[blockIdx.x * 2 + 1] = GI; }
}
uint32_t launch_zc_fold_skip(const F128d* a, const F128d* b, const F128d* w64, uint64_t n_words, const F128d* eq_lo,
                             uint32_t lo_bits, const F128d* eq_hi, F128d* part, cudaStream_t s) {
  if (eq_hi && lo_bits == ZC_SKIP_DEFER_LO_BITS && (n_words & ((1ull << lo_bits) - 1)) == 0 &&
      (n_words >> lo_bits) >= (uint64_t)sm_count() * 8) {
    // two resident blocks per SM, each looping over its share of the chunks
    const uint64_t n_chunks = n_words >> lo_bits;
    const uint32_t blocks = (uint32_t)sm_count() * 2;
    const int smem = (int)(BYTE_TABLE_SMEM_ENTRIES * sizeof(F128d));
    set_dynamic_smem((const void*)zc_fold_skip_defer_kernel, smem);
    zc_fold_skip_defer_kernel<<<blocks, 256, smem, s>>>(a, b, w64, n_chunks, eq_lo, eq_hi, part);
    LAUNCH_OK();
    return blocks;
  }
  uint64_t n_chunks = (n_words + (1ull << lo_bits) - 1) >> lo_bits;
  uint32_t blocks = (uint32_t)std::min<uint64_t>(n_chunks, (uint64_t)sm_count() * 8);
  zc_fold_skip_kernel<<<blocks, 256, 0, s>>>(a, b, w64, n_words, eq_lo, lo_bits, eq_hi, part);
  LAUNCH_OK();
  return blocks;
}

// The first multilinear fold at rho straight from the bits: the skip-folded pair of word
// w is (sum_s lo_s w_s, sum_s hi_s w_s), so its fold is
//   A'[w] = sum_s lo_s (1 + rho) w_s + sum_s hi_s rho w_s,
// two byte-table sums with the weights pre-scaled by (1 + rho) and rho (no per-word
// multiply). Then the next message over the pairs (A'[2j], A'[2j+1]) with eq(j).
__global__ void zc_scaled_tables_kernel(const F128d* __restrict__ w64, F128d rho, F128d* __restrict__ tabs) {
  __shared__ F128d ws[2][64];
  if (threadIdx.x < 64) {
    F128d v = rho * w64[threadIdx.x];
    ws[1][threadIdx.x] = v;                    // rho * w
    ws[0][threadIdx.x] = v + w64[threadIdx.x];  // (1 + rho) * w
  }
  __syncthreads();
  for (uint32_t e = threadIdx.x; e < 2 * 2048; e += blockDim.x) {
    uint32_t t = e >> 11, c = (e >> 8) & 7, v = e & 255;
    F128d acc = f128_zero();
    for (int k = 0; k < 8; ++k)
      if ((v >> k) & 1) acc += ws[t][8 * c + k];
    tabs[e] = acc;
  }
}
__global__ void __launch_bounds__(256)
zc_fold2_kernel(const F128d* __restrict__ a, const F128d* __restrict__ b, const F128d* __restrict__ tabs,
                uint64_t n_pairs, uint64_t live_pairs, const F128d* __restrict__ eq_lo, uint32_t lo_bits,
                const F128d* __restrict__ eq_hi, F128d* __restrict__ aout, F128d* __restrict__ bout,
                F128d* __restrict__ part) {
  extern __shared__ __align__(16) F128d T[];  // [2][8][256]: (1 + rho) w tables, then rho w tables
  __shared__ F128d sh[32];
  for (uint32_t e = threadIdx.x; e < 4096; e += blockDim.x) T[e] = tabs[e];
  __syncthreads();
  const F128d* T0 = T;
  const F128d* T1 = T + 2048;
  const uint64_t chunk = 1ull << lo_bits;
  const uint64_t n_chunks = (n_pairs + chunk - 1) / chunk;
  F128d G1 = f128_zero(), GI = f128_zero();
  for (uint64_t ch = blockIdx.x; ch < n_chunks; ch += gridDim.x) {
    F128d g1 = f128_zero(), gi = f128_zero();
    uint64_t end = min(n_pairs, (ch + 1) * chunk);
    for (uint64_t j = ch * chunk + threadIdx.x; j < end; j += blockDim.x) {
      if (j >= live_pairs) {  // zero words: zero outputs, nothing added to the message
        aout[2 * j] = aout[2 * j + 1] = bout[2 * j] = bout[2 * j + 1] = f128_zero();
        continue;
      }
      F128d A[2], B[2];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        F128d av = a[2 * j + h], bv = b[2 * j + h];
        F128d sa = f128_zero(), sb = f128_zero();
#pragma unroll
        for (int c = 0; c < 8; ++c) {
          sa += T0[c * 256 + ((av.lo >> (8 * c)) & 255)] + T1[c * 256 + ((av.hi >> (8 * c)) & 255)];
          sb += T0[c * 256 + ((bv.lo >> (8 * c)) & 255)] + T1[c * 256 + ((bv.hi >> (8 * c)) & 255)];
        }
        A[h] = sa;
        B[h] = sb;
      }
      aout[2 * j] = A[0]; aout[2 * j + 1] = A[1];
      bout[2 * j] = B[0]; bout[2 * j + 1] = B[1];
      F128d e = eq_lo[j & (chunk - 1)];
      g1 += mul_call(e, mul_call(A[1], B[1]));
      gi += mul_call(e, mul_call(A[0] + A[1], B[0] + B[1]));
    }
    g1 = block_xor(g1, sh);
    gi = block_xor(gi, sh);
    if (threadIdx.x == 0) {
      F128d hh = eq_hi ? eq_hi[ch] : f128_one();
      G1 += hh * g1;
      GI += hh * gi;
    }
  }
  if (threadIdx.x == 0) { part[blockIdx.x * 2] = G1; part[blockIdx.x * 2 + 1] = GI; }
}
uint32_t launch_zc_fold2(const F128d* a, const F128d* b, const F128d* w64, F128d rho, F128d* tabs, uint64_t n_pairs,
                         uint64_t live_pairs, const F128d* eq_lo, uint32_t lo_bits, const F128d* eq_hi, F128d* aout,
                         F128d* bout, F128d* part, cudaStream_t s) {
  live_pairs = std::min(live_pairs, n_pairs);
  zc_scaled_tables_kernel<<<16, 256, 0, s>>>(w64, rho, tabs);
  LAUNCH_OK();
  set_dynamic_smem((const void*)zc_fold2_kernel, 4096 * 16);
  uint64_t n_chunks = (n_pairs + (1ull << lo_bits) - 1) >> lo_bits;
  uint32_t blocks = (uint32_t)std::min<uint64_t>(n_chunks, (uint64_t)sm_count() * 3);
  zc_fold2_kernel<<<blocks, 256, 4096 * 16, s>>>(a, b, tabs, n_pairs, live_pairs, eq_lo, lo_bits, eq_hi, aout, bout,
                                                  part);
  LAUNCH_OK();
  return blocks;
}

// ------------------------------------------------------------------ fused publication
// Called by every block after thread 0 stored its `width` partials at part[block * width]:
// the block takes a ticket; the block that takes the last one reduces all partials (the
// other blocks' stores are visible to it after their fences and the atomic), writes the
// message to mapped memory, then the sequence number, and resets the counter.
__device__ void publish_if_last(const F128d* part, uint32_t width, const FusedPublish& pub, F128d* sh) {
  __shared__ uint32_t ticket;
  if (threadIdx.x == 0) {
    __threadfence();
    ticket = atomicAdd(pub.counter, 1u);
  }
  __syncthreads();
  if (ticket != gridDim.x - 1) return;
  __threadfence();
  for (uint32_t j = 0; j < width; ++j) {
    F128d acc = f128_zero();
    for (uint32_t b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
      const F128d* p = part + (uint64_t)b * width + j;
      acc += f128(__ldcg(&p->lo), __ldcg(&p->hi));
    }
    acc = block_xor(acc, sh);
    if (threadIdx.x == 0) {
      volatile F128d* o = pub.out;
      o[j].lo = acc.lo;
      o[j].hi = acc.hi;
    }
  }
  if (threadIdx.x == 0) {
    *pub.counter = 0;
    __threadfence_system();
    *(volatile uint32_t*)pub.flag = pub.seq;
  }
}

// ------------------------------------------------------------------ pair fold + message
// Folds of at least this many pairs take their products by r from byte tables. A block's
// table build costs about as much shared-memory traffic as 300 table products, so the
// table form also keeps at least PAIR_FOLD_TABLE_MIN_BLOCK_PAIRS pairs (4 table products
// each) per block.
constexpr uint64_t PAIR_FOLD_TABLE_MIN_PAIRS = uint64_t(1) << 17;
constexpr uint64_t PAIR_FOLD_TABLE_MIN_BLOCK_PAIRS = 512;
// Fold the low variable of two vectors at r (out[i] = in[2i] + r (in[2i+1] + in[2i]))
// and, unless `msg` is false, emit the pair message over the folded vectors:
//   g1 = sum_j eq(j) A1 B1, ginf = sum_j eq(j) (A0 + A1)(B0 + B1), (A0, A1) = out[2j..2j+2).
// eq_lo == nullptr means eq = 1. n_pairs = output length / 2 (>= 1).
// TBL: the four products by r come from byte tables of r in shared memory (load/store
// pipe) while the message's products of two variables stay integer multiplies; the
// block builds its table first, so this form is used where each block folds enough pairs
// to pay for that. Otherwise r is split once per block for mul_split.
template <bool TBL>
__global__ void __launch_bounds__(256, TBL ? 3 : 2)
pair_fold_kernel(const F128d* __restrict__ ain, const F128d* __restrict__ bin, uint64_t n_pairs, uint64_t live_pairs,
                 F128d r, const F128d* __restrict__ r_dev, const F128d* __restrict__ eq_lo, uint32_t lo_bits,
                 const F128d* __restrict__ eq_hi, F128d* __restrict__ aout, F128d* __restrict__ bout,
                 F128d* __restrict__ part, int msg, FusedPublish pub) {
  extern __shared__ __align__(16) F128d rtab[];  // TBL: build_byte_table's BYTE_TABLE_SMEM_ENTRIES
  __shared__ F128d sh[32];
  __shared__ F128split rs;  // the fold challenge, split once
  if (TBL) {
    build_byte_table(r_dev ? *r_dev : r, rtab);
  } else {
    if (threadIdx.x == 0) rs = split_factor(r_dev ? *r_dev : r);
    __syncthreads();
  }
  auto by_r = [&](F128d v) { return TBL ? mul_table(v, rtab) : mul_split_call(v, &rs); };
  const uint64_t chunk = 1ull << lo_bits;
  const uint64_t n_chunks = (n_pairs + chunk - 1) / chunk;
  F128d G1 = f128_zero(), GI = f128_zero();
  for (uint64_t ch = blockIdx.x; ch < n_chunks; ch += gridDim.x) {
    F128d g1 = f128_zero(), gi = f128_zero();
    uint64_t end = min(n_pairs, (ch + 1) * chunk);
    for (uint64_t j = ch * chunk + threadIdx.x; j < end; j += blockDim.x) {
      if (j >= live_pairs) {  // zero inputs: zero outputs, nothing added to the message
        aout[2 * j] = aout[2 * j + 1] = bout[2 * j] = bout[2 * j + 1] = f128_zero();
        continue;
      }
      F128d x0 = ain[4 * j], x1 = ain[4 * j + 1], x2 = ain[4 * j + 2], x3 = ain[4 * j + 3];
      F128d y0 = bin[4 * j], y1 = bin[4 * j + 1], y2 = bin[4 * j + 2], y3 = bin[4 * j + 3];
      F128d A0 = x0 + by_r(x1 + x0), A1 = x2 + by_r(x3 + x2);
      F128d B0 = y0 + by_r(y1 + y0), B1 = y2 + by_r(y3 + y2);
      aout[2 * j] = A0; aout[2 * j + 1] = A1;
      bout[2 * j] = B0; bout[2 * j + 1] = B1;
      if (msg) {
        F128d t1 = mul_call(A1, B1), ti = mul_call(A0 + A1, B0 + B1);
        if (eq_lo) {
          F128d e = eq_lo[j & (chunk - 1)];
          t1 = mul_call(e, t1);
          ti = mul_call(e, ti);
        }
        g1 += t1;
        gi += ti;
      }
    }
    if (msg) {
      g1 = block_xor(g1, sh);
      gi = block_xor(gi, sh);
      if (threadIdx.x == 0) {
        F128d h = (eq_lo && eq_hi) ? eq_hi[ch] : f128_one();
        G1 += h * g1;
        GI += h * gi;
      }
    }
  }
  if (msg && threadIdx.x == 0) { part[blockIdx.x * 2] = G1; part[blockIdx.x * 2 + 1] = GI; }
  if (msg && pub.out) publish_if_last(part, 2, pub, sh);
}
uint32_t launch_pair_fold(const F128d* ain, const F128d* bin, uint64_t n_pairs, uint64_t live_pairs, F128d r,
                          const F128d* r_dev, const F128d* eq_lo, uint32_t lo_bits, const F128d* eq_hi, F128d* aout,
                          F128d* bout, F128d* part, bool msg, cudaStream_t s, FusedPublish pub) {
  live_pairs = std::min(live_pairs, n_pairs);
  uint64_t n_chunks = (n_pairs + (1ull << lo_bits) - 1) >> lo_bits;
  if (n_pairs >= PAIR_FOLD_TABLE_MIN_PAIRS) {
    // three resident blocks per SM (74 KB of shared memory each), each building its table
    // once for its share of the chunks
    const int smem = (int)(BYTE_TABLE_SMEM_ENTRIES * sizeof(F128d));
    set_dynamic_smem((const void*)pair_fold_kernel<true>, smem);
    uint32_t blocks = (uint32_t)std::min<uint64_t>(std::min<uint64_t>(n_chunks, (uint64_t)sm_count() * 6),
                                                   n_pairs / PAIR_FOLD_TABLE_MIN_BLOCK_PAIRS);
    pair_fold_kernel<true><<<blocks, 256, smem, s>>>(ain, bin, n_pairs, live_pairs, r, r_dev, eq_lo, lo_bits, eq_hi,
                                                     aout, bout, part, msg ? 1 : 0, pub);
    LAUNCH_OK();
    return blocks;
  }
  uint32_t blocks = (uint32_t)std::min<uint64_t>(n_chunks, (uint64_t)sm_count() * 8);
  pair_fold_kernel<false><<<blocks, 256, 0, s>>>(ain, bin, n_pairs, live_pairs, r, r_dev, eq_lo, lo_bits, eq_hi, aout,
                                                 bout, part, msg ? 1 : 0, pub);
  LAUNCH_OK();
  return blocks;
}

// ------------------------------------------------------------------ lincheck
__global__ void lc_eq_inner_kernel(const F128d* __restrict__ w64, const F128d* __restrict__ er, uint32_t K,
                                   F128d* __restrict__ eqi) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < K) eqi[i] = w64[i & 63] * er[i >> 6];
}
void launch_lc_eq_inner(const F128d* w64, const F128d* er, uint32_t K, F128d* eqi, cudaStream_t s) {
  lc_eq_inner_kernel<<<(K + 255) / 256, 256, 0, s>>>(w64, er, K, eqi);
  LAUNCH_OK();
}
// One warp per column: consecutive lanes read consecutive row indices.
__global__ void csc_fold_kernel(const uint32_t* __restrict__ col_ptr, const uint32_t* __restrict__ rows,
                                uint32_t K, const F128d* __restrict__ eqi, F128d* __restrict__ out) {
  uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  uint32_t n_warps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t c = warp; c < K; c += n_warps) {
    F128d acc = f128_zero();
    for (uint32_t p = col_ptr[c] + lane; p < col_ptr[c + 1]; p += 32) acc += eqi[__ldg(rows + p)];
    acc = warp_xor(acc);
    if (lane == 0) out[c] = acc;
  }
}
void launch_csc_fold(const uint32_t* col_ptr, const uint32_t* rows, uint32_t K, const F128d* eqi, F128d* out,
                     cudaStream_t s) {
  uint32_t blocks = std::min<uint32_t>((K + 7) / 8, (uint32_t)sm_count() * 16);
  csc_fold_kernel<<<blocks, 256, 0, s>>>(col_ptr, rows, K, eqi, out);
  LAUNCH_OK();
}

// ---- Keccak-f lincheck columns: ca = eq^T A_0 and cb = eq^T B_0 of the Keccak-f block
// R1CS (the walker of KeccakLincheckCircuit::fold_alpha_batched, crates/flock-prover/src/
// r1cs_hashes/keccak.rs:692-829), as the adjoint of the constraint map. With st_r the
// state before round r and phi = pi o rho o theta, the rows are
//   A[Z] = B[Z] = z_Z;  A[s0] = st_0;  B[s0] = z_Z;  A[s24] = st_24;  B[s24] = z_Z;
//   A[t_r(x,y,z)] = phi(st_r)[x+1,y,z] + z_Z;  B[t_r(x,y,z)] = phi(st_r)[x+2,y,z];
//   st_{r+1} = phi(st_r) + t_r + RC_r z_Z,
// so with lambda_24 = eq[s24] (A) or 0 (B) and, for r = 23..0,
//   column t_r = lambda_{r+1};  lambda_r = phi^T(lambda_{r+1} + eq[t_r] shifted by 1 (A) / 2 (B) in x),
// column s0 = eq[s0] (A only) + lambda_0, and column Z collects eq[Z], the "+ z_Z" rows
// (A: all t rows; B: s0 and s24 rows) and <lambda_{r+1}, RC_r> for every round.
// phi^T = theta^T o (pi o rho)^T:
//   (pi o rho)^T: out[a,b,c] = in[b, 2(a-b) mod 5, c + rho(a,b)]
//   theta^T: out[x,y,z] = in[x,y,z] + sum_y' in[x+1,y',z] + sum_y' in[x-1,y',z+1].
// One block per side; the 1600-word vectors live in shared memory.
constexpr uint32_t KW_THREADS = 512;
constexpr uint32_t KW_STATE = 1600;
constexpr uint32_t KW_S24_WORD = 2048 / 64, KW_T_WORD = 4160 / 64, KW_Z = 4096;
__device__ __forceinline__ uint32_t kw_pos(uint32_t base_word, uint32_t s) { return (base_word + s % 25) * 64 + s / 25; }

__global__ void __launch_bounds__(KW_THREADS)
keccak_lincheck_columns_kernel(const F128d* __restrict__ eqi, F128d* __restrict__ ca, F128d* __restrict__ cb,
                               KeccakColumnConsts kc) {
  extern __shared__ F128d kw_sh[];
  F128d* lam = kw_sh;                // lambda, then mu in place
  F128d* P = lam + KW_STATE;         // (pi o rho)^T mu
  F128d* C = P + KW_STATE;           // column sums of P: C[x + 5 z]
  __shared__ F128d red[KW_THREADS / 32];
  const bool bside = blockIdx.x == 1;
  F128d* out = bside ? cb : ca;
  const uint32_t shift = bside ? 2 : 1, tid = threadIdx.x;
  F128d zacc = f128_zero();  // this thread's share of column Z beyond eq[Z]
  for (uint32_t s = tid; s < KW_STATE; s += KW_THREADS) {
    const F128d e = eqi[kw_pos(KW_S24_WORD, s)];
    if (bside) { lam[s] = f128_zero(); zacc += e; }
    else lam[s] = e;
  }
  __syncthreads();
  for (int r = 23; r >= 0; --r) {
    const uint32_t tb = KW_T_WORD + 25u * r;
    for (uint32_t s = tid; s < KW_STATE; s += KW_THREADS) {
      const F128d l = lam[s];
      out[kw_pos(tb, s)] = l;
      if (s % 25 == 0 && ((kc.rc[r] >> (s / 25)) & 1)) zacc += l;
      const uint32_t x = s % 5;
      const F128d e = eqi[kw_pos(tb, s - x + (x + 5 - shift) % 5)];
      if (!bside) zacc += e;
      lam[s] = l + e;
    }
    __syncthreads();
    for (uint32_t o = tid; o < KW_STATE; o += KW_THREADS) {
      const uint32_t a = o % 5, b = (o / 5) % 5, c = o / 25;
      const uint32_t y = (2 * (a + 5 - b)) % 5;
      P[o] = lam[b + 5 * y + 25 * ((c + kc.rho[a + 5 * b]) & 63)];
    }
    __syncthreads();
    for (uint32_t q = tid; q < 320; q += KW_THREADS) {
      const uint32_t x = q % 5, z = q / 5;
      F128d acc = f128_zero();
      for (uint32_t y = 0; y < 5; ++y) acc += P[x + 5 * y + 25 * z];
      C[q] = acc;
    }
    __syncthreads();
    for (uint32_t s = tid; s < KW_STATE; s += KW_THREADS) {
      const uint32_t x = s % 5, z = s / 25;
      lam[s] = P[s] + C[(x + 1) % 5 + 5 * z] + C[(x + 4) % 5 + 5 * ((z + 1) & 63)];
    }
    __syncthreads();
  }
  for (uint32_t s = tid; s < KW_STATE; s += KW_THREADS) {
    const uint32_t p = kw_pos(0, s);
    const F128d e = eqi[p];
    if (bside) { out[p] = lam[s]; zacc += e; }
    else out[p] = lam[s] + e;
  }
  const F128d tot = block_xor(zacc, red);
  if (tid == 0) out[KW_Z] = eqi[KW_Z] + tot;
}
void launch_keccak_lincheck_columns(const F128d* eqi, F128d* ca, F128d* cb, const KeccakColumnConsts& kc,
                                    cudaStream_t s) {
  const int smem = (int)((2 * KW_STATE + 320) * sizeof(F128d));
  set_dynamic_smem((const void*)keccak_lincheck_columns_kernel, smem);
  keccak_lincheck_columns_kernel<<<2, KW_THREADS, smem, s>>>(eqi, ca, cb, kc);
  LAUNCH_OK();
}

// z_vec[128 cc + t] = sum_row eq(row) * bit_t(z[(cc << nu) + row]). Block = (cc, row split),
// thread = bit t; rows staged through shared memory.
constexpr uint32_t ZV_TILE = 256;
__global__ void __launch_bounds__(128)
lc_zvec_kernel(const F128d* __restrict__ z, uint32_t nu, uint32_t n_split, const F128d* __restrict__ eq,
               F128d* __restrict__ part) {
  __shared__ F128d wz[ZV_TILE];
  __shared__ F128d we[ZV_TILE];
  __shared__ F128d we4[ZV_TILE / 4][16];  // we4[q][v] = sum of we[4 q + k] over the bits k of v
  uint32_t cc = blockIdx.x / n_split, sp = blockIdx.x % n_split;
  uint64_t rows = 1ull << nu, per = rows / n_split;
  uint64_t r0 = sp * per;
  uint32_t t = threadIdx.x, limb = t >> 5, sh = t & 31;
  F128d acc = f128_zero();
  for (uint64_t base = r0; base < r0 + per; base += ZV_TILE) {
    uint32_t n = (uint32_t)(ZV_TILE < r0 + per - base ? (uint64_t)ZV_TILE : r0 + per - base);
    __syncthreads();
    for (uint32_t i = t; i < n; i += blockDim.x) {
      wz[i] = z[((uint64_t)cc << nu) + base + i];
      we[i] = eq[base + i];
    }
    __syncthreads();
    // four rows at a time: their bits t index the subset sums of their eq weights (rows
    // past n are left out of every subset sum)
    const uint32_t groups = (n + 3) / 4;
    for (uint32_t i = t; i < groups * 16; i += blockDim.x) {
      const uint32_t q = i >> 4, v = i & 15;
      F128d s4 = f128_zero();
#pragma unroll
      for (uint32_t k = 0; k < 4; ++k)
        if (((v >> k) & 1) && 4 * q + k < n) s4 += we[4 * q + k];
      we4[q][v] = s4;
    }
    __syncthreads();
    for (uint32_t q = 0; q < groups; ++q) {
      const uint32_t* w0 = reinterpret_cast<const uint32_t*>(&wz[4 * q]) + limb;  // 4 words per row
      const uint32_t v = ((w0[0] >> sh) & 1) | (((w0[4] >> sh) & 1) << 1) | (((w0[8] >> sh) & 1) << 2) |
                         (((w0[12] >> sh) & 1) << 3);
      acc += we4[q][v];
    }
  }
  part[(uint64_t)blockIdx.x * 128 + t] = acc;
}
__global__ void lc_zvec_reduce_kernel(const F128d* __restrict__ part, uint32_t n_split, uint32_t n_out,
                                      F128d* __restrict__ zv) {
  uint32_t o = blockIdx.x * blockDim.x + threadIdx.x;  // o = 128 cc + t
  if (o >= n_out) return;
  uint32_t cc = o >> 7, t = o & 127;
  F128d acc = f128_zero();
  for (uint32_t sp = 0; sp < n_split; ++sp) acc += part[((uint64_t)cc * n_split + sp) * 128 + t];
  zv[o] = acc;
}
void launch_lc_zvec(const F128d* z, uint32_t nu, uint32_t used_chunks, const F128d* eq, F128d* part, F128d* zv,
                    cudaStream_t s) {
  uint32_t n_split = 1;
  while ((uint64_t)used_chunks * n_split < (uint64_t)sm_count() * 8 && (n_split << 1) <= (1u << nu) / 64)
    n_split <<= 1;
  lc_zvec_kernel<<<used_chunks * n_split, 128, 0, s>>>(z, nu, n_split, eq, part);
  LAUNCH_OK();
  uint32_t n_out = used_chunks * 128;
  lc_zvec_reduce_kernel<<<(n_out + 127) / 128, 128, 0, s>>>(part, n_split, n_out, zv);
  LAUNCH_OK();
}

// comb = alpha comb_a + comb_b (+ beta at pin); message over the top variable:
//   e1 = sum_i comb[h+i] zv[h+i], einf = sum_i (comb[h+i] + comb[i]) (zv[h+i] + zv[i]).
__global__ void lc_start_kernel(const F128d* __restrict__ ca, const F128d* __restrict__ cb, F128d alpha, F128d beta,
                                uint32_t pin, uint32_t K, F128d* __restrict__ comb, const F128d* __restrict__ zv,
                                F128d* __restrict__ part) {
  __shared__ F128d sh[32];
  uint32_t h = K / 2;
  F128d e1 = f128_zero(), ei = f128_zero();
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < h; i += gridDim.x * blockDim.x) {
    F128d c0 = alpha * ca[i] + cb[i], c1 = alpha * ca[i + h] + cb[i + h];
    if (i == pin) c0 += beta;
    if (i + h == pin) c1 += beta;
    comb[i] = c0; comb[i + h] = c1;
    F128d z0 = zv[i], z1 = zv[i + h];
    e1 += c1 * z1;
    ei += (c0 + c1) * (z0 + z1);
  }
  e1 = block_xor(e1, sh);
  ei = block_xor(ei, sh);
  if (threadIdx.x == 0) { part[blockIdx.x * 2] = e1; part[blockIdx.x * 2 + 1] = ei; }
}
uint32_t launch_lc_start(const F128d* ca, const F128d* cb, F128d alpha, F128d beta, uint32_t pin, uint32_t K,
                         F128d* comb, const F128d* zv, F128d* part, cudaStream_t s) {
  uint32_t blocks = std::max(1u, std::min((K / 2 + 255) / 256, 256u));
  lc_start_kernel<<<blocks, 256, 0, s>>>(ca, cb, alpha, beta, pin, K, comb, zv, part);
  LAUNCH_OK();
  return blocks;
}
// A union slot's share of the lincheck comb: out[i] = weight (alpha ca[i] + cb[i]), plus
// beta at the slot's const-pin column.
__global__ void lc_slot_comb_kernel(const F128d* __restrict__ ca, const F128d* __restrict__ cb, F128d alpha,
                                    F128d weight, F128d beta, uint32_t pin, uint32_t K, F128d* __restrict__ out) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < K; i += gridDim.x * blockDim.x) {
    F128d c = weight * (alpha * ca[i] + cb[i]);
    if (i == pin) c += beta;
    out[i] = c;
  }
}
void launch_lc_slot_comb(const F128d* ca, const F128d* cb, F128d alpha, F128d weight, F128d beta, uint32_t pin,
                         uint32_t K, F128d* out, cudaStream_t s) {
  lc_slot_comb_kernel<<<std::max(1u, std::min((K + 255) / 256, 1024u)), 256, 0, s>>>(ca, cb, alpha, weight, beta, pin,
                                                                                    K, out);
  LAUNCH_OK();
}
// First top-variable message of a built comb against zv (pairs (i, i + K/2)).
__global__ void lc_top_message_kernel(const F128d* __restrict__ comb, const F128d* __restrict__ zv, uint32_t K,
                                      F128d* __restrict__ part) {
  __shared__ F128d sh[32];
  uint32_t h = K / 2;
  F128d e1 = f128_zero(), ei = f128_zero();
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < h; i += gridDim.x * blockDim.x) {
    F128d c0 = comb[i], c1 = comb[i + h], z0 = zv[i], z1 = zv[i + h];
    e1 += c1 * z1;
    ei += (c0 + c1) * (z0 + z1);
  }
  e1 = block_xor(e1, sh);
  ei = block_xor(ei, sh);
  if (threadIdx.x == 0) { part[blockIdx.x * 2] = e1; part[blockIdx.x * 2 + 1] = ei; }
}
uint32_t launch_lc_top_message(const F128d* comb, const F128d* zv, uint32_t K, F128d* part, cudaStream_t s) {
  uint32_t blocks = std::max(1u, std::min((K / 2 + 255) / 256, 256u));
  lc_top_message_kernel<<<blocks, 256, 0, s>>>(comb, zv, K, part);
  LAUNCH_OK();
  return blocks;
}

// Bind the top variable of comb and zv (length len -> len/2) in place and emit the next
// top-variable message over the bound vectors (pairs (i, i + len/4)).
__global__ void lc_round_kernel(F128d* __restrict__ comb, F128d* __restrict__ zv, uint32_t len, F128d r, int msg,
                                F128d* __restrict__ part, FusedPublish pub) {
  __shared__ F128d sh[32];
  uint32_t h = len / 2, q = h / 2;
  F128d e1 = f128_zero(), ei = f128_zero();
  if (q == 0) {
    // len == 2: single bind, no message
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      comb[0] = comb[0] + r * (comb[1] + comb[0]);
      zv[0] = zv[0] + r * (zv[1] + zv[0]);
    }
  } else {
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < q; i += gridDim.x * blockDim.x) {
      F128d c0 = comb[i] + r * (comb[i + h] + comb[i]);
      F128d c1 = comb[i + q] + r * (comb[i + q + h] + comb[i + q]);
      F128d z0 = zv[i] + r * (zv[i + h] + zv[i]);
      F128d z1 = zv[i + q] + r * (zv[i + q + h] + zv[i + q]);
      comb[i] = c0; comb[i + q] = c1;
      zv[i] = z0; zv[i + q] = z1;
      if (msg) {
        e1 += c1 * z1;
        ei += (c0 + c1) * (z0 + z1);
      }
    }
  }
  e1 = block_xor(e1, sh);
  ei = block_xor(ei, sh);
  if (threadIdx.x == 0) { part[blockIdx.x * 2] = e1; part[blockIdx.x * 2 + 1] = ei; }
  if (pub.out) publish_if_last(part, 2, pub, sh);
}
uint32_t launch_lc_round(F128d* comb, F128d* zv, uint32_t len, F128d r, bool msg, F128d* part, cudaStream_t s,
                         FusedPublish pub) {
  uint32_t q = len / 4;
  uint32_t blocks = std::max(1u, std::min((q + 255) / 256, 256u));
  lc_round_kernel<<<blocks, 256, 0, s>>>(comb, zv, len, r, msg ? 1 : 0, part, pub);
  LAUNCH_OK();
  return blocks;
}
// (<w, comb_a>, <w, comb_b>), w[c] = er[c >> 6] * zp[c & 63].
__global__ void lc_matrix_evals_kernel(const F128d* __restrict__ ca, const F128d* __restrict__ cb,
                                       const F128d* __restrict__ er, const F128d* __restrict__ zp, uint32_t K,
                                       F128d* __restrict__ part) {
  __shared__ F128d sh[32];
  F128d ea = f128_zero(), eb = f128_zero();
  for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < K; c += gridDim.x * blockDim.x) {
    F128d w = er[c >> 6] * zp[c & 63];
    ea += w * ca[c];
    eb += w * cb[c];
  }
  ea = block_xor(ea, sh);
  eb = block_xor(eb, sh);
  if (threadIdx.x == 0) { part[blockIdx.x * 2] = ea; part[blockIdx.x * 2 + 1] = eb; }
}
uint32_t launch_lc_matrix_evals(const F128d* ca, const F128d* cb, const F128d* er, const F128d* zp, uint32_t K,
                                F128d* part, cudaStream_t s) {
  uint32_t blocks = std::max(1u, std::min((K + 255) / 256, 256u));
  lc_matrix_evals_kernel<<<blocks, 256, 0, s>>>(ca, cb, er, zp, K, part);
  LAUNCH_OK();
  return blocks;
}
// out[b] = sum_k et[k] * zv[b + 128 k]; one block per b.
__global__ void lc_s_hat_v_kernel(const F128d* __restrict__ zv, const F128d* __restrict__ et, uint32_t n_tail,
                                  F128d* __restrict__ out) {
  __shared__ F128d sh[32];
  uint32_t bb = blockIdx.x;
  F128d acc = f128_zero();
  for (uint32_t k = threadIdx.x; k < n_tail; k += blockDim.x) acc += et[k] * zv[bb + 128 * k];
  acc = block_xor(acc, sh);
  if (threadIdx.x == 0) out[bb] = acc;
}
void launch_lc_s_hat_v(const F128d* zv, const F128d* et, uint32_t n_tail, F128d* out, cudaStream_t s) {
  lc_s_hat_v_kernel<<<128, 128, 0, s>>>(zv, et, n_tail, out);
  LAUNCH_OK();
}

// ------------------------------------------------------------------ merged open
// W[d] = sum_c fold_one_slot(er_c[row] * ec_c[col], table_c) for d < area (row = d mod 2^nu,
// col = d >> nu), else 0; round-0 prime over (q, W): u0 = sum q[2i] W[2i],
// u2 = sum (q[2i] + q[2i+1]) (W[2i] + W[2i+1]).
__device__ __forceinline__ F128d fold_slot(F128d x, const F128d* tab) {
  F128d acc = f128_zero();
#pragma unroll
  for (int k = 0; k < 8; ++k) acc += tab[k * 256 + ((x.lo >> (8 * k)) & 255)];
#pragma unroll
  for (int k = 0; k < 8; ++k) acc += tab[(8 + k) * 256 + ((x.hi >> (8 * k)) & 255)];
  return acc;
}
// Jagged unrank of a union's committed stack: slot s holds dense [base, base + rows * cols),
// column-major with `rows` (the declared count) words per column, its first column at
// union chunk-column col_off.
__device__ __forceinline__ bool jagged_unrank(const JaggedSegs& g, uint64_t d, uint64_t& row, uint64_t& col) {
  for (uint32_t s = 0; s < g.n; ++s) {
    const uint64_t end = g.base[s] + g.rows[s] * g.cols[s];
    if (d >= g.base[s] && d < end) {
      const uint64_t local = d - g.base[s];
      col = g.col_off[s] + local / g.rows[s];
      row = local % g.rows[s];
      return true;
    }
  }
  return false;
}
template <bool JAGGED>
__global__ void __launch_bounds__(512, 1)
mo_build_w_kernel(const F128d* __restrict__ q, const F128d* __restrict__ er0, const F128d* __restrict__ ec0,
                  const F128d* __restrict__ er1, const F128d* __restrict__ ec1, const F128d* __restrict__ tables,
                  uint32_t nu, uint64_t area, uint64_t n, F128d* __restrict__ w, F128d* __restrict__ part,
                  JaggedSegs segs) {
  extern __shared__ __align__(16) F128d tab[];  // 2 x 16 x 256
  __shared__ F128d sh[32];
  for (uint32_t i = threadIdx.x; i < 2 * 16 * 256; i += blockDim.x) tab[i] = tables[i];
  __syncthreads();
  const uint64_t rmask = (1ull << nu) - 1;
  F128d u0 = f128_zero(), u2 = f128_zero();
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n / 2; i += (uint64_t)gridDim.x * blockDim.x) {
    if (2 * i >= area) {  // q and W are zero from the area on
      w[2 * i] = w[2 * i + 1] = f128_zero();
      continue;
    }
    F128d W[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
      uint64_t d = 2 * i + k;
      F128d acc = f128_zero();
      uint64_t row = d & rmask, col = d >> nu;
      if (d < area && (!JAGGED || jagged_unrank(segs, d, row, col)))
        acc = fold_slot(mul_call(er0[row], ec0[col]), tab) + fold_slot(mul_call(er1[row], ec1[col]), tab + 16 * 256);
      W[k] = acc;
      w[d] = acc;
    }
    F128d q0 = q[2 * i], q1 = q[2 * i + 1];
    u0 += mul_call(q0, W[0]);
    u2 += mul_call(q0 + q1, W[0] + W[1]);
  }
  u0 = block_xor(u0, sh);
  u2 = block_xor(u2, sh);
  if (threadIdx.x == 0) { part[blockIdx.x * 2] = u0; part[blockIdx.x * 2 + 1] = u2; }
}
// The same weight under identity compaction with tall columns (col = d >> nu): in column c
// the map x -> fold_slot(x ec_i[c], table_i) is GF(2)-linear, so the block builds its byte
// tables once per (column, part) work item and W[d] = M0_c(er0[row]) + M1_c(er1[row]) is
// 32 table lookups and no multiply; only the message's products stay integer multiplies.
// Work item = 2^(nu - part_log) consecutive rows of one column.
__global__ void __launch_bounds__(768, 1)
mo_build_w_cols_kernel(const F128d* __restrict__ q, const F128d* __restrict__ er0, const F128d* __restrict__ ec0,
                       const F128d* __restrict__ er1, const F128d* __restrict__ ec1, const F128d* __restrict__ tables,
                       uint32_t nu, uint32_t part_log, uint64_t area, uint64_t n, F128d* __restrict__ w,
                       F128d* __restrict__ part) {
  extern __shared__ __align__(16) F128d ct[];  // column tables M0, M1, then M1's scratch
  __shared__ F128d sh[32];
  F128d* T0 = ct;
  F128d* T1 = ct + BYTE_TABLE_ENTRIES;
  const uint64_t items = (n >> nu) << part_log, rows = 1ull << (nu - part_log);
  F128d u0 = f128_zero(), u2 = f128_zero();
  for (uint64_t it = blockIdx.x; it < items; it += gridDim.x) {
    const uint64_t col = it >> part_log, d0 = (col << nu) + ((it & ((1ull << part_log) - 1)) << (nu - part_log));
    const bool used = d0 < area;  // block-uniform
    if (!used) {  // q and W are zero from the area on: zero weights, nothing added to the message
      for (uint64_t j = threadIdx.x; j < rows; j += blockDim.x) w[d0 + j] = f128_zero();
      continue;
    }
    __syncthreads();  // the previous item's tables are no longer read
    {
      // M0's images (its scratch lies inside M1's table), then M1's
      if (threadIdx.x < 128) byte_table_images(T0)[threadIdx.x] = fold_slot(mul_call(ec0[col], unit_power(threadIdx.x)), tables);
      __syncthreads();
      byte_table_from_images(T0);
      if (threadIdx.x < 128)
        byte_table_images(T1)[threadIdx.x] = fold_slot(mul_call(ec1[col], unit_power(threadIdx.x)), tables + 16 * 256);
      __syncthreads();
      byte_table_from_images(T1);
    }
    for (uint64_t j = threadIdx.x; j < rows / 2; j += blockDim.x) {
      const uint64_t d = d0 + 2 * j, row = d & ((1ull << nu) - 1);
      F128d W0 = f128_zero(), W1 = f128_zero();
      if (d < area) W0 = mul_table(er0[row], T0) + mul_table(er1[row], T1);
      if (d + 1 < area) W1 = mul_table(er0[row + 1], T0) + mul_table(er1[row + 1], T1);
      w[d] = W0;
      w[d + 1] = W1;
      const F128d q0 = q[d], q1 = q[d + 1];
      u0 += mul_call(q0, W0);
      u2 += mul_call(q0 + q1, W0 + W1);
    }
  }
  u0 = block_xor(u0, sh);
  u2 = block_xor(u2, sh);
  if (threadIdx.x == 0) { part[blockIdx.x * 2] = u0; part[blockIdx.x * 2 + 1] = u2; }
}
// Columns of at least 2^MO_COLS_MIN_NU rows take the column-table form.
constexpr uint32_t MO_COLS_MIN_NU = 14;
uint32_t launch_mo_build_w(const F128d* q, const F128d* er0, const F128d* ec0, const F128d* er1, const F128d* ec1,
                           const F128d* tables, uint32_t nu, uint64_t area, uint64_t n, F128d* w, F128d* part,
                           cudaStream_t s, const JaggedSegs* segs) {
  if (!segs && nu >= MO_COLS_MIN_NU && (n >> nu) >= 1 && (n & ((1ull << nu) - 1)) == 0) {
    // work items of at least 2^13 rows, about eight per SM in all
    uint32_t part_log = 0;
    while (nu - part_log > 13 && ((n >> nu) << part_log) < (uint64_t)sm_count() * 8) ++part_log;
    const uint64_t items = (n >> nu) << part_log;
    const uint32_t blocks = (uint32_t)std::min<uint64_t>(items, (uint64_t)sm_count());
    const int smem = (int)((BYTE_TABLE_ENTRIES + BYTE_TABLE_SMEM_ENTRIES) * sizeof(F128d));
    set_dynamic_smem((const void*)mo_build_w_cols_kernel, smem);
    mo_build_w_cols_kernel<<<blocks, 768, smem, s>>>(q, er0, ec0, er1, ec1, tables, nu, part_log, area, n, w, part);
    LAUNCH_OK();
    return blocks;
  }
  size_t smem = 2 * 16 * 256 * sizeof(F128d);
  uint32_t blocks = (uint32_t)std::min<uint64_t>((n / 2 + 511) / 512, (uint64_t)sm_count());
  if (segs) {
    set_dynamic_smem((const void*)mo_build_w_kernel<true>, (int)smem);
    mo_build_w_kernel<true><<<blocks, 512, smem, s>>>(q, er0, ec0, er1, ec1, tables, nu, area, n, w, part, *segs);
  } else {
    set_dynamic_smem((const void*)mo_build_w_kernel<false>, (int)smem);
    mo_build_w_kernel<false><<<blocks, 512, smem, s>>>(q, er0, ec0, er1, ec1, tables, nu, area, n, w, part,
                                                       JaggedSegs());
  }
  LAUNCH_OK();
  return blocks;
}

// ------------------------------------------------------------------ Ligerito
// b[i] = eq(i) (the hi table carries the scale).
__global__ void lg_eq_fill_kernel(const F128d* __restrict__ eq_lo, uint32_t lo_bits, const F128d* __restrict__ eq_hi,
                                  uint64_t n, F128d* __restrict__ out, int add) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  F128d e = eq_at(eq_lo, lo_bits, eq_hi, i);
  if (add) out[i] += e;
  else out[i] = e;
}
// The same fill one chunk (2^lo_bits entries sharing eq_hi[chunk]) per block iteration:
// the first half of a chunk takes its products by eq_hi[chunk] from the chunk's byte
// tables, the second half from its split form; each thread forms one of each per
// iteration, so the load/store and multiply pipes share the products.
__global__ void __launch_bounds__(256, 2)
lg_eq_fill_tbl_kernel(const F128d* __restrict__ eq_lo, uint32_t lo_bits, const F128d* __restrict__ eq_hi, uint64_t n,
                      F128d* __restrict__ out, int add) {
  extern __shared__ __align__(16) F128d htab[];  // build_byte_table's BYTE_TABLE_SMEM_ENTRIES
  __shared__ F128split hs;
  const uint64_t chunk = 1ull << lo_bits, n_chunks = n >> lo_bits;
  for (uint64_t ch = blockIdx.x; ch < n_chunks; ch += gridDim.x) {
    __syncthreads();  // the previous chunk's table and split are no longer read
    const F128d h = eq_hi[ch];
    if (threadIdx.x == 0) hs = split_factor(h);
    build_byte_table(h, htab);
    F128d* o = out + ch * chunk;
    const uint64_t half = chunk / 2;
    for (uint64_t i = threadIdx.x; i < half; i += blockDim.x) {
      const F128d e0 = mul_table(eq_lo[i], htab);
      const F128d e1 = mul_split(eq_lo[half + i], hs);
      if (add) {
        o[i] += e0;
        o[half + i] += e1;
      } else {
        o[i] = e0;
        o[half + i] = e1;
      }
    }
  }
}
// b[i] = eq_a(i) + eq_b(i) for two eq splits with the same lo_bits (the basis eq and the
// first OOD eq in one pass over b): per chunk, the products by eq_hi_a[chunk] from its byte
// tables and those by eq_hi_b[chunk] from its split form, one of each per entry.
__global__ void __launch_bounds__(256, 2)
lg_eq_fill2_tbl_kernel(const F128d* __restrict__ lo_a, const F128d* __restrict__ hi_a, const F128d* __restrict__ lo_b,
                       const F128d* __restrict__ hi_b, uint32_t lo_bits, uint64_t n, F128d* __restrict__ out) {
  extern __shared__ __align__(16) F128d htab[];  // build_byte_table's BYTE_TABLE_SMEM_ENTRIES
  __shared__ F128split hs;
  const uint64_t chunk = 1ull << lo_bits, n_chunks = n >> lo_bits;
  for (uint64_t ch = blockIdx.x; ch < n_chunks; ch += gridDim.x) {
    __syncthreads();  // the previous chunk's table and split are no longer read
    if (threadIdx.x == 0) hs = split_factor(hi_b[ch]);
    build_byte_table(hi_a[ch], htab);
    F128d* o = out + ch * chunk;
    for (uint64_t i = threadIdx.x; i < chunk; i += blockDim.x) o[i] = mul_table(lo_a[i], htab) + mul_split(lo_b[i], hs);
  }
}
__global__ void lg_eq_fill2_kernel(const F128d* __restrict__ lo_a, const F128d* __restrict__ hi_a,
                                   const F128d* __restrict__ lo_b, const F128d* __restrict__ hi_b, uint32_t lo_bits,
                                   uint64_t n, F128d* __restrict__ out) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = eq_at(lo_a, lo_bits, hi_a, i) + eq_at(lo_b, lo_bits, hi_b, i);
}
void launch_lg_eq_fill2(const F128d* lo_a, const F128d* hi_a, const F128d* lo_b, const F128d* hi_b, uint32_t lo_bits,
                        uint64_t n, F128d* out, cudaStream_t s) {
  if (lo_bits >= 12 && (n >> lo_bits) >= (uint64_t)sm_count() * 2 && (n & ((1ull << lo_bits) - 1)) == 0) {
    const int smem = (int)(BYTE_TABLE_SMEM_ENTRIES * sizeof(F128d));
    set_dynamic_smem((const void*)lg_eq_fill2_tbl_kernel, smem);
    const uint32_t blocks = (uint32_t)std::min<uint64_t>(n >> lo_bits, (uint64_t)sm_count() * 2);
    lg_eq_fill2_tbl_kernel<<<blocks, 256, smem, s>>>(lo_a, hi_a, lo_b, hi_b, lo_bits, n, out);
    LAUNCH_OK();
    return;
  }
  lg_eq_fill2_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(lo_a, hi_a, lo_b, hi_b, lo_bits, n, out);
  LAUNCH_OK();
}
// Chunks of at least 2^12 entries (one table build per chunk), and enough of them to give
// every SM two blocks, use the table form.
constexpr uint32_t LG_EQ_FILL_TABLE_MIN_LO_BITS = 12;
void launch_lg_eq_fill(const F128d* eq_lo, uint32_t lo_bits, const F128d* eq_hi, uint64_t n, F128d* out, bool add,
                       cudaStream_t s) {
  if (eq_hi && lo_bits >= LG_EQ_FILL_TABLE_MIN_LO_BITS && (n >> lo_bits) >= (uint64_t)sm_count() * 2 &&
      (n & ((1ull << lo_bits) - 1)) == 0) {
    const int smem = (int)(BYTE_TABLE_SMEM_ENTRIES * sizeof(F128d));
    set_dynamic_smem((const void*)lg_eq_fill_tbl_kernel, smem);
    const uint32_t blocks = (uint32_t)std::min<uint64_t>(n >> lo_bits, (uint64_t)sm_count() * 2);
    lg_eq_fill_tbl_kernel<<<blocks, 256, smem, s>>>(eq_lo, lo_bits, eq_hi, n, out, add ? 1 : 0);
    LAUNCH_OK();
    return;
  }
  lg_eq_fill_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(eq_lo, lo_bits, eq_hi, n, out, add ? 1 : 0);
  LAUNCH_OK();
}
// sum_i f[i * stride] (F128 words) * eq(i), chunked.
__global__ void lg_dot_eq_kernel(const F128d* __restrict__ f, uint32_t stride, const F128d* __restrict__ eq_lo,
                                 uint32_t lo_bits, const F128d* __restrict__ eq_hi, uint64_t n,
                                 F128d* __restrict__ part) {
  __shared__ F128d sh[32];
  const uint64_t chunk = 1ull << lo_bits;
  const uint64_t n_chunks = (n + chunk - 1) / chunk;
  F128d G = f128_zero();
  for (uint64_t ch = blockIdx.x; ch < n_chunks; ch += gridDim.x) {
    F128d g = f128_zero();
    uint64_t end = min(n, (ch + 1) * chunk);
    for (uint64_t i = ch * chunk + threadIdx.x; i < end; i += blockDim.x) g += f[i * stride] * eq_lo[i & (chunk - 1)];
    g = block_xor(g, sh);
    if (threadIdx.x == 0) G += (eq_hi ? eq_hi[ch] : f128_one()) * g;
  }
  if (threadIdx.x == 0) part[blockIdx.x] = G;
}
// The same sum with chunks of 2^13 words and unit stride, reordered so that every
// per-word product is by a block constant:
//   sum_i f[i] eq(i) = sum_a eq_lo[a] h[a],  h[a] = sum_chunks eq_hi[chunk] f[chunk 2^13 + a].
// Thread t of the 512 owns the 16 low indices a = t + 512 k and accumulates its block's
// share of h[a] chunk by chunk; the products by the chunk's eq_hi come half from its byte
// tables, half from its split form. Then 16 products by eq_lo[a] and the block reduction.
constexpr uint32_t DOT_EQ_TBL_LO_BITS = 13;
__global__ void __launch_bounds__(512, 1)
lg_dot_eq_tbl_kernel(const F128d* __restrict__ f, const F128d* __restrict__ eq_lo, const F128d* __restrict__ eq_hi,
                     uint64_t n_chunks, F128d* __restrict__ part) {
  extern __shared__ __align__(16) F128d htab[];  // build_byte_table's BYTE_TABLE_SMEM_ENTRIES
  __shared__ F128split hs;
  __shared__ F128d sh[32];
  F128d h[16];
#pragma unroll
  for (int k = 0; k < 16; ++k) h[k] = f128_zero();
  for (uint64_t ch = blockIdx.x; ch < n_chunks; ch += gridDim.x) {
    __syncthreads();  // the previous chunk's table and split are no longer read
    const F128d e = eq_hi[ch];
    if (threadIdx.x == 0) hs = split_factor(e);
    build_byte_table(e, htab);
    const F128d* fc = f + (ch << DOT_EQ_TBL_LO_BITS) + threadIdx.x;
#pragma unroll
    for (int k = 0; k < 16; ++k) {
      const F128d x = fc[512 * k];
      h[k] += (k & 1) ? mul_split(x, hs) : mul_table(x, htab);
    }
  }
  F128d g = f128_zero();
#pragma unroll
  for (int k = 0; k < 16; ++k) g += mul_call(h[k], eq_lo[threadIdx.x + 512 * k]);
  g = block_xor(g, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = g;
}
uint32_t launch_lg_dot_eq(const F128d* f, uint32_t stride, const F128d* eq_lo, uint32_t lo_bits, const F128d* eq_hi,
                          uint64_t n, uint64_t live, F128d* part, cudaStream_t s) {
  live = std::min(live, n);  // f is zero from `live` on
  if (stride == 1 && eq_hi && lo_bits == DOT_EQ_TBL_LO_BITS && (n & ((1ull << lo_bits) - 1)) == 0 &&
      (n >> lo_bits) >= (uint64_t)sm_count()) {
    const uint64_t n_chunks = std::max<uint64_t>(1, (live + (1ull << lo_bits) - 1) >> lo_bits);
    const uint32_t blocks = (uint32_t)sm_count();
    const int smem = (int)(BYTE_TABLE_SMEM_ENTRIES * sizeof(F128d));
    set_dynamic_smem((const void*)lg_dot_eq_tbl_kernel, smem);
    lg_dot_eq_tbl_kernel<<<blocks, 512, smem, s>>>(f, eq_lo, eq_hi, n_chunks, part);
    LAUNCH_OK();
    return blocks;
  }
  n = std::max<uint64_t>(live, 1);
  uint64_t n_chunks = (n + (1ull << lo_bits) - 1) >> lo_bits;
  uint32_t blocks = (uint32_t)std::min<uint64_t>(n_chunks, (uint64_t)sm_count() * 8);
  lg_dot_eq_kernel<<<blocks, 256, 0, s>>>(f, stride, eq_lo, lo_bits, eq_hi, n, part);
  LAUNCH_OK();
  return blocks;
}

// Round message with block pairing d: pairs (lo, lo + d), lo = 2 d blk + k.
//   u0 = sum f[lo] b[lo], u2 = sum (f[lo] + f[hi]) (b[lo] + b[hi]).
// F128 (base) variant: outputs 2 words per block; F256 variant: 4 words (u0.c0, u0.c1, u2.c0, u2.c1).
// The pairing distances are powers of two (the kernels take log2 d).
static uint32_t log2_distance(uint64_t d) {
  if (d == 0 || (d & (d - 1))) throw std::runtime_error("Ligerito pair distance must be a power of two");
  uint32_t l = 0;
  while ((uint64_t(1) << l) < d) ++l;
  return l;
}
__device__ __forceinline__ uint64_t pair_lo(uint64_t i, uint32_t d_log) {
  return ((i >> d_log) << (d_log + 1)) | (i & ((1ull << d_log) - 1));
}
__global__ void lg_message128_kernel(const F128d* __restrict__ f, const F128d* __restrict__ b, uint64_t n, uint64_t f_live,
                                     uint32_t d_log, F128d* __restrict__ part, FusedPublish pub) {
  __shared__ F128d sh[32];
  F128d u0 = f128_zero(), u2 = f128_zero();
  for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n / 2; p += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t lo = pair_lo(p, d_log), hi = lo + (1ull << d_log);
    if (lo >= f_live) continue;  // f[lo] = f[hi] = 0: the pair adds nothing
    F128d f0 = f[lo], f1 = f[hi], b0 = b[lo], b1 = b[hi];
    u0 += f0 * b0;
    u2 += (f0 + f1) * (b0 + b1);
  }
  u0 = block_xor(u0, sh);
  u2 = block_xor(u2, sh);
  if (threadIdx.x == 0) { part[blockIdx.x * 2] = u0; part[blockIdx.x * 2 + 1] = u2; }
  if (pub.out) publish_if_last(part, 2, pub, sh);
}
uint32_t launch_lg_message128(const F128d* f, const F128d* b, uint64_t n, uint64_t f_live, uint64_t d, F128d* part,
                              cudaStream_t s, FusedPublish pub) {
  uint32_t blocks = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>((n / 2 + 255) / 256, (uint64_t)sm_count() * 8));
  lg_message128_kernel<<<blocks, 256, 0, s>>>(f, b, n, f_live, log2_distance(d), part, pub);
  LAUNCH_OK();
  return blocks;
}
__global__ void lg_message256_kernel(const F256d* __restrict__ f, const F256d* __restrict__ b, uint64_t n, uint64_t f_live,
                                     uint32_t d_log, F128d* __restrict__ part, FusedPublish pub) {
  __shared__ F128d sh[32];
  F256d u0 = f256(f128_zero(), f128_zero()), u2 = u0;
  for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n / 2; p += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t lo = pair_lo(p, d_log), hi = lo + (1ull << d_log);
    if (lo >= f_live) continue;  // f[lo] = f[hi] = 0: the pair adds nothing
    F256d f0 = f[lo], f1 = f[hi], b0 = b[lo], b1 = b[hi];
    u0 += f256_mul_call(f0, b0);
    u2 += f256_mul_call(f0 + f1, b0 + b1);
  }
  F128d r0 = block_xor(u0.c0, sh), r1 = block_xor(u0.c1, sh), r2 = block_xor(u2.c0, sh), r3 = block_xor(u2.c1, sh);
  if (threadIdx.x == 0) {
    part[blockIdx.x * 4] = r0; part[blockIdx.x * 4 + 1] = r1;
    part[blockIdx.x * 4 + 2] = r2; part[blockIdx.x * 4 + 3] = r3;
  }
  if (pub.out) publish_if_last(part, 4, pub, sh);
}
uint32_t launch_lg_message256(const F256d* f, const F256d* b, uint64_t n, uint64_t f_live, uint64_t d, F128d* part,
                              cudaStream_t s, FusedPublish pub) {
  uint32_t blocks = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>((n / 2 + 255) / 256, (uint64_t)sm_count() * 8));
  lg_message256_kernel<<<blocks, 256, 0, s>>>(f, b, n, f_live, log2_distance(d), part, pub);
  LAUNCH_OK();
  return blocks;
}
// o[i] = v[lo] + r (v[hi] + v[lo]), i = blk d + k, lo = 2 d blk + k. The products by r.c0
// come from byte tables of r.c0 (load/store pipe), those by r.c1 from its split form
// (multiply pipe); grid-stride, so each block's table serves many elements.
__global__ void __launch_bounds__(256, 2)
lg_fold128_kernel(const F128d* __restrict__ f, const F128d* __restrict__ b, uint64_t n_out, F256d r,
                  const F256d* __restrict__ r_dev, uint32_t d_log, F256d* __restrict__ fo, F256d* __restrict__ bo) {
  extern __shared__ __align__(16) F128d rtab[];  // build_byte_table's BYTE_TABLE_SMEM_ENTRIES
  __shared__ F128split r1s;
  const F256d rv = r_dev ? *r_dev : r;
  if (threadIdx.x == 0) r1s = split_factor(rv.c1);
  build_byte_table(rv.c0, rtab);
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n_out; i += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t lo = pair_lo(i, d_log), hi = lo + (1ull << d_log);
    F128d f0 = f[lo], df = f[hi] + f0, b0 = b[lo], db = b[hi] + b0;
    fo[i] = f256(f0 + mul_table(df, rtab), mul_split(df, r1s));
    bo[i] = f256(b0 + mul_table(db, rtab), mul_split(db, r1s));
  }
}
void launch_lg_fold128(const F128d* f, const F128d* b, uint64_t n_out, F256d r, const F256d* r_dev, uint64_t d,
                       F256d* fo, F256d* bo, cudaStream_t s) {
  const int smem = (int)(BYTE_TABLE_SMEM_ENTRIES * sizeof(F128d));
  set_dynamic_smem((const void*)lg_fold128_kernel, smem);
  // at least 2048 elements per block (two table products each) for one table build
  const uint64_t blocks = std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)sm_count() * 2, n_out / 2048));
  lg_fold128_kernel<<<(unsigned)blocks, 256, smem, s>>>(f, b, n_out, r, r_dev, log2_distance(d), fo, bo);
  LAUNCH_OK();
}
__global__ void lg_fold256_kernel(const F256d* __restrict__ f, const F256d* __restrict__ b, uint64_t n_out, F256d r,
                                  const F256d* __restrict__ r_dev, uint32_t d_log, F256d* __restrict__ fo,
                                  F256d* __restrict__ bo) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_out) return;
  const uint64_t lo = pair_lo(i, d_log), hi = lo + (1ull << d_log);
  F256d f0 = f[lo], b0 = b[lo];
  const F256d rv = r_dev ? *r_dev : r;
  fo[i] = f0 + f256_mul_call(rv, f[hi] + f0);
  bo[i] = b0 + f256_mul_call(rv, b[hi] + b0);
}
void launch_lg_fold256(const F256d* f, const F256d* b, uint64_t n_out, F256d r, const F256d* r_dev, uint64_t d,
                       F256d* fo, F256d* bo, cudaStream_t s) {
  lg_fold256_kernel<<<(unsigned)((n_out + 255) / 256), 256, 0, s>>>(f, b, n_out, r, r_dev, log2_distance(d), fo, bo);
  LAUNCH_OK();
}
// One round's fold (at r, pairs d_fold apart) fused with the next round's message over the
// folded vectors (pairs d_msg apart): each thread folds the two outputs of one message pair,
// stores them, and accumulates u0 = sum f0 b0, u2 = sum (f0 + f1)(b0 + b1) over them. Same
// index maps as lg_fold256_kernel and lg_message256_kernel; one pass instead of two.
__device__ __forceinline__ void lg_fold_at(const F256d* __restrict__ f, const F256d* __restrict__ b, F256d r,
                                        uint32_t d_log, uint64_t i, F256d& fi, F256d& bi) {
  const uint64_t lo = pair_lo(i, d_log), hi = lo + (1ull << d_log);
  const F256d f0 = f[lo], b0 = b[lo];
  fi = f0 + f256_mul_call(r, f[hi] + f0);
  bi = b0 + f256_mul_call(r, b[hi] + b0);
}
// TBL: the products by r come from byte tables of r.c0 and r.c1 plus the split form of
// r.c0 + r.c1 (the Karatsuba terms of F256 product, see operator* in field.cuh): per pair
// 8 table products on the load/store pipe beside 4 + 6 integer-multiply products. One
// 512-thread block per SM holds the two tables (141 KB).
template <bool TBL>
__global__ void __launch_bounds__(TBL ? 512 : 256, TBL ? 1 : 2)
lg_fold_msg256_kernel(const F256d* __restrict__ f, const F256d* __restrict__ b, uint64_t n_out, uint64_t f_live, F256d r,
                      uint32_t dlog_fold, uint32_t dlog_msg, F256d* __restrict__ fo, F256d* __restrict__ bo,
                      F128d* __restrict__ part, FusedPublish pub) {
  extern __shared__ __align__(16) F128d rtab[];  // TBL: tables of r.c0 and r.c1
  __shared__ F128d sh[32];
  __shared__ F128split rsum;
  if (TBL) {
    if (threadIdx.x == 0) rsum = split_factor(r.c0 + r.c1);
    build_byte_table(r.c0, rtab);
    build_byte_table(r.c1, rtab + BYTE_TABLE_ENTRIES);  // its scratch follows the second table
  }
  // fold of entry i (see lg_fold_at)
  auto fold_at = [&](uint64_t i, F256d& fi, F256d& bi) {
    if (TBL) {
      const uint64_t lo = pair_lo(i, dlog_fold), hi = lo + (1ull << dlog_fold);
      const F256d f0 = f[lo], b0 = b[lo], df = f[hi] + f0, db = b[hi] + b0;
      const F128d* T0 = rtab;
      const F128d* T1 = rtab + BYTE_TABLE_ENTRIES;
      F128d p0 = mul_table(df.c0, T0), p1 = mul_table(df.c1, T1), p2 = mul_split_call(df.c0 + df.c1, &rsum);
      fi = f0 + f256(p0 + mul_by_x_inv(p1), p2 + p0);
      p0 = mul_table(db.c0, T0);
      p1 = mul_table(db.c1, T1);
      p2 = mul_split_call(db.c0 + db.c1, &rsum);
      bi = b0 + f256(p0 + mul_by_x_inv(p1), p2 + p0);
    } else {
      lg_fold_at(f, b, r, dlog_fold, i, fi, bi);
    }
  };
  auto fold_b_at = [&](uint64_t i) {  // f is zero at both inputs of i: only b folds
    const uint64_t lo = pair_lo(i, dlog_fold), hi = lo + (1ull << dlog_fold);
    const F256d b0 = b[lo], db = b[hi] + b0;
    fo[i] = f256(f128_zero(), f128_zero());
    if (TBL) {
      const F128d p0 = mul_table(db.c0, rtab), p1 = mul_table(db.c1, rtab + BYTE_TABLE_ENTRIES),
                  p2 = mul_split_call(db.c0 + db.c1, &rsum);
      bo[i] = b0 + f256(p0 + mul_by_x_inv(p1), p2 + p0);
    } else {
      bo[i] = b0 + f256_mul_call(r, db);
    }
  };
  F256d u0 = f256(f128_zero(), f128_zero()), u2 = u0;
  for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n_out / 2; p += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t olo = pair_lo(p, dlog_msg), ohi = olo + (1ull << dlog_msg);
    if (pair_lo(olo, dlog_fold) >= f_live) {  // f is zero at every input of both entries
      fold_b_at(olo);
      fold_b_at(ohi);
      continue;
    }
    F256d fl, bl, fh, bh;
    fold_at(olo, fl, bl);
    fo[olo] = fl;
    bo[olo] = bl;
    u0 += f256_mul_call(fl, bl);
    fold_at(ohi, fh, bh);
    fo[ohi] = fh;
    bo[ohi] = bh;
    u2 += f256_mul_call(fl + fh, bl + bh);
  }
  F128d r0 = block_xor(u0.c0, sh), r1 = block_xor(u0.c1, sh), r2 = block_xor(u2.c0, sh), r3 = block_xor(u2.c1, sh);
  if (threadIdx.x == 0) {
    part[blockIdx.x * 4] = r0; part[blockIdx.x * 4 + 1] = r1;
    part[blockIdx.x * 4 + 2] = r2; part[blockIdx.x * 4 + 3] = r3;
  }
  if (pub.out) publish_if_last(part, 4, pub, sh);
}
// The first fold, of the base (F128) vectors at r, fused with the next message: the
// products r.c0 (f[hi] + f[lo]) and r.c1 (f[hi] + f[lo]) come from byte tables of r.c0 and
// r.c1 (8 table products per message pair on the load/store pipe) and the message's two
// F256 products of variables (6 F128 products) from integer multiplies. One 512-thread
// block per SM holds the two tables.
__global__ void __launch_bounds__(512, 1)
lg_fold_msg128_kernel(const F128d* __restrict__ f, const F128d* __restrict__ b, uint64_t n_out, uint64_t f_live, F256d r,
                      uint32_t dlog_fold, uint32_t dlog_msg, F256d* __restrict__ fo, F256d* __restrict__ bo,
                      F128d* __restrict__ part, FusedPublish pub) {
  extern __shared__ __align__(16) F128d rtab[];  // tables of r.c0 and r.c1
  __shared__ F128d sh[32];
  const F128d* T0 = rtab;
  const F128d* T1 = rtab + BYTE_TABLE_ENTRIES;
  build_byte_table(r.c0, rtab);
  build_byte_table(r.c1, rtab + BYTE_TABLE_ENTRIES);  // its scratch follows the second table
  auto fold_at = [&](uint64_t i, F256d& fi, F256d& bi) {
    const uint64_t lo = pair_lo(i, dlog_fold), hi = lo + (1ull << dlog_fold);
    const F128d f0 = f[lo], df = f[hi] + f0, b0 = b[lo], db = b[hi] + b0;
    fi = f256(f0 + mul_table(df, T0), mul_table(df, T1));
    bi = f256(b0 + mul_table(db, T0), mul_table(db, T1));
  };
  auto fold_b_at = [&](uint64_t i) {  // f is zero at both inputs of i: only b folds
    const uint64_t lo = pair_lo(i, dlog_fold), hi = lo + (1ull << dlog_fold);
    const F128d b0 = b[lo], db = b[hi] + b0;
    fo[i] = f256(f128_zero(), f128_zero());
    bo[i] = f256(b0 + mul_table(db, T0), mul_table(db, T1));
  };
  F256d u0 = f256(f128_zero(), f128_zero()), u2 = u0;
  for (uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; p < n_out / 2; p += (uint64_t)gridDim.x * blockDim.x) {
    const uint64_t olo = pair_lo(p, dlog_msg), ohi = olo + (1ull << dlog_msg);
    if (pair_lo(olo, dlog_fold) >= f_live) {  // f is zero at every input of both entries
      fold_b_at(olo);
      fold_b_at(ohi);
      continue;
    }
    F256d fl, bl, fh, bh;
    fold_at(olo, fl, bl);
    fo[olo] = fl;
    bo[olo] = bl;
    u0 += f256_mul_call(fl, bl);
    fold_at(ohi, fh, bh);
    fo[ohi] = fh;
    bo[ohi] = bh;
    u2 += f256_mul_call(fl + fh, bl + bh);
  }
  F128d r0 = block_xor(u0.c0, sh), r1 = block_xor(u0.c1, sh), r2 = block_xor(u2.c0, sh), r3 = block_xor(u2.c1, sh);
  if (threadIdx.x == 0) {
    part[blockIdx.x * 4] = r0; part[blockIdx.x * 4 + 1] = r1;
    part[blockIdx.x * 4 + 2] = r2; part[blockIdx.x * 4 + 3] = r3;
  }
  if (pub.out) publish_if_last(part, 4, pub, sh);
}
uint32_t launch_lg_fold_msg128(const F128d* f, const F128d* b, uint64_t n_out, uint64_t f_live, F256d r, uint64_t d_fold,
                               uint64_t d_msg, F256d* fo, F256d* bo, F128d* part, cudaStream_t s, FusedPublish pub) {
  const int smem = (int)((BYTE_TABLE_ENTRIES + BYTE_TABLE_SMEM_ENTRIES) * sizeof(F128d));
  set_dynamic_smem((const void*)lg_fold_msg128_kernel, smem);
  // at least 512 message pairs per block for its two table builds
  const uint32_t blocks =
      (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>((uint64_t)sm_count(), n_out / 2 / 512));
  lg_fold_msg128_kernel<<<blocks, 512, smem, s>>>(f, b, n_out, f_live, r, log2_distance(d_fold), log2_distance(d_msg),
                                                   fo, bo, part, pub);
  LAUNCH_OK();
  return blocks;
}
// Folds of at least this many output entries use the table form, with at least
// LG_FOLD_TABLE_MIN_BLOCK_PAIRS message pairs per block for its two table builds.
constexpr uint64_t LG_FOLD_TABLE_MIN_OUT = uint64_t(1) << 17;
constexpr uint64_t LG_FOLD_TABLE_MIN_BLOCK_PAIRS = 512;
uint32_t launch_lg_fold_msg256(const F256d* f, const F256d* b, uint64_t n_out, uint64_t f_live, F256d r, uint64_t d_fold,
                               uint64_t d_msg, F256d* fo, F256d* bo, F128d* part, cudaStream_t s, FusedPublish pub) {
  if (n_out >= LG_FOLD_TABLE_MIN_OUT) {
    const int smem = (int)((BYTE_TABLE_ENTRIES + BYTE_TABLE_SMEM_ENTRIES) * sizeof(F128d));
    set_dynamic_smem((const void*)lg_fold_msg256_kernel<true>, smem);
    const uint32_t blocks = (uint32_t)std::max<uint64_t>(
        1, std::min<uint64_t>((uint64_t)sm_count(), n_out / 2 / LG_FOLD_TABLE_MIN_BLOCK_PAIRS));
    lg_fold_msg256_kernel<true><<<blocks, 512, smem, s>>>(f, b, n_out, f_live, r, log2_distance(d_fold),
                                                          log2_distance(d_msg), fo, bo, part, pub);
    LAUNCH_OK();
    return blocks;
  }
  uint32_t blocks = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>((n_out / 2 + 255) / 256, (uint64_t)sm_count() * 8));
  lg_fold_msg256_kernel<false><<<blocks, 256, 0, s>>>(f, b, n_out, f_live, r, log2_distance(d_fold),
                                                      log2_distance(d_msg), fo, bo, part, pub);
  LAUNCH_OK();
  return blocks;
}
// f' = (f.c0, f.c1) interleaved as base values; b' = (b, u b).
__global__ void lg_code_switch_kernel(const F256d* __restrict__ f, const F256d* __restrict__ b, uint64_t n,
                                      F256d* __restrict__ fo, F256d* __restrict__ bo) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  F256d fv = f[i], bv = b[i];
  fo[2 * i] = f256_base(fv.c0);
  fo[2 * i + 1] = f256_base(fv.c1);
  bo[2 * i] = bv;
  bo[2 * i + 1] = f256(mul_by_x_inv(bv.c1), bv.c0 + bv.c1);
}
void launch_lg_code_switch(const F256d* f, const F256d* b, uint64_t n, F256d* fo, F256d* bo, cudaStream_t s) {
  lg_code_switch_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(f, b, n, fo, bo);
  LAUNCH_OK();
}
// The code switch fused with the next message (pairs (2i, 2i + 1) of the switched vectors).
// The switched f entries are base-field, so both products of pair i are base x F256, two
// F128 products each instead of three:
//   u0 += f.c0 b = (f.c0 b.c0, f.c0 b.c1),
//   u2 += (f.c0 + f.c1)(b + u b) = s (b.c0 + x^-1 b.c1, b.c0),  s = f.c0 + f.c1,
// with u b = (x^-1 b.c1, b.c0 + b.c1) as the switch writes it.
__global__ void lg_switch_msg_kernel(const F256d* __restrict__ f, const F256d* __restrict__ b, uint64_t n, uint64_t f_live,
                                     F256d* __restrict__ fo, F256d* __restrict__ bo, F128d* __restrict__ part,
                                     FusedPublish pub) {
  __shared__ F128d sh[32];
  F128d u00 = f128_zero(), u01 = f128_zero(), u20 = f128_zero(), u21 = f128_zero();
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const F256d fv = f[i], bv = b[i];
    const F128d ub0 = mul_by_x_inv(bv.c1);
    fo[2 * i] = f256_base(fv.c0);
    fo[2 * i + 1] = f256_base(fv.c1);
    bo[2 * i] = bv;
    bo[2 * i + 1] = f256(ub0, bv.c0 + bv.c1);
    if (i >= f_live) continue;  // f[i] = 0: both products vanish
    const F128d sv = fv.c0 + fv.c1;
    u00 += mul_call(fv.c0, bv.c0);
    u01 += mul_call(fv.c0, bv.c1);
    u20 += mul_call(sv, bv.c0 + ub0);
    u21 += mul_call(sv, bv.c0);
  }
  F128d r0 = block_xor(u00, sh), r1 = block_xor(u01, sh), r2 = block_xor(u20, sh), r3 = block_xor(u21, sh);
  if (threadIdx.x == 0) {
    part[blockIdx.x * 4] = r0; part[blockIdx.x * 4 + 1] = r1;
    part[blockIdx.x * 4 + 2] = r2; part[blockIdx.x * 4 + 3] = r3;
  }
  if (pub.out) publish_if_last(part, 4, pub, sh);
}
uint32_t launch_lg_switch_msg(const F256d* f, const F256d* b, uint64_t n, uint64_t f_live, F256d* fo, F256d* bo,
                              F128d* part, cudaStream_t s, FusedPublish pub) {
  uint32_t blocks = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>((n + 255) / 256, (uint64_t)sm_count() * 8));
  lg_switch_msg_kernel<<<blocks, 256, 0, s>>>(f, b, n, f_live, fo, bo, part, pub);
  LAUNCH_OK();
  return blocks;
}
// mat[i] = f[i mod msg].c0
__global__ void lg_replicate_kernel(const F256d* __restrict__ f, uint64_t msg, uint64_t total, F128d* __restrict__ mat) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < total) mat[i] = f[i & (msg - 1)].c0;
}
void launch_lg_replicate(const F256d* f, uint64_t msg, uint64_t total, F128d* mat, cudaStream_t s) {
  lg_replicate_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(f, msg, total, mat);
  LAUNCH_OK();
}
// Pending eq basis e = eq(z) over the (base-valued) f of length n: stores e, returns per
// block (answer = sum f e, u0 = sum f[2j] e[2j], u2 = sum (f0 + f1)(e0 + e1)).
__global__ void lg_intro_eq_kernel(const F256d* __restrict__ f, const F128d* __restrict__ eq_lo, uint32_t lo_bits,
                                   const F128d* __restrict__ eq_hi, uint64_t n, F128d* __restrict__ pend,
                                   F128d* __restrict__ part, FusedPublish pub) {
  __shared__ F128d sh[32];
  F128d ans = f128_zero(), u0 = f128_zero(), u2 = f128_zero();
  for (uint64_t j = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; j < n / 2; j += (uint64_t)gridDim.x * blockDim.x) {
    F128d e0 = eq_at(eq_lo, lo_bits, eq_hi, 2 * j), e1 = eq_at(eq_lo, lo_bits, eq_hi, 2 * j + 1);
    pend[2 * j] = e0;
    pend[2 * j + 1] = e1;
    F128d f0 = f[2 * j].c0, f1 = f[2 * j + 1].c0;
    F128d p0 = f0 * e0;
    ans += p0 + f1 * e1;
    u0 += p0;
    u2 += (f0 + f1) * (e0 + e1);
  }
  ans = block_xor(ans, sh);
  u0 = block_xor(u0, sh);
  u2 = block_xor(u2, sh);
  if (threadIdx.x == 0) { part[blockIdx.x * 3] = ans; part[blockIdx.x * 3 + 1] = u0; part[blockIdx.x * 3 + 2] = u2; }
  if (pub.out) publish_if_last(part, 3, pub, sh);
}
uint32_t launch_lg_intro_eq(const F256d* f, const F128d* eq_lo, uint32_t lo_bits, const F128d* eq_hi, uint64_t n,
                            F128d* pend, F128d* part, cudaStream_t s, FusedPublish pub) {
  uint32_t blocks = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>((n / 2 + 255) / 256, (uint64_t)sm_count() * 8));
  lg_intro_eq_kernel<<<blocks, 256, 0, s>>>(f, eq_lo, lo_bits, eq_hi, n, pend, part, pub);
  LAUNCH_OK();
  return blocks;
}
// Induced basis of the queried positions. The level's codeword is the NTT (layers
// [log_rate, log_d)) of the message replicated 2^log_rate times, so for weights w_q at
// positions pos_q
//   basis = R^T . L_rate^T ... L_{log_d-1}^T . (sum_q w_q e_{pos_q}),
// with the transposed butterfly (u, v) -> (u + v, v + t (u + v)) and R^T the sum over
// the replicas. One scatter, log_d - log_rate transposed layers and the replica fold.
__global__ void lg_scatter_kernel(const uint64_t* __restrict__ pos, const F128d* __restrict__ w, uint32_t n_q,
                                  F128d* __restrict__ y) {
  uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n_q) return;
  unsigned long long* p = reinterpret_cast<unsigned long long*>(y + pos[q]);
  atomicXor(p, (unsigned long long)w[q].lo);
  atomicXor(p + 1, (unsigned long long)w[q].hi);
}
__global__ void ntt_t_layer_kernel(F128d* __restrict__ y, uint32_t log_d, uint32_t layer, const F128d* __restrict__ tw) {
  uint64_t pair = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (pair >= (1ull << (log_d - 1))) return;
  uint32_t sh = log_d - layer - 1;
  uint64_t blk = pair >> sh, within = pair & ((1ull << sh) - 1);
  uint64_t i0 = (blk << (sh + 1)) + within, i1 = i0 + (1ull << sh);
  F128d t = tw[(1ull << layer) - 1 + blk];
  F128d u = y[i0], v = y[i1], sum = u + v;
  y[i0] = sum;
  y[i1] = blk == 0 ? v : v + t * sum;  // the first block's twiddle is zero in every layer
}
// basis[i] = sum_rep y[rep * n + i]; with the split f (length 2n):
// a = sum f[2i] basis[i], s = sum (f[2i] + f[2i+1]) basis[i].
__global__ void lg_induced_fold_kernel(const F128d* __restrict__ y, uint32_t ln, uint32_t log_rate,
                                       const F256d* __restrict__ f, F128d* __restrict__ basis, F128d* __restrict__ part,
                                       FusedPublish pub) {
  __shared__ F128d sh[32];
  uint64_t n = 1ull << ln;
  F128d A = f128_zero(), Sm = f128_zero();
  for (uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    F128d acc = f128_zero();
    for (uint64_t rep = 0; rep < (1ull << log_rate); ++rep) acc += y[rep * n + i];
    basis[i] = acc;
    F128d f0 = f[2 * i].c0, f1 = f[2 * i + 1].c0;
    A += f0 * acc;
    Sm += (f0 + f1) * acc;
  }
  A = block_xor(A, sh);
  Sm = block_xor(Sm, sh);
  if (threadIdx.x == 0) { part[blockIdx.x * 2] = A; part[blockIdx.x * 2 + 1] = Sm; }
  if (pub.out) publish_if_last(part, 2, pub, sh);
}
// Several consecutive transposed layers in one launch: layers layer_hi, layer_hi - 1, ...,
// layer_hi - nl + 1 (pair distances 2^sh_min, ..., 2^(sh_min + nl - 1), sh_min =
// log_d - 1 - layer_hi) act within groups of 2^nl positions spaced 2^sh_min apart, so one
// block stages a group in shared memory and runs all nl layers there (one launch and one
// global pass instead of nl). Group g: base = (g >> sh_min) << (sh_min + nl) | (g mod
// 2^sh_min); position t of the group is base + t 2^sh_min. The butterfly is ntt_t_layer's.
constexpr uint32_t NTT_T_FUSED = 6;  // layers per fused pass (64-position groups)
constexpr uint32_t NTT_T_FUSED_MAX_LOG = 16;  // transforms of at most 2^16 positions use it
__global__ void __launch_bounds__(256)
ntt_t_fused_kernel(F128d* __restrict__ y, uint32_t log_d, uint32_t layer_hi, uint32_t nl,
                   const F128d* __restrict__ tw) {
  __shared__ F128d g[4][1u << NTT_T_FUSED];  // four groups per 256-thread block
  const uint32_t P = 1u << nl, sh_min = log_d - 1 - layer_hi;
  const uint64_t n_groups = 1ull << (log_d - nl);
  const uint32_t sub = threadIdx.x >> 6, t = threadIdx.x & 63;  // 64 threads per group
  const uint64_t gi = (uint64_t)blockIdx.x * 4 + sub;
  const bool have = gi < n_groups;  // group-uniform
  const uint64_t base = have ? (((gi >> sh_min) << (sh_min + nl)) | (gi & ((1ull << sh_min) - 1))) : 0;
  if (have && t < P) g[sub][t] = y[base + ((uint64_t)t << sh_min)];
  __syncthreads();
  for (uint32_t k = 0; k < nl; ++k) {
    const uint32_t layer = layer_hi - k, sh = sh_min + k;
    if (have && t < P / 2) {
      // pair t of the group at group distance 2^k
      const uint32_t lo = ((t >> k) << (k + 1)) | (t & ((1u << k) - 1)), hi = lo + (1u << k);
      const uint64_t i0 = base + ((uint64_t)lo << sh_min);
      const uint64_t blk = i0 >> (sh + 1);
      const F128d u = g[sub][lo], v = g[sub][hi], sum = u + v;
      g[sub][lo] = sum;
      g[sub][hi] = blk == 0 ? v : v + mul_call(tw[(1ull << layer) - 1 + blk], sum);  // first block: twiddle zero
    }
    __syncthreads();
  }
  if (have && t < P) y[base + ((uint64_t)t << sh_min)] = g[sub][t];
}
uint32_t launch_lg_induced(const uint64_t* pos, const F128d* w, uint32_t n_q, uint32_t ln, uint32_t log_rate,
                           const F128d* tw, const F256d* f, F128d* y, F128d* basis, F128d* part, cudaStream_t s,
                           FusedPublish pub) {
  uint32_t log_d = ln + log_rate;
  CUDA_OK(cudaMemsetAsync(y, 0, (sizeof(F128d)) << log_d, s));
  lg_scatter_kernel<<<(n_q + 127) / 128, 128, 0, s>>>(pos, w, n_q, y);
  LAUNCH_OK();
  uint64_t pairs = 1ull << (log_d - 1);
  // transposed layers from log_d - 1 down to log_rate: for the small levels (launch-latency
  // bound) up to NTT_T_FUSED per launch; the large ones one per launch (their fused groups
  // would be strided and half the threads idle in every layer: slower, measured)
  const uint32_t per_launch = log_d <= NTT_T_FUSED_MAX_LOG ? NTT_T_FUSED : 1;
  for (int layer = (int)log_d - 1; layer >= (int)log_rate;) {
    const uint32_t nl = std::min<uint32_t>(per_launch, (uint32_t)(layer - (int)log_rate + 1));
    if (nl >= 2) {
      const uint64_t n_groups = 1ull << (log_d - nl);
      ntt_t_fused_kernel<<<(unsigned)((n_groups + 3) / 4), 256, 0, s>>>(y, log_d, (uint32_t)layer, nl, tw);
    } else {
      ntt_t_layer_kernel<<<(unsigned)((pairs + 255) / 256), 256, 0, s>>>(y, log_d, (uint32_t)layer, tw);
    }
    LAUNCH_OK();
    layer -= (int)nl;
  }
  uint64_t n = 1ull << ln;
  uint32_t blocks = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>((n + 255) / 256, (uint64_t)sm_count() * 8));
  lg_induced_fold_kernel<<<blocks, 256, 0, s>>>(y, ln, log_rate, f, basis, part, pub);
  LAUNCH_OK();
  return blocks;
}
// Glue a pending basis into b with weight beta.
//   eq mode      : b[i].c0 += beta * p[i]
//   induced mode : b[2i].c0 += beta * p[i], b[2i+1].c1 += beta * p[i]  (u * base = (0, base))
__global__ void lg_glue_kernel(F256d* __restrict__ b, const F128d* __restrict__ p, F128d beta, uint64_t n,
                               int induced) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  F128d v = beta * p[i];
  if (induced) {
    b[2 * i].c0 += v;
    b[2 * i + 1].c1 += v;
  } else {
    b[i].c0 += v;
  }
}
void launch_lg_glue(F256d* b, const F128d* p, F128d beta, uint64_t n, bool induced, cudaStream_t s) {
  lg_glue_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(b, p, beta, n, induced ? 1 : 0);
  LAUNCH_OK();
}

}  // namespace gpu
}  // namespace flock
