// Commitment kernels: the lane-major codeword fill, the additive NTT over GF(2^128)
// (LCH novel basis, neighbours-last: at layer l pairs are 2^(log_d - l - 1) apart and
// share the twiddle of their block; crates/flock-core/src/ntt/additive_ntt_f128.rs:
// 627-648), Merkle trees over codeword rows (crates/flock-core/src/merkle.rs:593-620)
// and the row / capped-path gathers of Ligerito openings
// (crates/flock-core/src/pcs/ligerito.rs:4582-4610, merkle.rs:663-690).
//
// Layout: codewords are position-major SoA, data[pos * lanes + lane]; a Merkle leaf is
// one position's `lanes` words. Trees are flat: leaves [0, N), then each level, root last.
#include "kernels.h"
#include "sha256.cuh"
#include <atomic>

namespace flock {
namespace gpu {

// cw[(rep * D + p) * lanes + l] = q[l * D + p]: 2^(log_pos - log_dim) replicas of the
// transposed lane-major stack (the state after the first log_inv_rate NTT layers).
// Tiled through shared memory: a 32-position x 32-lane tile per block.
__global__ void fill_lane_major_kernel(const F128d* __restrict__ q, F128d* __restrict__ cw, uint32_t lanes,
                                       uint32_t log_dim, uint64_t n_pos) {
  __shared__ F128d tile[32][33];
  uint64_t p0 = (uint64_t)blockIdx.x * 32;
  uint32_t l0 = blockIdx.y * 32;
  uint64_t D = 1ull << log_dim;
  // read: lane-major, consecutive threads -> consecutive positions
  for (int ly = threadIdx.y; ly < 32; ly += blockDim.y) {
    uint32_t l = l0 + ly;
    uint64_t p = p0 + threadIdx.x;
    if (l < lanes && p < n_pos) tile[ly][threadIdx.x] = q[(uint64_t)l * D + (p & (D - 1))];
  }
  __syncthreads();
  // write: position-major, consecutive threads -> consecutive lanes
  for (int py = threadIdx.y; py < 32; py += blockDim.y) {
    uint64_t p = p0 + py;
    uint32_t l = l0 + threadIdx.x;
    if (l < lanes && p < n_pos) cw[p * lanes + l] = tile[threadIdx.x][py];
  }
}

void launch_fill_lane_major(const F128d* q, F128d* cw, uint32_t lanes, uint32_t log_dim, uint32_t log_pos,
                            cudaStream_t s) {
  uint64_t n_pos = 1ull << log_pos;
  dim3 grid((unsigned)((n_pos + 31) / 32), (lanes + 31) / 32), block(32, 8);
  fill_lane_major_kernel<<<grid, block, 0, s>>>(q, cw, lanes, log_dim, n_pos);
  LAUNCH_OK();
}

// One butterfly layer: thread per (pair, lane). tw[(1 << layer) - 1 + block].
__global__ void ntt_layer_kernel(F128d* __restrict__ data, uint32_t lanes, uint32_t log_d, uint32_t layer,
                                 const F128d* __restrict__ tw) {
  uint64_t gid = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  uint64_t n_pairs = 1ull << (log_d - 1);
  if (gid >= n_pairs * lanes) return;
  uint64_t pair = gid / lanes;
  uint32_t l = (uint32_t)(gid - pair * lanes);
  uint32_t sh = log_d - layer - 1;
  uint64_t block = pair >> sh, within = pair & ((1ull << sh) - 1);
  uint64_t i0 = (block << (sh + 1)) + within, i1 = i0 + (1ull << sh);
  F128d t = tw[(1ull << layer) - 1 + block];
  F128d u = data[i0 * lanes + l], v = data[i1 * lanes + l];
  F128d nu = block == 0 ? u : u + v * t;  // the first block's twiddle is zero in every layer
  data[i0 * lanes + l] = nu;
  data[i1 * lanes + l] = v + nu;
}

// Table layers: butterfly layers whose twiddle blocks are large. Each block of a launch
// handles a contiguous share of one twiddle block's butterflies (2^cpb_log launch blocks
// per twiddle block), builds that twiddle's byte tables once and takes half of its
// products from them (load/store pipe), the other half from split twiddles (multiply
// pipe). The butterflies of twiddle block b of a layer are the contiguous element ranges
// u = [b 2^(sh+1) lanes, + 2^sh lanes) and v = u + 2^sh lanes, sh = log_d - layer - 1
// (lane-minor layout); the first twiddle block's twiddle is zero in every layer.
//
// Two layers per pass: twiddle block b of `layer` spans the quarters x0..x3 of
// Q = lanes 2^(sh-1) elements each; `layer` pairs (x0, x2) and (x1, x3) by t_b (table),
// layer + 1 pairs (x0, x1) by t_2b and (x2, x3) by t_2b+1 (split). One read and one write
// of the data per two layers.
__global__ void __launch_bounds__(256, 3)
ntt_layer2_tbl_kernel(F128d* __restrict__ data, uint32_t lanes, uint32_t log_d, uint32_t layer,
                      const F128d* __restrict__ tw, uint32_t cpb_log) {
  extern __shared__ __align__(16) F128d ttab[];  // build_byte_table's BYTE_TABLE_SMEM_ENTRIES
  __shared__ F128split s0, s1;
  const uint64_t b = blockIdx.x >> cpb_log, part = blockIdx.x & ((1ull << cpb_log) - 1);
  const uint32_t sh = log_d - layer - 1;
  const uint64_t Q = ((uint64_t)lanes) << (sh - 1);
  const uint64_t per = Q >> cpb_log;
  F128d* x = data + ((b << (sh + 1)) * lanes) + part * per;
  const bool zero = (b == 0);  // block-uniform: t_b and t_2b are zero
  if (threadIdx.x == 0) {
    s0 = split_factor(tw[(2ull << layer) - 1 + 2 * b]);
    s1 = split_factor(tw[(2ull << layer) - 1 + 2 * b + 1]);
  }
  if (!zero) build_byte_table(tw[(1ull << layer) - 1 + b], ttab);
  else __syncthreads();
  for (uint64_t k = threadIdx.x; k < per; k += blockDim.x) {
    F128d a0 = x[k], a1 = x[Q + k], a2 = x[2 * Q + k], a3 = x[3 * Q + k];
    if (!zero) {
      a0 += mul_table(a2, ttab);
      a1 += mul_table(a3, ttab);
    }
    a2 += a0;
    a3 += a1;
    if (!zero) a0 += mul_split(a1, s0);  // inline: 7-11 % faster than the out-of-line call here
    a1 += a0;
    a2 += mul_split(a3, s1);
    a3 += a2;
    x[k] = a0;
    x[Q + k] = a1;
    x[2 * Q + k] = a2;
    x[3 * Q + k] = a3;
  }
}
// One layer per pass (for an odd table layer): per thread and iteration one butterfly by
// table and one by the split twiddle, the next iteration's operands loaded before this
// one's products.
__global__ void __launch_bounds__(256, 2)
ntt_layer_tbl_kernel(F128d* __restrict__ data, uint32_t lanes, uint32_t log_d, uint32_t layer,
                     const F128d* __restrict__ tw, uint32_t cpb_log) {
  extern __shared__ __align__(16) F128d ttab[];  // build_byte_table's BYTE_TABLE_SMEM_ENTRIES
  __shared__ F128split ts;
  const uint64_t b = blockIdx.x >> cpb_log, part = blockIdx.x & ((1ull << cpb_log) - 1);
  const uint32_t sh = log_d - layer - 1;
  const uint64_t M = ((uint64_t)lanes) << sh;  // butterflies of twiddle block b
  const uint64_t per = M >> cpb_log;           // this block's share (even: cpb_log < sh)
  F128d* u = data + ((b << (sh + 1)) * lanes) + part * per;
  F128d* v = u + M;
  const bool zero = (b == 0);  // block-uniform
  if (!zero) {
    const F128d t = tw[(1ull << layer) - 1 + b];
    if (threadIdx.x == 0) ts = split_factor(t);
    build_byte_table(t, ttab);
  }
  const uint64_t half = per / 2;
  uint64_t k = threadIdx.x;
  F128d u0, v0, u1, v1;
  if (k < half) {
    u0 = u[k];
    v0 = v[k];
    u1 = u[half + k];
    v1 = v[half + k];
  }
  for (; k < half; k += blockDim.x) {
    const uint64_t kn = k + blockDim.x;
    F128d p0, q0, p1, q1;
    if (kn < half) {
      p0 = u[kn];
      q0 = v[kn];
      p1 = u[half + kn];
      q1 = v[half + kn];
    }
    const F128d n0 = zero ? u0 : u0 + mul_table(v0, ttab);
    const F128d n1 = zero ? u1 : u1 + mul_split_call(v1, &ts);
    u[k] = n0;
    v[k] = v0 + n0;
    u[half + k] = n1;
    v[half + k] = v1 + n1;
    u0 = p0;
    v0 = q0;
    u1 = p1;
    v1 = q1;
  }
}
// A layer is a table layer while its twiddle blocks hold at least this many butterflies
// (a table build costs about as much shared-memory traffic as 300 table products), each
// launch block getting at least NTT_TBL_MIN_BLOCK_BUTTERFLIES of them, and while the
// transform is large enough to give every SM two such launch blocks.
constexpr uint64_t NTT_TBL_MIN_TWIDDLE_BUTTERFLIES = uint64_t(1) << 11;
constexpr uint64_t NTT_TBL_MIN_BLOCK_BUTTERFLIES = uint64_t(1) << 12;

// Several consecutive layers [layer, layer + nl) fused through shared memory. A block
// owns 2^nl positions spaced 2^(log_d - layer - nl) apart (one residue class inside a
// block of the first fused layer) for a slice of lanes; each fused layer pairs positions
// within that set. Fused layer k meets 2^k twiddles; the block stages all 2^nl - 1 of them
// once, already split for mul_split, after the positions' data.
constexpr uint32_t NTT_MAX_THREADS = 320;  // with 3 blocks per SM: at most 64 registers a thread
template <int NL>
__global__ void __launch_bounds__(NTT_MAX_THREADS, 3)
ntt_fused_kernel(F128d* __restrict__ data, uint32_t lanes, uint32_t log_d, uint32_t layer, const F128d* __restrict__ tw,
                 uint32_t lane_tile) {
  extern __shared__ F128d sm[];  // [2^NL][lane_tile], then F128split[2^NL - 1]
  const uint32_t P = 1u << NL;
  F128split* tws = reinterpret_cast<F128split*>(sm + P * lane_tile);
  uint32_t stride_log = log_d - layer - NL;  // spacing of the positions in this group
  uint64_t n_groups = 1ull << (log_d - NL);
  uint64_t lane_tiles = (lanes + lane_tile - 1) / lane_tile;
  uint64_t gidx = blockIdx.x / lane_tiles;
  uint32_t lt = (uint32_t)(blockIdx.x % lane_tiles);
  if (gidx >= n_groups) return;
  // group -> (outer block of the first fused layer, residue within stride)
  uint64_t outer = gidx >> stride_log, resid = gidx & ((1ull << stride_log) - 1);
  uint64_t base = (outer << (stride_log + NL)) + resid;
  uint32_t l0 = lt * lane_tile;
  uint32_t nl_here = min(lane_tile, lanes - l0);
  // twiddle (k, blk) at tws[2^k - 1 + blk]: its global block at layer + k is (outer << k) + blk
  for (uint32_t t = threadIdx.x; t < P - 1; t += blockDim.x) {
    const uint32_t k = 31 - __clz(t + 1), blk = t + 1 - (1u << k);
    const F128d v = tw[(1ull << (layer + k)) - 1 + (outer << k) + blk];
    const uint64_t hl[3] = {v.lo, v.hi, v.lo ^ v.hi};
#pragma unroll
    for (int q = 0; q < 3; ++q) {  // split_factor(v), stored as it is formed
      const uint32_t y0 = (uint32_t)hl[q], y1 = (uint32_t)(hl[q] >> 32);
      split_classes(y0, tws[t].w[3 * q]);
      split_classes(y1, tws[t].w[3 * q + 1]);
      split_classes(y0 ^ y1, tws[t].w[3 * q + 2]);
    }
  }
  for (uint32_t i = threadIdx.x; i < P * nl_here; i += blockDim.x) {
    uint32_t pos = i / nl_here, l = i - pos * nl_here;
    sm[pos * lane_tile + l] = data[(base + ((uint64_t)pos << stride_log)) * lanes + l0 + l];
  }
  __syncthreads();
  // (pair, lane) of this thread's first butterfly and the step between its butterflies
  const uint32_t pr0 = threadIdx.x / nl_here, ln0 = threadIdx.x - pr0 * nl_here;
  const uint32_t dpr = blockDim.x / nl_here, dln = blockDim.x - dpr * nl_here;
#pragma unroll
  for (int k = 0; k < NL; ++k) {
    const uint32_t half = P >> (k + 1);  // pairing distance inside the group (in group positions)
    uint32_t pr = pr0, l = ln0;
    for (uint32_t i = threadIdx.x; i < (P / 2) * nl_here; i += blockDim.x) {
      uint32_t blk = pr / half, w = pr - blk * half;
      uint32_t i0 = blk * 2 * half + w, i1 = i0 + half;
      F128d u = sm[i0 * lane_tile + l], v = sm[i1 * lane_tile + l];
      // the first block's twiddle is zero in every layer
      F128d nu = (outer == 0 && blk == 0) ? u : u + mul_split(v, tws[(1u << k) - 1 + blk]);
      sm[i0 * lane_tile + l] = nu;
      sm[i1 * lane_tile + l] = v + nu;
      pr += dpr;
      l += dln;
      if (l >= nl_here) {
        l -= nl_here;
        ++pr;
      }
    }
    __syncthreads();
  }
  for (uint32_t i = threadIdx.x; i < P * nl_here; i += blockDim.x) {
    uint32_t pos = i / nl_here, l = i - pos * nl_here;
    data[(base + ((uint64_t)pos << stride_log)) * lanes + l0 + l] = sm[pos * lane_tile + l];
  }
}

// Threads per fused-NTT block for a lane tile: among the multiples of 32 in [192, 320], the
// one with the most busy resident warps per SM (resident warps, capped at 32, times the
// fraction of threads with a butterfly in a layer's passes). Cached per device and tile.
template <int NL>
static uint32_t ntt_block_threads(uint32_t lane_tile, size_t smem) {
  static std::atomic<uint32_t> cache[MAX_DEVICES][65];
  int dev = 0;
  CUDA_OK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= MAX_DEVICES || lane_tile > 64) throw std::runtime_error("fused NTT: bad device or lane tile");
  uint32_t best = cache[dev][lane_tile].load(std::memory_order_relaxed);
  if (best) return best;
  const uint32_t butterflies = (1u << (NL - 1)) * lane_tile;
  double best_score = -1.0;
  for (uint32_t t = 192; t <= NTT_MAX_THREADS; t += 32) {
    int blocks = 0;
    CUDA_OK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, ntt_fused_kernel<NL>, (int)t, smem));
    const uint32_t passes = (butterflies + t - 1) / t;
    const double score = std::min(blocks * t / 32.0, 32.0) * butterflies / (double)(passes * t);
    if (score > best_score + 1e-9) {
      best_score = score;
      best = t;
    }
  }
  cache[dev][lane_tile].store(best, std::memory_order_relaxed);
  return best;
}

void launch_ntt(F128d* data, uint32_t lanes, uint32_t log_d, uint32_t start_layer, const F128d* tw, cudaStream_t s) {
  const int NL = 6;  // layers fused per pass
  uint32_t layer = start_layer;
  uint32_t lane_tile = lanes < 64 ? lanes : 64;
  const size_t tw_bytes = ((1u << NL) - 1) * sizeof(F128split);
  // the top layers, whose twiddles are each shared by many butterflies: table layers, two
  // per launch
  const uint64_t butterflies = (uint64_t)lanes << (log_d - 1);
  const bool tables = butterflies >= (uint64_t)sm_count() * 2 * NTT_TBL_MIN_BLOCK_BUTTERFLIES;
  auto table_layer = [&](uint32_t l) {
    return tables && l + 1 < log_d && ((uint64_t)lanes << (log_d - l - 1)) >= NTT_TBL_MIN_TWIDDLE_BUTTERFLIES;
  };
  // launch blocks per twiddle block: about eight per SM in all, and each with at least
  // NTT_TBL_MIN_BLOCK_BUTTERFLIES of the `share` butterflies of its twiddle block
  auto blocks_log = [&](uint32_t l, uint64_t share, uint32_t max_log) {
    uint32_t c = 0;
    while (c < max_log && ((uint64_t)1 << (l + c + 1)) <= (uint64_t)sm_count() * 8 &&
           (share >> (c + 1)) >= NTT_TBL_MIN_BLOCK_BUTTERFLIES)
      ++c;
    return c;
  };
  const int tbl_smem = (int)(BYTE_TABLE_SMEM_ENTRIES * sizeof(F128d));
  while (table_layer(layer)) {
    const uint32_t sh = log_d - layer - 1;
    if (table_layer(layer + 1) && sh >= 2) {
      // radix-4 units of 4 elements; a block's share counted in butterflies (2 per unit)
      const uint32_t c = blocks_log(layer, (uint64_t)lanes << sh, sh - 1);
      set_dynamic_smem((const void*)ntt_layer2_tbl_kernel, tbl_smem);
      ntt_layer2_tbl_kernel<<<(unsigned)(1ull << (layer + c)), 256, tbl_smem, s>>>(data, lanes, log_d, layer, tw, c);
      LAUNCH_OK();
      layer += 2;
    } else {
      const uint32_t c = blocks_log(layer, (uint64_t)lanes << sh, sh - 1);
      set_dynamic_smem((const void*)ntt_layer_tbl_kernel, tbl_smem);
      ntt_layer_tbl_kernel<<<(unsigned)(1ull << (layer + c)), 256, tbl_smem, s>>>(data, lanes, log_d, layer, tw, c);
      LAUNCH_OK();
      layer += 1;
    }
  }
  while (layer < log_d) {
    uint32_t remaining = log_d - layer;
    if (remaining >= (uint32_t)NL) {
      uint64_t n_groups = 1ull << (log_d - NL);
      uint64_t lane_tiles = (lanes + lane_tile - 1) / lane_tile;
      size_t smem = (size_t)(1u << NL) * lane_tile * sizeof(F128d) + tw_bytes;
      set_dynamic_smem((const void*)ntt_fused_kernel<NL>, (int)((1u << NL) * 64 * sizeof(F128d) + tw_bytes));
      const uint32_t threads = ntt_block_threads<NL>(lane_tile, smem);
      ntt_fused_kernel<NL><<<(unsigned)(n_groups * lane_tiles), threads, smem, s>>>(data, lanes, log_d, layer, tw,
                                                                                     lane_tile);
      LAUNCH_OK();
      layer += NL;
    } else {
      uint64_t work = (1ull << (log_d - 1)) * lanes;
      ntt_layer_kernel<<<(unsigned)((work + 255) / 256), 256, 0, s>>>(data, lanes, log_d, layer, tw);
      LAUNCH_OK();
      layer += 1;
    }
  }
}

// ---- Merkle
__global__ void merkle_leaves_kernel(const F128d* __restrict__ rows, uint32_t lanes, uint64_t n_leaves,
                                     uint32_t* __restrict__ tree) {
  uint64_t p = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n_leaves) return;
  const uint32_t* w = (const uint32_t*)(rows + p * lanes);
  uint32_t out[8];
  sha256_words([&](uint32_t i) { return __ldg(w + i); }, lanes * 4, out);
#pragma unroll
  for (int i = 0; i < 8; ++i) tree[p * 8 + i] = out[i];
}
__global__ void merkle_level_kernel(uint32_t* __restrict__ tree, uint64_t in_off, uint64_t n_out) {
  uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_out) return;
  const uint32_t* l = tree + (in_off + 2 * i) * 8;
  uint32_t out[8];
  sha256_words([&](uint32_t k) { return l[k]; }, 16, out);
  uint64_t o = in_off + 2 * n_out + i;
#pragma unroll
  for (int k = 0; k < 8; ++k) tree[o * 8 + k] = out[k];
}
// The top of the tree, from a level of n_in <= MERKLE_TOP_NODES nodes up to the level of
// n_cap nodes (the cap), in one block: each level's nodes are hashed by the block's
// threads, then a barrier.
constexpr uint32_t MERKLE_TOP_NODES = 2048;
__global__ void __launch_bounds__(1024) merkle_top_kernel(uint32_t* __restrict__ tree, uint64_t in_off, uint32_t n_in,
                                                         uint32_t n_cap) {
  uint64_t off = in_off;
  for (uint32_t len = n_in; len > n_cap; len /= 2) {
    const uint32_t nout = len / 2;
    for (uint32_t i = threadIdx.x; i < nout; i += blockDim.x) {
      const uint32_t* l = tree + (off + 2 * (uint64_t)i) * 8;
      uint32_t out[8];
      sha256_words([&](uint32_t k) { return l[k]; }, 16, out);
      const uint64_t o = off + len + i;
#pragma unroll
      for (int k = 0; k < 8; ++k) tree[o * 8 + k] = out[k];
    }
    __syncthreads();
    off += len;
  }
}
void launch_merkle(const F128d* rows, uint32_t lanes, uint64_t n_leaves, uint32_t cap_depth, uint8_t* tree,
                   cudaStream_t s) {
  // levels above the cap are never read (the cap is the commitment, paths stop below it)
  const uint64_t n_cap = uint64_t(1) << cap_depth;
  if (n_cap > n_leaves) throw std::runtime_error("Merkle cap wider than the leaf level");
  merkle_leaves_kernel<<<(unsigned)((n_leaves + 127) / 128), 128, 0, s>>>(rows, lanes, n_leaves, (uint32_t*)tree);
  LAUNCH_OK();
  uint64_t off = 0, len = n_leaves;
  while (len > MERKLE_TOP_NODES && len > n_cap) {
    uint64_t nout = len / 2;
    merkle_level_kernel<<<(unsigned)((nout + 127) / 128), 128, 0, s>>>((uint32_t*)tree, off, nout);
    LAUNCH_OK();
    off += len;
    len = nout;
  }
  if (len > n_cap) {
    merkle_top_kernel<<<1, 1024, 0, s>>>((uint32_t*)tree, off, (uint32_t)len, (uint32_t)n_cap);
    LAUNCH_OK();
  }
}

// ---- transcript proof of work (challenger.rs:1100-1140): the smallest nonce in
// [start, start + count) whose SHA256(digest || nonce_le) has `bits` leading zero bits,
// or ~0. Each block folds its minimum into *dmin; the last block to
// finish (ticket counter) reads and resets *dmin, writes the result to mapped host memory,
// then the sequence number, and resets the counter: one launch per search, no copies.
__global__ void __launch_bounds__(256) pow_kernel(uint4 dlo, uint4 dhi, uint32_t bits, uint64_t start, uint64_t count,
                                                  unsigned long long* dmin, uint32_t* counter, unsigned long long* out,
                                                  uint32_t* flag, uint32_t seq) {
  __shared__ unsigned long long bmin;
  __shared__ uint32_t ticket;
  if (threadIdx.x == 0) bmin = ~0ull;
  __syncthreads();
  const uint64_t i = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < count) {
    const uint64_t nonce = start + i;
    uint32_t w[16];
    w[0] = bswap32(dlo.x); w[1] = bswap32(dlo.y); w[2] = bswap32(dlo.z); w[3] = bswap32(dlo.w);
    w[4] = bswap32(dhi.x); w[5] = bswap32(dhi.y); w[6] = bswap32(dhi.z); w[7] = bswap32(dhi.w);
    w[8] = bswap32((uint32_t)nonce);
    w[9] = bswap32((uint32_t)(nonce >> 32));
    w[10] = 0x80000000u;
#pragma unroll
    for (int k = 11; k < 15; ++k) w[k] = 0;
    w[15] = 320;
    uint32_t st[8];
    sha256_init(st);
    sha256_compress(st, w);
    bool ok = true;
    uint32_t need = bits;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      if (need >= 32) { ok &= st[k] == 0; need -= 32; }
      else if (need > 0) { ok &= (st[k] >> (32 - need)) == 0; need = 0; }
    }
    if (ok) atomicMin(&bmin, (unsigned long long)nonce);
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    if (bmin != ~0ull) atomicMin(dmin, bmin);
    __threadfence();
    ticket = atomicAdd(counter, 1u);
  }
  __syncthreads();
  if (threadIdx.x == 0 && ticket == gridDim.x - 1) {
    __threadfence();
    const unsigned long long m = atomicExch(dmin, ~0ull);
    *counter = 0;
    *(volatile unsigned long long*)out = m;
    __threadfence_system();
    *(volatile uint32_t*)flag = seq;
  }
}
void launch_pow(const uint32_t digest_le[8], uint32_t bits, uint64_t start, uint64_t count, unsigned long long* d_min,
                uint32_t* d_counter, unsigned long long* out, uint32_t* flag, uint32_t seq, cudaStream_t s) {
  uint4 lo = make_uint4(digest_le[0], digest_le[1], digest_le[2], digest_le[3]);
  uint4 hi = make_uint4(digest_le[4], digest_le[5], digest_le[6], digest_le[7]);
  pow_kernel<<<(unsigned)((count + 255) / 256), 256, 0, s>>>(lo, hi, bits, start, count, d_min, d_counter, out, flag,
                                                             seq);
  LAUNCH_OK();
}

// ---- openings
__global__ void gather_rows_kernel(const F128d* __restrict__ mat, uint32_t lanes, const uint64_t* __restrict__ pos,
                                   uint32_t n, F128d* __restrict__ out) {
  uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n * lanes) return;
  uint32_t q = i / lanes, l = i - q * lanes;
  out[i] = mat[pos[q] * lanes + l];
}
void launch_gather_rows(const F128d* mat, uint32_t lanes, const uint64_t* d_pos, uint32_t n, F128d* out,
                        cudaStream_t s) {
  uint32_t work = n * lanes;
  gather_rows_kernel<<<(work + 255) / 256, 256, 0, s>>>(mat, lanes, d_pos, n, out);
  LAUNCH_OK();
}
__global__ void gather_paths_kernel(const uint8_t* __restrict__ tree, uint64_t n_leaves,
                                    const uint64_t* __restrict__ pos, uint32_t n, uint32_t cap_depth,
                                    uint8_t* __restrict__ out) {
  uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= n) return;
  uint32_t depth = 0;
  while ((1ull << depth) < n_leaves) ++depth;
  uint32_t plen = depth - cap_depth;
  uint64_t start = 0, len = n_leaves, idx = pos[q];
  for (uint32_t k = 0; k < plen; ++k) {  // 32-byte nodes: two 16-byte copies (tree and out are 16-byte aligned)
    const uint4* src = reinterpret_cast<const uint4*>(tree + (start + (idx ^ 1)) * 32);
    uint4* dst = reinterpret_cast<uint4*>(out + ((uint64_t)q * plen + k) * 32);
    dst[0] = src[0];
    dst[1] = src[1];
    start += len;
    len >>= 1;
    idx >>= 1;
  }
}
void launch_gather_paths(const uint8_t* tree, uint64_t n_leaves, const uint64_t* d_pos, uint32_t n,
                         uint32_t cap_depth, uint8_t* out, cudaStream_t s) {
  gather_paths_kernel<<<(n + 127) / 128, 128, 0, s>>>(tree, n_leaves, d_pos, n, cap_depth, out);
  LAUNCH_OK();
}

}  // namespace gpu
}  // namespace flock
