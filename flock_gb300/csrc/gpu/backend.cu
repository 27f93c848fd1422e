// The device backend of prove_fast: owns every witness-sized buffer in HBM for the
// life of a setup (z, a, b, the L0 codeword and tree, the zerocheck / merged-open fold
// buffers, the Ligerito F256 state and level codewords) and runs each bulk step of the
// protocol as sm_103a kernels on one stream. The host keeps only the transcript and the
// O(m)-sized arithmetic between rounds; every round message comes back as a handful of
// field elements.
#include "backend.h"
#include "../host/tables.h"
#include <atomic>
#include <thread>

namespace flock {
namespace gpu {

namespace {

// Constant tables are per device (module constants and cudaMalloc'd tables live in each
// device's context); a process may drive several devices.
std::mutex g_consts_mu;
bool g_consts_done[MAX_DEVICES] = {};
void upload_constants_once() {
  int dev = 0;
  CUDA_OK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= MAX_DEVICES) throw std::runtime_error("device index out of range");
  std::lock_guard<std::mutex> g(g_consts_mu);
  if (g_consts_done[dev]) return;
  [] {
    const SkipTables& st = skip_tables();
    // eq factor of the three small zerocheck constants (bit j of K selects c_j or 1 + c_j)
    const uint8_t c[3] = {0xF7, 0x53, 0xB5};
    uint8_t mulk[8][256], e2[4];
    for (int K = 0; K < 8; ++K) {
      uint8_t e = 1;
      for (int j = 0; j < 3; ++j) e = gf8_mul(e, ((K >> j) & 1) ? c[j] : (uint8_t)(c[j] ^ 1));
      for (int v = 0; v < 256; ++v) mulk[K][v] = gf8_mul(e, (uint8_t)v);
    }
    for (int K2 = 0; K2 < 4; ++K2) {
      uint8_t e = 1;
      for (int j = 0; j < 2; ++j) e = gf8_mul(e, ((K2 >> j) & 1) ? c[j + 1] : (uint8_t)(c[j + 1] ^ 1));
      e2[K2] = e;
    }
    // word 4M + K2 of an xo carries eq weight x^M * phi8(e2[K2]) (times D * eq_o(xo))
    F128 wconst[64];
    for (int M = 0; M < 16; ++M) {
      F128 xm = F128::one();
      for (int i = 0; i < M; ++i) xm = mul_by_x(xm);
      for (int K2 = 0; K2 < 4; ++K2) wconst[4 * M + K2] = xm * phi8(e2[K2]);
    }
    upload_zc_consts(st.ext.data(), reinterpret_cast<const F128d*>(phi8_table().data()), mulk,
                     reinterpret_cast<const F128d*>(wconst));
    upload_witness_constants();
  }();
  g_consts_done[dev] = true;
}

inline F128d dev(F128 v) { F128d r; r.lo = v.lo; r.hi = v.hi; return r; }
inline F256d dev(F256 v) { F256d r; r.c0 = dev(v.c0); r.c1 = dev(v.c1); return r; }
inline F128 host(F128d v) { return F128(v.lo, v.hi); }

}  // namespace

template <class T>
static T* dmalloc(size_t n, std::vector<void*>& owned, uint64_t& counter) {
  void* p = nullptr;
  if (n == 0) n = 1;
  CUDA_OK(cudaMalloc(&p, n * sizeof(T)));
  owned.push_back(p);
  counter += n * sizeof(T);
  return static_cast<T*>(p);
}

// Entries of the split eq tables of the skip fold (over L coordinates) and of every
// later zerocheck fold round (over the suffixes of L - 1, L - 2, ..., 0 coordinates).
// Round i splits its n = L - 1 - i coordinates as lo + hi with lo = zc_round_lo_bits(n).
static uint32_t zc_round_lo_bits(uint32_t n) {
  // chunks of 2^10 pairs where the round has enough of them for the table form, else of
  // 2^8 (one pair per thread: four times the blocks of a small, latency-bound round)
  return std::min(n, n >= 17 ? 10u : 8u);
}
static uint64_t zc_tables_entries(uint32_t L) {
  uint64_t total = (uint64_t(1) << 10) + (uint64_t(1) << (L - 10));
  for (uint32_t i = 0; i < L; ++i) {
    uint32_t n = L - 1 - i, lo = zc_round_lo_bits(n);
    total += (uint64_t(1) << lo) + (uint64_t(1) << (n - lo));
  }
  return total;
}

// Device bytes a backend for this statement holds after its first prove (the buffers of
// the constructor, the Ligerito level codewords and trees, the twiddle tables).
uint64_t GpuBackend::estimate_device_bytes(const Statement& S) {
  const uint64_t W = uint64_t(1) << (S.m - 7), K = uint64_t(1) << S.k_log, n_pos = uint64_t(1) << S.k_code;
  uint64_t b = 0;
  for (const SlotInfo& t : S.slots) b += t.count * input_record_bytes(t.hash);
  b += 3 * W * 16;                          // z, a, b
  if (!S.identity) b += S.committed_words * 16;  // the compacted stack
  b += n_pos * S.lanes * 16 + 2 * n_pos * 32;  // L0 codeword and tree
  b += (W / 2 * 2 + W * 2 + 64) * 16;       // zerocheck folds
  b += zc_tables_entries(S.m - 7) * 16;
  b += 6 * K * 16;                          // lincheck vectors
  for (const SlotInfo& t : S.slots) {
    b += 2 * (uint64_t(16) << t.k_log);
    if (t.csc_a) b += 4 * (t.csc_a->col_ptr.size() + t.csc_a->rows_flat.size() + t.csc_b->col_ptr.size() + t.csc_b->rows_flat.size());
  }
  b += (W + W + W / 2) * 16;                // merged weight and fold buffers
  b += W * 16 + 4 * (W / 2) * 32 + (W / 2) * 16;  // Ligerito basis, f/b ping-pong, pending
  b += (uint64_t(1) << 20) * 16 + 4096 * 16 + (size_t(96) << 20) + (size_t(8) << 20);  // partials, scratch, staging
  b += n_pos * 16;                          // L0 twiddles
  // recursive levels: codeword 2^(log_cols + rate) x 2^k, tree, twiddles
  const LigeritoParams& P = S.lig;
  uint32_t split_dim = (P.log_n - P.initial_k) + 1;
  for (uint32_t i = 0; i < P.r; ++i) {
    uint32_t k = P.recursive_ks[i], rate = P.log_inv_rates[i + 1];
    uint32_t log_cols = split_dim - k;
    uint64_t bl = uint64_t(1) << (log_cols + rate);
    b += bl * (uint64_t(1) << k) * 16 + 2 * bl * 32 + bl * 16;
    split_dim = (split_dim - k) + 1;
  }
  return b;
}

GpuBackend::GpuBackend(const Statement& s) : S(s) {
  CUDA_OK(cudaGetDevice(&device_));
  CUDA_OK(cudaStreamCreateWithFlags(&st_, cudaStreamNonBlocking));
  upload_constants_once();
  W_ = uint64_t(1) << (S.m - 7);
  K_ = 1u << S.k_log;
  zc_live_words_ = (S.slots.size() == 1 && S.slots[0].offset == 0)
                       ? std::min<uint64_t>(W_, S.slots[0].used_cols << S.nu)
                       : W_;
  const uint64_t W = W_;
  in_bytes_ = 0;
  for (const SlotInfo& t : S.slots) in_bytes_ += (size_t)t.count * input_record_bytes(t.hash);
  in_bytes_ = std::max<size_t>(in_bytes_, 16);
  d_in_ = dmalloc<uint8_t>(in_bytes_, owned_, device_bytes_);
  CUDA_OK(cudaMallocHost(&h_in_, in_bytes_));
  z_ = dmalloc<F128d>(W, owned_, device_bytes_);
  a_ = dmalloc<F128d>(W, owned_, device_bytes_);
  b_ = dmalloc<F128d>(W, owned_, device_bytes_);
  // chunk columns the witness never writes stay zero for the life of the backend
  CUDA_OK(cudaMemset(z_, 0, W * 16));
  CUDA_OK(cudaMemset(a_, 0, W * 16));
  CUDA_OK(cudaMemset(b_, 0, W * 16));
  n_pos0_ = uint64_t(1) << S.k_code;
  cw0_ = dmalloc<F128d>(n_pos0_ * S.lanes, owned_, device_bytes_);
  tree0_ = dmalloc<uint8_t>((2 * n_pos0_) * 32, owned_, device_bytes_);
  // fold buffers: round 2 writes W words per vector (zc2), later rounds alternate (zc1, zc2)
  zc1a_ = dmalloc<F128d>(W / 2, owned_, device_bytes_);
  zc1b_ = dmalloc<F128d>(W / 2, owned_, device_bytes_);
  zc2a_ = dmalloc<F128d>(W, owned_, device_bytes_);
  zc2b_ = dmalloc<F128d>(W, owned_, device_bytes_);
  zc_w64_ = dmalloc<F128d>(64, owned_, device_bytes_);
  comb_ = dmalloc<F128d>(K_, owned_, device_bytes_);
  zv_ = dmalloc<F128d>(K_, owned_, device_bytes_);
  zvcap_ = dmalloc<F128d>(K_, owned_, device_bytes_);
  uint32_t k_max = 0;
  for (const SlotInfo& t : S.slots) {
    SlotDev sd;
    sd.K = 1u << t.k_log;
    k_max = std::max(k_max, sd.K);
    sd.ca = dmalloc<F128d>(sd.K, owned_, device_bytes_);
    sd.cb = dmalloc<F128d>(sd.K, owned_, device_bytes_);
    if (t.hash != HASH_KECCAK) {
      const Csc& A = *t.csc_a;
      const Csc& B = *t.csc_b;
      sd.cola = dmalloc<uint32_t>(A.col_ptr.size(), owned_, device_bytes_);
      sd.rowa = dmalloc<uint32_t>(A.rows_flat.size(), owned_, device_bytes_);
      sd.colb = dmalloc<uint32_t>(B.col_ptr.size(), owned_, device_bytes_);
      sd.rowb = dmalloc<uint32_t>(B.rows_flat.size(), owned_, device_bytes_);
      CUDA_OK(cudaMemcpy(sd.cola, A.col_ptr.data(), A.col_ptr.size() * 4, cudaMemcpyHostToDevice));
      CUDA_OK(cudaMemcpy(sd.rowa, A.rows_flat.data(), A.rows_flat.size() * 4, cudaMemcpyHostToDevice));
      CUDA_OK(cudaMemcpy(sd.colb, B.col_ptr.data(), B.col_ptr.size() * 4, cudaMemcpyHostToDevice));
      CUDA_OK(cudaMemcpy(sd.rowb, B.rows_flat.data(), B.rows_flat.size() * 4, cudaMemcpyHostToDevice));
    }
    slot_dev_.push_back(sd);
  }
  eqi_ = dmalloc<F128d>(k_max, owned_, device_bytes_);
  ca_ = slot_dev_[0].ca;
  cb_ = slot_dev_[0].cb;
  Q_ = S.committed_words;
  q_ = S.identity ? z_ : dmalloc<F128d>(Q_, owned_, device_bytes_);
  mw_ = dmalloc<F128d>(W, owned_, device_bytes_);
  moAq_ = dmalloc<F128d>(W / 2, owned_, device_bytes_);
  moAw_ = dmalloc<F128d>(W / 2, owned_, device_bytes_);
  moBq_ = dmalloc<F128d>(W / 4, owned_, device_bytes_);
  moBw_ = dmalloc<F128d>(W / 4, owned_, device_bytes_);
  lb128_ = dmalloc<F128d>(W, owned_, device_bytes_);
  for (int k = 0; k < 2; ++k) {
    lf_[k] = dmalloc<F256d>(W / 2, owned_, device_bytes_);
    lb_[k] = dmalloc<F256d>(W / 2, owned_, device_bytes_);
  }
  pend_ = dmalloc<F128d>(W / 2, owned_, device_bytes_);
  part_cap_ = 1u << 20;
  part_ = dmalloc<F128d>(part_cap_, owned_, device_bytes_);
  red_ = dmalloc<F128d>(4096, owned_, device_bytes_);
  CUDA_OK(cudaMallocHost(&h_red_, 4096 * sizeof(F128d)));
  scr_cap_ = size_t(96) << 20;
  scr_ = dmalloc<uint8_t>(scr_cap_, owned_, device_bytes_);
  stage_cap_ = size_t(8) << 20;
  d_stage_ = dmalloc<uint8_t>(stage_cap_, owned_, device_bytes_);
  CUDA_OK(cudaMallocHost(&h_stage_, stage_cap_));
  CUDA_OK(cudaHostAlloc(&h_pub_, 64 * sizeof(F128d), cudaHostAllocMapped));
  CUDA_OK(cudaHostGetDevicePointer(&d_pub_, h_pub_, 0));
  CUDA_OK(cudaHostAlloc(&h_flag_, 64, cudaHostAllocMapped));
  CUDA_OK(cudaHostGetDevicePointer(&d_flag_, h_flag_, 0));
  *(volatile uint32_t*)h_flag_ = 0;
  pub_counter_ = dmalloc<uint32_t>(1, owned_, device_bytes_);
  CUDA_OK(cudaMemsetAsync(pub_counter_, 0, sizeof(uint32_t), st_));
  zc_tabs_cap_ = zc_tables_entries(S.m - 7);
  zc_tabs_ = dmalloc<F128d>(zc_tabs_cap_, owned_, device_bytes_);
  CUDA_OK(cudaStreamCreateWithFlags(&pow_st_, cudaStreamNonBlocking));
  d_pow_ = dmalloc<unsigned long long>(1, owned_, device_bytes_);
  CUDA_OK(cudaMemset(d_pow_, 0xFF, sizeof(unsigned long long)));
  pow_counter_ = dmalloc<uint32_t>(1, owned_, device_bytes_);
  CUDA_OK(cudaMemset(pow_counter_, 0, sizeof(uint32_t)));
  CUDA_OK(cudaHostAlloc(&h_pow_, sizeof(unsigned long long), cudaHostAllocMapped));
  CUDA_OK(cudaHostGetDevicePointer(&d_pow_out_, h_pow_, 0));
  CUDA_OK(cudaHostAlloc(&h_pow_flag_, 64, cudaHostAllocMapped));
  CUDA_OK(cudaHostGetDevicePointer(&d_pow_flag_, h_pow_flag_, 0));
  *(volatile uint32_t*)h_pow_flag_ = 0;
  // twiddles of the L0 transform; host tables used by every prove
  tw0_ = twiddles(S.k_code);
  (void)moore_inverse();
  CUDA_OK(cudaDeviceSynchronize());
}

GpuBackend::~GpuBackend() {
  cudaStreamSynchronize(st_);
  for (void* p : owned_) cudaFree(p);
  for (auto& kv : tw_) cudaFree(kv.second);
  for (auto& L : levels_) { cudaFree(L.mat); cudaFree(L.tree); }
  for (cudaEvent_t e : ev_pool_) cudaEventDestroy(e);
  cudaFreeHost(h_in_);
  cudaFreeHost(h_red_);
  cudaFreeHost(h_stage_);
  cudaFreeHost(h_pow_);
  cudaFreeHost(h_pow_flag_);
  cudaFreeHost(h_pub_);
  cudaFreeHost(h_flag_);
  cudaStreamDestroy(pow_st_);
  cudaStreamDestroy(st_);
}

const F128d* GpuBackend::twiddles(uint32_t log_d) {
  auto it = tw_.find(log_d);
  if (it != tw_.end()) return it->second;
  auto tw = ntt_twiddles(log_d);
  F128d* d = nullptr;
  CUDA_OK(cudaMalloc(&d, std::max<size_t>(1, tw.size()) * sizeof(F128d)));
  device_bytes_ += std::max<size_t>(1, tw.size()) * sizeof(F128d);
  // Ordered on this backend's stream: a plain cudaMemcpy from pageable memory may return
  // before its DMA lands, and kernels on a non-blocking stream are not ordered after it.
  CUDA_OK(cudaMemcpyAsync(d, tw.data(), tw.size() * sizeof(F128d), cudaMemcpyHostToDevice, st_));
  CUDA_OK(cudaStreamSynchronize(st_));
  tw_[log_d] = d;
  return d;
}

// ---- stage timing
const char* GpuBackend::stage_name(int s) {
  static const char* names[ST_COUNT] = {"witness", "l0_fill", "l0_ntt", "l0_merkle", "zc_round1", "zc_fold_skip",
                                        "zc_folds", "lincheck", "mo_build_w", "mo_rounds", "ligerito", "lg_ntt",
                                        "lg_merkle"};
  return (s >= 0 && s < ST_COUNT) ? names[s] : "?";
}
cudaEvent_t GpuBackend::event() {
  if (ev_used_ == ev_pool_.size()) {
    cudaEvent_t e;
    CUDA_OK(cudaEventCreate(&e));
    ev_pool_.push_back(e);
  }
  return ev_pool_[ev_used_++];
}
GpuBackend::Mark::Mark(GpuBackend* be, int stage) : b(be), st(stage), l0(launch_count()) {
  if ((b->timing_mask_ >> st) & 1) {
    cudaEvent_t a = b->event();
    CUDA_OK(cudaEventRecord(a, b->st_));
    b->spans_.push_back({st, a, nullptr, 0});
  }
}
GpuBackend::Mark::~Mark() {
  if (((b->timing_mask_ >> st) & 1) && !b->spans_.empty()) {
    cudaEvent_t e = b->event();
    if (cudaEventRecord(e, b->st_) == cudaSuccess) {
      b->spans_.back().b = e;
      b->spans_.back().launches = launch_count() - l0;
    }
  }
}
void GpuBackend::begin_prove(const void* d_inputs) {
  lg_pend_fold_.active = false;
  lg_pend_switch_ = false;
  lg_pend_basis_ = false;
  d_user_inputs_ = d_inputs;
  h2d_ = d2h_ = 0;
  spans_.clear();
  ev_used_ = 0;
}
void GpuBackend::stage_ms(double out[ST_COUNT], uint32_t launches[ST_COUNT]) {
  for (int i = 0; i < ST_COUNT; ++i) { out[i] = 0; launches[i] = 0; }
  CUDA_OK(cudaStreamSynchronize(st_));
  for (auto& sp : spans_) {
    if (!sp.b) continue;
    float ms = 0;
    CUDA_OK(cudaEventElapsedTime(&ms, sp.a, sp.b));
    out[sp.st] += ms;
    launches[sp.st] += (uint32_t)sp.launches;
  }
}

// ---- proof of work
uint64_t GpuBackend::gpu_pow(const std::array<uint8_t, 32>& digest, uint32_t bits) {
  std::lock_guard<std::mutex> g(pow_mu_);
  uint32_t words[8];
  memcpy(words, digest.data(), 32);
  // ~e^-16 chance that a window of 16 * 2^bits nonces holds no solution; then the next one
  const uint64_t window = uint64_t(16) << bits;
  for (uint64_t start = 0;; start += window) {
    const uint32_t seq = ++pow_seq_;
    launch_pow(words, bits, start, window, d_pow_, pow_counter_, d_pow_out_, d_pow_flag_, seq, pow_st_);
    wait_flag(h_pow_flag_, seq, pow_st_);
    const unsigned long long v = *(volatile unsigned long long*)h_pow_;
    if (v != ~0ull) return v;
  }
}
PowSearchFn GpuBackend::pow_search() {
  return [this](const std::array<uint8_t, 32>& digest, uint32_t bits) -> uint64_t {
    // Up to 8 bits (256 compressions expected) the host search with the SHA-2 instructions
    // (a few microseconds) beats a device launch and its round trip
    if (bits <= 8) return pow_search_host(digest, bits);
    return gpu_pow(digest, bits);
  };
}

// ---- staging helpers
void* GpuBackend::scratch(size_t bytes) {
  size_t off = (scr_off_ + 255) & ~size_t(255);
  if (off + bytes > scr_cap_) throw std::runtime_error("device scratch exhausted");
  scr_off_ = off + bytes;
  return scr_ + off;
}
const void* GpuBackend::upload(const void* src, size_t bytes) {
  size_t off = (stage_off_ + 255) & ~size_t(255);
  if (off + bytes > stage_cap_) {
    sync();
    off = 0;
  }
  memcpy(h_stage_ + off, src, bytes);
  CUDA_OK(cudaMemcpyAsync(d_stage_ + off, h_stage_ + off, bytes, cudaMemcpyHostToDevice, st_));
  h2d_ += bytes;
  stage_off_ = off + bytes;
  return d_stage_ + off;
}
const F128d* GpuBackend::upload(const std::vector<F128>& v) {
  return static_cast<const F128d*>(upload(v.data(), v.size() * sizeof(F128)));
}
void GpuBackend::sync() {
  CUDA_OK(cudaStreamSynchronize(st_));
  stage_off_ = 0;
}
std::vector<F128> GpuBackend::reduce(uint32_t n_blocks, uint32_t width) {
  if ((uint64_t)n_blocks * width > part_cap_) throw std::runtime_error("partials buffer too small");
  if (width > 64) {
    launch_reduce_parts(part_, n_blocks, width, red_, st_);
    return fetch(red_, width);
  }
  // round messages: one block reduces and publishes into mapped host memory
  uint32_t seq = ++seq_;
  launch_reduce_publish(part_, n_blocks, width, d_pub_, d_flag_, seq, st_);
  return read_published(seq, width);
}
std::vector<F128> GpuBackend::read_published(uint32_t seq, uint32_t width) {
  wait_published(seq);
  std::vector<F128> out(width);
  const volatile F128d* p = h_pub_;
  for (uint32_t j = 0; j < width; ++j) out[j] = F128(p[j].lo, p[j].hi);
  d2h_ += width * sizeof(F128d) + sizeof(uint32_t);
  return out;
}
// Wait for the published sequence number (the stream keeps running; no synchronisation):
// a short hot spin for the common case of a message a few microseconds away, then a spin
// that yields the core on every pass, so that concurrent provers' host work (assists,
// transcripts) is not starved by waiting threads. A stalled stream is reported after 20 s.
void GpuBackend::wait_published(uint32_t seq) { wait_flag(h_flag_, seq, st_); }
void GpuBackend::wait_flag(const uint32_t* flag, uint32_t seq, cudaStream_t stream) {
  const volatile uint32_t* f = flag;
  uint64_t spins = 0;
  double t0 = 0;
  while (*f != seq) {
    ++spins;
    if (spins > 2048) std::this_thread::yield();
    if ((spins & 0x3FFF) == 0) {
      double t = now_ms();
      if (t0 == 0) t0 = t;
      else if (t - t0 > 20000) throw std::runtime_error("device result not published within 20 s");
      cudaError_t e = cudaStreamQuery(stream);
      if (e != cudaSuccess && e != cudaErrorNotReady) CUDA_OK(e);
    }
  }
  std::atomic_thread_fence(std::memory_order_acquire);
}
std::vector<F128> GpuBackend::fetch(const F128d* d, size_t n) {
  std::vector<F128> out(n);
  F128d* h = h_red_;
  bool big = n > 4096;
  if (big) h = reinterpret_cast<F128d*>(out.data());
  CUDA_OK(cudaMemcpyAsync(h, d, n * sizeof(F128d), cudaMemcpyDeviceToHost, st_));
  d2h_ += n * sizeof(F128d);
  sync();
  if (!big) memcpy(out.data(), h, n * sizeof(F128d));
  return out;
}

// eq(point) split as lo (first lo_bits coordinates) x hi (rest, times scale).
GpuBackend::EqSplit GpuBackend::eq_split(const std::vector<F128>& point, F128 scale, uint32_t max_lo) {
  EqSplit e;
  uint32_t n = (uint32_t)point.size();
  e.lo_bits = std::min(n, max_lo);
  uint32_t hi_bits = n - e.lo_bits;
  const F128d* dp = upload(point);
  F128d* lo = static_cast<F128d*>(scratch((size_t(16)) << e.lo_bits));
  F128d* hi = static_cast<F128d*>(scratch((size_t(16)) << hi_bits));
  launch_eq_split(dp, e.lo_bits, hi_bits, dev(scale), lo, hi, st_);
  e.lo = lo;
  e.hi = hi;
  return e;
}

GpuBackend::EqSplit GpuBackend::eq_split_dev(const F128d* dp, uint32_t n, F128 scale, uint32_t max_lo) {
  EqSplit e;
  e.lo_bits = std::min(n, max_lo);
  uint32_t hi_bits = n - e.lo_bits;
  F128d* lo = static_cast<F128d*>(scratch((size_t(16)) << e.lo_bits));
  F128d* hi = static_cast<F128d*>(scratch((size_t(16)) << hi_bits));
  launch_eq_split(dp, e.lo_bits, hi_bits, dev(scale), lo, hi, st_);
  e.lo = lo;
  e.hi = hi;
  return e;
}

// ------------------------------------------------------------------ witness + commit
void GpuBackend::witness(const std::vector<const uint8_t*>& slot_inputs) {
  scr_off_ = 0;
  if (S.slots.size() != 1 || !S.identity) {
    // union: each slot's records are staged into consecutive regions of the input buffer;
    // the padded buffers are cleared (rows past a count, unused columns and gaps are zero)
    // and each slot's witness is written into its aligned block
    size_t off = 0;
    std::vector<size_t> offs;
    for (size_t t = 0; t < S.slots.size(); ++t) {
      const size_t bytes = (size_t)S.slots[t].count * input_record_bytes(S.slots[t].hash);
      offs.push_back(off);
      if (bytes) {
        memcpy(h_in_ + off, slot_inputs[t], bytes);
        CUDA_OK(cudaMemcpyAsync(d_in_ + off, h_in_ + off, bytes, cudaMemcpyHostToDevice, st_));
      }
      h2d_ += bytes;
      off += bytes;
    }
    Mark mk(this, ST_WITNESS);
    CUDA_OK(cudaMemsetAsync(z_, 0, W_ * 16, st_));
    CUDA_OK(cudaMemsetAsync(a_, 0, W_ * 16, st_));
    CUDA_OK(cudaMemsetAsync(b_, 0, W_ * 16, st_));
    for (size_t t = 0; t < S.slots.size(); ++t) {
      const SlotInfo& T = S.slots[t];
      if (!T.count) continue;
      const size_t w0 = T.offset >> 7;
      launch_witness((int)T.hash, d_in_ + offs[t], (uint32_t)T.count, S.nu, z_ + w0, a_ + w0, b_ + w0,
                     (uint32_t)T.used_cols, st_);
    }
    return;
  }
  const uint8_t* inputs = slot_inputs[0];
  const void* src = d_user_inputs_;
  if (!src) {
    // Host inputs: staged into pinned memory by the host thread pool, 8 MiB at a time, each
    // group's copy to the device queued as soon as it is staged (it overlaps the next
    // group's staging).
    const size_t GROUP = size_t(8) << 20, CHUNK = size_t(512) << 10;
    for (size_t g0 = 0; g0 < in_bytes_; g0 += GROUP) {
      const size_t glen = std::min(GROUP, in_bytes_ - g0);
      parallel_for((glen + CHUNK - 1) / CHUNK, [&](size_t c) {
        const size_t off = g0 + c * CHUNK;
        memcpy(h_in_ + off, inputs + off, std::min(CHUNK, g0 + glen - off));
      });
      CUDA_OK(cudaMemcpyAsync(d_in_ + g0, h_in_ + g0, glen, cudaMemcpyHostToDevice, st_));
    }
    h2d_ += in_bytes_;
    src = d_in_;
  }
  Mark mk(this, ST_WITNESS);
  launch_witness((int)S.hash, src, S.n_blocks, S.nu, z_, a_, b_, (uint32_t)S.geo.used_cols, st_);
}

void GpuBackend::commit_l0(uint32_t cap_depth, std::vector<Hash>& cap) {
  if (!S.identity) {
    // height-n_t compaction: each slot's used columns, the first `count` words of each,
    // stacked column after column (one strided copy per slot), then the zero tail
    Mark mk(this, ST_L0_FILL);
    uint64_t cursor = 0;
    for (const SlotInfo& T : S.slots) {
      if (!T.count || !T.used_cols) continue;
      CUDA_OK(cudaMemcpy2DAsync(q_ + cursor, T.count * 16, z_ + (T.offset >> 7), (size_t(16) << S.nu), T.count * 16,
                                T.used_cols, cudaMemcpyDeviceToDevice, st_));
      cursor += T.count * T.used_cols;
    }
    if (Q_ > cursor) CUDA_OK(cudaMemsetAsync(q_ + cursor, 0, (Q_ - cursor) * 16, st_));
  }
  { Mark mk(this, ST_L0_FILL); launch_fill_lane_major(q_, cw0_, S.lanes, S.log_dim, S.k_code, st_); }
  { Mark mk(this, ST_L0_NTT); launch_ntt(cw0_, S.lanes, S.k_code, 1, tw0_, st_); }
  { Mark mk(this, ST_L0_MERKLE); launch_merkle(cw0_, S.lanes, n_pos0_, cap_depth, tree0_, st_); }
  cap = read_cap(tree0_, n_pos0_, cap_depth);
}

std::vector<Hash> GpuBackend::read_cap(const uint8_t* tree, uint64_t n_leaves, uint32_t cap_depth) {
  uint64_t l = uint64_t(1) << cap_depth;
  std::vector<Hash> cap(l);
  CUDA_OK(cudaMemcpyAsync(cap.data(), tree + (2 * n_leaves - 2 * l) * 32, l * 32, cudaMemcpyDeviceToHost, st_));
  d2h_ += l * 32;
  sync();
  return cap;
}

// ------------------------------------------------------------------ zerocheck
void GpuBackend::zc_round1(const std::vector<F128>& r, std::vector<F128>& ab, std::vector<F128>& c,
                           std::vector<F128>& svc) {
  scr_off_ = 0;
  const uint32_t m = S.m;
  const auto& fixed = zc_fixed_challenges();
  for (int i = 0; i < 7; ++i)
    if (r[6 + i] != fixed[i]) throw std::runtime_error("zerocheck round 1 expects the fixed challenges at r[6..13)");
  std::vector<F128> outer(r.begin() + 13, r.end());
  EqSplit e = eq_split(outer, F128::one(), 10);
  uint32_t nab = 0, nsvc = 0;
  F128d* part_svc = part_ + part_cap_ / 2;
  {
    Mark mk(this, ST_ZC_ROUND1);
    launch_zc_round1(a_, b_, z_, m, zc_live_words_, e.lo, e.lo_bits, e.hi, part_, &nab, part_svc, &nsvc, st_);
  }
  if ((uint64_t)nab * 64 > part_cap_ / 2 || (uint64_t)nsvc * 128 > part_cap_ / 2)
    throw std::runtime_error("round-1 partials exceed the partials buffer");
  launch_reduce_parts(part_, nab, 64, red_, st_);
  launch_reduce_parts(part_svc, nsvc, 128, red_ + 64, st_);
  auto v = fetch(red_, 192);
  // D = prod (1 + g_i)^-1 over the medium constants' g_i = x^1, x^2, x^4, x^8
  static const F128 D = [] {
    F128 d = F128::one();
    for (int e : {1, 2, 4, 8}) d = d * inv(F128::one() + F128(1ull << e, 0));
    return d;
  }();
  ab.assign(64, F128());
  svc.assign(128, F128());
  for (int i = 0; i < 64; ++i) ab[i] = D * v[i];
  for (int i = 0; i < 128; ++i) svc[i] = D * v[64 + i];
  // P_c(i) = sum_s phi8(unit_s(i)) * S_s with S_s = sum_x eq(x) bit_s(z_x); row x = 2w + h
  // splits eq(r[6..m], x) = eq(r_6, h) * eq(r[7..m], w), so S_s = (1 + r_6) svc[s] + r_6 svc[64 + s].
  // phi8 is additive: sum over the set bits b of unit_s(i) of phi8(2^b) * S_s.
  const SkipTables& st = skip_tables();
  F128 T[8][64];
  for (int s = 0; s < 64; ++s) {
    F128 Ss = (F128::one() + r[6]) * svc[s] + r[6] * svc[64 + s];
    for (int bit = 0; bit < 8; ++bit) T[bit][s] = phi8((uint8_t)(1u << bit)) * Ss;
  }
  c.assign(64, F128());
  for (int i = 0; i < 64; ++i) {
    F128 acc;
    for (int s = 0; s < 64; ++s) {
      uint8_t u = st.unit[s][i];
      while (u) {
        int bit = __builtin_ctz(u);
        acc += T[bit][s];
        u &= u - 1;
      }
    }
    c[i] = acc;
  }
}

void GpuBackend::zc_fold_skip(const std::vector<F128>& w, const std::vector<F128>& eq_point, F128& g1, F128& gi) {
  scr_off_ = 0;
  const uint32_t L = (uint32_t)eq_point.size();  // m - 7
  if (L < 10) throw std::runtime_error("zerocheck skip fold needs m >= 17");
  const F128d* dw = upload(w);
  const F128d* dp = upload(eq_point);
  // Every later fold round i uses eq over the suffix eq_point[1 + i ..]: build all the
  // split tables now, in one launch.
  zc_desc_.clear();
  uint64_t total = 0;
  auto add = [&](uint32_t off, uint32_t n) {
    EqDesc d;
    d.p_off = off;
    d.n = n;
    d.out_off = total;
    d.scale = dev(F128::one());
    zc_desc_.push_back(d);
    total += uint64_t(1) << n;
  };
  add(0, 10);
  add(10, L - 10);
  for (uint32_t i = 0; i < L; ++i) {  // round i: eq over eq_point[1 + i ..), L - 1 - i coordinates
    uint32_t n = L - 1 - i, lo = zc_round_lo_bits(n);
    add(1 + i, lo);
    add(1 + i + lo, n - lo);
  }
  if (total != zc_tables_entries(L)) throw std::runtime_error("zerocheck eq tables: size mismatch");
  const EqDesc* ddesc = static_cast<const EqDesc*>(upload(zc_desc_.data(), zc_desc_.size() * sizeof(EqDesc)));
  uint32_t nb;
  {
    Mark mk(this, ST_ZC_FOLD_SKIP);
    launch_eq_tables(dp, ddesc, (uint32_t)zc_desc_.size(), total, zc_tabs_, st_);
    // words from zc_live_words_ on are zero and add nothing to the message
    nb = launch_zc_fold_skip(a_, b_, dw, zc_live_words_, zc_tabs_, 10, zc_tabs_ + zc_desc_[1].out_off, part_, st_);
    CUDA_OK(cudaMemcpyAsync(zc_w64_, dw, 64 * sizeof(F128d), cudaMemcpyDeviceToDevice, st_));
  }
  auto v = reduce(nb, 2);
  g1 = v[0];
  gi = v[1];
  zc_cur_a_ = nullptr;  // the skip-folded vectors live only implicitly (a, b bits and the weights)
  zc_cur_b_ = nullptr;
  zc_len_ = 2 * W_;
  zc_live_ = 2 * zc_live_words_;
  zc_round_ = 0;
}

void GpuBackend::zc_fold(F128 rho, const std::vector<F128>& eq_point, F128& g1, F128& gi) {
  uint64_t n_pairs = zc_len_ / 4;
  if ((uint64_t(1) << eq_point.size()) != n_pairs) throw std::runtime_error("zerocheck fold: eq size mismatch");
  size_t k = 2 + 2 * zc_round_;
  if (k + 1 >= zc_desc_.size() || zc_desc_[k].n + zc_desc_[k + 1].n != eq_point.size())
    throw std::runtime_error("zerocheck fold: round tables out of step");
  const EqDesc& lo = zc_desc_[k];
  const EqDesc& hi = zc_desc_[k + 1];
  // pairs (4 entries in, 2 out) from live_pairs on read only the zero tail
  const uint64_t live_pairs = std::min<uint64_t>(n_pairs, (zc_live_ + 3) / 4);
  // round 0 writes W words per vector into zc2; later rounds alternate zc1 <-> zc2
  F128d* oa = (zc_round_ == 0 || zc_cur_a_ == zc1a_) ? zc2a_ : zc1a_;
  F128d* ob = (zc_round_ == 0 || zc_cur_a_ == zc1a_) ? zc2b_ : zc1b_;
  uint32_t nb, pub_seq = 0;
  {
    Mark mk(this, ST_ZC_FOLDS);
    if (zc_round_ == 0) {
      F128d* tabs = static_cast<F128d*>(scratch(4096 * sizeof(F128d)));
      nb = launch_zc_fold2(a_, b_, zc_w64_, dev(rho), tabs, n_pairs, live_pairs, zc_tabs_ + lo.out_off, lo.n,
                           zc_tabs_ + hi.out_off, oa, ob, part_, st_);
    } else {
      FusedPublish fp = fused_publish();
      launch_pair_fold(zc_cur_a_, zc_cur_b_, n_pairs, live_pairs, dev(rho), nullptr, zc_tabs_ + lo.out_off, lo.n,
                       zc_tabs_ + hi.out_off, oa, ob, part_, true, st_, fp);
      nb = 0;
      pub_seq = fp.seq;
    }
  }
  auto v = pub_seq ? read_published(pub_seq, 2) : reduce(nb, 2);
  g1 = v[0];
  gi = v[1];
  zc_cur_a_ = oa;
  zc_cur_b_ = ob;
  zc_len_ /= 2;
  zc_live_ = std::min(zc_len_, 2 * live_pairs);
  zc_round_++;
}

void GpuBackend::zc_final(F128 rho, F128& ae, F128& be) {
  if (zc_len_ != 2) throw std::runtime_error("zerocheck final fold expects two values");
  auto av = fetch(zc_cur_a_, 2);
  auto bv = fetch(zc_cur_b_, 2);
  ae = av[0] + rho * (av[1] + av[0]);
  be = bv[0] + rho * (bv[1] + bv[0]);
}

// ------------------------------------------------------------------ lincheck
void GpuBackend::lc_comb(const std::vector<F128>& skip_w, const std::vector<F128>& xir) {
  scr_off_ = 0;
  const F128d* dw = upload(skip_w);
  for (size_t t = 0; t < S.slots.size(); ++t) {
    // slot t folds its own matrices by skip_w (x) eq(xir[.. k_log_t - 6])
    const SlotInfo& T = S.slots[t];
    const SlotDev& sd = slot_dev_[t];
    const F128d* der = upload(build_eq(std::vector<F128>(xir.begin(), xir.begin() + (T.k_log - 6))));
    Mark mk(this, ST_LINCHECK);
    launch_lc_eq_inner(dw, der, sd.K, eqi_, st_);
    lc_fold_slot(T.hash, sd);
  }
}

void GpuBackend::lc_fold_slot(HashKind hash, const SlotDev& sd) {
  if (hash == HASH_KECCAK) {
    // the walker's column folds on the device (no materialised matrices)
    static const KeccakColumnConsts kc = [] {
      KeccakColumnConsts c{};
      for (int r = 0; r < 24; ++r) c.rc[r] = kr1cs::RC[r];
      for (int a = 0; a < 5; ++a)
        for (int b = 0; b < 5; ++b) c.rho[a + 5 * b] = (uint8_t)(kr1cs::RHO[a][b] % 64);
      return c;
    }();
    CUDA_OK(cudaMemsetAsync(sd.ca, 0, sd.K * 16, st_));
    CUDA_OK(cudaMemsetAsync(sd.cb, 0, sd.K * 16, st_));
    launch_keccak_lincheck_columns(eqi_, sd.ca, sd.cb, kc, st_);
    return;
  }
  launch_csc_fold(sd.cola, sd.rowa, sd.K, eqi_, sd.ca, st_);
  launch_csc_fold(sd.colb, sd.rowb, sd.K, eqi_, sd.cb, st_);
}

void GpuBackend::lc_zvec(const std::vector<F128>& x_outer) {
  scr_off_ = 0;
  const uint32_t nu = S.nu;
  const F128d* dp = upload(x_outer);
  F128d* eq = static_cast<F128d*>(scratch(size_t(16) << nu));
  Mark mk(this, ST_LINCHECK);
  launch_eq_table(dp, nu, dev(F128::one()), eq, st_);
  // a single slot folds its used columns only; a union folds every union column (the
  // gaps and unused columns of z are zero)
  uint32_t used = S.slots.size() == 1 ? (uint32_t)S.slots[0].used_cols : K_ / 128;
  if ((uint64_t)used * 128 < K_) CUDA_OK(cudaMemsetAsync(zv_ + used * 128, 0, (K_ - used * 128) * 16, st_));
  launch_lc_zvec(z_, nu, used, eq, part_, zv_, st_);
  CUDA_OK(cudaMemcpyAsync(zvcap_, zv_, K_ * 16, cudaMemcpyDeviceToDevice, st_));
  lc_len_ = K_;
}

void GpuBackend::lc_start(F128 alpha, const std::vector<SlotComb>& sc, F128& e1, F128& ei) {
  uint32_t nb;
  if (S.slots.size() == 1 && sc[0].offset == 0 && sc[0].weight == F128::one()) {
    Mark mk(this, ST_LINCHECK);
    nb = launch_lc_start(ca_, cb_, dev(alpha), dev(sc[0].beta), sc[0].pin, K_, comb_, zv_, part_, st_);
  } else {
    Mark mk(this, ST_LINCHECK);
    CUDA_OK(cudaMemsetAsync(comb_, 0, size_t(K_) * 16, st_));
    for (size_t t = 0; t < S.slots.size(); ++t)
      launch_lc_slot_comb(slot_dev_[t].ca, slot_dev_[t].cb, dev(alpha), dev(sc[t].weight), dev(sc[t].beta), sc[t].pin,
                          slot_dev_[t].K, comb_ + sc[t].offset, st_);
    nb = launch_lc_top_message(comb_, zv_, K_, part_, st_);
  }
  auto v = reduce(nb, 2);
  e1 = v[0];
  ei = v[1];
}

void GpuBackend::lc_round(F128 r, bool last, F128& e1, F128& ei) {
  FusedPublish fp = last ? FusedPublish() : fused_publish();
  { Mark mk(this, ST_LINCHECK); launch_lc_round(comb_, zv_, lc_len_, dev(r), !last, part_, st_, fp); }
  lc_len_ /= 2;
  if (!last) {
    auto v = read_published(fp.seq, 2);
    e1 = v[0];
    ei = v[1];
  }
}

void GpuBackend::lc_partial(std::vector<F128>& zp) {
  if (lc_len_ != 64) throw std::runtime_error("lincheck partial expects 64 values");
  zp = fetch(zv_, 64);
}

void GpuBackend::lc_matrix_evals(const std::vector<F128>& rest, const std::vector<F128>& zp,
                                 std::vector<Pair128>& evals) {
  for (size_t t = 0; t < S.slots.size(); ++t) {
    scr_off_ = 0;
    const SlotInfo& T = S.slots[t];
    const F128d* der = upload(build_eq(std::vector<F128>(rest.begin(), rest.begin() + (T.k_log - 6))));
    const F128d* dzp = upload(zp);
    uint32_t nb;
    {
      Mark mk(this, ST_LINCHECK);
      nb = launch_lc_matrix_evals(slot_dev_[t].ca, slot_dev_[t].cb, der, dzp, slot_dev_[t].K, part_, st_);
    }
    auto v = reduce(nb, 2);
    evals.push_back({v[0], v[1]});
  }
}

void GpuBackend::lc_s_hat_v(const std::vector<F128>& tail, std::vector<F128>& out) {
  auto et = build_eq(tail);
  const F128d* det = upload(et);
  { Mark mk(this, ST_LINCHECK); launch_lc_s_hat_v(zvcap_, det, (uint32_t)et.size(), red_, st_); }
  out = fetch(red_, 128);
}

// ------------------------------------------------------------------ merged open
uint32_t GpuBackend::launch_build_w(const std::vector<WeightClaim>& cl, uint32_t nu, uint64_t area) {
  if (cl.size() != 2) throw std::runtime_error("merged open expects the AB and C claims");
  F128d* er[2];
  F128d* ec[2];
  for (int i = 0; i < 2; ++i) {
    // the row and column tables of one claim in one launch, from the point (z_row | z_col)
    std::vector<F128> rc(cl[i].z_row);
    rc.insert(rc.end(), cl[i].z_col.begin(), cl[i].z_col.end());
    const F128d* prc = upload(rc);
    er[i] = static_cast<F128d*>(scratch(size_t(16) << cl[i].z_row.size()));
    ec[i] = static_cast<F128d*>(scratch(size_t(16) << cl[i].z_col.size()));
    launch_eq_split(prc, (uint32_t)cl[i].z_row.size(), (uint32_t)cl[i].z_col.size(), dev(F128::one()), er[i], ec[i],
                    st_);
  }
  std::vector<F128> tabs(cl[0].table);
  tabs.insert(tabs.end(), cl[1].table.begin(), cl[1].table.end());
  const F128d* dt = upload(tabs);
  if (S.slots.size() == 1 && S.identity)
    return launch_mo_build_w(q_, er[0], ec[0], er[1], ec[1], dt, nu, area, Q_, mw_, part_, st_);
  JaggedSegs g;
  uint64_t base = 0;
  for (const SlotInfo& T : S.slots) {
    if (!T.count || !T.used_cols) continue;
    if (g.n == 4) throw std::runtime_error("the merged weight supports at most four non-empty slots");
    g.base[g.n] = base;
    g.rows[g.n] = T.count;
    g.cols[g.n] = T.used_cols;
    g.col_off[g.n] = T.col_offset(S.nu);
    base += T.count * T.used_cols;
    g.n++;
  }
  return launch_mo_build_w(q_, er[0], ec[0], er[1], ec[1], dt, nu, area, Q_, mw_, part_, st_, &g);
}

void GpuBackend::mo_build_w(const std::vector<WeightClaim>& cl, uint32_t nu, uint64_t area, F128& u0, F128& u2) {
  scr_off_ = 0;
  uint32_t nb;
  {
    Mark mk(this, ST_MO_BUILD_W);
    nb = launch_build_w(cl, nu, area);
  }
  auto v = reduce(nb, 2);
  u0 = v[0];
  u2 = v[1];
  mo_q_ = q_;
  mo_w_ = mw_;
  mo_len_ = Q_;
  mo_live_ = std::min<uint64_t>(Q_, area);
}

void GpuBackend::mo_round(F128 r, bool last, F128& g1, F128& gi) {
  if (mo_len_ == 2) {
    auto q = fetch(mo_q_, 2);
    mo_final_ = q[0] + r * (q[1] + q[0]);
    mo_len_ = 1;
    return;
  }
  F128d* oq = (mo_q_ == moAq_) ? moBq_ : moAq_;
  F128d* ow = (mo_q_ == moAq_) ? moBw_ : moAw_;
  uint64_t n_pairs = mo_len_ / 4;
  const uint64_t live_pairs = std::min<uint64_t>(n_pairs, (mo_live_ + 3) / 4);
  // chunking only sets the work split: 2^10 pairs per chunk for the table form's rounds,
  // 2^8 (one pair per thread) for the small, latency-bound ones
  uint32_t chunk_bits = std::min<uint32_t>(n_pairs >= (uint64_t(1) << 17) ? 10 : 8, ceil_log2(n_pairs));
  FusedPublish fp;
  if (!last) fp = fused_publish();
  {
    Mark mk(this, ST_MO_ROUNDS);
    launch_pair_fold(mo_q_, mo_w_, n_pairs, live_pairs, dev(r), nullptr, nullptr, chunk_bits, nullptr, oq, ow, part_,
                     !last, st_, fp);
  }
  mo_q_ = oq;
  mo_w_ = ow;
  mo_len_ /= 2;
  mo_live_ = std::min(mo_len_, 2 * live_pairs);
  if (!last) {
    auto v = read_published(fp.seq, 2);
    g1 = v[0];
    gi = v[1];
  }
}

F128 GpuBackend::mo_q_eval() {
  if (mo_len_ == 1) return mo_final_;
  return fetch(mo_q_, 1)[0];
}

// ------------------------------------------------------------------ Ligerito
void GpuBackend::lg_basis_eq(F128 gamma, const std::vector<F128>& rho) {
  lg_flush_fold();
  scr_off_ = 0;
  if ((uint64_t(1) << rho.size()) != Q_) throw std::runtime_error("Ligerito basis size mismatch");
  lg_pend_basis_ = true;  // filled with the first OOD eq (lg_add_eq) or alone (lg_flush_basis)
  lg_basis_gamma_ = gamma;
  lg_basis_rho_ = rho;
  lg_base_ = true;
  lg_n_ = Q_;
  lg_live_ = std::min<uint64_t>(Q_, S.dense_words);  // q is zero from the dense words on
  lg_cur_ = 0;
}

F128 GpuBackend::lg_eval_eq(const std::vector<F128>& zp) {
  lg_flush_pending();  // reads q only: a held-back basis fill stays held back
  scr_off_ = 0;
  if (!lg_base_) throw std::runtime_error("OOD evaluation expects the committed base vector");
  // chunks of 2^13 words (one eq_hi table each) where there are enough of them for every SM
  EqSplit e = eq_split(zp, F128::one(), (Q_ >> 13) >= (uint64_t)sm_count() ? 13 : 10);
  uint32_t nb;
  // q is zero from the dense words on (the zero tail of the committed vector)
  { Mark mk(this, ST_LIGERITO); nb = launch_lg_dot_eq(q_, 1, e.lo, e.lo_bits, e.hi, Q_, S.dense_words, part_, st_); }
  return reduce(nb, 1)[0];
}

void GpuBackend::lg_add_eq(F128 beta, const std::vector<F128>& zp) {
  lg_flush_pending();
  scr_off_ = 0;
  if (!lg_base_) throw std::runtime_error("basis update expects the base stage");
  EqSplit e = eq_split(zp, beta, 13);
  if (lg_pend_basis_) {
    // b = gamma eq(rho) + beta eq(z) in one pass
    lg_pend_basis_ = false;
    EqSplit eb = eq_split(lg_basis_rho_, lg_basis_gamma_, 13);
    if (eb.lo_bits != e.lo_bits) throw std::runtime_error("basis and OOD eq splits differ");
    Mark mk(this, ST_LIGERITO);
    launch_lg_eq_fill2(eb.lo, eb.hi, e.lo, e.hi, e.lo_bits, Q_, lb128_, st_);
    return;
  }
  { Mark mk(this, ST_LIGERITO); launch_lg_eq_fill(e.lo, e.lo_bits, e.hi, Q_, lb128_, true, st_); }
}

void GpuBackend::lg_flush_basis() {
  if (!lg_pend_basis_) return;
  lg_pend_basis_ = false;
  EqSplit e = eq_split(lg_basis_rho_, lg_basis_gamma_, 13);  // chunks of 2^13 entries: one eq_hi table each
  Mark mk(this, ST_LIGERITO);
  launch_lg_eq_fill(e.lo, e.lo_bits, e.hi, Q_, lb128_, false, st_);
}

Msg256 GpuBackend::lg_message(size_t d) {
  lg_flush_basis();  // the base message reads b
  if (lg_pend_switch_ && (d == 1 || 2 * lg_n_ == d)) {
    // code switch and the message over its pairs (2i, 2i + 1) in one pass
    lg_pend_switch_ = false;
    const int nx = lg_cur_ ^ 1;
    FusedPublish fp = fused_publish();
    {
      Mark mk(this, ST_LIGERITO);
      launch_lg_switch_msg(lf_[lg_cur_], lb_[lg_cur_], lg_n_, lg_live_, lf_[nx], lb_[nx], part_, st_, fp);
    }
    lg_cur_ = nx;
    lg_n_ *= 2;
    lg_live_ = std::min(lg_n_, 2 * lg_live_);
    auto v = read_published(fp.seq, 4);
    Msg256 m;
    m.u0 = F256(v[0], v[1]);
    m.u2 = F256(v[2], v[3]);
    return m;
  }
  if (lg_pend_switch_) lg_flush_fold();  // a code switch followed by a message with other pairs
  if (lg_pend_fold_.active) {
    // fold and message in one pass (over the base vectors for the first fold)
    const uint64_t n_out = lg_n_ / 2;
    const size_t dm = (d == 1 || n_out == d) ? 1 : d;
    const int nx = lg_pend_fold_.base ? 0 : lg_cur_ ^ 1;
    FusedPublish fp = fused_publish();
    {
      Mark mk(this, ST_LIGERITO);
      if (lg_pend_fold_.base)
        launch_lg_fold_msg128(q_, lb128_, n_out, lg_live_, dev(lg_pend_fold_.r), lg_pend_fold_.d, dm, lf_[0], lb_[0],
                              part_, st_, fp);
      else
        launch_lg_fold_msg256(lf_[lg_cur_], lb_[lg_cur_], n_out, lg_live_, dev(lg_pend_fold_.r), lg_pend_fold_.d, dm,
                              lf_[nx], lb_[nx], part_, st_, fp);
    }
    if (lg_pend_fold_.base) lg_base_ = false;
    lg_pend_fold_.active = false;
    lg_cur_ = nx;
    lg_n_ = n_out;
    lg_live_ = fold_live(lg_live_, lg_pend_fold_.d);
    auto v = read_published(fp.seq, 4);
    Msg256 m;
    m.u0 = F256(v[0], v[1]);
    m.u2 = F256(v[2], v[3]);
    return m;
  }
  uint64_t n = lg_n_;
  if (d == 1 || n == d) d = 1;
  Msg256 m;
  if (lg_base_) {
    FusedPublish fp = fused_publish();
    { Mark mk(this, ST_LIGERITO); launch_lg_message128(q_, lb128_, n, lg_live_, d, part_, st_, fp); }
    auto v = read_published(fp.seq, 2);
    m.u0 = F256(v[0]);
    m.u2 = F256(v[1]);
  } else {
    FusedPublish fp = fused_publish();
    { Mark mk(this, ST_LIGERITO); launch_lg_message256(lf_[lg_cur_], lb_[lg_cur_], n, lg_live_, d, part_, st_, fp); }
    auto v = read_published(fp.seq, 4);
    m.u0 = F256(v[0], v[1]);
    m.u2 = F256(v[2], v[3]);
  }
  return m;
}

void GpuBackend::lg_flush_fold() {
  lg_flush_basis();
  lg_flush_pending();
}

void GpuBackend::lg_flush_pending() {
  if (lg_pend_fold_.active && lg_pend_fold_.base) lg_flush_basis();  // the base fold reads b
  if (lg_pend_switch_) {
    lg_pend_switch_ = false;
    const int nx = lg_cur_ ^ 1;
    {
      Mark mk(this, ST_LIGERITO);
      launch_lg_code_switch(lf_[lg_cur_], lb_[lg_cur_], lg_n_, lf_[nx], lb_[nx], st_);
    }
    lg_cur_ = nx;
    lg_n_ *= 2;
    lg_live_ = std::min(lg_n_, 2 * lg_live_);
  }
  if (!lg_pend_fold_.active) return;
  lg_pend_fold_.active = false;
  const uint64_t n_out = lg_n_ / 2;
  if (lg_pend_fold_.base) {
    {
      Mark mk(this, ST_LIGERITO);
      launch_lg_fold128(q_, lb128_, n_out, dev(lg_pend_fold_.r), nullptr, lg_pend_fold_.d, lf_[0], lb_[0], st_);
    }
    lg_cur_ = 0;
    lg_base_ = false;
    lg_n_ = n_out;
    lg_live_ = fold_live(lg_live_, lg_pend_fold_.d);
    return;
  }
  const int nx = lg_cur_ ^ 1;
  {
    Mark mk(this, ST_LIGERITO);
    launch_lg_fold256(lf_[lg_cur_], lb_[lg_cur_], n_out, dev(lg_pend_fold_.r), nullptr, lg_pend_fold_.d, lf_[nx], lb_[nx],
                      st_);
  }
  lg_cur_ = nx;
  lg_n_ = n_out;
  lg_live_ = fold_live(lg_live_, lg_pend_fold_.d);
}

void GpuBackend::lg_fold(F256 r, size_t d) {
  lg_flush_fold();
  // held back: the next message runs fused with it, any other call performs it first
  lg_pend_fold_.active = true;
  lg_pend_fold_.base = lg_base_;
  lg_pend_fold_.r = r;
  lg_pend_fold_.d = d;
}

void GpuBackend::lg_code_switch() {
  lg_flush_fold();
  if (lg_base_) throw std::runtime_error("code switch before the first fold");
  if (2 * lg_n_ > W_ / 2) throw std::runtime_error("code switch exceeds the Ligerito buffers");
  lg_pend_switch_ = true;  // performed by the next message, or by lg_flush_fold
}

void GpuBackend::lg_commit(uint32_t level, uint32_t log_cols, uint32_t log_lanes, uint32_t log_rate,
                           uint32_t cap_depth, std::vector<Hash>& cap) {
  lg_flush_fold();
  if (lg_n_ != (uint64_t(1) << (log_cols + log_lanes))) throw std::runtime_error("Ligerito commit size mismatch");
  if (levels_.size() < level + 1) levels_.resize(level + 1);
  Level& L = levels_[level];
  uint64_t block_len = uint64_t(1) << (log_cols + log_rate);
  uint32_t lanes = 1u << log_lanes;
  if (L.block_len != block_len || L.lanes != lanes) {
    if (L.mat) {
      cudaFree(L.mat);
      cudaFree(L.tree);
      device_bytes_ -= L.block_len * L.lanes * sizeof(F128d) + 2 * L.block_len * 32;
    }
    CUDA_OK(cudaMalloc(&L.mat, block_len * lanes * sizeof(F128d)));
    CUDA_OK(cudaMalloc(&L.tree, 2 * block_len * 32));
    device_bytes_ += block_len * lanes * sizeof(F128d) + 2 * block_len * 32;
    L.block_len = block_len;
    L.lanes = lanes;
  }
  const F128d* tw = twiddles(log_cols + log_rate);
  { Mark mk(this, ST_LIGERITO); launch_lg_replicate(lf_[lg_cur_], lg_n_, block_len * lanes, L.mat, st_); }
  { Mark mk(this, ST_LG_NTT); launch_ntt(L.mat, lanes, log_cols + log_rate, log_rate, tw, st_); }
  { Mark mk(this, ST_LG_MERKLE); launch_merkle(L.mat, lanes, block_len, cap_depth, L.tree, st_); }
  cap = read_cap(L.tree, block_len, cap_depth);
}

Msg256 GpuBackend::lg_introduce_eq(const std::vector<F128>& zp, F128& answer) {
  lg_flush_fold();
  scr_off_ = 0;
  if ((uint64_t(1) << zp.size()) != lg_n_) throw std::runtime_error("OOD point size mismatch");
  EqSplit e = eq_split(zp, F128::one(), 10);
  FusedPublish fp = fused_publish();
  { Mark mk(this, ST_LIGERITO); launch_lg_intro_eq(lf_[lg_cur_], e.lo, e.lo_bits, e.hi, lg_n_, pend_, part_, st_, fp); }
  auto v = read_published(fp.seq, 3);
  answer = v[0];
  pend_induced_ = false;
  pend_n_ = lg_n_;
  Msg256 m;
  m.u0 = F256(v[1]);
  m.u2 = F256(v[2]);
  return m;
}

Msg256 GpuBackend::lg_introduce_induced(uint32_t ln, uint32_t log_rate, const std::vector<uint64_t>& pos,
                                        const std::vector<F128>& w, const std::vector<std::vector<F128>>&) {
  lg_flush_fold();
  scr_off_ = 0;
  if ((uint64_t(2) << ln) != lg_n_) throw std::runtime_error("induced basis size mismatch");
  if (pos.size() != w.size()) throw std::runtime_error("induced basis: one weight per position");
  uint32_t log_d = ln + log_rate;
  for (uint64_t p : pos)
    if (p >> log_d) throw std::runtime_error("induced basis: position outside the codeword");
  uint32_t nq = (uint32_t)w.size();
  const uint64_t* dpos = static_cast<const uint64_t*>(upload(pos.data(), pos.size() * 8));
  const F128d* dw = upload(w);
  F128d* y = static_cast<F128d*>(scratch(size_t(16) << log_d));
  const F128d* tw = twiddles(log_d);
  FusedPublish fp = fused_publish();
  {
    Mark mk(this, ST_LIGERITO);
    launch_lg_induced(dpos, dw, nq, ln, log_rate, tw, lf_[lg_cur_], y, pend_, part_, st_, fp);
  }
  auto v = read_published(fp.seq, 2);
  pend_induced_ = true;
  pend_n_ = uint64_t(1) << ln;
  Msg256 m;
  m.u0 = F256(v[0]);
  m.u2 = F256(v[1], v[1]);
  return m;
}

void GpuBackend::lg_glue(F128 beta) {
  lg_flush_fold();
  Mark mk(this, ST_LIGERITO);
  launch_lg_glue(lb_[lg_cur_], pend_, dev(beta), pend_n_, pend_induced_, st_);
}

void GpuBackend::lg_open(uint32_t level, const std::vector<uint64_t>& pos, uint32_t cap_depth,
                         std::vector<std::vector<F128>>& rows, std::vector<Hash>& paths) {
  lg_flush_fold();
  scr_off_ = 0;
  const F128d* mat;
  const uint8_t* tree;
  uint32_t lanes;
  uint64_t n_leaves;
  if (level == 0) { mat = cw0_; tree = tree0_; lanes = S.lanes; n_leaves = n_pos0_; }
  else { mat = levels_.at(level).mat; tree = levels_.at(level).tree; lanes = levels_[level].lanes; n_leaves = levels_[level].block_len; }
  uint32_t n = (uint32_t)pos.size();
  for (uint64_t p : pos)
    if (p >= n_leaves) throw std::runtime_error("opening position out of range");
  uint32_t depth = 0;
  while ((uint64_t(1) << depth) < n_leaves) ++depth;
  uint32_t plen = depth - cap_depth;
  const uint64_t* dpos = static_cast<const uint64_t*>(upload(pos.data(), n * 8));
  F128d* drows = static_cast<F128d*>(scratch((size_t)n * lanes * 16));
  uint8_t* dpaths = static_cast<uint8_t*>(scratch((size_t)n * plen * 32 + 32));
  {
    Mark mk(this, ST_LIGERITO);
    launch_gather_rows(mat, lanes, dpos, n, drows, st_);
    launch_gather_paths(tree, n_leaves, dpos, n, cap_depth, dpaths, st_);
  }
  std::vector<F128> hr((size_t)n * lanes);
  std::vector<Hash> hp((size_t)n * plen);
  CUDA_OK(cudaMemcpyAsync(hr.data(), drows, hr.size() * 16, cudaMemcpyDeviceToHost, st_));
  if (plen) CUDA_OK(cudaMemcpyAsync(hp.data(), dpaths, hp.size() * 32, cudaMemcpyDeviceToHost, st_));
  d2h_ += hr.size() * 16 + (plen ? hp.size() * 32 : 0);
  sync();
  for (uint32_t q = 0; q < n; ++q) rows.emplace_back(hr.begin() + (size_t)q * lanes, hr.begin() + (size_t)(q + 1) * lanes);
  paths.insert(paths.end(), hp.begin(), hp.end());
}

std::vector<F256> GpuBackend::lg_residual() {
  lg_flush_fold();
  std::vector<F256> out(lg_n_);
  CUDA_OK(cudaMemcpyAsync(out.data(), lf_[lg_cur_], lg_n_ * sizeof(F256d), cudaMemcpyDeviceToHost, st_));
  d2h_ += lg_n_ * sizeof(F256d);
  sync();
  return out;
}

}  // namespace gpu
}  // namespace flock
