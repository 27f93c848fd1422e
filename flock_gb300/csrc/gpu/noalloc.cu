// flock_gb300_commit_cap_noalloc: the L0 commitment (witness -> lane-major fill -> additive
// NTT -> Merkle tree -> cap) of a batch whose working set fits a fixed, file-scope device
// array, for callers that must not have the library allocate device memory.
//
// Device memory: g_noalloc_scratch (NOALLOC_SCRATCH_BYTES) and g_noalloc_twiddles, both
// static module storage. No cudaMalloc / cudaFree or allocating library routine is called.
// First call on a device: the symbol addresses are looked up (cudaGetSymbolAddress) and
// the twiddle tables and witness constants are copied in (synchronous copies); this set-up
// should happen before any stream capture. Every call is synchronous: it returns after its
// work on the caller's stream has finished and the cap is in host memory.
// Limit: codewords of at most 2^13 rows (committed stacks of m <= 25): up to 2^11 BLAKE3,
// 2^10 SHA-256 or 2^9 Keccak-f instances; the scratch they need stays below the 32 MiB.
#include "kernels.h"
#include "../host/setup.h"
#include "../host/tables.h"
#include "../../../include/flock_gb300.h"
#include <cstdio>
#include <mutex>

namespace flock {
namespace gpu {
namespace {

constexpr size_t NOALLOC_SCRATCH_BYTES = size_t(32) << 20;
constexpr uint32_t NOALLOC_MAX_LOG_CODE = 13;

__device__ __align__(256) uint8_t g_noalloc_scratch[NOALLOC_SCRATCH_BYTES];
// twiddles of the size-2^k transform at [2^k, 2^(k+1) - 1), k = 1..NOALLOC_MAX_LOG_CODE
__device__ __align__(256) F128d g_noalloc_twiddles[size_t(1) << (NOALLOC_MAX_LOG_CODE + 1)];

struct DeviceState {
  bool ready = false;
  uint8_t* scratch = nullptr;
  F128d* twiddles = nullptr;
};
DeviceState g_state[MAX_DEVICES];
std::mutex g_mu[MAX_DEVICES];

void setup_device(DeviceState& st) {
  void* p = nullptr;
  CUDA_OK(cudaGetSymbolAddress(&p, g_noalloc_scratch));
  st.scratch = static_cast<uint8_t*>(p);
  CUDA_OK(cudaGetSymbolAddress(&p, g_noalloc_twiddles));
  st.twiddles = static_cast<F128d*>(p);
  for (uint32_t k = 1; k <= NOALLOC_MAX_LOG_CODE; ++k) {
    std::vector<F128> tw = ntt_twiddles(k);
    CUDA_OK(cudaMemcpy(st.twiddles + (size_t(1) << k), tw.data(), tw.size() * sizeof(F128), cudaMemcpyHostToDevice));
  }
  upload_witness_constants();
  CUDA_OK(cudaDeviceSynchronize());  // the synchronous copies above may return before their DMA lands
  st.ready = true;
}

}  // namespace
}  // namespace gpu
void set_last_error(const std::string& msg);  // capi.cu: read by flock_gb300_last_error
}  // namespace flock

using namespace flock;
using namespace flock::gpu;

extern "C" int flock_gb300_commit_cap_noalloc(int hash_kind, const void* d_inputs, uint64_t n_blocks, uint8_t* cap_out,
                                              size_t cap_out_bytes, size_t* cap_len, void* stream) {
  auto fail = [](int code, const char* msg) {
    set_last_error(msg);
    return code;
  };
  set_last_error("");
  if (hash_kind < 0 || hash_kind > 2) return fail(FLOCK_GB300_EINVAL, "unknown hash kind");
  if (!d_inputs || !cap_out || !cap_len) return fail(FLOCK_GB300_EINVAL, "null argument");
  if (n_blocks < 8 || (n_blocks & (n_blocks - 1)) || n_blocks > (uint64_t(1) << 24))
    return fail(FLOCK_GB300_EINVAL, "n_blocks must be a power of two in [8, 2^24]");
  // geometry of the single-slot full-utilisation statement (no host containers)
  uint32_t k_log = hash_kind == 0 ? b3r1cs::K_LOG : (hash_kind == 1 ? s2r1cs::K_LOG : kr1cs::K_LOG);
  uint64_t useful = hash_kind == 0 ? b3r1cs::USEFUL_BITS : (hash_kind == 1 ? s2r1cs::USEFUL_BITS : kr1cs::USEFUL_BITS);
  uint32_t nu = 0;
  while ((uint64_t(1) << nu) < n_blocks) ++nu;
  UnionGeometry geo = union_geometry(k_log, useful, nu);
  if (!geo.identity) return fail(FLOCK_GB300_EINVAL, "batch too small for a full-utilisation statement");
  // the Ligerito parameters, log_dim and cap depth exactly as make_statement derives them
  // for flock_gb300_prove_fast (the cap depth is the top stratum of level 0's schedule)
  LigeritoParams lig;
  try {
    lig = ligerito_params_for(geo.dense_m);
  } catch (const std::exception&) {
    return fail(FLOCK_GB300_EINVAL, "no Ligerito configuration for this size");
  }
  const uint32_t log_batch = lig.initial_k, lanes = geo.commit_lanes(log_batch);
  const uint32_t log_dim = geo.dense_m - 7 - log_batch, k_code = log_dim + 1;
  if (lig.log_n != geo.dense_m - 7 || lig.initial_log_msg_cols != log_dim || lig.log_inv_rates[0] != 1)
    return fail(FLOCK_GB300_EINVAL, "Ligerito configuration does not match the committed geometry");
  const uint32_t cap_depth = lig.sched[0].cap_depth();
  const uint64_t W = uint64_t(1) << (geo.m - 7), n_pos = uint64_t(1) << k_code;
  const size_t need = 3 * W * 16 + n_pos * lanes * 16 + 2 * n_pos * 32;
  if (k_code > NOALLOC_MAX_LOG_CODE || need > NOALLOC_SCRATCH_BYTES) {
    static thread_local char msg[200];
    snprintf(msg, sizeof(msg), "batch needs %zu bytes of scratch; the static scratch holds %zu bytes (at most 2^%u codeword rows)",
             need, NOALLOC_SCRATCH_BYTES, NOALLOC_MAX_LOG_CODE);
    return fail(FLOCK_GB300_EINVAL, msg);
  }
  const size_t cap_bytes = (size_t(32) << cap_depth);
  if (cap_out_bytes < cap_bytes) return fail(FLOCK_GB300_EINVAL, "cap_out too small");
  try {
    int dev = 0;
    CUDA_OK(cudaGetDevice(&dev));
    if (dev < 0 || dev >= MAX_DEVICES) return fail(FLOCK_GB300_EINVAL, "device index out of range");
    std::lock_guard<std::mutex> g(g_mu[dev]);
    DeviceState& st = g_state[dev];
    if (!st.ready) setup_device(st);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    F128d* z = reinterpret_cast<F128d*>(st.scratch);
    F128d* a = z + W;  // a = A z and b = B z of the witness kernel: written, not used here
    F128d* b = a + W;
    F128d* cw = b + W;
    uint8_t* tree = reinterpret_cast<uint8_t*>(cw + n_pos * lanes);
    const uint64_t used_words = geo.used_cols << nu;
    // chunk columns past the witness must read as zero
    CUDA_OK(cudaMemsetAsync(z + used_words, 0, (W - used_words) * 16, s));
    launch_witness(hash_kind, d_inputs, (uint32_t)n_blocks, nu, z, a, b, (uint32_t)geo.used_cols, s);
    launch_fill_lane_major(z, cw, lanes, log_dim, k_code, s);
    launch_ntt(cw, lanes, k_code, 1, st.twiddles + (size_t(1) << k_code), s);
    launch_merkle(cw, lanes, n_pos, cap_depth, tree, s);
    CUDA_OK(cudaMemcpyAsync(cap_out, tree + (2 * n_pos - 2 * (uint64_t(1) << cap_depth)) * 32, cap_bytes,
                            cudaMemcpyDeviceToHost, s));
    CUDA_OK(cudaStreamSynchronize(s));
    *cap_len = cap_bytes;
    return FLOCK_GB300_OK;
  } catch (const std::exception& e) {
    set_last_error(e.what());
    return FLOCK_GB300_ECUDA;
  }
}
