// Throughput of the GF(2^128) product that every multiply-bound kernel of the path uses
// (field.cuh `mul`), measured on the device: the integer-pipe roofline of the NTT, the
// sumcheck folds and the Ligerito folds. sm_103a has no carry-less multiply, so these
// kernels are bound by the integer multiply pipe rather than by HBM; this figure is their
// peak, taken the same way a copy kernel gives the HBM peak.
#include "kernels.h"
#include "../../../include/flock_gb300.h"

namespace flock {
namespace gpu {
namespace {

constexpr int MUL_CHAINS = 4;
constexpr int MUL_THREADS = 256;
constexpr int MUL_BLOCKS_PER_SM = 8;

// Each thread runs MUL_CHAINS independent chains x <- x * y of `iters` products; the
// chains' XOR is stored so no product is dead.
__global__ void __launch_bounds__(MUL_THREADS) mul_rate_kernel(const F128d* __restrict__ in, F128d* __restrict__ out,
                                                               int iters) {
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  F128d x[MUL_CHAINS];
  const F128d y = in[t & 1023];
#pragma unroll
  for (int c = 0; c < MUL_CHAINS; ++c) x[c] = in[(t + 17 * c + 5) & 1023];
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < MUL_CHAINS; ++c) x[c] = x[c] * y;
  }
  F128d acc = f128_zero();
#pragma unroll
  for (int c = 0; c < MUL_CHAINS; ++c) acc += x[c];
  out[t] = acc;
}

}  // namespace
}  // namespace gpu
void set_last_error(const std::string& msg);
}  // namespace flock

using namespace flock;
using namespace flock::gpu;

extern "C" int flock_gb300_f128_mul_rate(int iters, double* muls_per_s) {
  set_last_error("");
  if (!muls_per_s || iters < 1 || iters > (1 << 16)) {
    set_last_error("iters must be in [1, 65536] and muls_per_s non-null");
    return FLOCK_GB300_EINVAL;
  }
  F128d* in = nullptr;
  F128d* out = nullptr;
  cudaStream_t s = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = FLOCK_GB300_OK;
  try {
    const uint32_t blocks = (uint32_t)sm_count() * MUL_BLOCKS_PER_SM;
    const size_t n_out = (size_t)blocks * MUL_THREADS;
    CUDA_OK(cudaMalloc(&in, 1024 * sizeof(F128d)));
    CUDA_OK(cudaMalloc(&out, n_out * sizeof(F128d)));
    F128d h[1024];
    uint64_t st = 0x9E3779B97F4A7C15ull;
    for (auto& v : h) {
      st = st * 6364136223846793005ull + 1442695040888963407ull;
      v.lo = st;
      st = st * 6364136223846793005ull + 1442695040888963407ull;
      v.hi = st | 1;
    }
    CUDA_OK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    CUDA_OK(cudaMemcpyAsync(in, h, sizeof(h), cudaMemcpyHostToDevice, s));
    CUDA_OK(cudaEventCreate(&e0));
    CUDA_OK(cudaEventCreate(&e1));
    mul_rate_kernel<<<blocks, MUL_THREADS, 0, s>>>(in, out, iters);  // warm-up (clocks ramp)
    LAUNCH_OK();
    CUDA_OK(cudaEventRecord(e0, s));
    mul_rate_kernel<<<blocks, MUL_THREADS, 0, s>>>(in, out, iters);
    LAUNCH_OK();
    CUDA_OK(cudaEventRecord(e1, s));
    CUDA_OK(cudaEventSynchronize(e1));
    float ms = 0;
    CUDA_OK(cudaEventElapsedTime(&ms, e0, e1));
    *muls_per_s = (double)n_out * MUL_CHAINS * iters / (ms * 1e-3);
  } catch (const std::exception& ex) {
    set_last_error(ex.what());
    rc = FLOCK_GB300_ECUDA;
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (s) cudaStreamDestroy(s);
  if (in) cudaFree(in);
  if (out) cudaFree(out);
  return rc;
}
