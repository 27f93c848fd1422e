// Throughput of the GF(2^128) products the multiply-bound kernels of the path use, measured
// on the device: the integer-multiply product (field.cuh `mul`), the roofline of products
// of two variables, and the mixed table / split form of products by a block constant (the
// NTT table layers, the challenge folds). sm_103a has no carry-less multiply, so these
// kernels are bound by the integer multiply and shared-memory pipes rather than by HBM;
// these figures are their peaks, taken the same way a copy kernel gives the HBM peak.
#include "kernels.h"
#include "../../../include/flock_gb300.h"

namespace flock {
void set_last_error(const std::string& msg);
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

// Products by one constant per block in the form the table kernels use: of each thread's
// MUL_CHAINS chains x <- x * y + s, half take the product from the block's byte tables of y
// (load/store pipe), half from its split form (multiply pipe).
__global__ void __launch_bounds__(MUL_THREADS) table_mix_rate_kernel(const F128d* __restrict__ in,
                                                                     F128d* __restrict__ out, int iters) {
  extern __shared__ __align__(16) F128d ytab[];  // build_byte_table's BYTE_TABLE_SMEM_ENTRIES
  __shared__ F128split ys;
  const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
  const F128d y = in[blockIdx.x & 1023];
  if (threadIdx.x == 0) ys = split_factor(y);
  build_byte_table(y, ytab);
  F128d x[MUL_CHAINS];
  const F128d sft = in[(t + 3) & 1023];
#pragma unroll
  for (int c = 0; c < MUL_CHAINS; ++c) x[c] = in[(t + 17 * c + 5) & 1023];
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int c = 0; c < MUL_CHAINS; ++c)
      x[c] = (c < MUL_CHAINS / 2 ? mul_table(x[c], ytab) : mul_split(x[c], ys)) + sft;
  }
  F128d acc = f128_zero();
#pragma unroll
  for (int c = 0; c < MUL_CHAINS; ++c) acc += x[c];
  out[t] = acc;
}

// Times `kernel` (warm-up launch, then one timed launch) on blocks_per_sm x SMs blocks.
template <typename K>
int rate_of(K kernel, uint32_t blocks_per_sm, size_t smem, int iters, double* per_s) {
  F128d* in = nullptr;
  F128d* out = nullptr;
  cudaStream_t s = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = FLOCK_GB300_OK;
  try {
    const uint32_t blocks = (uint32_t)sm_count() * blocks_per_sm;
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
    if (smem) CUDA_OK(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    CUDA_OK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    CUDA_OK(cudaMemcpyAsync(in, h, sizeof(h), cudaMemcpyHostToDevice, s));
    CUDA_OK(cudaEventCreate(&e0));
    CUDA_OK(cudaEventCreate(&e1));
    kernel<<<blocks, MUL_THREADS, smem, s>>>(in, out, iters);  // warm-up (clocks ramp)
    LAUNCH_OK();
    CUDA_OK(cudaEventRecord(e0, s));
    kernel<<<blocks, MUL_THREADS, smem, s>>>(in, out, iters);
    LAUNCH_OK();
    CUDA_OK(cudaEventRecord(e1, s));
    CUDA_OK(cudaEventSynchronize(e1));
    float ms = 0;
    CUDA_OK(cudaEventElapsedTime(&ms, e0, e1));
    *per_s = (double)n_out * MUL_CHAINS * iters / (ms * 1e-3);
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

}  // namespace
}  // namespace gpu
}  // namespace flock

using namespace flock;
using namespace flock::gpu;

extern "C" int flock_gb300_f128_mul_rate(int iters, double* muls_per_s) {
  set_last_error("");
  if (!muls_per_s || iters < 1 || iters > (1 << 16)) {
    set_last_error("iters must be in [1, 65536] and muls_per_s non-null");
    return FLOCK_GB300_EINVAL;
  }
  return rate_of(mul_rate_kernel, MUL_BLOCKS_PER_SM, 0, iters, muls_per_s);
}

extern "C" int flock_gb300_f128_table_mix_rate(int iters, double* products_per_s) {
  set_last_error("");
  if (!products_per_s || iters < 1 || iters > (1 << 16)) {
    set_last_error("iters must be in [1, 65536] and products_per_s non-null");
    return FLOCK_GB300_EINVAL;
  }
  // three 256-thread blocks per SM fit beside their 74 KB tables
  return rate_of(table_mix_rate_kernel, 3, BYTE_TABLE_SMEM_ENTRIES * sizeof(F128d), iters, products_per_s);
}
