// Round messages published straight into mapped host memory: the host waits on a
// sequence flag instead of a stream synchronisation and a device-to-host copy.
#include "kernels.h"

namespace flock {
namespace gpu {

__global__ void reduce_publish_kernel(const F128d* __restrict__ part, uint32_t nb, uint32_t width,
                                      volatile F128d* out, volatile uint32_t* flag, uint32_t seq) {
  __shared__ F128d sh[32];
  for (uint32_t j = 0; j < width; ++j) {
    F128d acc = f128_zero();
    for (uint32_t b = threadIdx.x; b < nb; b += blockDim.x) acc += part[(uint64_t)b * width + j];
    acc = warp_xor(acc);
    const uint32_t w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
    __syncthreads();
    if (l == 0) sh[w] = acc;
    __syncthreads();
    if (w == 0) {
      F128d r = l < nw ? sh[l] : f128_zero();
      r = warp_xor(r);
      if (l == 0) {
        out[j].lo = r.lo;
        out[j].hi = r.hi;
      }
    }
  }
  if (threadIdx.x == 0) {
    __threadfence_system();
    *flag = seq;
  }
}
void launch_reduce_publish(const F128d* part, uint32_t nb, uint32_t width, F128d* out_mapped, uint32_t* flag_mapped,
                           uint32_t seq, cudaStream_t s) {
  reduce_publish_kernel<<<1, 256, 0, s>>>(part, nb, width, out_mapped, flag_mapped, seq);
  LAUNCH_OK();
}

// Several eq tables in one launch: table k = scale_k * eq(point[off_k .. off_k + n_k)) at out + out_k.
__global__ void eq_tables_kernel(const F128d* __restrict__ point, const EqDesc* __restrict__ desc, uint32_t n_desc,
                                 uint64_t total, F128d* __restrict__ out) {
  __shared__ EqDesc sd[64];
  for (uint32_t i = threadIdx.x; i < n_desc; i += blockDim.x) sd[i] = desc[i];
  __syncthreads();
  for (uint64_t e = (uint64_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += (uint64_t)gridDim.x * blockDim.x) {
    uint32_t k = 0;
    while (k + 1 < n_desc && sd[k + 1].out_off <= e) ++k;
    const EqDesc& d = sd[k];
    uint64_t i = e - d.out_off;
    F128d v = d.scale;
    for (uint32_t j = 0; j < d.n; ++j) {
      F128d r = point[d.p_off + j];
      if (!((i >> j) & 1)) r.lo ^= 1;
      v = v * r;
    }
    out[e] = v;
  }
}
void launch_eq_tables(const F128d* point, const EqDesc* d_desc, uint32_t n_desc, uint64_t total, F128d* out,
                      cudaStream_t s) {
  if (n_desc > 64) throw std::runtime_error("too many eq tables in one launch");
  uint32_t blocks = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>((total + 255) / 256, (uint64_t)sm_count() * 8));
  eq_tables_kernel<<<blocks, 256, 0, s>>>(point, d_desc, n_desc, total, out);
  LAUNCH_OK();
}

}  // namespace gpu
}  // namespace flock
