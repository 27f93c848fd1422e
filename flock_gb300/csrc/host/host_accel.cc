// Host arithmetic for the CUDA library's host code: the GF(2^128) product and the SHA-256
// compression, built by the host compiler (not nvcc) so that they can use the target's
// crypto extensions (PMULL and the SHA-2 instructions on aarch64; the portable forms
// elsewhere). The protocol driver, the transcript, the ring switch and the multipoint
// assist, which nvcc compiles as part of the library, call these (field.h, hashes.h).
#include "field.h"
#include "hashes.h"

namespace flock {

F128 mul_host_accel(const F128& a, const F128& b) { return mul_impl(a, b); }

void sha256_compress_host_accel(uint32_t st[8], const uint8_t* p) { Sha256::compress_impl(st, p); }

}  // namespace flock
