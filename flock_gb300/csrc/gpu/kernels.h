// Launchers of the sm_103a kernels behind the prove_fast backend. Every launcher runs
// on the caller's stream; none allocates device memory (the one-time constant uploads
// excepted: upload_zc_consts and the witness constants live in module memory).
#pragma once
#include <cuda_runtime.h>
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include "field.cuh"

#define CUDA_OK(x)                                                                          \
  do {                                                                                      \
    cudaError_t e__ = (x);                                                                  \
    if (e__ != cudaSuccess)                                                                 \
      throw std::runtime_error(std::string("CUDA error ") + cudaGetErrorString(e__) + " at " + \
                               __FILE__ + ":" + std::to_string(__LINE__));                  \
  } while (0)

namespace flock {
namespace gpu {

// Kernel launches made by this library (all threads); read through flock_gb300_launch_count.
uint64_t launch_count();
void note_launch();
constexpr int MAX_DEVICES = 64;
// Raises `kernel`'s dynamic shared-memory limit to `bytes` on the current device, once per
// (kernel, device, size); thread-safe (provers on several threads launch the same kernels).
void set_dynamic_smem(const void* kernel, int bytes);
#define LAUNCH_OK()                    \
  do {                                 \
    CUDA_OK(cudaGetLastError());       \
    ::flock::gpu::note_launch();       \
  } while (0)

int sm_count();

// witness.cu — writes chunk columns [0, used_chunks) of z, a, b
void upload_witness_constants();  // once per process (synchronous symbol copies)
void launch_witness(int hash, const void* d_inputs, uint32_t n_inst, uint32_t nu, F128d* z, F128d* a, F128d* b,
                    uint32_t used_chunks, cudaStream_t s);

// commit.cu
void launch_fill_lane_major(const F128d* q, F128d* cw, uint32_t lanes, uint32_t log_dim, uint32_t log_pos,
                            cudaStream_t s);
void launch_ntt(F128d* data, uint32_t lanes, uint32_t log_d, uint32_t start_layer, const F128d* tw, cudaStream_t s);
// Leaves and the levels up to the cap level (2^cap_depth nodes); the levels above it are
// not computed.
void launch_merkle(const F128d* rows, uint32_t lanes, uint64_t n_leaves, uint32_t cap_depth, uint8_t* tree,
                   cudaStream_t s);
void launch_pow(const uint32_t digest_le[8], uint32_t bits, uint64_t start, uint64_t count, unsigned long long* d_min,
                uint32_t* d_counter, unsigned long long* out, uint32_t* flag, uint32_t seq, cudaStream_t s);
void launch_gather_rows(const F128d* mat, uint32_t lanes, const uint64_t* d_pos, uint32_t n, F128d* out,
                        cudaStream_t s);
void launch_gather_paths(const uint8_t* tree, uint64_t n_leaves, const uint64_t* d_pos, uint32_t n,
                         uint32_t cap_depth, uint8_t* out, cudaStream_t s);

// sumcheck.cu. Kernels returning a block count wrote per-block partials of the stated
// width into `part`; launch_reduce_parts XORs them.
void launch_eq_table(const F128d* d_point, uint32_t n, F128d scale, F128d* out, cudaStream_t s);
// The lo and hi tables of an eq split (lo unscaled, hi times scale) in one launch.
void launch_eq_split(const F128d* d_point, uint32_t lo_bits, uint32_t hi_bits, F128d scale, F128d* lo, F128d* hi,
                     cudaStream_t s);
void launch_reduce_parts(const F128d* part, uint32_t n_blocks, uint32_t width, F128d* out, cudaStream_t s);

void upload_zc_consts(const uint8_t* ext, const F128d* phi8, const uint8_t mulk[8][256], const F128d* wconst);
// Round-1 partials: P_ab rows of width 64 into part_ab, s_hat_v_c rows of width 128 into part_svc.
// Words of z, a and b from live_words on are zero (the zero tail of a single slot's chunk
// columns) and are not read.
void launch_zc_round1(const F128d* a, const F128d* b, const F128d* z, uint32_t m, uint64_t live_words,
                      const F128d* eq_lo, uint32_t lo_bits, const F128d* eq_hi, F128d* part_ab, uint32_t* nrows_ab,
                      F128d* part_svc, uint32_t* nrows_svc, cudaStream_t s);
uint32_t launch_zc_fold_skip(const F128d* a, const F128d* b, const F128d* w64, uint64_t n_words, const F128d* eq_lo,
                             uint32_t lo_bits, const F128d* eq_hi, F128d* part, cudaStream_t s);       // width 2
// First multilinear fold (at rho) of the skip-folded a, b, computed from the bits; writes
// n_pairs * 2 words of each folded vector and the next message. tabs: 4096-word scratch.
// Pairs from live_pairs on have zero inputs: their outputs are written as zeros and they
// add nothing to the message.
uint32_t launch_zc_fold2(const F128d* a, const F128d* b, const F128d* w64, F128d rho, F128d* tabs, uint64_t n_pairs,
                         uint64_t live_pairs, const F128d* eq_lo, uint32_t lo_bits, const F128d* eq_hi, F128d* aout,
                         F128d* bout, F128d* part, cudaStream_t s);                                     // width 2
// In-kernel publication of a round message: the last block to finish (a device-wide
// ticket counter) XOR-reduces every block's partials, writes the message to mapped host
// memory and then the sequence number, as launch_reduce_publish does in a launch of its
// own. counter must be zero before the launch; the last block resets it.
struct FusedPublish {
  F128d* out = nullptr;        // mapped host memory (null: no publication)
  uint32_t* flag = nullptr;    // mapped host memory
  uint32_t* counter = nullptr; // device memory
  uint32_t seq = 0;
};
// r_dev (when not null) is the device address of the challenge, read by the kernel. Pairs
// from live_pairs on have zero inputs (zeros written, nothing added to the message).
uint32_t launch_pair_fold(const F128d* ain, const F128d* bin, uint64_t n_pairs, uint64_t live_pairs, F128d r,
                          const F128d* r_dev, const F128d* eq_lo, uint32_t lo_bits, const F128d* eq_hi, F128d* aout,
                          F128d* bout, F128d* part, bool msg, cudaStream_t s,
                          FusedPublish pub = FusedPublish());  // width 2

void launch_lc_eq_inner(const F128d* w64, const F128d* er, uint32_t K, F128d* eqi, cudaStream_t s);
void launch_csc_fold(const uint32_t* col_ptr, const uint32_t* rows, uint32_t K, const F128d* eqi, F128d* out,
                     cudaStream_t s);
// Keccak-f block R1CS: writes the nonzero entries of ca = eq^T A_0 and cb = eq^T B_0 (the
// caller zeroes both K-word vectors first). rc = the 24 round constants, rho[a + 5 b] = the
// rotation offset of lane (a, b) mod 64.
struct KeccakColumnConsts {
  uint64_t rc[24];
  uint8_t rho[25];
};
void launch_keccak_lincheck_columns(const F128d* eqi, F128d* ca, F128d* cb, const KeccakColumnConsts& kc,
                                    cudaStream_t s);
void launch_lc_zvec(const F128d* z, uint32_t nu, uint32_t used_chunks, const F128d* eq, F128d* part, F128d* zv,
                    cudaStream_t s);
uint32_t launch_lc_start(const F128d* ca, const F128d* cb, F128d alpha, F128d beta, uint32_t pin, uint32_t K,
                         F128d* comb, const F128d* zv, F128d* part, cudaStream_t s);                   // width 2
uint32_t launch_lc_round(F128d* comb, F128d* zv, uint32_t len, F128d r, bool msg, F128d* part, cudaStream_t s,
                         FusedPublish pub = FusedPublish());
// Union lincheck: one slot's weighted comb (out = weight (alpha ca + cb), + beta at pin),
// and the first message of a comb built that way.
void launch_lc_slot_comb(const F128d* ca, const F128d* cb, F128d alpha, F128d weight, F128d beta, uint32_t pin,
                         uint32_t K, F128d* out, cudaStream_t s);
uint32_t launch_lc_top_message(const F128d* comb, const F128d* zv, uint32_t K, F128d* part, cudaStream_t s);  // width 2
uint32_t launch_lc_matrix_evals(const F128d* ca, const F128d* cb, const F128d* er, const F128d* zp, uint32_t K,
                                F128d* part, cudaStream_t s);                                          // width 2
void launch_lc_s_hat_v(const F128d* zv, const F128d* et, uint32_t n_tail, F128d* out, cudaStream_t s);

// The committed stack of a union with non-identity compaction, as at most four slot
// segments (dense [base, base + rows * cols), column-major, first column col_off).
struct JaggedSegs {
  uint32_t n = 0;
  uint64_t base[4] = {0, 0, 0, 0}, rows[4] = {1, 1, 1, 1}, cols[4] = {0, 0, 0, 0}, col_off[4] = {0, 0, 0, 0};
};
// segs == nullptr: the aligned layout (row = d mod 2^nu, col = d >> nu).
uint32_t launch_mo_build_w(const F128d* q, const F128d* er0, const F128d* ec0, const F128d* er1, const F128d* ec1,
                           const F128d* tables, uint32_t nu, uint64_t area, uint64_t n, F128d* w, F128d* part,
                           cudaStream_t s, const JaggedSegs* segs = nullptr);                          // width 2

void launch_lg_eq_fill(const F128d* eq_lo, uint32_t lo_bits, const F128d* eq_hi, uint64_t n, F128d* out, bool add,
                       cudaStream_t s);
// b = eq_a + eq_b for two eq splits (lo tables unscaled, hi tables carrying the scales) with
// the same lo_bits, in one pass.
void launch_lg_eq_fill2(const F128d* lo_a, const F128d* hi_a, const F128d* lo_b, const F128d* hi_b, uint32_t lo_bits,
                        uint64_t n, F128d* out, cudaStream_t s);
uint32_t launch_lg_dot_eq(const F128d* f, uint32_t stride, const F128d* eq_lo, uint32_t lo_bits, const F128d* eq_hi,
                          uint64_t n, uint64_t live, F128d* part, cudaStream_t s);  // f zero from `live` on                                    // width 1
// f_live: f is zero from that entry on (pairs wholly past it add nothing and are skipped).
uint32_t launch_lg_message128(const F128d* f, const F128d* b, uint64_t n, uint64_t f_live, uint64_t d, F128d* part,
                              cudaStream_t s, FusedPublish pub = FusedPublish());
uint32_t launch_lg_message256(const F256d* f, const F256d* b, uint64_t n, uint64_t f_live, uint64_t d, F128d* part,
                              cudaStream_t s, FusedPublish pub = FusedPublish());
void launch_lg_fold128(const F128d* f, const F128d* b, uint64_t n_out, F256d r, const F256d* r_dev, uint64_t d,
                       F256d* fo, F256d* bo, cudaStream_t s);
// The first fold (of the base vectors into F256 vectors) fused with the next message,
// like launch_lg_fold_msg256.
// f_live: the input f is zero from that entry on; message pairs whose inputs all lie past
// it fold only b (their f outputs are written as zero) and add nothing to the message.
uint32_t launch_lg_fold_msg128(const F128d* f, const F128d* b, uint64_t n_out, uint64_t f_live, F256d r, uint64_t d_fold,
                               uint64_t d_msg, F256d* fo, F256d* bo, F128d* part, cudaStream_t s, FusedPublish pub);
uint32_t launch_lg_fold_msg256(const F256d* f, const F256d* b, uint64_t n_out, uint64_t f_live, F256d r, uint64_t d_fold,
                               uint64_t d_msg, F256d* fo, F256d* bo, F128d* part, cudaStream_t s,
                               FusedPublish pub = FusedPublish());                                  // width 4
void launch_lg_fold256(const F256d* f, const F256d* b, uint64_t n_out, F256d r, const F256d* r_dev, uint64_t d,
                       F256d* fo, F256d* bo, cudaStream_t s);
void launch_lg_code_switch(const F256d* f, const F256d* b, uint64_t n, F256d* fo, F256d* bo, cudaStream_t s);
// The code switch and the round message over the switched vectors with pairs one apart,
// in one pass; published like launch_lg_message256 (four words).
uint32_t launch_lg_switch_msg(const F256d* f, const F256d* b, uint64_t n, uint64_t f_live, F256d* fo, F256d* bo,
                              F128d* part, cudaStream_t s, FusedPublish pub);
void launch_lg_replicate(const F256d* f, uint64_t msg, uint64_t total, F128d* mat, cudaStream_t s);
uint32_t launch_lg_intro_eq(const F256d* f, const F128d* eq_lo, uint32_t lo_bits, const F128d* eq_hi, uint64_t n,
                            F128d* pend, F128d* part, cudaStream_t s,
                            FusedPublish pub = FusedPublish());  // width 3
uint32_t launch_lg_induced(const uint64_t* pos, const F128d* w, uint32_t n_q, uint32_t ln, uint32_t log_rate,
                           const F128d* tw, const F256d* f, F128d* y, F128d* basis, F128d* part,
                           cudaStream_t s, FusedPublish pub = FusedPublish());  // width 2
void launch_lg_glue(F256d* b, const F128d* p, F128d beta, uint64_t n, bool induced, cudaStream_t s);

// rounds.cu
// XOR-reduce width-wide partials with one block and publish the sums to mapped host
// memory, then set *flag = seq (after a system-scope fence).
void launch_reduce_publish(const F128d* part, uint32_t nb, uint32_t width, F128d* out_mapped, uint32_t* flag_mapped,
                           uint32_t seq, cudaStream_t s);
struct EqDesc {
  uint32_t p_off, n;   // coordinates point[p_off .. p_off + n)
  uint64_t out_off;    // first entry in the output (tables in increasing out_off)
  F128d scale;
};
void launch_eq_tables(const F128d* point, const EqDesc* d_desc, uint32_t n_desc, uint64_t total, F128d* out,
                      cudaStream_t s);

}  // namespace gpu
}  // namespace flock
