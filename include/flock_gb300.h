/* flock_gb300 — C ABI of the GB300 prove_fast path.
 *
 * Drop-in boundary for the reference's prove_fast entry points
 *   Blake3Setup::new / prove_fast        crates/flock-prover/src/r1cs_hashes/blake3.rs:1589-1652, 1669-1685
 *   Sha256HybridSetup::new / prove_fast  crates/flock-prover/src/r1cs_hashes/sha2.rs:1185-1268, 1289-1306
 *   KeccakSetup::new / prove_fast        crates/flock-prover/src/r1cs_hashes/keccak.rs:847-909, 922-938
 * and for the reference's own C ABI of its CUDA prover
 *   flock_cuda_prove_blake3 / flock_cuda_free / flock_cuda_device_count
 *                                        cuda-ghash/prove_ffi.cu:366-420
 *
 * Conventions (those of prove_ffi.cu): plain pointers and sizes, int status codes (0 = ok),
 * no exceptions across the boundary, output bytes malloc'd by the library and released
 * with flock_gb300_free. Unlike prove_ffi.cu, statement constants (R1CS matrices, GF(2^8)
 * tables, Ligerito configurations) are derived inside the library, and there is no
 * process-global lock: each setup owns its device buffers and stream, and calls on one
 * setup are serialised by that setup's own lock.
 */
#ifndef FLOCK_GB300_H
#define FLOCK_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Hash kinds (the three single-type registries of prove_fast). */
#define FLOCK_GB300_BLAKE3 0
#define FLOCK_GB300_SHA256 1
#define FLOCK_GB300_KECCAK 2

/* Status codes. */
#define FLOCK_GB300_OK 0
#define FLOCK_GB300_EINVAL 1   /* bad argument: kind, count, sizes, null pointers */
#define FLOCK_GB300_ECUDA 2    /* a CUDA call failed (message in flock_gb300_last_error) */
#define FLOCK_GB300_EINTERNAL 3
#define FLOCK_GB300_PENDING 4  /* flock_gb300_server_poll: not finished yet */

typedef struct flock_gb300_setup flock_gb300_setup;

/* Input record layouts (little-endian, packed):
 *   BLAKE3  : { u32 cv[8]; u32 m[16]; u64 counter; u32 block_len; u32 flags; }  112 bytes
 *             (Compression, blake3.rs:1232)
 *   SHA-256 : { u32 h[8]; u32 w[16]; }                                           96 bytes
 *             (sha2.rs:1332)
 *   Keccak  : { u64 lanes[25]; }  bit j of lane i = state bit 64 i + j           200 bytes
 *             (keccak.rs:922) */
size_t flock_gb300_input_record_bytes(int hash_kind);

/* Setup::new(n_blocks): builds the statement (matrices, registry digest, Ligerito
 * parameters) and allocates the device buffers of one prove of this shape on the
 * current CUDA device. n_blocks must be a power of two >= 8 (full utilisation).
 * Replaces Blake3Setup::new / Sha256HybridSetup::new / KeccakSetup::new. */
int flock_gb300_setup_new(int hash_kind, uint64_t n_blocks, flock_gb300_setup** out);
void flock_gb300_setup_free(flock_gb300_setup* setup);

/* Committed dimension m, commit lanes t, log2 of the L0 codeword length and the 32-byte
 * registry digest of a setup (any output pointer may be null). */
int flock_gb300_setup_info(const flock_gb300_setup* setup, uint32_t* m, uint32_t* lanes, uint32_t* log_code_len,
                           uint8_t digest[32]);

/* prove_fast(inputs, &mut FsChallenger::new(domain)) on the GPU. n_inputs must equal the
 * setup's n_blocks (the reference asserts the same). On success *out receives a malloc'd
 * proof bundle of *out_len bytes:
 *   u64 proof_len | proof_len bytes : bincode(R1csProofMergedLigerito)   (proof.rs:43-48)
 *   u64 cap_len   | cap_len x 32    : Commitment cap (the L0 Merkle cap)
 *   16 bytes ab_value | 16 bytes c_value : R1csClaim values (F128 lo, hi little-endian)
 * SHA-256 over the bundle without its two length words is the digest of
 * crates/flock-prover/tests/union_m6_fixtures.rs:166-180.
 * Replaces Blake3Setup::prove_fast (blake3.rs:1669), Sha256HybridSetup::prove_fast
 * (sha2.rs:1289), KeccakSetup::prove_fast (keccak.rs:922) and flock_cuda_prove_blake3
 * (cuda-ghash/prove_ffi.cu:420). */
int flock_gb300_prove_fast(flock_gb300_setup* setup, const void* inputs, size_t n_inputs, const uint8_t* domain,
                           size_t domain_len, uint8_t** out, size_t* out_len);

/* prove_fast with the input records already in device memory (a device pointer on the
 * setup's device, n_inputs packed records, left unmodified). Same output as
 * flock_gb300_prove_fast; the host-to-device copy of the inputs is skipped. No
 * reference counterpart: the reference proves from host slices only. */
int flock_gb300_prove_fast_device(flock_gb300_setup* setup, const void* d_inputs, size_t n_inputs,
                                  const uint8_t* domain, size_t domain_len, uint8_t** out, size_t* out_len);

/* The CUDA stream (cudaStream_t) every kernel of this setup runs on. */
int flock_gb300_setup_stream(const flock_gb300_setup* setup, void** stream);

/* Device-time breakdown. Each prove records CUDA events around the stages whose bit is
 * set in stage_mask (0 = none, the default); flock_gb300_last_stage_ms then fills up to
 * `cap` entries of milliseconds and kernel launch counts per stage (names from
 * flock_gb300_stage_name) and returns the stage count. */
int flock_gb300_set_stage_timing(flock_gb300_setup* setup, uint32_t stage_mask);
int flock_gb300_last_stage_ms(flock_gb300_setup* setup, double* ms, uint32_t* launches, int cap);
const char* flock_gb300_stage_name(int stage);

/* Bytes copied host-to-device and device-to-host by the last prove on this setup. */
int flock_gb300_last_transfer_bytes(const flock_gb300_setup* setup, uint64_t* h2d, uint64_t* d2h);

/* Kernel launches issued by the library so far (all setups, all threads). */
uint64_t flock_gb300_launch_count(void);

/* Host wall-clock milliseconds of the last prove on this setup:
 * [witness, commit, zerocheck, lincheck, open, total, multipoint assist (its own thread),
 *  time the open phase waited for the assist]. */
int flock_gb300_last_phase_ms(const flock_gb300_setup* setup, double out[8]);

/* The L0 commitment cap of a batch without any device allocation by the library.
 *
 * For callers that cannot let a library allocate device memory: inside a pre-reserved
 * memory budget (an HBM-budgeted serving process), or on a stream whose work must not be
 * interleaved with allocator calls. Runs witness generation, the lane-major codeword fill,
 * the additive NTT and the Merkle tree of the batch's committed stack in a fixed static
 * device array (32 MiB, codewords of at most 2^13 rows: up to 2^11 BLAKE3, 2^10 SHA-256 or
 * 2^9 Keccak-f instances); larger batches are rejected with FLOCK_GB300_EINVAL and a message
 * naming the bytes needed. d_inputs: n_blocks packed input records in device memory. On success
 * cap_out receives the 2^c x 32-byte Merkle cap, identical to the cap in the bundle of
 * flock_gb300_prove_fast for the same inputs, and *cap_len its length. The call is
 * synchronous: it returns after its work on `stream` (a cudaStream_t, 0 = legacy default)
 * has completed and the cap has been copied to cap_out.
 * The first call on a device looks up the static arrays and copies the twiddle tables in
 * (synchronous copies): make it before any stream capture. The chunk columns past the
 * witness are cleared on every call (nothing needs to start zeroed). All calls on a device
 * share the one static array: calls are serialised by a per-device lock, and the caller
 * must not run two of them concurrently through other means (e.g. from two processes
 * sharing a context). No reference counterpart: the reference commits only inside
 * prove_fast. */
int flock_gb300_commit_cap_noalloc(int hash_kind, const void* d_inputs, uint64_t n_blocks, uint8_t* cap_out,
                                   size_t cap_out_bytes, size_t* cap_len, void* stream);

/* ---- batched and served proving (no reference counterpart: the reference proves one
 * statement per call). Independent proofs run concurrently on the device, each on its own
 * stream and buffers, admitted against a device-memory budget; every bundle is byte-
 * identical to the one flock_gb300_prove_fast returns for the same request. */
typedef struct {
  int hash_kind;
  uint64_t n_blocks;       /* power of two >= 8 */
  const void* inputs;      /* n_blocks host records (copied at submission) */
  const uint8_t* domain;   /* transcript domain bytes */
  size_t domain_len;
} flock_gb300_request;

typedef struct {
  int status;              /* FLOCK_GB300_OK or an error code */
  uint8_t* bundle;         /* malloc'd proof bundle (release with flock_gb300_free) */
  size_t bundle_len;
  double latency_ms;       /* submission to completion */
} flock_gb300_result;

/* Device bytes a prover of (hash_kind, n_blocks) holds: the figure the batch and serving
 * entry points admit requests by (witness, L0 codeword and tree, sumcheck and Ligerito
 * buffers, scratch). Builds (and caches) the statement on the calling thread. No
 * reference counterpart. */
int flock_gb300_estimate_device_bytes(int hash_kind, uint64_t n_blocks, uint64_t* bytes);

/* Proves n requests with `workers` concurrent provers within hbm_budget_bytes of device
 * memory (a request larger than the budget still runs, alone). results[i] answers reqs[i];
 * returns the first failing status, or 0. */
int flock_gb300_prove_batch(const flock_gb300_request* reqs, size_t n, int workers, uint64_t hbm_budget_bytes,
                            flock_gb300_result* results);

/* A serving loop: requests are admitted as workers and memory free up, and proofs that
 * arrive while others run overlap with them on the device. Provers are cached per
 * statement shape and evicted least-recently-used when the budget needs room. */
typedef struct flock_gb300_server flock_gb300_server;
int flock_gb300_server_new(uint64_t hbm_budget_bytes, int workers, flock_gb300_server** out);
int flock_gb300_server_submit(flock_gb300_server* server, const flock_gb300_request* req, uint64_t* ticket);
/* Waits up to wait_ms (< 0: until done) for a ticket. Returns FLOCK_GB300_PENDING while it
 * runs; once done fills *result (each ticket's result is returned once). */
int flock_gb300_server_poll(flock_gb300_server* server, uint64_t ticket, int wait_ms, flock_gb300_result* result);
/* flock_gb300_prove_batch on a server's provers: the provers cached by earlier requests
 * (device buffers, twiddles, constant tables) are reused, so a steady stream of batches pays
 * no allocation. May run alongside submit/poll on the same server. */
int flock_gb300_server_prove_batch(flock_gb300_server* server, const flock_gb300_request* reqs, size_t n,
                                   flock_gb300_result* results);
void flock_gb300_server_free(flock_gb300_server* server);

/* The reference's proof file / wire format of a bundle (crates/flock-prover/src/proof_io.rs:238-252,
 * R1csProofBundleLigerito::to_bytes): "FLOCK" | version 21 | flavor 2 | bincode(Commitment,
 * proof), with the commitment's PcsParams those of the setup for (hash_kind, n_blocks).
 * Host-only (no device work); *out is malloc'd, release with flock_gb300_free. */
int flock_gb300_proof_io(int hash_kind, uint64_t n_blocks, const uint8_t* bundle, size_t bundle_len, uint8_t** out,
                         size_t* out_len);

/* ---- mixed multi-type union proofs: several hash types with arbitrary declared counts in
 * one proof (prover::prove_fast_ligerito_union, crates/flock-prover/src/prover.rs:587-620,
 * over UnionInstance::new(&Registry::new(types, nu), counts), crates/flock-core/src/union.rs,
 * schedule.rs:337-690). */
typedef struct flock_gb300_union_setup flock_gb300_union_setup;
/* A registry of n_types distinct hash kinds at uniform row capacity 2^nu (3 <= nu <= 24).
 * Registry::new sorts the types into slot order (k_log descending, stable); that order is
 * written to slot_kinds[0 .. n_types) and every per-slot argument below follows it. The
 * registry digest is computed here. */
int flock_gb300_union_setup_new(const int* hash_kinds, size_t n_types, uint32_t nu, flock_gb300_union_setup** out,
                                int* slot_kinds);
void flock_gb300_union_setup_free(flock_gb300_union_setup* setup);
/* prove_fast_ligerito_union(&UnionInstance::new(&registry, counts), pcs_params, slots,
 * &mut FsChallenger::new(domain)) on the GPU. counts[t] <= 2^nu declared invocations of slot
 * t (zero allowed); inputs[t] points at counts[t] host records of slot t's hash (the records
 * of flock_gb300_prove_fast); rows past a count are the zero dummy rows of the reference's
 * generate_witness_batch_major_partial drivers. *out receives a bundle in the format of
 * flock_gb300_prove_fast (the proof's lincheck carries one matrix-evaluation pair per slot).
 * Provers are cached per counts vector on the setup (device buffers sized for 2^(M-7)
 * words). */
int flock_gb300_prove_union(flock_gb300_union_setup* setup, const uint64_t* counts, const void* const* inputs,
                            const uint8_t* domain, size_t domain_len, uint8_t** out, size_t* out_len);
/* MixedProofBundleLigerito::to_bytes (crates/flock-prover/src/proof_io.rs:254-282) of a
 * union bundle: "FLOCK" | 21 | flavor 4 | registry id (u8) | counts (Vec<u64>) | Commitment |
 * proof. Only the built-in tiers have a registry id (mixed.rs:55-97: BLAKE3 + SHA-256 at nu 7
 * or 10); other registries get FLOCK_GB300_EINVAL. Host-only. */
int flock_gb300_mixed_proof_io(const flock_gb300_union_setup* setup, const uint64_t* counts, const uint8_t* bundle,
                               size_t bundle_len, uint8_t** out, size_t* out_len);

/* Measurement helper (no reference counterpart): products per second of the device
 * GF(2^128) multiply that the NTT and sumcheck kernels use, from `iters` chained products
 * per thread on a full grid (about 256 gives a ~10 ms launch). The integer-pipe peak that
 * the multiply-bound kernels are compared against. Allocates and frees its own buffers. */
int flock_gb300_f128_mul_rate(int iters, double* muls_per_s);

/* Measurement helper (no reference counterpart): products per second by a per-block
 * constant in the mixed form the table kernels use (half the products from the constant's
 * shared-memory byte tables, half from its split form), `iters` chained products per
 * thread on a full grid. The peak that the constant-operand kernels (NTT table layers,
 * challenge folds) are compared against. Allocates and frees its own buffers. */
int flock_gb300_f128_table_mix_rate(int iters, double* products_per_s);

/* Releases a bundle returned by flock_gb300_prove_fast (cuda-ghash/prove_ffi.cu:417 flock_cuda_free). */
void flock_gb300_free(uint8_t* p);

/* Number of visible CUDA devices (cuda-ghash/prove_ffi.cu:410 flock_cuda_device_count). */
int flock_gb300_device_count(void);

/* Message of the last failed call on this thread ("" if none). */
const char* flock_gb300_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* FLOCK_GB300_H */
