// Device backend of prove_fast (one setup = one statement shape, one stream, buffers
// allocated once and reused by every prove of that shape).
#pragma once
#include "kernels.h"
#include "../host/prover.h"
#include <map>
#include <mutex>

namespace flock {
namespace gpu {

class GpuBackend : public ProverBackend {
 public:
  explicit GpuBackend(const Statement& s);
  ~GpuBackend() override;
  GpuBackend(const GpuBackend&) = delete;
  GpuBackend& operator=(const GpuBackend&) = delete;

  void witness(const std::vector<const uint8_t*>& slot_inputs) override;
  void commit_l0(uint32_t cap_depth, std::vector<Hash>& cap) override;
  void zc_round1(const std::vector<F128>& r, std::vector<F128>& ab, std::vector<F128>& c,
                 std::vector<F128>& s_hat_v_c) override;
  void zc_fold_skip(const std::vector<F128>& w, const std::vector<F128>& eq_point, F128& g1, F128& ginf) override;
  void zc_fold(F128 rho, const std::vector<F128>& eq_point, F128& g1, F128& ginf) override;
  void zc_final(F128 rho, F128& a_eval, F128& b_eval) override;
  void lc_comb(const std::vector<F128>& skip_w, const std::vector<F128>& x_inner_rest) override;
  void lc_zvec(const std::vector<F128>& x_outer) override;
  void lc_start(F128 alpha, const std::vector<SlotComb>& slots, F128& e1, F128& einf) override;
  void lc_round(F128 r, bool last, F128& e1, F128& einf) override;
  void lc_partial(std::vector<F128>& z_partial64) override;
  void lc_matrix_evals(const std::vector<F128>& rest_point, const std::vector<F128>& zp,
                       std::vector<Pair128>& evals) override;
  void lc_s_hat_v(const std::vector<F128>& tail, std::vector<F128>& out128) override;
  void mo_build_w(const std::vector<WeightClaim>& claims, uint32_t nu, uint64_t area, F128& u0, F128& u2) override;
  void mo_round(F128 r, bool last, F128& g1, F128& ginf) override;
  F128 mo_q_eval() override;
  void lg_basis_eq(F128 gamma, const std::vector<F128>& rho) override;
  F128 lg_eval_eq(const std::vector<F128>& z) override;
  void lg_add_eq(F128 beta, const std::vector<F128>& z) override;
  Msg256 lg_message(size_t d) override;
  void lg_fold(F256 r, size_t d) override;
  void lg_code_switch() override;
  void lg_commit(uint32_t level, uint32_t log_cols, uint32_t log_lanes, uint32_t log_rate, uint32_t cap_depth,
                 std::vector<Hash>& cap) override;
  Msg256 lg_introduce_eq(const std::vector<F128>& z, F128& answer) override;
  Msg256 lg_introduce_induced(uint32_t log_msg_cols, uint32_t log_rate, const std::vector<uint64_t>& positions,
                              const std::vector<F128>& w, const std::vector<std::vector<F128>>& what) override;
  bool induced_from_positions() const override { return true; }
  void lg_glue(F128 beta) override;
  void lg_open(uint32_t level, const std::vector<uint64_t>& positions, uint32_t cap_depth,
               std::vector<std::vector<F128>>& rows, std::vector<Hash>& paths) override;
  std::vector<F256> lg_residual() override;
  // Proof-of-work searches of 6 or more bits run on the device (own stream, thread-safe:
  // the forked multipoint transcript grinds concurrently with the main one).
  PowSearchFn pow_search() override;
  // Device-time breakdown of a prove (CUDA events on the backend's stream).
  enum Stage {
    ST_WITNESS, ST_L0_FILL, ST_L0_NTT, ST_L0_MERKLE, ST_ZC_ROUND1, ST_ZC_FOLD_SKIP, ST_ZC_FOLDS, ST_LINCHECK,
    ST_MO_BUILD_W, ST_MO_ROUNDS, ST_LIGERITO, ST_LG_NTT, ST_LG_MERKLE, ST_COUNT
  };
  static const char* stage_name(int s);
  // bit s of `mask` records CUDA events around stage s (0: none)
  void set_stage_timing(uint32_t mask) { timing_mask_ = mask; }
  // Called before each prove: clears transfer counters and stage events.
  void begin_prove(const void* d_inputs);
  // Milliseconds per stage of the last prove and the launches counted in each.
  void stage_ms(double out[ST_COUNT], uint32_t launches[ST_COUNT]);
  uint64_t h2d_bytes() const { return h2d_; }
  uint64_t d2h_bytes() const { return d2h_; }

  cudaStream_t stream() const { return st_; }
  uint64_t device_bytes() const { return device_bytes_; }
  static uint64_t estimate_device_bytes(const Statement& S);
  int device() const { return device_; }
  // Device views for tests of single stages.
  const F128d* z() const { return z_; }
  const F128d* codeword0() const { return cw0_; }
  const uint8_t* tree0() const { return tree0_; }
  uint64_t words() const { return W_; }

 private:
  struct EqSplit {
    const F128d* lo = nullptr;
    const F128d* hi = nullptr;
    uint32_t lo_bits = 0;
  };
  struct Level {
    F128d* mat = nullptr;
    uint8_t* tree = nullptr;
    uint64_t block_len = 0;
    uint32_t lanes = 0;
  };

  void* scratch(size_t bytes);
  const void* upload(const void* src, size_t bytes);
  const F128d* upload(const std::vector<F128>& v);
  void sync();
  std::vector<F128> reduce(uint32_t n_blocks, uint32_t width);
  std::vector<F128> fetch(const F128d* d, size_t n);
  EqSplit eq_split(const std::vector<F128>& point, F128 scale, uint32_t max_lo);
  EqSplit eq_split_dev(const F128d* d_point, uint32_t n, F128 scale, uint32_t max_lo);
  // build the merged-open weight and launch its round-0 reduction (per-block partials)
  uint32_t launch_build_w(const std::vector<WeightClaim>& cl, uint32_t nu, uint64_t area);
  const F128d* twiddles(uint32_t log_d);
  std::vector<Hash> read_cap(const uint8_t* tree, uint64_t n_leaves, uint32_t cap_depth);

  struct Mark {
    GpuBackend* b;
    int st;
    uint64_t l0;
    Mark(GpuBackend* be, int stage);
    ~Mark();
  };
  friend struct Mark;
  cudaEvent_t event();

  const Statement& S;
  int device_ = 0;
  uint32_t timing_mask_ = 0;
  std::vector<cudaEvent_t> ev_pool_;
  size_t ev_used_ = 0;
  struct Span { int st; cudaEvent_t a, b; uint64_t launches; };
  std::vector<Span> spans_;
  uint64_t h2d_ = 0, d2h_ = 0;
  uint64_t device_bytes_ = 0;
  const void* d_user_inputs_ = nullptr;
  cudaStream_t st_ = nullptr;
  uint64_t W_ = 0;
  uint32_t K_ = 0;
  std::vector<void*> owned_;
  std::map<uint32_t, F128d*> tw_;

  size_t in_bytes_ = 0;
  uint8_t* d_in_ = nullptr;
  uint8_t* h_in_ = nullptr;
  F128d *z_ = nullptr, *a_ = nullptr, *b_ = nullptr;
  // the committed stack: z_ itself under identity compaction, else its own Q_ words
  F128d* q_ = nullptr;
  uint64_t Q_ = 0;
  // per-slot lincheck state: the slot's column folds and its matrices (CSC) on the device
  struct SlotDev {
    F128d *ca = nullptr, *cb = nullptr;
    uint32_t *cola = nullptr, *rowa = nullptr, *colb = nullptr, *rowb = nullptr;
    uint32_t K = 0;
  };
  std::vector<SlotDev> slot_dev_;
  void lc_fold_slot(HashKind hash, const SlotDev& sd);
  uint64_t n_pos0_ = 0;
  F128d* cw0_ = nullptr;
  uint8_t* tree0_ = nullptr;
  const F128d* tw0_ = nullptr;

  F128d *zc1a_ = nullptr, *zc1b_ = nullptr, *zc2a_ = nullptr, *zc2b_ = nullptr;
  F128d *zc_cur_a_ = nullptr, *zc_cur_b_ = nullptr;
  uint64_t zc_len_ = 0;
  // Words of z, a and b that can be nonzero (a single slot's witness fills chunk-columns
  // c < used_cols of word (c << nu) + instance; the tail is cleared at allocation and never
  // written), and the live entries of the current zerocheck vectors: the zerocheck kernels
  // skip the zero tail.
  uint64_t zc_live_words_ = 0;
  uint64_t zc_live_ = 0;
  uint32_t zc_round_ = 0;
  F128d* zc_w64_ = nullptr;  // skip-point Lagrange weights (device)

  F128d *eqi_ = nullptr, *ca_ = nullptr, *cb_ = nullptr, *comb_ = nullptr, *zv_ = nullptr, *zvcap_ = nullptr;
  uint32_t *cola_ = nullptr, *rowa_ = nullptr, *colb_ = nullptr, *rowb_ = nullptr;
  uint32_t lc_len_ = 0;

  F128d *mw_ = nullptr, *moAq_ = nullptr, *moAw_ = nullptr, *moBq_ = nullptr, *moBw_ = nullptr;
  const F128d* mo_q_ = nullptr;
  const F128d* mo_w_ = nullptr;
  uint64_t mo_len_ = 0;
  uint64_t mo_live_ = 0;  // entries of q and W that can be nonzero (both are zero from the area on)
  F128 mo_final_;

  F128d* lb128_ = nullptr;
  F256d* lf_[2] = {nullptr, nullptr};
  F256d* lb_[2] = {nullptr, nullptr};
  int lg_cur_ = 0;
  bool lg_base_ = true;
  // An F256 fold is held back until the next call: a message over the folded vectors then
  // runs fused with it (one pass); any other call first performs it on its own.
  struct PendingFold {
    bool active = false;
    bool base = false;  // the first fold: of the base vectors q_ and lb128_ into lf_[0], lb_[0]
    F256 r;
    size_t d = 0;
  };
  PendingFold lg_pend_fold_;
  // A code switch is held back the same way: the next message (pairs one apart) runs fused
  // with it; any other call first performs it on its own (lg_flush_fold does both).
  bool lg_pend_switch_ = false;
  // The basis eq fill is held back too: the first OOD sample's eq is added in the same pass
  // over b (launch_lg_eq_fill2); any other use of b performs it alone first.
  bool lg_pend_basis_ = false;
  F128 lg_basis_gamma_;
  std::vector<F128> lg_basis_rho_;
  void lg_flush_basis();
  void lg_flush_pending();  // the held-back code switch and fold
  void lg_flush_fold();     // lg_flush_basis, then lg_flush_pending
  uint64_t lg_n_ = 0;
  // f (the folded committed vector) is zero from entry lg_live_ on: the committed vector's
  // zero tail, halved through the folds, doubled by the code switch
  uint64_t lg_live_ = 0;
  static uint64_t fold_live(uint64_t live, uint64_t d) {  // output i is live when f[pair_lo(i, d)] may be nonzero
    return (live / (2 * d)) * d + std::min<uint64_t>(d, live % (2 * d));
  }
  F128d* pend_ = nullptr;
  bool pend_induced_ = false;
  uint64_t pend_n_ = 0;
  std::vector<Level> levels_;

  // mapped pinned memory the message reductions publish into
  F128d* h_pub_ = nullptr;
  F128d* d_pub_ = nullptr;
  uint32_t* h_flag_ = nullptr;
  uint32_t* d_flag_ = nullptr;
  uint32_t seq_ = 0;
  void wait_published(uint32_t seq);
  // Spin until the mapped flag holds seq (bounded: an error after 20 s, stream errors
  // reported as they occur).
  void wait_flag(const uint32_t* flag, uint32_t seq, cudaStream_t stream);
  std::vector<F128> read_published(uint32_t seq, uint32_t width);
  uint32_t* pub_counter_ = nullptr;  // ticket counter of in-kernel publication (device)
  FusedPublish fused_publish() { FusedPublish p; p.out = d_pub_; p.flag = d_flag_; p.counter = pub_counter_; p.seq = ++seq_; return p; }
  // eq tables of every zerocheck fold round, built once from the skip-fold point
  F128d* zc_tabs_ = nullptr;
  uint64_t zc_tabs_cap_ = 0;
  std::vector<EqDesc> zc_desc_;

  std::mutex pow_mu_;
  cudaStream_t pow_st_ = nullptr;
  unsigned long long* d_pow_ = nullptr;      // running minimum of the current search (device)
  uint32_t* pow_counter_ = nullptr;          // ticket counter of the current search (device)
  unsigned long long* h_pow_ = nullptr;      // result, mapped host memory
  unsigned long long* d_pow_out_ = nullptr;  // its device alias
  uint32_t* h_pow_flag_ = nullptr;           // sequence number of the last finished search (mapped)
  uint32_t* d_pow_flag_ = nullptr;
  uint32_t pow_seq_ = 0;
  uint64_t gpu_pow(const std::array<uint8_t, 32>& digest, uint32_t bits);

  F128d* part_ = nullptr;
  uint32_t part_cap_ = 0;
  F128d* red_ = nullptr;
  F128d* h_red_ = nullptr;
  uint8_t* scr_ = nullptr;
  size_t scr_cap_ = 0, scr_off_ = 0;
  uint8_t* d_stage_ = nullptr;
  uint8_t* h_stage_ = nullptr;
  size_t stage_cap_ = 0, stage_off_ = 0;
};

}  // namespace gpu
}  // namespace flock
