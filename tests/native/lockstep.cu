// Test harness: runs prove_fast with a backend that drives the CUDA backend and the CPU
// oracle side by side and compares every value each step returns (and the witness and
// L0 codeword), reporting the first step that diverges. Test infrastructure only.
//
//   lockstep <hash 0|1|2> <n_blocks> <seed>
#include "../../flock_gb300/csrc/gpu/backend.h"
#include "../../oracle/cpu_backend.h"
#include <cstdio>

using namespace flock;

struct Rng {
  uint64_t s;
  uint32_t next() {
    s += 0x9E3779B97F4A7C15ull;
    uint64_t z = s;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return (uint32_t)(z ^ (z >> 31));
  }
};

static int g_fail = 0;
static void check(const char* what, const void* a, const void* b, size_t bytes) {
  if (memcmp(a, b, bytes) == 0) return;
  size_t i = 0;
  while (((const uint8_t*)a)[i] == ((const uint8_t*)b)[i]) ++i;
  printf("MISMATCH in %s at byte %zu of %zu (F128 index %zu)\n", what, i, bytes, i / 16);
  g_fail = 1;
  throw std::runtime_error(std::string("divergence in ") + what);
}
static void check(const char* what, const std::vector<F128>& a, const std::vector<F128>& b) {
  if (a.size() != b.size()) { printf("MISMATCH in %s: sizes %zu vs %zu\n", what, a.size(), b.size()); throw std::runtime_error(what); }
  check(what, a.data(), b.data(), a.size() * 16);
}
static void check(const char* what, F128 a, F128 b) { check(what, &a, &b, 16); }
static void check(const char* what, const Msg256& a, const Msg256& b) { check(what, &a, &b, sizeof(Msg256)); }

struct Lockstep : ProverBackend {
  oracle::CpuBackend& C;
  gpu::GpuBackend& G;
  const Statement& S;
  Lockstep(oracle::CpuBackend& c, gpu::GpuBackend& g, const Statement& s) : C(c), G(g), S(s) {}
  template <class T> std::vector<T> dl(const void* d, size_t n) {
    std::vector<T> h(n);
    CUDA_OK(cudaStreamSynchronize(G.stream()));
    CUDA_OK(cudaMemcpy(h.data(), d, n * sizeof(T), cudaMemcpyDeviceToHost));
    return h;
  }
  void witness(const std::vector<const uint8_t*>& in) override {
    C.witness(in); G.witness(in);
    auto z = dl<F128>(G.z(), G.words());
    check("witness z", z, C.z);
    printf("  witness ok\n");
  }
  void commit_l0(uint32_t cd, std::vector<Hash>& cap) override {
    std::vector<Hash> c2;
    C.commit_l0(cd, cap); G.commit_l0(cd, c2);
    auto cw = dl<F128>(G.codeword0(), C.cw0.size());
    check("L0 codeword", cw, C.cw0);
    check("L0 cap", cap.data(), c2.data(), cap.size() * 32);
    printf("  commit ok\n");
  }
  void zc_round1(const std::vector<F128>& r, std::vector<F128>& ab, std::vector<F128>& c, std::vector<F128>& s) override {
    std::vector<F128> ab2, c2, s2;
    C.zc_round1(r, ab, c, s); G.zc_round1(r, ab2, c2, s2);
    check("zc round1 ab", ab, ab2); check("zc round1 c", c, c2); check("zc s_hat_v_c", s, s2);
    printf("  zc round1 ok\n");
  }
  void zc_fold_skip(const std::vector<F128>& w, const std::vector<F128>& e, F128& g1, F128& gi) override {
    F128 a, b; C.zc_fold_skip(w, e, g1, gi); G.zc_fold_skip(w, e, a, b);
    check("zc fold_skip g1", g1, a); check("zc fold_skip ginf", gi, b);
  }
  void zc_fold(F128 r, const std::vector<F128>& e, F128& g1, F128& gi) override {
    F128 a, b; C.zc_fold(r, e, g1, gi); G.zc_fold(r, e, a, b);
    check("zc fold g1", g1, a); check("zc fold ginf", gi, b);
  }
  void zc_final(F128 r, F128& ae, F128& be) override {
    F128 a, b; C.zc_final(r, ae, be); G.zc_final(r, a, b);
    check("zc final a", ae, a); check("zc final b", be, b);
    printf("  zerocheck ok\n");
  }
  void lc_comb(const std::vector<F128>& w, const std::vector<F128>& x) override { C.lc_comb(w, x); G.lc_comb(w, x); }
  void lc_zvec(const std::vector<F128>& x) override { C.lc_zvec(x); G.lc_zvec(x); }
  void lc_start(F128 al, const std::vector<SlotComb>& sc, F128& e1, F128& ei) override {
    F128 a, b; C.lc_start(al, sc, e1, ei); G.lc_start(al, sc, a, b);
    check("lc start e1", e1, a); check("lc start einf", ei, b);
  }
  void lc_round(F128 r, bool last, F128& e1, F128& ei) override {
    F128 a, b; C.lc_round(r, last, e1, ei); G.lc_round(r, last, a, b);
    if (!last) { check("lc round e1", e1, a); check("lc round einf", ei, b); }
  }
  void lc_partial(std::vector<F128>& zp) override {
    std::vector<F128> z2; C.lc_partial(zp); G.lc_partial(z2); check("lc z_partial", zp, z2);
  }
  void lc_matrix_evals(const std::vector<F128>& r, const std::vector<F128>& zp, std::vector<Pair128>& ev) override {
    std::vector<Pair128> e2; C.lc_matrix_evals(r, zp, ev); G.lc_matrix_evals(r, zp, e2);
    if (ev.size() != e2.size()) throw std::runtime_error("lc matrix eval count");
    for (size_t i = 0; i < ev.size(); ++i) { check("lc matrix ea", ev[i].first, e2[i].first); check("lc matrix eb", ev[i].second, e2[i].second); }
  }
  void lc_s_hat_v(const std::vector<F128>& t, std::vector<F128>& o) override {
    std::vector<F128> o2; C.lc_s_hat_v(t, o); G.lc_s_hat_v(t, o2); check("lc s_hat_v", o, o2);
    printf("  lincheck ok\n");
  }
  void mo_build_w(const std::vector<WeightClaim>& cl, uint32_t nu, uint64_t area, F128& u0, F128& u2) override {
    F128 a, b; C.mo_build_w(cl, nu, area, u0, u2); G.mo_build_w(cl, nu, area, a, b);
    check("mo build u0", u0, a); check("mo build u2", u2, b);
  }
  void mo_round(F128 r, bool last, F128& g1, F128& gi) override {
    F128 a, b; C.mo_round(r, last, g1, gi); G.mo_round(r, last, a, b);
    if (!last) { check("mo round g1", g1, a); check("mo round ginf", gi, b); }
  }
  F128 mo_q_eval() override {
    F128 a = C.mo_q_eval(), b = G.mo_q_eval(); check("mo q_eval", a, b);
    printf("  merged open ok\n");
    return a;
  }
  void lg_basis_eq(F128 g, const std::vector<F128>& rho) override { C.lg_basis_eq(g, rho); G.lg_basis_eq(g, rho); }
  F128 lg_eval_eq(const std::vector<F128>& z) override {
    F128 a = C.lg_eval_eq(z), b = G.lg_eval_eq(z); check("lg eval_eq", a, b); return a;
  }
  void lg_add_eq(F128 b, const std::vector<F128>& z) override { C.lg_add_eq(b, z); G.lg_add_eq(b, z); }
  Msg256 lg_message(size_t d) override {
    Msg256 a = C.lg_message(d), b = G.lg_message(d); check("lg message", a, b); return a;
  }
  void lg_fold(F256 r, size_t d) override { C.lg_fold(r, d); G.lg_fold(r, d); }
  void lg_code_switch() override { C.lg_code_switch(); G.lg_code_switch(); }
  void lg_commit(uint32_t lv, uint32_t lc, uint32_t ll, uint32_t lr, uint32_t cd, std::vector<Hash>& cap) override {
    std::vector<Hash> c2;
    C.lg_commit(lv, lc, ll, lr, cd, cap); G.lg_commit(lv, lc, ll, lr, cd, c2);
    check("lg commit cap", cap.data(), c2.data(), cap.size() * 32);
    printf("  ligerito level %u commit ok\n", lv);
  }
  Msg256 lg_introduce_eq(const std::vector<F128>& z, F128& ans) override {
    F128 a2;
    Msg256 a = C.lg_introduce_eq(z, ans), b = G.lg_introduce_eq(z, a2);
    check("lg intro_eq answer", ans, a2); check("lg intro_eq msg", a, b); return a;
  }
  Msg256 lg_introduce_induced(uint32_t ln, uint32_t lr, const std::vector<uint64_t>& pos, const std::vector<F128>& w,
                              const std::vector<std::vector<F128>>& wh) override {
    Msg256 a = C.lg_introduce_induced(ln, lr, pos, w, wh), b = G.lg_introduce_induced(ln, lr, pos, w, {});
    check("lg induced msg", a, b); return a;
  }
  void lg_glue(F128 b) override { C.lg_glue(b); G.lg_glue(b); }
  void lg_open(uint32_t lv, const std::vector<uint64_t>& pos, uint32_t cd, std::vector<std::vector<F128>>& rows,
               std::vector<Hash>& paths) override {
    std::vector<std::vector<F128>> r2; std::vector<Hash> p2;
    size_t r0 = rows.size(), p0 = paths.size();
    C.lg_open(lv, pos, cd, rows, paths); G.lg_open(lv, pos, cd, r2, p2);
    for (size_t i = 0; i < r2.size(); ++i) check("lg open row", rows[r0 + i], r2[i]);
    if (paths.size() - p0 != p2.size()) throw std::runtime_error("lg open path count");
    check("lg open paths", paths.data() + p0, p2.data(), p2.size() * 32);
  }
  std::vector<F256> lg_residual() override {
    auto a = C.lg_residual(), b = G.lg_residual();
    if (a.size() != b.size()) throw std::runtime_error("residual size");
    check("lg residual", a.data(), b.data(), a.size() * 32);
    printf("  ligerito ok\n");
    return a;
  }
};

int main(int argc, char** argv) {
  int hash = argc > 1 ? atoi(argv[1]) : 0;
  uint32_t n = argc > 2 ? (uint32_t)atoi(argv[2]) : 256;
  uint64_t seed = argc > 3 ? strtoull(argv[3], nullptr, 0) : 1;
  Statement S = make_statement((HashKind)hash, n);
  compute_registry_digest(S);
  size_t rec = input_record_bytes(S.hash);
  std::vector<uint8_t> in(rec * n);
  Rng r{seed};
  for (size_t i = 0; i < in.size(); i += 4) { uint32_t v = r.next(); memcpy(&in[i], &v, 4); }
  if (S.hash == HASH_BLAKE3)
    for (uint32_t i = 0; i < n; ++i) { uint32_t bl = 64, fl = 11; memcpy(&in[i * rec + 104], &bl, 4); memcpy(&in[i * rec + 108], &fl, 4); }
  printf("lockstep hash=%d n=%u m=%u lanes=%u\n", hash, n, S.m, S.lanes);
  try {
    oracle::CpuBackend C(S);
    gpu::GpuBackend G(S);
    Lockstep L(C, G, S);
    const char* dom = "lockstep";
    prove_fast(S, L, in.data(), (const uint8_t*)dom, strlen(dom));
  } catch (const std::exception& e) {
    printf("FAILED: %s\n", e.what());
    return 1;
  }
  printf("LOCKSTEP OK\n");
  return 0;
}
