// contract(A, B; algorithm = :TCI) (contraction.jl:399-434): crossinterpolate2 of
// the Contraction batch evaluator (contraction.jl:5-62, 103-335) on the device.
//
// The evaluator is an FEvaluator behind the solve's device value cache: for the
// points a prefill misses it builds the left environments of their row
// multi-indices and the right environments of their column multi-indices
// (evaluateleft / evaluateright, contraction.jl:112-176, kept in device memory
// and keyed by the fused index prefix / suffix, as the reference's leftcache /
// rightcache), one batched kernel pair per environment length, and contracts
// each pair over (link_a, link_b) (batchevaluate, :325-329).  A point list is
// a product with full-length rows, so its value is the full left environment
// (the reference's single-point evaluate splits at the midpoint, :180-196: the
// same number up to rounding).  Values are cached per point: the first product
// that asks for a point fixes its value, and the oracle follows the same rule.
#include "contract_tci.h"

#include <algorithm>
#include <cmath>
#include <string>
#include <unordered_map>

#include "tci_rng.h"

cudaError_t tci_env_level_launch(const double* A, const double* B, int ra, int s, int S, int ra2, int rb, int s2,
                                 int rb2, int right, int n, const double* const* parent, double* const* out,
                                 double* const* tmp, const int32_t* ii, const int32_t* jj, cudaStream_t st);
cudaError_t tci_env_dot_launch(const double* const* L, const double* const* R, const int32_t* len, int n, double* out,
                               cudaStream_t st);

namespace tci {

namespace {

int ct_fail(int code, const std::string& msg) {
  set_error(code, msg);
  return code;
}

#define CTT_TRY(x)                                                                \
  do {                                                                            \
    cudaError_t _e = (x);                                                         \
    if (_e != cudaSuccess) return ct_fail(TCI_ERR_CUDA, cudaGetErrorString(_e));  \
  } while (0)

// Device memory handed out in order from large chunks, released together.
class Arena {
 public:
  ~Arena() { release(); }
  double* take(size_t elems) {
    const size_t bytes = (elems * sizeof(double) + 255) / 256 * 256;
    if (chunks_.empty() || used_ + bytes > cap_) {
      const size_t want = std::max(bytes, (size_t)64 << 20);
      void* p = nullptr;
      if (cudaMalloc(&p, want) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
      }
      chunks_.push_back(p);
      cap_ = want;
      used_ = 0;
    }
    double* r = (double*)((char*)chunks_.back() + used_);
    used_ += bytes;
    return r;
  }
  void release() {
    for (void* p : chunks_) cudaFree(p);
    chunks_.clear();
    cap_ = used_ = 0;
  }

 private:
  std::vector<void*> chunks_;
  size_t cap_ = 0, used_ = 0;
};

// Growable device buffer for per-call scratch.
struct Scratch {
  void* p = nullptr;
  size_t cap = 0;
  ~Scratch() {
    if (p) cudaFree(p);
  }
  void* get(size_t bytes) {
    if (bytes <= cap) return p;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    if (cudaMalloc(&p, std::max(bytes, (size_t)1 << 20)) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    cap = std::max(bytes, (size_t)1 << 20);
    return p;
  }
};

class ContractionEval : public FEvaluator {
 public:
  ContractionEval(TT4&& a, TT4&& b, tci_value_fn vf, void* vuser, Engine& e)
      : a_(std::move(a)), b_(std::move(b)), vf_(vf), vuser_(vuser), e_(e) {
    L_ = (int)a_.cores.size();
    for (int n = 0; n <= L_; ++n) {
      ra_.push_back(n < L_ ? a_.cores[n].d[0] : 1);
      rb_.push_back(n < L_ ? b_.cores[n].d[0] : 1);
    }
  }
  ~ContractionEval() override {
    a_.release(e_);
    b_.release(e_);
  }
  int init() {
    one_ = arena_.take(1);
    if (!one_) return ct_fail(TCI_ERR_OOM, "device memory for the environments");
    const double v = 1.0;
    CTT_TRY(cudaMemcpy(one_, &v, sizeof(double), cudaMemcpyHostToDevice));
    left_[std::string()] = one_;
    right_[std::string()] = one_;
    return 0;
  }
  int s_in(int n) const { return (int)a_.cores[n].d[1]; }

  int values(Engine& e, const std::vector<FcProduct>& prods, const std::vector<FcMiss>& miss,
             double* out) override {
    const size_t u = miss.size();
    std::vector<std::string> lk(u), rk(u);
    for (size_t k = 0; k < u; ++k) {
      const FcProduct& p = prods[(size_t)miss[k].q];
      lk[k].assign((const char*)p.rows + (size_t)miss[k].i * p.rl, (size_t)p.rl);
      if (p.cl) rk[k].assign((const char*)p.cols + (size_t)miss[k].j * p.cl, (size_t)p.cl);
    }
    int rc = ensure(e, lk, false);
    if (!rc) rc = ensure(e, rk, true);
    if (rc) return rc;
    std::vector<const double*> lp(u), rp(u);
    std::vector<int32_t> len(u);
    for (size_t k = 0; k < u; ++k) {
      lp[k] = left_.at(lk[k]);
      rp[k] = right_.at(rk[k]);
      const size_t bond = lk[k].size();
      len[k] = (int32_t)(ra_[bond] * rb_[bond]);
    }
    const size_t pb = u * sizeof(void*);
    char* d = (char*)scr_.get(2 * pb + u * 4 + u * 8 + 64);
    if (!d) return ct_fail(TCI_ERR_OOM, "device memory for the contraction scratch");
    const double** dL = (const double**)d;
    const double** dR = (const double**)(d + pb);
    int32_t* dlen = (int32_t*)(d + 2 * pb);
    double* dout = (double*)(d + ((2 * pb + u * 4 + 7) / 8 * 8));
    cudaStream_t st = e.stream();
    CTT_TRY(cudaMemcpyAsync(dL, lp.data(), pb, cudaMemcpyHostToDevice, st));
    CTT_TRY(cudaMemcpyAsync(dR, rp.data(), pb, cudaMemcpyHostToDevice, st));
    CTT_TRY(cudaMemcpyAsync(dlen, len.data(), u * 4, cudaMemcpyHostToDevice, st));
    CTT_TRY(tci_env_dot_launch(dL, dR, dlen, (int)u, dout, st));
    CTT_TRY(cudaMemcpyAsync(out, dout, u * 8, cudaMemcpyDeviceToHost, st));
    CTT_TRY(cudaStreamSynchronize(st));
    if (vf_ && u) {  // contract(...; f): f applied to every value (contraction.jl:205-207, :331-333)
      const int frc = vf_(vuser_, (int64_t)u, out);
      if (frc) return ct_fail(TCI_ERR_GENERIC, "caller-supplied f failed (code " + std::to_string(frc) + ")");
    }
    return 0;
  }

 private:
  // Environments for every key (and every missing ancestor), level by level.
  int ensure(Engine& e, const std::vector<std::string>& keys, bool right) {
    auto& cache = right ? right_ : left_;
    std::vector<std::vector<std::string>> todo((size_t)L_ + 1);
    std::unordered_map<std::string, char> queued;
    for (const std::string& k0 : keys) {
      std::string k = k0;
      while (!k.empty() && !cache.count(k) && !queued.count(k)) {
        queued[k] = 1;
        todo[k.size()].push_back(k);
        k = right ? k.substr(1) : k.substr(0, k.size() - 1);
      }
    }
    for (size_t len = 1; len <= (size_t)L_; ++len) {
      auto& lvl = todo[len];
      if (lvl.empty()) continue;
      const int site = right ? L_ - (int)len : (int)len - 1;
      const Tensor4& A = a_.cores[(size_t)site];
      const Tensor4& B = b_.cores[(size_t)site];
      const int ra = (int)A.d[0], s = (int)A.d[1], S = (int)A.d[2], ra2 = (int)A.d[3];
      const int rb = (int)B.d[0], s2 = (int)B.d[2], rb2 = (int)B.d[3];
      const size_t outn = right ? (size_t)ra * rb : (size_t)ra2 * rb2;
      const size_t tmpn = right ? (size_t)rb2 * S * ra : (size_t)rb * S * ra2;
      const size_t n = lvl.size();
      std::vector<const double*> par(n);
      std::vector<double*> outp(n), tmpp(n);
      std::vector<int32_t> ii(n), jj(n);
      double* tmpbase = (double*)tmp_.get(n * tmpn * sizeof(double));
      if (!tmpbase) return ct_fail(TCI_ERR_OOM, "device memory for the environments");
      for (size_t q = 0; q < n; ++q) {
        const std::string& k = lvl[q];
        const std::string parent = right ? k.substr(1) : k.substr(0, k.size() - 1);
        par[q] = cache.at(parent);
        const int v = (uint8_t)(right ? k[0] : k.back());
        ii[q] = v % s;  // _unfuse_idx (contraction.jl:95-97): A's index fastest
        jj[q] = v / s;
        outp[q] = arena_.take(outn);
        if (!outp[q]) return ct_fail(TCI_ERR_OOM, "device memory for the environments");
        tmpp[q] = tmpbase + q * tmpn;
      }
      const size_t pb = n * sizeof(void*);
      char* d = (char*)scr2_.get(3 * pb + 2 * n * 4 + 64);
      if (!d) return ct_fail(TCI_ERR_OOM, "device memory for the environments");
      cudaStream_t st = e.stream();
      CTT_TRY(cudaMemcpyAsync(d, par.data(), pb, cudaMemcpyHostToDevice, st));
      CTT_TRY(cudaMemcpyAsync(d + pb, outp.data(), pb, cudaMemcpyHostToDevice, st));
      CTT_TRY(cudaMemcpyAsync(d + 2 * pb, tmpp.data(), pb, cudaMemcpyHostToDevice, st));
      CTT_TRY(cudaMemcpyAsync(d + 3 * pb, ii.data(), n * 4, cudaMemcpyHostToDevice, st));
      CTT_TRY(cudaMemcpyAsync(d + 3 * pb + n * 4, jj.data(), n * 4, cudaMemcpyHostToDevice, st));
      CTT_TRY(tci_env_level_launch(A.p, B.p, ra, s, S, ra2, rb, s2, rb2, right ? 1 : 0, (int)n,
                                   (const double* const*)d, (double* const*)(d + pb), (double* const*)(d + 2 * pb),
                                   (const int32_t*)(d + 3 * pb), (const int32_t*)(d + 3 * pb + n * 4), st));
      CTT_TRY(cudaStreamSynchronize(st));  // the pointer tables are reused by the next level
      for (size_t q = 0; q < n; ++q) cache[lvl[q]] = outp[q];
    }
    return 0;
  }

  TT4 a_, b_;
  tci_value_fn vf_;
  void* vuser_;
  Engine& e_;
  int L_ = 0;
  std::vector<int64_t> ra_, rb_;
  Arena arena_;
  Scratch scr_, scr2_, tmp_;
  double* one_ = nullptr;
  std::unordered_map<std::string, double*> left_, right_;
};

// _findinitialpivots (contraction.jl:385-397): random starts from the solve's
// RNG seed, each improved by optfirstpivot; starts whose |f| is zero dropped.
CoTask co_findinitialpivots(Engine& e, Solve& s, int nmax, uint64_t seed, std::vector<std::vector<uint8_t>>* out) {
  out->clear();
  const int L = s.L;
  tci_rng rng;
  tci_rng_seed(&rng, seed);
  std::vector<std::vector<uint8_t>> piv((size_t)nmax, std::vector<uint8_t>((size_t)L));
  for (auto& p : piv)
    for (int q = 0; q < L; ++q) p[(size_t)q] = (uint8_t)(tci_rng_uniform1(&rng, (uint64_t)s.d[(size_t)q]) - 1);
  std::vector<double> valf;
  CO_TRY(co_optfirstpivots(e, s, &piv, &valf, 1000));
  for (int q = 0; q < nmax; ++q)
    if (valf[(size_t)q] != 0.0) out->push_back(piv[(size_t)q]);
  co_return 0;
}

CoTask co_contract_tci(Engine& e, Solve& s, std::vector<std::vector<uint8_t>> pivots, int nmax, tci_opts o) {
  if (pivots.empty()) {
    CO_TRY(co_findinitialpivots(e, s, nmax, o.seed, &pivots));
    if (pivots.empty()) co_return ct_fail(TCI_ERR_GENERIC, "No initial pivots found.");
  }
  co_return co_await co_crossinterpolate2(e, s, std::move(pivots), o);
}

}  // namespace

int tt4_contract_tci(Engine& e, TT4&& a, TT4&& b, const std::vector<std::vector<uint8_t>>& pivots, int nmax,
                     tci_value_fn vf, void* vuser, const tci_opts& o, TT4& out) {
  const int L = (int)a.cores.size();
  if (L != (int)b.cores.size()) {
    a.release(e);
    b.release(e);
    return ct_fail(TCI_ERR_ARG, "Cannot contract tensor trains with different length.");
  }
  for (int n = 0; n < L; ++n)
    if (a.cores[(size_t)n].d[2] != b.cores[(size_t)n].d[1]) {
      a.release(e);
      b.release(e);
      return ct_fail(TCI_ERR_ARG, "Cannot contract tensor trains with non-matching site dimensions.");
    }
  std::vector<int64_t> ld((size_t)L), s1((size_t)L), s3((size_t)L);
  for (int n = 0; n < L; ++n) {
    s1[(size_t)n] = a.cores[(size_t)n].d[1];
    s3[(size_t)n] = b.cores[(size_t)n].d[2];
    ld[(size_t)n] = s1[(size_t)n] * s3[(size_t)n];
    if (ld[(size_t)n] > 256) {
      a.release(e);
      b.release(e);
      return ct_fail(TCI_ERR_ARG, "fused local dimensions must be at most 256");
    }
  }
  auto ev = std::make_shared<ContractionEval>(std::move(a), std::move(b), vf, vuser, e);
  int rc = ev->init();
  if (rc) return rc;
  Solve s;
  rc = solve_init_evaluator(s, L, ld.data(), ev);
  if (rc) return rc;
  for (const auto& p : pivots)
    for (int q = 0; q < L; ++q)
      if ((int64_t)p[(size_t)q] >= ld[(size_t)q]) return ct_fail(TCI_ERR_ARG, "pivot index out of range");
  CoTask t = co_contract_tci(e, s, pivots, nmax, o);
  rc = e.run(t, false);
  if (!rc) {  // the solve's site tensors become the result, legs split (contraction.jl:430-433)
    out.cores.clear();
    for (int n = 0; n < L; ++n) {
      Core& c = s.cores[(size_t)n];
      Tensor4 t4;
      t4.p = c.p;
      t4.d[0] = c.d0;
      t4.d[1] = s1[(size_t)n];
      t4.d[2] = s3[(size_t)n];
      t4.d[3] = c.d2;
      c.p = nullptr;
      out.cores.push_back(t4);
    }
  }
  e.release_solve(s);
  return rc;
}

}  // namespace tci
