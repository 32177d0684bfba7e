// C ABI of libtci_gpu.so (include/tci_gb300.h): thin wrappers that build the
// solve state, run the coroutine algorithm on the context's engine and copy
// results into caller buffers.
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <optional>
#include <thread>
#include <cstdlib>
#include <algorithm>
#include <condition_variable>
#include <deque>
#include <functional>
#include <numeric>

#include "contract.h"
#include "contract_tci.h"
#include "engine.h"
#include "tc_gemm.h"

using namespace tci;

// A context owns a pool of engines, each with its own stream and buffers.
// Single-solve entry points use the first; batched solves and the server spread
// solves over all of them so that one engine's host work and kernel tail
// overlap the others' kernels.
struct tci_ctx {
  // declaration order = reverse destruction order: the engines go first, then
  // the ring, then the pools their blocks came from
  std::unique_ptr<BlockPool> dpool;
  std::vector<std::unique_ptr<BlockPool>> hpools, spools;  // per engine: task records, task scratch
  std::unique_ptr<BlockPool> xpool;                        // pinned export buffers handed to the caller
  std::unique_ptr<ResidentQueue> rq;  // null: batched launches only
  std::vector<std::unique_ptr<Engine>> pool;
  Engine* engp = nullptr;
  // Recursive: a caller-supplied f runs while its call holds the lock, and a
  // finalizer it triggers (a garbage collector releasing another solve) may
  // destroy objects of the same context from inside it.  Entry points that
  // compute refuse to run there (Engine::run / run_tasks).
  std::recursive_mutex mu;
  int64_t peak_live = 0;  // most solves live at once in a batched / serving drive (stats)
  Engine& eng_ref() { return *engp; }
};

struct tci_solve {
  tci_ctx* ctx = nullptr;
  Solve s;
};

namespace {

int fail(int code, const std::string& msg) {
  set_error(code, msg);
  return code;
}

std::vector<std::vector<uint8_t>> to_pivots(const int64_t* piv, int64_t np, int L, const std::vector<int>& d,
                                            int* rc) {
  std::vector<std::vector<uint8_t>> out;
  *rc = 0;
  for (int64_t p = 0; p < np; ++p) {
    std::vector<uint8_t> v(L);
    for (int q = 0; q < L; ++q) {
      int64_t x = piv[p * L + q];
      if (x < 1 || x > d[q]) {
        *rc = fail(TCI_ERR_ARG, "pivot index out of range");
        return {};
      }
      v[q] = (uint8_t)(x - 1);
    }
    out.push_back(v);
  }
  return out;
}

// Points (np x L, row-major, 1-based int64) -> flat 0-based uint8 multi-indices,
// range-checked; large inputs are split over host threads.
int pack_points(const int64_t* pts, int64_t np, int L, const std::vector<int>& d, std::vector<uint8_t>& out) {
  out.resize((size_t)np * (size_t)L);
  auto run = [&](int64_t p0, int64_t p1) {
    bool ok = true;
    for (int64_t p = p0; p < p1; ++p) {
      const int64_t* x = pts + p * L;
      uint8_t* o = out.data() + (size_t)p * L;
      for (int q = 0; q < L; ++q) {
        ok &= x[q] >= 1 && x[q] <= d[q];
        o[q] = (uint8_t)(x[q] - 1);
      }
    }
    return ok;
  };
  const int64_t work = np * (int64_t)L;
  int nt = work >= (1 << 22) ? (int)std::min<int64_t>(8, std::max(1u, std::thread::hardware_concurrency())) : 1;
  bool ok = true;
  if (nt == 1) {
    ok = run(0, np);
  } else {
    std::vector<std::thread> th;
    std::vector<char> res(nt, 1);
    const int64_t per = (np + nt - 1) / nt;
    for (int t = 0; t < nt; ++t)
      th.emplace_back([&, t] { res[t] = run(std::min(np, t * per), std::min(np, (t + 1) * per)); });
    for (auto& x : th) x.join();
    for (char r : res) ok &= r != 0;
  }
  if (!ok) return fail(TCI_ERR_ARG, "pivot index out of range");
  return 0;
}

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

// HBM estimate used for admission: L * d^2 * r_max^2 doubles.
double solve_estimate_bytes(const tci_request& r) {
  double dmax = 1;
  for (int q = 0; q < r.L; ++q) dmax = std::max<double>(dmax, (double)r.localdims[q]);
  double rmax = r.opts.maxbonddim > 0 ? (double)r.opts.maxbonddim : 1e9;
  double full = 1;  // d^(L/2) bound on the rank
  for (int q = 0; q < r.L / 2; ++q) full = std::min(full * dmax, 1e9);
  rmax = std::min(rmax, full);
  return (double)r.L * dmax * dmax * rmax * rmax * 8.0;
}

}  // namespace

extern "C" {

void tci_opts_default(tci_opts* o) {
  std::memset(o, 0, sizeof(*o));
  o->tolerance = 1e-8;
  o->maxbonddim = 0;
  o->maxiter = 20;
  o->sweepstrategy = TCI_SWEEP_BACKANDFORTH;
  o->normalizeerror = 1;
  o->ncheckhistory = 3;
  o->maxnglobalpivot = 5;
  o->nsearchglobalpivot = 5;
  o->strictlynested = 0;
  o->checkconvglobalpivot = 1;
  o->tolmarginglobalsearch = 10.0;
  o->seed = 0;
}

const char* tci_last_error(void) { return last_message(); }

int tci_f_lookup(const char* name, int* fid) {
  static const struct {
    const char* n;
    int id;
  } tab[] = {{"lorentz", TCI_F_LORENTZ}, {"served", TCI_F_SERVED}, {"qtt1d", TCI_F_QTT1D},
             {"qtt2d", TCI_F_QTT2D},     {"dense", TCI_F_DENSE}, {"product", TCI_F_PRODUCT}};
  for (auto& e : tab)
    if (std::strcmp(e.n, name) == 0) {
      *fid = e.id;
      return 0;
    }
  return fail(TCI_ERR_ARG, std::string("unknown function ") + name);
}

int tci_ctx_create(int device, size_t hbm_budget, tci_ctx** out) {
  *out = nullptr;
  // Engines = host threads of the batched/served paths.  Resident mode (the
  // default) feeds one persistent kernel through a ring in pinned memory;
  // TCI_RESIDENT=0 selects one batched launch per engine step instead.
  bool resident = true;
  if (const char* s = std::getenv("TCI_RESIDENT")) resident = std::atoi(s) != 0;
  // Resident mode: one engine per host core up to 16 (measured on a 16-core host
  // with 10 000-request served steps: the SMs were inside tasks 79 % of the
  // kernel's time with 8 engines, 84 % with 12 and 86 % with 16).
  const unsigned hw = std::thread::hardware_concurrency();
  int neng = resident ? (int)std::min(16u, std::max(4u, hw ? hw : 12u)) : 8;
  if (const char* s = std::getenv("TCI_ENGINES")) neng = std::max(1, std::min(32, std::atoi(s)));
  std::unique_ptr<tci_ctx> c(new tci_ctx());
  c->dpool.reset(new BlockPool(BlockPool::DEVICE, device, true));
  c->xpool.reset(new BlockPool(BlockPool::HOST, device, true));
  for (int i = 0; i < neng; ++i) {
    c->pool.emplace_back(new Engine(device));
    int rc = c->pool.back()->init();  // fails first when there is no device
    if (rc) return rc;
    if (i == 0 && !c->dpool->reserve_slab()) return fail(TCI_ERR_OOM, "device memory for site tensors");
    c->pool.back()->set_device_pool(c->dpool.get());
    c->hpools.emplace_back(new BlockPool(BlockPool::HOST, device, false));
    c->spools.emplace_back(new BlockPool(BlockPool::DEVICE, device, false));
    if (resident && !c->hpools.back()->reserve_slab()) return fail(TCI_ERR_OOM, "pinned host memory");
  }
  c->engp = c->pool[0].get();
  if (resident) {
    c->rq.reset(new ResidentQueue());
    int idle_us = 20000;
    if (const char* s = std::getenv("TCI_RESIDENT_IDLE_US")) idle_us = std::max(100, std::atoi(s));
    int rc = c->rq->init(device, c->pool[0]->num_sms, idle_us);
    if (rc) return rc;
    // single solves and the API calls on them run on the resident kernel too
    c->pool[0]->attach_ring(c->rq.get(), c->hpools[0].get(), c->spools[0].get());
  }
  if (hbm_budget == 0) {
    size_t fr = 0, tot = 0;
    cudaMemGetInfo(&fr, &tot);
    hbm_budget = (size_t)(0.8 * (double)fr);
  }
  for (auto& e : c->pool) e->hbm_budget = hbm_budget;
  *out = c.release();
  return 0;
}

int tci_ctx_destroy(tci_ctx* ctx) {
  delete ctx;
  return 0;
}

uintptr_t tci_ctx_stream(tci_ctx* ctx) { return (uintptr_t)ctx->eng_ref().stream(); }

int tci_ctx_synchronize(tci_ctx* ctx) {
  for (auto& eng : ctx->pool) {
    cudaError_t e = cudaStreamSynchronize(eng->stream());
    if (e != cudaSuccess) return fail(TCI_ERR_CUDA, cudaGetErrorString(e));
  }
  return 0;
}

int tci_ctx_set_resident_limits(tci_ctx* ctx, int32_t idle_us, int64_t wait_us) {
  if (idle_us < 100 || wait_us < 1) return fail(TCI_ERR_ARG, "idle_us must be >= 100 and wait_us >= 1");
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  if (!ctx->rq) return 0;  // batched launches only: nothing waits
  int rc = ctx->rq->stop();  // the next launch takes the new limits
  ctx->rq->qc->idle_us = idle_us;
  ctx->rq->wait_ns = (unsigned long long)wait_us * 1000ull;
  return rc;
}

int tci_ctx_stats(tci_ctx* ctx, tci_stats* out, int32_t reset) {
  tci_stats t{};
  for (auto& e : ctx->pool) {
    const tci_stats& s = e->stats;
    t.steps += s.steps;
    t.launches += s.launches;
    t.tasks += s.tasks;
    t.kernel_ms += s.kernel_ms;
    t.feval += s.feval;
    t.lu_updates += s.lu_updates;
    t.h2d_bytes += s.h2d_bytes;
    t.d2h_bytes += s.d2h_bytes;
    t.host_launch_ms += s.host_launch_ms;
    t.host_wait_ms += s.host_wait_ms;
    t.host_resume_ms += s.host_resume_ms;
    t.task_cycles += s.task_cycles;
    t.feval_tabulated += s.feval_tabulated;
    t.tc_ms += s.tc_ms;
    t.tc_flops += s.tc_flops;
    t.dense_macs += s.dense_macs;
    if (reset) e->stats = tci_stats{};
  }
  t.peak_live = ctx->peak_live;
  if (reset) ctx->peak_live = 0;
  if (ctx->rq) {
    t.kernel_ms += ctx->rq->kernel_ms;
    t.launches += ctx->rq->launches;
    if (reset) {
      ctx->rq->kernel_ms = 0;
      ctx->rq->launches = 0;
    }
  }
  *out = t;
  return 0;
}

// ---------------------------------------------------------------- solves
static int make_solve(tci_ctx* ctx, int32_t L, const int64_t* localdims, int32_t fid, const double* fparams,
                      int64_t nparams, tci_solve** out) {
  auto* h = new tci_solve();
  h->ctx = ctx;
  int rc = solve_init(h->s, L, localdims, fid, fparams, nparams, nullptr, 0);
  if (rc) {
    delete h;
    *out = nullptr;
    return rc;
  }
  *out = h;
  return 0;
}

// A solve whose f is caller-supplied runs on plain step launches: its value
// cache is filled by separate kernels between steps, which a persistent kernel
// holding every SM would keep waiting.
static int run_solve(tci_ctx* ctx, Solve& s, CoTask& t) {
  if (!s.fcache) return ctx->eng_ref().run(t);
  if (ctx->rq) {
    int rc = ctx->rq->stop();
    if (rc) return rc;
  }
  return ctx->eng_ref().run(t, false);
}

int tci_solve_create(tci_ctx* ctx, int32_t L, const int64_t* localdims, int32_t fid, const double* fparams,
                     int64_t nparams, const int64_t* pivots, int64_t np, tci_solve** out) {
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  int rc = make_solve(ctx, L, localdims, fid, fparams, nparams, out);
  if (rc) return rc;
  auto piv = to_pivots(pivots, np, L, (*out)->s.d, &rc);
  if (!rc) {
    CoTask t = co_construct(ctx->eng_ref(), (*out)->s, piv);
    rc = run_solve(ctx, (*out)->s, t);
  }
  if (rc) {
    ctx->eng_ref().release_solve((*out)->s);
    delete *out;
    *out = nullptr;
  }
  return rc;
}

int tci_solve_destroy(tci_solve* s) {
  if (!s) return 0;
  std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
  s->ctx->eng_ref().release_solve(s->s);
  delete s;
  return 0;
}

int tci_fcache_stats(const tci_solve* s, int64_t* entries, int64_t* evaluated, int64_t* calls) {
  if (!s) return fail(TCI_ERR_ARG, "null solve");
  const FCache* c = s->s.fcache.get();
  if (entries) *entries = c ? (int64_t)c->count : 0;
  if (evaluated) *evaluated = c ? c->evaluated : 0;
  if (calls) *calls = c ? c->calls : 0;
  return 0;
}

int tci_crossinterpolate2(tci_ctx* ctx, int32_t L, const int64_t* localdims, int32_t fid,
                          const double* fparams, int64_t nparams, const int64_t* pivots, int64_t np,
                          const tci_opts* opts, tci_solve** out) {
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  int rc = make_solve(ctx, L, localdims, fid, fparams, nparams, out);
  if (rc) return rc;
  std::vector<int64_t> ones;
  if (!pivots || np == 0) {
    ones.assign(L, 1);
    pivots = ones.data();
    np = 1;
  }
  auto piv = to_pivots(pivots, np, L, (*out)->s.d, &rc);
  if (!rc) {
    tci_opts o;
    if (opts)
      o = *opts;
    else
      tci_opts_default(&o);
    CoTask t = co_crossinterpolate2(ctx->eng_ref(), (*out)->s, piv, o);
    rc = run_solve(ctx, (*out)->s, t);
  }
  if (rc) {
    ctx->eng_ref().release_solve((*out)->s);
    delete *out;
    *out = nullptr;
  }
  return rc;
}

int tci_optimize(tci_solve* s, const tci_opts* opts) {
  std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
  tci_opts o;
  if (opts)
    o = *opts;
  else
    tci_opts_default(&o);
  CoTask t = co_optimize(s->ctx->eng_ref(), s->s, o);
  return run_solve(s->ctx, s->s, t);
}

int tci_updatepivots(tci_solve* s, int32_t b, int32_t leftorthogonal, double reltol, double abstol,
                     int64_t maxbonddim) {
  std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
  if (b < 1 || b > s->s.L - 1) return fail(TCI_ERR_ARG, "bond index out of range");
  CoTask t = co_updatepivots(s->ctx->eng_ref(), s->s, b - 1, leftorthogonal != 0, reltol, abstol,
                             maxbonddim <= 0 ? TYPEMAX : maxbonddim, nullptr, nullptr);
  return run_solve(s->ctx, s->s, t);
}

int tci_sweep2site(tci_solve* s, int32_t niter, int32_t iter1, double abstol, int64_t maxbonddim,
                   int32_t sweepstrategy, int32_t strictlynested, int32_t fillsitetensors) {
  std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
  CoTask t = co_sweep2site(s->ctx->eng_ref(), s->s, niter, iter1, abstol, maxbonddim <= 0 ? TYPEMAX : maxbonddim,
                           sweepstrategy, strictlynested != 0, fillsitetensors != 0);
  return run_solve(s->ctx, s->s, t);
}

int tci_sweep1site(tci_solve* s, int32_t forward, double reltol, double abstol, int64_t maxbonddim,
                   int32_t updatetensors) {
  std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
  CoTask t = co_sweep1site(s->ctx->eng_ref(), s->s, forward != 0, reltol, abstol,
                           maxbonddim <= 0 ? TYPEMAX : maxbonddim, updatetensors != 0);
  return run_solve(s->ctx, s->s, t);
}

int tci_fillsitetensors(tci_solve* s) {
  std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
  CoTask t = co_fillsitetensors(s->ctx->eng_ref(), s->s);
  return run_solve(s->ctx, s->s, t);
}

int tci_addglobalpivots(tci_solve* s, const int64_t* pivots, int64_t np) {
  std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
  int rc = 0;
  auto piv = to_pivots(pivots, np, s->s.L, s->s.d, &rc);
  if (rc) return rc;
  rc = addglobalpivots(s->s, piv);
  if (!rc && !piv.empty()) s->ctx->eng_ref().release_cores(s->s);
  return rc;
}

int tci_addglobalpivots1sitesweep(tci_solve* s, const int64_t* pivots, int64_t np, double reltol,
                                  double abstol, int64_t maxbonddim) {
  int rc = tci_addglobalpivots(s, pivots, np);
  if (rc) return rc;
  // makecanonical! (tensorci2.jl:463-474)
  rc = tci_sweep1site(s, 1, 0.0, 0.0, 0, 0);
  if (!rc) rc = tci_sweep1site(s, 0, reltol, abstol, maxbonddim, 0);
  if (!rc) rc = tci_sweep1site(s, 1, reltol, abstol, maxbonddim, 1);
  return rc;
}

int tci_solve_length(const tci_solve* s, int32_t* L) {
  *L = s->s.L;
  return 0;
}

int tci_linkdims(const tci_solve* s, int64_t* out) {
  for (int b = 0; b < s->s.L - 1; ++b) out[b] = (int64_t)s->s.Iset[b + 1].n;
  return 0;
}

double tci_maxsamplevalue(const tci_solve* s) { return s->s.maxsample; }

int64_t tci_solve_nfeval(const tci_solve* s) { return s->s.nfeval; }

int tci_get_sets(const tci_solve* s, int32_t b, int64_t* I, int64_t* nI, int64_t* J, int64_t* nJ) {
  if (b < 1 || b > s->s.L) return fail(TCI_ERR_ARG, "site index out of range");
  const IndexSet& Is = s->s.Iset[b - 1];
  const IndexSet& Js = s->s.Jset[b - 1];
  *nI = (int64_t)Is.n;
  *nJ = (int64_t)Js.n;
  if (I)
    for (size_t i = 0; i < Is.n; ++i)
      for (int q = 0; q < Is.len; ++q) I[i * Is.len + q] = (int64_t)Is.at(i)[q] + 1;
  if (J)
    for (size_t j = 0; j < Js.n; ++j)
      for (int q = 0; q < Js.len; ++q) J[j * Js.len + q] = (int64_t)Js.at(j)[q] + 1;
  return 0;
}

// Iset[b] / Jset[b] <- the given multi-indices (1-based, row-major: nI x (b-1)
// and nJ x (L-b)); the site tensors are invalidated (tensorci2.jl:528-529 style
// replacement of the index sets, as a restart would do).
int tci_set_sets(tci_solve* s, int32_t b, const int64_t* I, int64_t nI, const int64_t* J, int64_t nJ) {
  std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
  Solve& v = s->s;
  if (b < 1 || b > v.L) return fail(TCI_ERR_ARG, "site index out of range");
  if (nI < 0 || nJ < 0) return fail(TCI_ERR_ARG, "negative set size");
  IndexSet Is, Js;
  Is.len = b - 1;
  Js.len = v.L - b;
  std::vector<uint8_t> buf((size_t)std::max(v.L, 1));
  for (int64_t i = 0; i < nI; ++i) {
    for (int q = 0; q < Is.len; ++q) {
      const int64_t x = I[i * Is.len + q];
      if (x < 1 || x > v.d[q]) return fail(TCI_ERR_ARG, "index out of range");
      buf[q] = (uint8_t)(x - 1);
    }
    if (Is.len == 0) ++Is.n; else Is.push(buf.data());
  }
  for (int64_t j = 0; j < nJ; ++j) {
    for (int q = 0; q < Js.len; ++q) {
      const int64_t x = J[j * Js.len + q];
      if (x < 1 || x > v.d[b + q]) return fail(TCI_ERR_ARG, "index out of range");
      buf[q] = (uint8_t)(x - 1);
    }
    if (Js.len == 0) ++Js.n; else Js.push(buf.data());
  }
  v.Iset[b - 1] = std::move(Is);
  v.Jset[b - 1] = std::move(Js);
  s->ctx->eng_ref().release_cores(v);
  return 0;
}

// bonderrors (tensorci2.jl:132-139): L-1 doubles
int tci_bonderrors(const tci_solve* s, double* out) {
  std::copy(s->s.bonderrors.begin(), s->s.bonderrors.end(), out);
  return 0;
}

int tci_get_core(const tci_solve* s, int32_t b, double* out, int64_t* dims) {
  if (b < 1 || b > s->s.L) return fail(TCI_ERR_ARG, "site index out of range");
  if (!s->s.cores_valid) return fail(TCI_ERR_GENERIC, "site tensors are not available");
  const Core& c = s->s.cores[b - 1];
  dims[0] = c.d0;
  dims[1] = c.d1;
  dims[2] = c.d2;
  if (out && c.elems()) {
    cudaError_t e = cudaMemcpyAsync(out, c.p, c.elems() * sizeof(double), cudaMemcpyDeviceToHost,
                                    s->ctx->eng_ref().stream());
    if (e == cudaSuccess) e = cudaStreamSynchronize(s->ctx->eng_ref().stream());
    if (e != cudaSuccess) return fail(TCI_ERR_CUDA, cudaGetErrorString(e));
    s->ctx->eng_ref().stats.d2h_bytes += (int64_t)(c.elems() * sizeof(double));
  }
  return 0;
}

int tci_get_cores_pinned(tci_ctx* ctx, int64_t n, tci_solve* const* solves, double** out, int64_t* total_elems) {
  *out = nullptr;
  *total_elems = 0;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  std::vector<const double*> src;
  std::vector<int64_t> len;
  int64_t total = 0;
  for (int64_t i = 0; i < n; ++i) {
    const Solve& s = solves[i]->s;
    if (!s.cores_valid) return fail(TCI_ERR_GENERIC, "site tensors are not available");
    for (const Core& c : s.cores) {
      src.push_back(c.p);
      len.push_back((int64_t)c.elems());
      total += (int64_t)c.elems();
    }
  }
  double* buf = (double*)ctx->xpool->alloc((size_t)std::max<int64_t>(total, 1) * sizeof(double));
  if (!buf) return fail(TCI_ERR_OOM, "pinned host memory for the export");
  int rc = ctx->eng_ref().gather_to_pinned(src, len, buf);
  if (rc) {
    ctx->xpool->free(buf);
    return rc;
  }
  *out = buf;
  *total_elems = total;
  return 0;
}

int tci_host_free(tci_ctx* ctx, void* p) {
  ctx->xpool->free(p);
  return 0;
}

int tci_get_core_dims_batched(int64_t n, tci_solve* const* solves, int64_t* dims) {
  int64_t q = 0;
  for (int64_t i = 0; i < n; ++i) {
    const Solve& s = solves[i]->s;
    if (!s.cores_valid) return fail(TCI_ERR_GENERIC, "site tensors are not available");
    for (const Core& c : s.cores) {
      dims[q++] = c.d0;
      dims[q++] = c.d1;
      dims[q++] = c.d2;
    }
  }
  return 0;
}

int tci_get_cores_batched(tci_ctx* ctx, int64_t n, tci_solve* const* solves, double* out,
                          const int64_t* out_offsets) {
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  std::vector<const double*> src;
  std::vector<int64_t> len;
  int64_t expect = -1;
  for (int64_t i = 0; i < n; ++i) {
    const Solve& s = solves[i]->s;
    if (!s.cores_valid) return fail(TCI_ERR_GENERIC, "site tensors are not available");
    int64_t pos = out_offsets[i];
    if (expect >= 0 && pos != expect) return fail(TCI_ERR_ARG, "out_offsets must be contiguous");
    for (const Core& c : s.cores) {
      src.push_back(c.p);
      len.push_back((int64_t)c.elems());
      pos += (int64_t)c.elems();
    }
    expect = pos;
  }
  if (n == 0) return 0;
  return ctx->eng_ref().gather_to_host(src, len, out + out_offsets[0]);
}

int tci_get_errors(const tci_solve* s, double* pivoterrors, int64_t* npe, double* bonderrors) {
  *npe = (int64_t)s->s.pivoterrors.size();
  if (pivoterrors) std::copy(s->s.pivoterrors.begin(), s->s.pivoterrors.end(), pivoterrors);
  if (bonderrors) std::copy(s->s.bonderrors.begin(), s->s.bonderrors.end(), bonderrors);
  return 0;
}

int tci_get_history(const tci_solve* s, int64_t* ranks, double* errors, int64_t* nglobal, int64_t* niter) {
  *niter = (int64_t)s->s.ranks.size();
  if (ranks) std::copy(s->s.ranks.begin(), s->s.ranks.end(), ranks);
  if (errors) std::copy(s->s.errors.begin(), s->s.errors.end(), errors);
  if (nglobal) std::copy(s->s.nglobal.begin(), s->s.nglobal.end(), nglobal);
  return 0;
}

int tci_evaluate(tci_solve* s, const int64_t* points, int64_t np, double* out) {
  std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
  std::vector<uint8_t> pts;
  int rc = pack_points(points, np, s->s.L, s->s.d, pts);
  if (rc) return rc;
  // up to 2^20 points per engine step (split into tasks inside co_evaluate)
  const int64_t chunk = 1 << 20;
  for (int64_t b = 0; b < np; b += chunk) {
    int64_t n = std::min(chunk, np - b);
    CoTask t = co_evaluate(s->ctx->eng_ref(), s->s, pts.data() + b * s->s.L, n, nullptr, out + b);
    rc = run_solve(s->ctx, s->s, t);
    if (rc) return rc;
  }
  return 0;
}

int tci_sum(tci_solve* s, double* out) {
  std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
  CoTask t = co_sum(s->ctx->eng_ref(), s->s, out);
  return run_solve(s->ctx, s->s, t);
}

namespace {

// evaluate() of the train held in s.cores at np points (packed 0-based local
// indices) with TF32 hi/lo split products on the tensor cores
// (tci_tc_evaluate_split); the first min(np, 256) points are also evaluated in
// FP64 and *err_est = max |split - fp64| / max |fp64| over them.
int split_evaluate(tci_ctx* ctx, Solve& s, const std::vector<uint8_t>& pts, int64_t np, double* out, double* err_est) {
  const int L = s.L;
  std::vector<int64_t> dims((size_t)(3 * L));
  std::vector<const double*> cores((size_t)L);
  for (int b = 0; b < L; ++b) {
    const Core& c = s.cores[(size_t)b];
    if (!c.p) return fail(TCI_ERR_GENERIC, "site tensors are not available (call fillsitetensors first)");
    dims[3 * b] = c.d0;
    dims[3 * b + 1] = c.d1;
    dims[3 * b + 2] = c.d2;
    cores[(size_t)b] = c.p;
  }
  if (L > 64 || !tci_tc_eval_supported(L, dims.data()))
    return fail(TCI_ERR_ARG, "split-precision evaluation needs bonds <= 128, at most 64 sites and "
                             "d * roundup(bond, 16) <= 512 per site");
  if (ctx->rq) {  // plain launches: the tensor-core kernel needs the SMs
    int rc = ctx->rq->stop();
    if (rc) return rc;
  }
  Engine& e = ctx->eng_ref();
  int dev = 0, nsm = 148;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int ns = (int)std::min<int64_t>(np, 256);
  const size_t ws = tci_tc_eval_workspace(L, dims.data());
  double* dpts = e.alloc_core(std::max<size_t>(((size_t)np * L + 7) / 8, 1));
  double* dout = e.alloc_core(std::max<size_t>((size_t)np + (size_t)ns + 1, 1));
  double* dws = e.alloc_core(ws / 8 + 1);
  int rc = 0;
  if (!dpts || !dout || !dws) rc = fail(TCI_ERR_OOM, "device memory for split-precision evaluation");
  int* derr = (int*)(dout + np + ns);
  std::vector<double> samp((size_t)ns);
  int herr = 0;
  auto ck = [&](cudaError_t ce) {
    if (!rc && ce != cudaSuccess) rc = fail(TCI_ERR_CUDA, cudaGetErrorString(ce));
  };
  if (!rc && np > 0) ck(cudaMemcpyAsync(dpts, pts.data(), (size_t)np * L, cudaMemcpyHostToDevice, e.stream()));
  if (!rc) ck(cudaMemsetAsync(derr, 0, sizeof(int), e.stream()));
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  if (!rc) ck(cudaEventCreate(&ev0));
  if (!rc) ck(cudaEventCreate(&ev1));
  if (!rc) ck(cudaEventRecord(ev0, e.stream()));
  if (!rc)
    ck(tci_tc_evaluate_split(L, dims.data(), cores.data(), (const uint8_t*)dpts, np, dout, ns, dout + np, dws, derr,
                             nsm, e.stream()));
  if (!rc) ck(cudaEventRecord(ev1, e.stream()));
  if (!rc && np > 0) ck(cudaMemcpyAsync(out, dout, (size_t)np * 8, cudaMemcpyDeviceToHost, e.stream()));
  if (!rc && ns > 0) ck(cudaMemcpyAsync(samp.data(), dout + np, (size_t)ns * 8, cudaMemcpyDeviceToHost, e.stream()));
  if (!rc) ck(cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, e.stream()));
  if (!rc) ck(cudaStreamSynchronize(e.stream()));
  if (!rc && herr) rc = fail(TCI_ERR_TIMEOUT, "tensor-core evaluation: a bounded wait ran out (code " +
                                                  std::to_string(herr) + ")");
  if (!rc) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, ev0, ev1) == cudaSuccess) e.stats.tc_ms += ms;
    // per point and site b >= 1: d_b products of (1 x r_{b-1}) (r_{b-1} x r_b)
    double fl = 0.0;
    for (int b = 1; b < L; ++b) fl += 2.0 * (double)dims[3 * b + 1] * (double)dims[3 * b] * (double)dims[3 * b + 2];
    e.stats.tc_flops += fl * (double)np;
  }
  if (ev0) cudaEventDestroy(ev0);
  if (ev1) cudaEventDestroy(ev1);
  if (!rc && err_est) {
    double dmax = 0, vmax = 0;
    for (int k = 0; k < ns; ++k) {
      dmax = std::max(dmax, std::fabs(out[k] - samp[(size_t)k]));
      vmax = std::max(vmax, std::fabs(samp[(size_t)k]));
    }
    *err_est = vmax > 0 ? dmax / vmax : dmax;
  }
  if (dpts) e.free_core(dpts);
  if (dout) e.free_core(dout);
  if (dws) e.free_core(dws);
  return rc;
}

}  // namespace

int tci_evaluate_prec(tci_solve* s, const int64_t* points, int64_t np, double* out, int32_t precision,
                      double* err_est) {
  if (precision == TCI_PREC_FP64) {
    if (err_est) *err_est = 0.0;
    return tci_evaluate(s, points, np, out);
  }
  if (precision != TCI_PREC_TF32X3) return fail(TCI_ERR_ARG, "unknown precision");
  std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
  std::vector<uint8_t> pts;
  int rc = pack_points(points, np, s->s.L, s->s.d, pts);
  if (rc) return rc;
  return split_evaluate(s->ctx, s->s, pts, np, out, err_est);
}

// ---------------------------------------------------------------- batches / serving
namespace {
struct Job {
  tci_solve* solve = nullptr;
  std::optional<CoTask> task;
  bool started = false, done = false;
  double arrival = 0, t_start = 0, t_done = 0;  // seconds since the drive started
  int rc = 0;
  tci_request req{};  // the request (its arrays owned below for server jobs)
  std::vector<int64_t> dims_own;
  std::vector<double> params_own;
  double est = 0;     // HBM estimate
  int64_t id = -1;    // server request id
  double t_submit = 0;  // server: absolute submit time
};

// Source of jobs beyond the initial list (the server's queue): pull appends
// newly submitted jobs and their admission order and tells whether more may
// come; on_done reports a finished job.  Both are called under the drive lock.
struct JobFeed {
  std::function<bool(std::deque<Job>&, std::vector<int64_t>&)> pull;
  std::function<void(Job&)> on_done;
};

// Drive jobs with continuous batching, one host thread per engine of the
// context's pool.  arrival == nullptr: every request is available at t = 0.
// Each thread admits requests from the shared queue (by arrival time, the live
// cap and the HBM estimate) onto its own engine, completes its engine's batch
// when ready (resuming those solves, which queue their next tasks) and
// relaunches it.  Solves never move between engines, so the only shared state
// is the admission queue and the counters below.
struct DriveShared {
  std::mutex mu;
  int64_t next = 0, live = 0, finished = 0;
  double live_bytes = 0;
  int first_rc = 0;
  std::string first_msg;
  int fatal = 0;
  std::string fatal_msg;
};

int drive(tci_ctx* ctx, std::deque<Job>& jobs, bool use_arrival, int64_t max_live, bool keep, JobFeed* feed) {
  auto& pool = ctx->pool;
  const int G = (int)pool.size();
  int64_t n = (int64_t)jobs.size();
  if (max_live <= 0) max_live = feed ? 1024 : std::max<int64_t>(n, 1);
  const double t0 = now_s();
  const double budget = (double)pool[0]->hbm_budget;
  for (auto& j : jobs) j.est = solve_estimate_bytes(j.req);
  // Admission order: by arrival when there are arrival times; otherwise the
  // largest solves first, so that the longest serial chains do not start last
  // and leave the device with a tail of a few live solves.  Jobs from the feed
  // are admitted in submission order.
  std::vector<int64_t> order(n);
  std::iota(order.begin(), order.end(), 0);
  if (!use_arrival)
    std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) { return jobs[a].est > jobs[b].est; });
  DriveShared sh;
  bool feed_open = feed != nullptr;

  auto worker = [&](int g) {
    Engine& e = *pool[g];
    std::vector<Job*> mine;  // live jobs on this engine (deque elements do not move)
    auto finish = [&](Job* jp) {
      Job& j = *jp;
      j.done = true;
      j.t_done = now_s() - t0;
      j.rc = j.task->h.promise().rc;
      std::string msg = j.rc ? std::string(last_message()) : std::string();
      j.task.reset();
      if (!keep) e.release_solve(j.solve->s);
      std::lock_guard<std::mutex> lk(sh.mu);
      if (j.rc && !sh.first_rc && !feed) {  // a server reports errors per request
        sh.first_rc = j.rc;
        sh.first_msg = msg;
      }
      --sh.live;
      ++sh.finished;
      sh.live_bytes -= j.est;
      if (feed) feed->on_done(j);
    };
    auto reap = [&]() {
      size_t w = 0;
      for (size_t k = 0; k < mine.size(); ++k) {
        Job* jp = mine[k];
        if (jp->task && jp->task->h.done())
          finish(jp);
        else
          mine[w++] = jp;
      }
      mine.resize(w);
    };
    // take at most a fair share of the live cap so every engine gets work
    const int64_t share = std::max<int64_t>(1, (max_live + G - 1) / G);
    double last_progress = now_s(), last_done = last_progress;
    double last_switch = now_s();
    for (;;) {
      // Kernel variant by load (worker 0): with fewer live solves than SMs and no
      // admission waiting, every task gets a whole SM (k512); from two live
      // solves per SM on, two task CTAs share an SM (k256).  Tasks are
      // planned for k256's budget, which k512 satisfies, so a switch only
      // relaunches the kernel; tasks published meanwhile wait in the ring.
      if (g == 0 && ctx->rq) {
        int64_t live;
        bool admit_waiting;
        {
          std::lock_guard<std::mutex> lk(sh.mu);
          live = sh.live;
          admit_waiting = sh.next < (int64_t)order.size() && sh.live < max_live &&
                          (!use_arrival || jobs[order[sh.next]].arrival <= now_s() - t0);
        }
        const tci_kernel_set* cur = ctx->rq->ks;
        const int nsm = ctx->rq->num_sms;
        const tci_kernel_set* want = cur;
        if (cur == &tci_k256::kernels && live > 0 && live < nsm && !admit_waiting) want = &tci_k512::kernels;
        if (cur == &tci_k512::kernels && live >= 2 * nsm) want = &tci_k256::kernels;
        if (want != cur && now_s() - last_switch > 0.02) {
          last_switch = now_s();
          int rc = ctx->rq->stop();
          if (!rc) rc = ctx->rq->start(want);
          if (rc) {
            std::lock_guard<std::mutex> lk(sh.mu);
            sh.fatal = rc;
            sh.fatal_msg = last_message();
            return;
          }
        }
      }
      // admission
      for (;;) {
        Job* jp = nullptr;
        {
          std::lock_guard<std::mutex> lk(sh.mu);
          if (sh.fatal) return;
          if (feed_open && sh.next >= (int64_t)order.size()) {
            const size_t before = jobs.size();
            feed_open = feed->pull(jobs, order);
            for (size_t q = before; q < jobs.size(); ++q) jobs[q].est = solve_estimate_bytes(jobs[q].req);
          }
          double t = now_s() - t0;
          if (sh.next < (int64_t)order.size() && sh.live < max_live && (int64_t)mine.size() < share &&
              (!use_arrival || jobs[order[sh.next]].arrival <= t) &&
              (sh.live == 0 || sh.live_bytes + jobs[order[sh.next]].est <= budget)) {
            jp = &jobs[order[sh.next++]];
            ++sh.live;
            sh.live_bytes += jp->est;
            ctx->peak_live = std::max(ctx->peak_live, sh.live);
          }
        }
        if (!jp) break;
        Job& j = *jp;
        j.t_start = now_s() - t0;
        const tci_request& r = j.req;
        int rc = r.fid >= TCI_F_USER
                     ? fail(TCI_ERR_ARG, "batched solves take registered device functions only")
                     : make_solve(ctx, r.L, r.localdims, r.fid, r.fparams, r.nparams, &j.solve);
        if (rc) {
          j.started = j.done = true;
          j.rc = rc;
          std::lock_guard<std::mutex> lk(sh.mu);
          if (!sh.first_rc && !feed) {
            sh.first_rc = rc;
            sh.first_msg = last_message();
          }
          --sh.live;
          ++sh.finished;
          sh.live_bytes -= j.est;
          if (feed) feed->on_done(j);
          continue;
        }
        std::vector<std::vector<uint8_t>> piv(1, std::vector<uint8_t>(r.L, 0));
        j.task.emplace(co_crossinterpolate2(e, j.solve->s, piv, r.opts));
        j.started = true;
        mine.push_back(jp);
        j.task->h.resume();
      }
      reap();
      auto fatal = [&](int rc) {
        std::lock_guard<std::mutex> lk(sh.mu);
        sh.fatal = rc;
        sh.fatal_msg = last_message();
      };
      if (e.resident()) {
        // publish what the solves queued, resume those whose tasks are done
        int rc = e.submit();
        if (rc) return fatal(rc);
        bool progressed = false;
        rc = e.poll(progressed);
        if (rc) return fatal(rc);
        reap();
        const double tnow = now_s();
        if (progressed) {
          last_progress = last_done = tnow;
          continue;
        }
        if (!e.idle()) continue;
        if (e.has_flights()) {
          if (tnow - last_progress > 2e-3) {  // the kernel may have left on its idle limit
            rc = ctx->rq->ensure_alive();
            if (rc) return fatal(rc);
            last_progress = tnow;
          }
          if (tnow - last_done > 120.0) {
            set_error(TCI_ERR_TIMEOUT, "resident mode: no task finished for 120 s");
            return fatal(TCI_ERR_TIMEOUT);
          }
          std::this_thread::yield();
          continue;
        }
      } else {
        bool progressed = false;
        if (e.inflight() && e.ready()) {
          int rc = e.complete();
          if (rc) return fatal(rc);
          reap();
          progressed = true;
        }
        if (!e.inflight() && !e.idle()) {
          int rc = e.launch();
          if (rc) return fatal(rc);
          progressed = true;
        }
        if (progressed) continue;
        if (e.inflight()) {  // nothing else to do here: wait for the GPU
          int rc = e.complete();
          if (rc) return fatal(rc);
          reap();
          continue;
        }
      }
      if (!mine.empty()) {  // live solves but no pending task: cannot happen
        std::lock_guard<std::mutex> lk(sh.mu);
        sh.fatal = TCI_ERR_GENERIC;
        sh.fatal_msg = "engine stalled with live solves";
        return;
      }
      double wait = 0;
      {
        std::lock_guard<std::mutex> lk(sh.mu);
        if (sh.fatal) return;
        if (sh.next >= (int64_t)order.size()) {
          if (!feed_open) return;  // nothing left for this engine
          wait = 2e-4;             // the server's queue is empty: look again shortly
        } else if (use_arrival) {
          wait = jobs[order[sh.next]].arrival - (now_s() - t0);
        }
      }
      if (wait > 0)
        std::this_thread::sleep_for(std::chrono::duration<double>(std::min(wait, 1e-3)));
      else
        std::this_thread::yield();
    }
  };
  if (ctx->rq) {
    int rc = ctx->rq->start(&tci_k256::kernels);
    if (rc) return rc;
    for (int g = 0; g < G; ++g) pool[g]->set_resident(ctx->rq.get(), ctx->hpools[g].get(), ctx->spools[g].get());
  }
  std::vector<std::thread> threads;
  for (int g = 1; g < G; ++g) threads.emplace_back(worker, g);
  worker(0);
  for (auto& t : threads) t.join();
  if (ctx->rq) {
    // every published task is done once the kernel has left (a CTA leaves only
    // when it finds no published ticket, and the workers have stopped)
    int rc = ctx->rq->stop();
    for (int g = 0; g < G; ++g) {
      pool[g]->abandon();  // nothing is left here unless a fatal error stopped the workers
      pool[g]->set_resident(nullptr, nullptr, nullptr);
    }
    if (rc && !sh.fatal) return rc;
  }
  if (sh.fatal) return fail(sh.fatal, sh.fatal_msg);
  if (sh.first_rc) set_error(sh.first_rc, sh.first_msg);
  return sh.first_rc;
}
}  // namespace

int tci_crossinterpolate2_batched(tci_ctx* ctx, int64_t n, const tci_request* reqs, int64_t max_live,
                                  tci_solve** out) {
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  std::deque<Job> jobs((size_t)n);
  for (int64_t i = 0; i < n; ++i) jobs[i].req = reqs[i];
  int rc = drive(ctx, jobs, false, max_live, true, nullptr);
  for (int64_t i = 0; i < n; ++i) out[i] = jobs[i].solve;
  return rc;
}

int tci_serve_run(tci_ctx* ctx, int64_t n, const tci_request* reqs, const double* arrival, int64_t max_live,
                  double* latency, int64_t* rank, double* wall) {
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  std::deque<Job> jobs((size_t)n);
  for (int64_t i = 0; i < n; ++i) {
    jobs[i].req = reqs[i];
    jobs[i].arrival = arrival ? arrival[i] : 0.0;
  }
  double t0 = now_s();
  int rc = drive(ctx, jobs, arrival != nullptr, max_live, false, nullptr);
  if (wall) *wall = now_s() - t0;
  for (int64_t i = 0; i < n; ++i) {
    if (latency) latency[i] = jobs[i].t_done - jobs[i].arrival;
    if (rank) rank[i] = jobs[i].solve ? solve_rank(jobs[i].solve->s) : -1;
    if (jobs[i].solve) delete jobs[i].solve;
  }
  return rc;
}

// ---------------------------------------------------------------- incremental server
}  // extern "C"

struct tci_server {
  tci_ctx* ctx = nullptr;
  int64_t max_live = 0;
  std::mutex mu;
  std::condition_variable cv;
  std::deque<Job> incoming;  // submitted, not yet handed to the drive
  struct Done {
    int64_t id, rank;
    int32_t status;
    double latency;
  };
  std::vector<Done> completed;
  bool stopping = false;
  int64_t next_id = 0;
  int rc = 0;
  std::string msg;
  std::thread th;
};

namespace {
void server_main(tci_server* srv) {
  tci_ctx* ctx = srv->ctx;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);  // the server owns the context until it stops
  std::deque<Job> jobs;
  JobFeed feed;
  feed.pull = [srv](std::deque<Job>& js, std::vector<int64_t>& order) {
    std::lock_guard<std::mutex> l(srv->mu);
    while (!srv->incoming.empty()) {
      js.push_back(std::move(srv->incoming.front()));
      srv->incoming.pop_front();
      Job& j = js.back();
      j.req.localdims = j.dims_own.data();  // the arrays moved with the job
      j.req.fparams = j.params_own.empty() ? nullptr : j.params_own.data();
      order.push_back((int64_t)js.size() - 1);
    }
    return !srv->stopping;
  };
  feed.on_done = [srv](Job& j) {
    tci_server::Done d;
    d.id = j.id;
    d.status = j.rc;
    d.rank = (j.solve && !j.rc) ? solve_rank(j.solve->s) : -1;
    d.latency = now_s() - j.t_submit;
    if (j.solve) {
      delete j.solve;  // its device memory went back at the end of the solve
      j.solve = nullptr;
    }
    std::lock_guard<std::mutex> l(srv->mu);
    srv->completed.push_back(d);
    srv->cv.notify_all();
  };
  int rc = drive(ctx, jobs, false, srv->max_live, false, &feed);
  std::lock_guard<std::mutex> l(srv->mu);
  srv->rc = rc;
  if (rc) srv->msg = last_message();
  srv->cv.notify_all();
}
}  // namespace

extern "C" {

int tci_serve_start(tci_ctx* ctx, int64_t max_live, tci_server** out) {
  auto* srv = new tci_server();
  srv->ctx = ctx;
  srv->max_live = max_live;
  srv->th = std::thread(server_main, srv);
  *out = srv;
  return 0;
}

int tci_serve_submit(tci_server* srv, const tci_request* req, int64_t* id) {
  if (req->L < 2) return fail(TCI_ERR_GENERIC, "localdims should have at least 2 elements!");
  Job j;
  j.req = *req;
  j.dims_own.assign(req->localdims, req->localdims + req->L);
  if (req->nparams > 0) j.params_own.assign(req->fparams, req->fparams + req->nparams);
  j.req.localdims = j.dims_own.data();
  j.req.fparams = j.params_own.empty() ? nullptr : j.params_own.data();
  j.t_submit = now_s();
  std::lock_guard<std::mutex> l(srv->mu);
  if (srv->stopping) return fail(TCI_ERR_ARG, "the server is stopping");
  j.id = srv->next_id++;
  *id = j.id;
  srv->incoming.push_back(std::move(j));
  return 0;
}

int tci_serve_poll(tci_server* srv, int64_t cap, int64_t* ids, int32_t* status, int64_t* ranks, double* latency,
                   int64_t* n, int32_t timeout_ms) {
  std::unique_lock<std::mutex> l(srv->mu);
  if (timeout_ms > 0 && srv->completed.empty())
    srv->cv.wait_for(l, std::chrono::milliseconds(timeout_ms), [&] { return !srv->completed.empty() || srv->rc; });
  const int64_t k = std::min<int64_t>(cap, (int64_t)srv->completed.size());
  for (int64_t q = 0; q < k; ++q) {
    const auto& d = srv->completed[(size_t)q];
    if (ids) ids[q] = d.id;
    if (status) status[q] = d.status;
    if (ranks) ranks[q] = d.rank;
    if (latency) latency[q] = d.latency;
  }
  srv->completed.erase(srv->completed.begin(), srv->completed.begin() + k);
  *n = k;
  if (srv->rc) return fail(srv->rc, srv->msg);
  return 0;
}

int tci_serve_stop(tci_server* srv) {
  {
    std::lock_guard<std::mutex> l(srv->mu);
    srv->stopping = true;
  }
  if (srv->th.joinable()) srv->th.join();
  const int rc = srv->rc;
  const std::string msg = srv->msg;
  delete srv;
  if (rc) return fail(rc, msg);
  return 0;
}

// ---------------------------------------------------------------- f and host helpers
int tci_feval(tci_ctx* ctx, int32_t fid, const double* fparams, int64_t nparams, int32_t L,
              const int64_t* localdims, const int64_t* points, int64_t np, double* out) {
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  Solve s;
  int rc = solve_init(s, L, localdims, fid, fparams, nparams, nullptr, 0);
  if (rc) return rc;
  std::vector<uint8_t> pts;
  rc = pack_points(points, np, L, s.d, pts);
  if (rc) return rc;
  const int64_t chunk = 1 << 20;
  for (int64_t b = 0; b < np; b += chunk) {
    int64_t n = std::min(chunk, np - b);
    CoTask t = co_evaluate(ctx->eng_ref(), s, pts.data() + b * L, n, out + b, nullptr);
    rc = run_solve(ctx, s, t);
    if (rc) return rc;
  }
  return 0;
}

int tci_optfirstpivot(tci_ctx* ctx, int32_t fid, const double* fparams, int64_t nparams, int32_t L,
                      const int64_t* localdims, int64_t* pivot, int32_t maxsweep) {
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  Solve s;
  int rc = solve_init(s, L, localdims, fid, fparams, nparams, nullptr, 0);
  if (rc) return rc;
  std::vector<std::vector<uint8_t>> piv = to_pivots(pivot, 1, L, s.d, &rc);
  if (rc) return rc;
  std::vector<double> valf;
  CoTask t = co_optfirstpivots(ctx->eng_ref(), s, &piv, &valf, maxsweep > 0 ? maxsweep : 1000);
  rc = run_solve(ctx, s, t);
  if (rc) return rc;
  for (int q = 0; q < L; ++q) pivot[q] = (int64_t)piv[0][(size_t)q] + 1;
  return 0;
}

int tci_estimatetrueerror(tci_solve* s, int32_t nsearch, const int64_t* initialpoints, int64_t np, uint64_t seed,
                          int64_t cap, int64_t* pivots, double* errors, int64_t* nout) {
  std::lock_guard<std::recursive_mutex> lk(s->ctx->mu);
  const int L = s->s.L;
  int rc = 0;
  std::vector<std::vector<uint8_t>> starts;
  if (np > 0) {
    starts = to_pivots(initialpoints, np, L, s->s.d, &rc);
    if (rc) return rc;
  } else {
    if (nsearch <= 0) return fail(TCI_ERR_GENERIC, "No search is performed");
    tci_rng rng;
    tci_rng_seed(&rng, seed);
    starts.assign((size_t)nsearch, std::vector<uint8_t>((size_t)L));
    for (auto& p : starts)
      for (int q = 0; q < L; ++q) p[(size_t)q] = (uint8_t)(tci_rng_uniform1(&rng, (uint64_t)s->s.d[(size_t)q]) - 1);
  }
  std::vector<std::pair<std::vector<uint8_t>, double>> res;
  CoTask t = co_estimatetrueerror(s->ctx->eng_ref(), s->s, std::move(starts), &res);
  rc = run_solve(s->ctx, s->s, t);
  if (rc) return rc;
  *nout = (int64_t)res.size();
  for (int64_t k = 0; k < std::min<int64_t>(cap, (int64_t)res.size()); ++k) {
    for (int q = 0; q < L; ++q) pivots[k * L + q] = (int64_t)res[(size_t)k].first[(size_t)q] + 1;
    errors[k] = res[(size_t)k].second;
  }
  return 0;
}

int tci_convergencecriterion(const int64_t* ranks, const double* errors, const int64_t* nglobalpivots,
                             int64_t n, double tolerance, int64_t maxbonddim, int64_t ncheckhistory,
                             int32_t checkconvglobalpivot) {
  std::vector<i64> r(ranks, ranks + n), g(nglobalpivots, nglobalpivots + n);
  std::vector<double> e(errors, errors + n);
  return convergencecriterion(r, e, g, tolerance, maxbonddim, ncheckhistory, checkconvglobalpivot != 0) ? 1 : 0;
}

// ---------------------------------------------------------------- rrLU
int tci_rrlu(tci_ctx* ctx, const double* A, int64_t m, int64_t n, int64_t maxrank, double reltol,
             double abstol, int32_t leftorthogonal, int64_t* rowperm, int64_t* colperm, double* L, double* U,
             int64_t* npivot, double* error) {
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  if (m < 0 || n < 0 || m > INT32_MAX || n > INT32_MAX || m * n > INT32_MAX)
    return fail(TCI_ERR_ARG, "matrix size out of range");
  Engine& e = ctx->eng_ref();
  Req r;
  r.t.kind = TCI_TASK_RRLU;
  r.t.m = (int32_t)m;
  r.t.n = (int32_t)n;
  int64_t kmax = std::min<int64_t>(maxrank <= 0 ? INT64_MAX : maxrank, std::min(m, n));
  r.t.maxrank = (int32_t)kmax;
  r.t.kcap = (int32_t)kmax;
  r.t.reltol = reltol;
  r.t.abstol = abstol;
  r.t.leftorth = leftorthogonal ? 1 : 0;
  r.t.post = TCI_POST_FACTORS;
  r.ain_host = A;
  // factors (m*n doubles) followed by the full permutations (m + n int32)
  size_t out_elems = (size_t)(m * n) + ((size_t)(m + n) * 4 + 7) / 8;
  double* dout = e.alloc_core(out_elems);
  if (!dout) return fail(TCI_ERR_OOM, "device memory");
  r.t.core_out = dout;
  std::vector<Req*> reqs{&r};
  int rc = e.run_tasks(reqs);
  if (rc) {
    e.free_core(dout);
    return rc;
  }
  const tci_result_head* h = r.head();
  const int K = h->npivot;
  std::vector<double> F(out_elems);
  cudaError_t ce = cudaMemcpyAsync(F.data(), dout, out_elems * 8, cudaMemcpyDeviceToHost, e.stream());
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(e.stream());
  e.free_core(dout);
  if (ce != cudaSuccess) return fail(TCI_ERR_CUDA, cudaGetErrorString(ce));
  const int32_t* perms = (const int32_t*)(F.data() + m * n);
  if (rowperm)
    for (int64_t i = 0; i < m; ++i) rowperm[i] = perms[i] + 1;
  if (colperm)
    for (int64_t j = 0; j < n; ++j) colperm[j] = perms[m + j] + 1;
  // L = tril(A[:, 1:K]), U = triu(A[1:K, :]), unit diagonal on L or U (matrixlu.jl:162-174)
  if (L)
    for (int64_t j = 0; j < K; ++j)
      for (int64_t i = 0; i < m; ++i)
        L[i + j * m] = i < j ? 0.0 : (i == j && leftorthogonal ? 1.0 : F[i + j * m]);
  if (U)
    for (int64_t j = 0; j < n; ++j)
      for (int64_t i = 0; i < K; ++i)
        U[i + j * K] = i > j ? 0.0 : (i == j && !leftorthogonal ? 1.0 : F[i + j * m]);
  if (npivot) *npivot = K;
  if (error) *error = h->error;
  if (h->status & TCI_ST_NAN) return fail(TCI_ERR_NAN, "lu.L contains NaNs");
  return 0;
}

int tci_rrlu_batched(tci_ctx* ctx, int64_t nmat, const double* A, const int64_t* offsets, const int64_t* ms,
                     const int64_t* ns, int64_t maxrank, double reltol, double abstol, int32_t leftorthogonal,
                     int64_t* piv, const int64_t* piv_offsets, int64_t* npivots, double* errors) {
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  Engine& e = ctx->eng_ref();
  std::vector<Req> rs((size_t)nmat);
  std::vector<Req*> ptrs;
  for (int64_t i = 0; i < nmat; ++i) {
    Req& r = rs[i];
    if (ms[i] * ns[i] > INT32_MAX) return fail(TCI_ERR_ARG, "matrix size out of range");
    r.t.kind = TCI_TASK_RRLU;
    r.t.m = (int32_t)ms[i];
    r.t.n = (int32_t)ns[i];
    int64_t kmax = std::min<int64_t>(maxrank <= 0 ? INT64_MAX : maxrank, std::min(ms[i], ns[i]));
    r.t.maxrank = (int32_t)kmax;
    r.t.kcap = (int32_t)kmax;
    r.t.reltol = reltol;
    r.t.abstol = abstol;
    r.t.leftorth = leftorthogonal ? 1 : 0;
    r.t.post = TCI_POST_NONE;
    r.ain_host = A + offsets[i];
    ptrs.push_back(&r);
  }
  int rc = e.run_tasks(ptrs);
  if (rc) return rc;
  int bad = 0;
  for (int64_t i = 0; i < nmat; ++i) {
    const Req& r = rs[i];
    const tci_result_head* h = r.head();
    npivots[i] = h->npivot;
    errors[i] = h->error;
    if (h->status & TCI_ST_NAN) bad = 1;
    if (piv) {
      int64_t* o = piv + piv_offsets[i];
      for (int k = 0; k < h->npivot; ++k) {
        o[k] = r.rowperm()[k] + 1;
        o[r.t.kcap + k] = r.colperm()[k] + 1;
      }
    }
  }
  if (bad) return fail(TCI_ERR_NAN, "lu.L contains NaNs");
  return 0;
}

// ---------------------------------------------------------------- autotuner
namespace {

// Seeded calibration matrices of one tuning bucket: A = G1 diag(10^(-k/4)) G2^T
// + 1e-12 noise (the decay of the batched-rrLU workload), Gaussian G1, G2; the
// terms beyond k = 48 (below 1e-12) are left to the noise.
struct TuneRng {
  uint64_t s;
  uint64_t next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
  }
  double uniform() { return ((double)(next() >> 11) + 0.5) * (1.0 / 9007199254740992.0); }
  double normal() {
    const double u = uniform(), v = uniform();
    return std::sqrt(-2.0 * std::log(u)) * std::cos(6.283185307179586 * v);
  }
};

// Calibration matrices of a bucket, two kinds in equal numbers:
//  - low rank: U diag(10^(-k/4)) V^T + 1e-12 noise, rank <= 48 (a factorization
//    stops near rank 40 and never reaches a small trailing block unless the
//    matrix is small);
//  - graded: u_ij 10^(-(p_i + q_j)/c), u uniform in [-1, 1] and p, q random
//    permutations of the rows and columns, c = 0.18 min(m, n): the pivots
//    decay like 10^(-2k/c) and reach reltol 1e-10 near k = 0.9 min(m, n), so
//    the factorization ends in the trailing blocks the tail size acts on.
void tune_matrix_lowrank(TuneRng& g, int64_t m, int64_t n, std::vector<double>& A) {
  const int64_t r = std::min<int64_t>(std::min(m, n), 48);
  std::vector<double> G1((size_t)(m * r)), G2((size_t)(n * r));
  for (auto& x : G1) x = g.normal();
  for (auto& x : G2) x = g.normal();
  A.assign((size_t)(m * n), 0.0);
  for (int64_t k = 0; k < r; ++k) {
    const double sk = std::pow(10.0, -(double)k / 4.0);
    for (int64_t j = 0; j < n; ++j) {
      const double y = sk * G2[(size_t)(j + n * k)];
      for (int64_t i = 0; i < m; ++i) A[(size_t)(i + m * j)] += G1[(size_t)(i + m * k)] * y;
    }
  }
  for (auto& x : A) x += 1e-12 * g.normal();
}

void tune_matrix_graded(TuneRng& g, int64_t m, int64_t n, std::vector<double>& A) {
  const double c = std::max(1.0, 0.18 * (double)std::min(m, n));
  auto scales = [&](int64_t k) {
    std::vector<int64_t> p((size_t)k);
    for (int64_t i = 0; i < k; ++i) p[(size_t)i] = i;
    for (int64_t i = k - 1; i > 0; --i) std::swap(p[(size_t)i], p[(size_t)(g.next() % (uint64_t)(i + 1))]);
    std::vector<double> s((size_t)k);
    for (int64_t i = 0; i < k; ++i) s[(size_t)i] = std::pow(10.0, -(double)p[(size_t)i] / c);
    return s;
  };
  const std::vector<double> rs = scales(m), cs = scales(n);
  A.resize((size_t)(m * n));
  for (int64_t j = 0; j < n; ++j)
    for (int64_t i = 0; i < m; ++i) A[(size_t)(i + m * j)] = (2.0 * g.uniform() - 1.0) * rs[(size_t)i] * cs[(size_t)j];
}

struct TuneSet {
  std::vector<std::vector<double>> mats;
  std::vector<int64_t> ms, ns;
};

// Seeded calibration set of bucket bk: enough matrices for about three tasks per
// CTA of the batched launch (capped at 24 M elements, at least one per CTA).
TuneSet tune_set(int bk, uint64_t seed, int64_t grid) {
  static const int64_t lo[6] = {8, 25, 49, 97, 161, 257}, hi[6] = {24, 48, 96, 160, 256, 320};
  const int size = bk / 2, elong = bk % 2;
  const double mid = 0.5 * (double)(lo[size] + hi[size]);
  const double avg = mid * mid * (elong ? 3.0 : 1.0);
  const int64_t nmat = std::max(grid, std::min<int64_t>(3 * grid, (int64_t)(24e6 / avg)));
  TuneRng g{seed};
  TuneSet S;
  S.mats.resize((size_t)nmat);
  S.ms.resize((size_t)nmat);
  S.ns.resize((size_t)nmat);
  for (int64_t q = 0; q < nmat; ++q) {
    const int64_t s0 = lo[size] + (int64_t)(g.uniform() * (double)(hi[size] - lo[size] + 1));
    int64_t m = s0, n = s0;
    if (elong) {
      if (q & 2)
        n = 3 * s0;
      else
        m = 3 * s0;
    }
    S.ms[(size_t)q] = m;
    S.ns[(size_t)q] = n;
    if (q & 1)
      tune_matrix_lowrank(g, m, n, S.mats[(size_t)q]);
    else
      tune_matrix_graded(g, m, n, S.mats[(size_t)q]);
  }
  return S;
}

// Kernel milliseconds of one batched launch of the set's factorizations with
// tail size c (CUDA events around the step kernel).
int tune_time(Engine& e, const TuneSet& S, int32_t c, double& ms) {
  const size_t nmat = S.mats.size();
  std::vector<Req> rs(nmat);
  std::vector<Req*> ptrs;
  for (size_t q = 0; q < nmat; ++q) {
    Req& r = rs[q];
    r.t.kind = TCI_TASK_RRLU;
    r.t.m = (int32_t)S.ms[q];
    r.t.n = (int32_t)S.ns[q];
    r.t.maxrank = r.t.kcap = (int32_t)std::min(S.ms[q], S.ns[q]);
    r.t.reltol = 1e-10;
    r.t.leftorth = 1;
    r.t.post = TCI_POST_NONE;
    r.t.tail_elems = c;
    r.ain_host = S.mats[q].data();
    ptrs.push_back(&r);
  }
  const double k0 = e.stats.kernel_ms;
  const int rc = e.run_tasks(ptrs);
  ms = e.stats.kernel_ms - k0;
  return rc;
}

}  // namespace

int tci_autotune_rrlu(tci_ctx* ctx, int32_t reps, double* speedup, double* ms_default, double* ms_tuned) {
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  if (ctx->rq) {  // plain launches: the calibration times the batched step kernel
    int rc = ctx->rq->stop();
    if (rc) return rc;
  }
  Engine& e = ctx->eng_ref();
  const int32_t cands[] = {1, 96, 192, 384, 768, 1536};
  const int32_t dflt = 192;
  // a candidate replaces the default only if it is this much faster on the
  // calibration set and again on a fresh validation set
  const double margin = 0.98;
  reps = std::max(1, reps);
  const int64_t grid = (int64_t)e.num_sms * tci_k256::kernels.ctas_per_sm;
  double tot_def = 0.0, tot_best = 0.0;
  int32_t table[Engine::TUNE_BUCKETS];
  const bool timing = e.timing;
  e.timing = true;
  int rc = 0;
  for (int bk = 0; bk < Engine::TUNE_BUCKETS && !rc; ++bk) {
    const TuneSet S = tune_set(bk, 0x7a11ULL + (uint64_t)bk, grid);
    double warm = 0.0;
    rc = tune_time(e, S, dflt, warm);  // first launch of the set warms up
    std::vector<double> tmin(sizeof(cands) / sizeof(cands[0]), 1e300);
    for (int rep = 0; rep < reps && !rc; ++rep)  // candidates interleaved per repetition
      for (size_t ci = 0; ci < tmin.size() && !rc; ++ci) {
        double t = 0.0;
        rc = tune_time(e, S, cands[ci], t);
        tmin[ci] = std::min(tmin[ci], t);
      }
    if (rc) break;
    size_t best = 0, idef = 0;
    for (size_t ci = 0; ci < tmin.size(); ++ci) {
      if (tmin[ci] < tmin[best]) best = ci;
      if (cands[ci] == dflt) idef = ci;
    }
    int32_t choice = dflt;
    double t_def = tmin[idef], t_choice = tmin[idef];
    if (best != idef && tmin[best] < margin * tmin[idef]) {
      // confirm on a fresh set of the same bucket
      const TuneSet V = tune_set(bk, 0x5eedULL + (uint64_t)bk, grid);
      double vd = 1e300, vc = 1e300;
      rc = tune_time(e, V, dflt, warm);
      for (int rep = 0; rep < reps && !rc; ++rep) {
        double t = 0.0;
        rc = tune_time(e, V, dflt, t);
        vd = std::min(vd, t);
        if (!rc) rc = tune_time(e, V, cands[best], t);
        vc = std::min(vc, t);
      }
      if (rc) break;
      t_def = vd;
      t_choice = vd;
      if (vc < margin * vd) {
        choice = cands[best];
        t_choice = vc;
      }
    }
    table[bk] = choice;
    tot_def += t_def;
    tot_best += t_choice;
  }
  e.timing = timing;
  if (rc) return rc;
  for (auto& eng : ctx->pool)
    for (int bk = 0; bk < Engine::TUNE_BUCKETS; ++bk) eng->tail_table[bk] = table[bk];
  if (speedup) *speedup = tot_best > 0 ? tot_def / tot_best : 1.0;
  if (ms_default) *ms_default = tot_def;
  if (ms_tuned) *ms_tuned = tot_best;
  return 0;
}

int tci_autotune_table(tci_ctx* ctx, int32_t* table, int32_t* nbuckets, int32_t set) {
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  if (nbuckets) *nbuckets = Engine::TUNE_BUCKETS;
  if (!table) return 0;
  if (set) {
    for (int bk = 0; bk < Engine::TUNE_BUCKETS; ++bk)
      if (table[bk] < 0) return fail(TCI_ERR_ARG, "tail sizes must be >= 0 (0: the kernel's default)");
    for (auto& eng : ctx->pool)
      for (int bk = 0; bk < Engine::TUNE_BUCKETS; ++bk) eng->tail_table[bk] = table[bk];
  } else {
    for (int bk = 0; bk < Engine::TUNE_BUCKETS; ++bk) table[bk] = ctx->eng_ref().tail_table[bk];
  }
  return 0;
}

// ---------------------------------------------------------------- tensor-train contraction
}  // extern "C"

struct tci_tt4 {
  tci_ctx* ctx = nullptr;
  TT4 tt;
};

namespace {
int upload_tt4(Engine& e, int32_t L, const int64_t* dims, const double* const* cores, TT4& out) {
  out.cores.clear();
  for (int32_t b = 0; b < L; ++b) {
    Tensor4 c;
    for (int q = 0; q < 4; ++q) c.d[q] = dims[4 * b + q];
    for (int q = 0; q < 4; ++q)
      if (c.d[q] < 1 || c.d[q] > INT32_MAX) {
        out.release(e);
        return fail(TCI_ERR_DIM, "bad core dimensions");
      }
    if (!cores[b]) {
      out.release(e);
      return fail(TCI_ERR_ARG, "missing core");
    }
    c.p = e.alloc_core(c.elems());
    if (!c.p) {
      out.release(e);
      return fail(TCI_ERR_OOM, "device memory for the cores");
    }
    out.cores.push_back(c);
    cudaError_t ce = cudaMemcpyAsync(c.p, cores[b], c.elems() * sizeof(double), cudaMemcpyHostToDevice, e.stream());
    if (ce != cudaSuccess) {
      out.release(e);
      return fail(TCI_ERR_CUDA, cudaGetErrorString(ce));
    }
  }
  cudaError_t ce = cudaStreamSynchronize(e.stream());
  if (ce != cudaSuccess) {
    out.release(e);
    return fail(TCI_ERR_CUDA, cudaGetErrorString(ce));
  }
  return 0;
}
}  // namespace

extern "C" {

int tci_tt4_contract(tci_ctx* ctx, int32_t L, const int64_t* a_dims, const double* const* a_cores,
                     const int64_t* b_dims, const double* const* b_cores, int32_t algorithm, int32_t method,
                     double tolerance, int64_t maxbonddim, tci_tt4** out) {
  *out = nullptr;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  if (algorithm != TCI_CONTRACT_NAIVE && algorithm != TCI_CONTRACT_ZIPUP)
    return fail(TCI_ERR_ARG, "Unknown algorithm.");
  if (method != TCI_FACTORIZE_LU && method != TCI_FACTORIZE_CI) return fail(TCI_ERR_GENERIC, "Not implemented yet.");
  const bool ci = method == TCI_FACTORIZE_CI;
  if (L < 1) return fail(TCI_ERR_ARG, "empty tensor train");
  Engine& e = ctx->eng_ref();
  TT4 a, b;
  int rc = upload_tt4(e, L, a_dims, a_cores, a);
  if (!rc) rc = upload_tt4(e, L, b_dims, b_cores, b);
  if (!rc) rc = tt4_check_pair(a, b, true);
  std::unique_ptr<tci_tt4> res(new tci_tt4());
  res->ctx = ctx;
  if (!rc) {
    if (algorithm == TCI_CONTRACT_NAIVE) {
      rc = tt4_contract_naive(e, a, b, res->tt);
      if (!rc && (tolerance > 0 || maxbonddim > 0))
        rc = tt4_compress(e, res->tt, tolerance, maxbonddim, true, ci);
    } else {
      rc = tt4_contract_zipup(e, a, b, tolerance, maxbonddim, res->tt, ci);
    }
  }
  a.release(e);
  b.release(e);
  if (rc) {
    res->tt.release(e);
    return rc;
  }
  *out = res.release();
  return 0;
}

int tci_tt4_contract_prec(tci_ctx* ctx, int32_t L, const int64_t* a_dims, const double* const* a_cores,
                          const int64_t* b_dims, const double* const* b_cores, int32_t algorithm, int32_t method,
                          double tolerance, int64_t maxbonddim, int32_t precision, double* err_est, tci_tt4** out) {
  if (precision == TCI_PREC_FP64) {
    if (err_est) *err_est = 0.0;
    return tci_tt4_contract(ctx, L, a_dims, a_cores, b_dims, b_cores, algorithm, method, tolerance, maxbonddim, out);
  }
  *out = nullptr;
  if (precision != TCI_PREC_TF32X3) return fail(TCI_ERR_ARG, "unknown precision");
  if (algorithm != TCI_CONTRACT_ZIPUP) return fail(TCI_ERR_ARG, "split precision is implemented for algorithm = :zipup");
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  if (method != TCI_FACTORIZE_LU && method != TCI_FACTORIZE_CI) return fail(TCI_ERR_GENERIC, "Not implemented yet.");
  if (L < 1) return fail(TCI_ERR_ARG, "empty tensor train");
  if (ctx->rq) {  // plain launches: the tensor-core kernels need the SMs
    int rc = ctx->rq->stop();
    if (rc) return rc;
  }
  Engine& e = ctx->eng_ref();
  TT4 a, b;
  int rc = upload_tt4(e, L, a_dims, a_cores, a);
  if (!rc) rc = upload_tt4(e, L, b_dims, b_cores, b);
  if (!rc) rc = tt4_check_pair(a, b, true);
  std::unique_ptr<tci_tt4> res(new tci_tt4());
  res->ctx = ctx;
  SplitRun split;
  if (!rc) rc = tt4_contract_zipup(e, a, b, tolerance, maxbonddim, res->tt, method == TCI_FACTORIZE_CI, &split);
  a.release(e);
  b.release(e);
  if (rc) {
    res->tt.release(e);
    return rc;
  }
  if (err_est) *err_est = split.max_rel_err;
  *out = res.release();
  return 0;
}

int tci_matmul(tci_ctx* ctx, int64_t M, int64_t N, int64_t K, const double* A, const double* B, double* C,
               int32_t precision, double* err_est) {
  if (M < 0 || N < 0 || K < 0) return fail(TCI_ERR_ARG, "negative matrix dimension");
  if (precision != TCI_PREC_FP64 && precision != TCI_PREC_TF32X3) return fail(TCI_ERR_ARG, "unknown precision");
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  if (err_est) *err_est = 0.0;
  if (M == 0 || N == 0) return 0;
  if (ctx->rq) {
    int rc = ctx->rq->stop();
    if (rc) return rc;
  }
  Engine& e = ctx->eng_ref();
  const size_t na = (size_t)(M * K), nb = (size_t)(K * N), nc = (size_t)(M * N);
  double* dA = e.alloc_core(std::max<size_t>(na, 1));
  double* dB = e.alloc_core(std::max<size_t>(nb, 1));
  double* dC = e.alloc_core(nc);
  int rc = 0;
  if (!dA || !dB || !dC) rc = fail(TCI_ERR_OOM, "device memory for the matrix product");
  if (!rc && na && cudaMemcpyAsync(dA, A, na * 8, cudaMemcpyHostToDevice, e.stream()) != cudaSuccess)
    rc = fail(TCI_ERR_CUDA, "copy of A");
  if (!rc && nb && cudaMemcpyAsync(dB, B, nb * 8, cudaMemcpyHostToDevice, e.stream()) != cudaSuccess)
    rc = fail(TCI_ERR_CUDA, "copy of B");
  if (!rc && K == 0 && cudaMemsetAsync(dC, 0, nc * 8, e.stream()) != cudaSuccess) rc = fail(TCI_ERR_CUDA, "memset");
  SplitRun split;
  if (!rc && K > 0) rc = device_matmul(e, dA, dB, dC, M, N, K, precision == TCI_PREC_TF32X3 ? &split : nullptr);
  if (!rc && cudaMemcpyAsync(C, dC, nc * 8, cudaMemcpyDeviceToHost, e.stream()) != cudaSuccess)
    rc = fail(TCI_ERR_CUDA, "copy of C");
  if (!rc && cudaStreamSynchronize(e.stream()) != cudaSuccess) rc = fail(TCI_ERR_CUDA, "synchronize");
  if (!rc && err_est) *err_est = split.max_rel_err;
  e.free_core(dA);
  e.free_core(dB);
  e.free_core(dC);
  return rc;
}

int tci_tt4_compress(tci_ctx* ctx, int32_t L, const int64_t* dims, const double* const* cores, int32_t method,
                     double tolerance, int64_t maxbonddim, int32_t normalizeerror, tci_tt4** out) {
  *out = nullptr;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  if (L < 1) return fail(TCI_ERR_ARG, "empty tensor train");
  if (method != TCI_FACTORIZE_LU && method != TCI_FACTORIZE_CI) return fail(TCI_ERR_GENERIC, "Not implemented yet.");
  Engine& e = ctx->eng_ref();
  std::unique_ptr<tci_tt4> res(new tci_tt4());
  res->ctx = ctx;
  int rc = upload_tt4(e, L, dims, cores, res->tt);
  if (!rc) rc = tt4_check(res->tt);
  if (!rc) rc = tt4_compress(e, res->tt, tolerance, maxbonddim, normalizeerror != 0, method == TCI_FACTORIZE_CI);
  if (rc) {
    res->tt.release(e);
    return rc;
  }
  *out = res.release();
  return 0;
}

int tci_tt4_contract_tci(tci_ctx* ctx, int32_t L, const int64_t* a_dims, const double* const* a_cores,
                         const int64_t* b_dims, const double* const* b_cores, const int64_t* initialpivots,
                         int64_t np, int32_t ninitialpivots, tci_value_fn f, void* user, const tci_opts* opts,
                         tci_tt4** out) {
  *out = nullptr;
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  if (L < 1) return fail(TCI_ERR_ARG, "empty tensor train");
  Engine& e = ctx->eng_ref();
  TT4 a, b;
  int rc = upload_tt4(e, L, a_dims, a_cores, a);
  if (!rc) rc = upload_tt4(e, L, b_dims, b_cores, b);
  if (rc) {
    a.release(e);
    b.release(e);
    return rc;
  }
  std::vector<std::vector<uint8_t>> piv;
  for (int64_t p = 0; p < np; ++p) {
    std::vector<uint8_t> v((size_t)L);
    for (int q = 0; q < L; ++q) {
      const int64_t x = initialpivots[p * L + q];
      const int64_t dq = a.cores[(size_t)q].d[1] * b.cores[(size_t)q].d[2];
      if (x < 1 || x > dq || dq > 256) {
        a.release(e);
        b.release(e);
        return fail(TCI_ERR_ARG, "pivot index out of range");
      }
      v[(size_t)q] = (uint8_t)(x - 1);
    }
    piv.push_back(v);
  }
  tci_opts o;
  if (opts)
    o = *opts;
  else
    tci_opts_default(&o);
  if (ctx->rq) {  // plain launches: the evaluator's kernels run between steps
    rc = ctx->rq->stop();
    if (rc) return rc;
  }
  std::unique_ptr<tci_tt4> res(new tci_tt4());
  res->ctx = ctx;
  rc = tt4_contract_tci(e, std::move(a), std::move(b), piv, ninitialpivots > 0 ? ninitialpivots : 10, f, user, o,
                        res->tt);
  if (rc) {
    res->tt.release(e);
    return rc;
  }
  *out = res.release();
  return 0;
}

int32_t tci_tt4_length(const tci_tt4* t) { return (int32_t)t->tt.cores.size(); }

int tci_tt4_dims(const tci_tt4* t, int64_t* dims) {
  for (size_t b = 0; b < t->tt.cores.size(); ++b)
    for (int q = 0; q < 4; ++q) dims[4 * b + q] = t->tt.cores[b].d[q];
  return 0;
}

int tci_tt4_get_core(const tci_tt4* t, int32_t b, double* out) {
  if (b < 1 || b > (int32_t)t->tt.cores.size()) return fail(TCI_ERR_ARG, "site index out of range");
  std::lock_guard<std::recursive_mutex> lk(t->ctx->mu);
  Engine& e = t->ctx->eng_ref();
  const Tensor4& c = t->tt.cores[b - 1];
  cudaError_t ce = cudaMemcpyAsync(out, c.p, c.elems() * sizeof(double), cudaMemcpyDeviceToHost, e.stream());
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(e.stream());
  if (ce != cudaSuccess) return fail(TCI_ERR_CUDA, cudaGetErrorString(ce));
  return 0;
}

int tci_tt4_destroy(tci_tt4* t) {
  if (!t) return 0;
  {
    std::lock_guard<std::recursive_mutex> lk(t->ctx->mu);
    t->tt.release(t->ctx->eng_ref());
  }
  delete t;
  return 0;
}

}  // extern "C"

// ---------------------------------------------------------------- tensor trains given by the caller
namespace {
// A solve holding only uploaded cores (no f): evaluate/sum run on its tables.
int upload_tt3(Engine& e, int32_t L, const int64_t* dims, const double* const* cores, Solve& s) {
  s.L = L;
  s.d.assign((size_t)L, 1);
  s.cores.assign((size_t)L, Core());
  for (int32_t b = 0; b < L; ++b) {
    Core& c = s.cores[b];
    c.d0 = dims[3 * b];
    c.d1 = dims[3 * b + 1];
    c.d2 = dims[3 * b + 2];
    if (c.d0 < 1 || c.d1 < 1 || c.d2 < 1 || c.d1 > 256 || (b > 0 && s.cores[b - 1].d2 != c.d0) ||
        (b == 0 && c.d0 != 1) || (b == L - 1 && c.d2 != 1)) {
      e.release_cores(s);
      return fail(TCI_ERR_DIM, "inconsistent tensor-train dimensions");
    }
    s.d[b] = (int)c.d1;
    c.p = e.alloc_core(c.elems());
    if (!c.p) {
      e.release_cores(s);
      return fail(TCI_ERR_OOM, "device memory for the cores");
    }
    cudaError_t ce = cudaMemcpyAsync(c.p, cores[b], c.elems() * sizeof(double), cudaMemcpyHostToDevice, e.stream());
    if (ce != cudaSuccess) {
      e.release_cores(s);
      return fail(TCI_ERR_CUDA, cudaGetErrorString(ce));
    }
  }
  cudaError_t ce = cudaStreamSynchronize(e.stream());
  if (ce != cudaSuccess) {
    e.release_cores(s);
    return fail(TCI_ERR_CUDA, cudaGetErrorString(ce));
  }
  s.cores_valid = true;
  return 0;
}
}  // namespace

extern "C" {

int tci_tt_evaluate(tci_ctx* ctx, int32_t L, const int64_t* dims, const double* const* cores, const int64_t* points,
                    int64_t np, double* out) {
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  if (L < 1) return fail(TCI_ERR_ARG, "empty tensor train");
  Engine& e = ctx->eng_ref();
  Solve s;
  int rc = upload_tt3(e, L, dims, cores, s);
  if (rc) return rc;
  std::vector<uint8_t> pts;
  rc = pack_points(points, np, L, s.d, pts);
  if (!rc) {
    const int64_t chunk = 1 << 20;
    for (int64_t b = 0; b < np && !rc; b += chunk) {
      const int64_t n = std::min(chunk, np - b);
      CoTask t = co_evaluate(e, s, pts.data() + b * L, n, nullptr, out + b);
      rc = e.run(t);
    }
  }
  e.release_cores(s);
  return rc;
}

int tci_tt_evaluate_prec(tci_ctx* ctx, int32_t L, const int64_t* dims, const double* const* cores,
                         const int64_t* points, int64_t np, double* out, int32_t precision, double* err_est) {
  if (precision == TCI_PREC_FP64) {
    if (err_est) *err_est = 0.0;
    return tci_tt_evaluate(ctx, L, dims, cores, points, np, out);
  }
  if (precision != TCI_PREC_TF32X3) return fail(TCI_ERR_ARG, "unknown precision");
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  if (L < 1) return fail(TCI_ERR_ARG, "empty tensor train");
  Engine& e = ctx->eng_ref();
  Solve s;
  int rc = upload_tt3(e, L, dims, cores, s);
  if (rc) return rc;
  std::vector<uint8_t> pts;
  rc = pack_points(points, np, L, s.d, pts);
  if (!rc) rc = split_evaluate(ctx, s, pts, np, out, err_est);
  e.release_cores(s);
  return rc;
}

int tci_tt_sum(tci_ctx* ctx, int32_t L, const int64_t* dims, const double* const* cores, double* out) {
  std::lock_guard<std::recursive_mutex> lk(ctx->mu);
  if (L < 1) return fail(TCI_ERR_ARG, "empty tensor train");
  Engine& e = ctx->eng_ref();
  Solve s;
  int rc = upload_tt3(e, L, dims, cores, s);
  if (rc) return rc;
  CoTask t = co_sum(e, s, out);
  rc = e.run(t);
  e.release_cores(s);
  return rc;
}

}  // extern "C"
