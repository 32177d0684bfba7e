// Host engine: index sets, the batched step loop and the TCI2 algorithm written
// as coroutines.  The algorithm follows tensorci2.jl step by step (citations at
// each function); every Pi evaluation, LU and site-tensor computation is a GPU
// task, and the only host work is integer bookkeeping of the pivot index sets,
// the convergence test and the random start points of the global pivot search.
#include "engine.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <numeric>
#include <thread>

cudaError_t tci_gather_launch(const void* table_dev, int n, double* dst_dev, int grid, cudaStream_t stream);
using tci_k256::tci_rrlu_big_fits;
using tci_k256::tci_rrlu_big_launch;
using tci_k256::tci_rrlu_big_scratch_bytes;

namespace tci {

namespace {
thread_local Error g_err;
const double QNAN = std::numeric_limits<double>::quiet_NaN();

double jmax(double a, double b) {
  if (a != a || b != b) return QNAN;
  return a > b ? a : b;
}
inline size_t a16(size_t x) { return (x + 15) & ~(size_t)15; }
inline size_t a8(size_t x) { return (x + 7) & ~(size_t)7; }

uint64_t hash_bytes(const uint8_t* p, int len) {
  uint64_t h = 1469598103934665603ULL;
  for (int i = 0; i < len; ++i) h = (h ^ p[i]) * 1099511628211ULL;
  return h ^ (h >> 29);
}
}  // namespace

void set_error(int code, const std::string& msg) {
  g_err.code = code;
  g_err.msg = msg;
}
int last_code() { return g_err.code; }
const char* last_message() { return g_err.msg.c_str(); }

static int fail(int code, const std::string& msg) {
  set_error(code, msg);
  return code;
}

static int reentry() {
  return fail(TCI_ERR_GENERIC, "the library was called to compute from inside a caller-supplied f");
}

// ---------------------------------------------------------------- index sets
bool IndexSet::contains(const uint8_t* v) const {
  for (size_t i = 0; i < n; ++i)
    if (len == 0 || std::memcmp(at(i), v, (size_t)len) == 0) return true;
  return false;
}

IndexSet kron_right(const IndexSet& I, int d) {
  IndexSet o;
  o.len = I.len + 1;
  o.n = I.n * (size_t)d;
  o.data.resize(o.n * (size_t)o.len);
  uint8_t* dst = o.data.data();
  const size_t il = (size_t)I.len;
  for (int j = 0; j < d; ++j)
    for (size_t i = 0; i < I.n; ++i) {
      if (il) std::memcpy(dst, I.data.data() + i * il, il);
      dst[il] = (uint8_t)j;
      dst += o.len;
    }
  return o;
}

IndexSet kron_left(int d, const IndexSet& J) {
  IndexSet o;
  o.len = J.len + 1;
  o.n = J.n * (size_t)d;
  o.data.resize(o.n * (size_t)o.len);
  uint8_t* dst = o.data.data();
  const size_t jl = (size_t)J.len;
  for (size_t j = 0; j < J.n; ++j)
    for (int i = 0; i < d; ++i) {
      dst[0] = (uint8_t)i;
      if (jl) std::memcpy(dst + 1, J.data.data() + j * jl, jl);
      dst += o.len;
    }
  return o;
}

namespace {
// Multi-indices of up to 16 bytes as two integers (bytes in order, zero padded):
// equal keys <=> equal multi-indices of one length.
struct Key16 {
  uint64_t lo, hi;
  bool operator==(const Key16& o) const { return lo == o.lo && hi == o.hi; }
};
inline uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ULL;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebULL;
  return z ^ (z >> 31);
}
inline Key16 key16(const uint8_t* v, int len) {
  Key16 k{0, 0};
  for (int q = 0; q < len && q < 8; ++q) k.lo |= (uint64_t)v[q] << (8 * q);
  for (int q = 8; q < len; ++q) k.hi |= (uint64_t)v[q] << (8 * (q - 8));
  return k;
}

// Base.union for lengths up to 16: open addressing over packed keys, in a table
// kept per thread (slots hold entry + 1; 0 = empty).
IndexSet union_small(const IndexSet& a, const IndexSet& b) {
  thread_local std::vector<uint32_t> table;
  thread_local std::vector<Key16> keys;
  IndexSet o;
  o.len = a.len;
  const size_t nmax = a.n + b.n;
  size_t cap = 16;
  while (cap < 2 * nmax + 1) cap <<= 1;
  if (table.size() < cap) table.resize(cap);
  if (keys.size() < nmax) keys.resize(nmax);
  uint32_t* const tab = table.data();  // (thread-local lookups hoisted out of the loop)
  Key16* const ks = keys.data();
  std::memset(tab, 0, cap * sizeof(uint32_t));
  o.data.resize(nmax * (size_t)a.len);
  uint8_t* dst = o.data.data();
  size_t cnt = 0;
  const size_t mask = cap - 1;
  for (const IndexSet* src : {&a, &b})
    for (size_t i = 0; i < src->n; ++i) {
      const uint8_t* v = src->data.data() + i * (size_t)a.len;
      const Key16 k = key16(v, a.len);
      size_t h = mix64(k.lo * 0x9e3779b97f4a7c15ULL ^ mix64(k.hi)) & mask;
      bool found = false;
      while (tab[h]) {
        if (ks[tab[h] - 1] == k) {
          found = true;
          break;
        }
        h = (h + 1) & mask;
      }
      if (!found) {
        tab[h] = (uint32_t)(cnt + 1);
        ks[cnt] = k;
        for (int q = 0; q < a.len; ++q) dst[q] = v[q];
        dst += a.len;
        ++cnt;
      }
    }
  o.n = cnt;
  o.data.resize(cnt * (size_t)a.len);
  return o;
}
}  // namespace

IndexSet set_union(const IndexSet& a, const IndexSet& b) {
  IndexSet o;
  o.len = a.len;
  if (a.len == 0) {  // entries are all the empty multi-index
    if (a.n + b.n > 0) o.n = 1;
    return o;
  }
  if (a.len <= 16 && a.n + b.n < ((size_t)1 << 31)) return union_small(a, b);
  size_t cap = 16;
  while (cap < 2 * (a.n + b.n) + 1) cap <<= 1;
  std::vector<int64_t> table(cap, -1);
  o.data.reserve((a.n + b.n) * a.len);
  for (const IndexSet* src : {&a, &b})
    for (size_t i = 0; i < src->n; ++i) {
      const uint8_t* v = src->at(i);
      size_t h = hash_bytes(v, a.len) & (cap - 1);
      bool found = false;
      while (table[h] >= 0) {
        if (std::memcmp(o.at((size_t)table[h]), v, a.len) == 0) {
          found = true;
          break;
        }
        h = (h + 1) & (cap - 1);
      }
      if (!found) {
        table[h] = (int64_t)o.n;
        o.push(v);
      }
    }
  return o;
}

IndexSet select(const IndexSet& s, const int32_t* idx, int k) {
  IndexSet o;
  o.len = s.len;
  if (s.len == 0) {
    o.n = (size_t)k;
    return o;
  }
  o.n = (size_t)k;
  o.data.resize((size_t)k * s.len);
  uint8_t* dst = o.data.data();
  for (int i = 0; i < k; ++i, dst += s.len) std::memcpy(dst, s.at((size_t)idx[i]), (size_t)s.len);
  return o;
}

// ---------------------------------------------------------------- GpuOp
bool GpuOp::await_ready() {
  if (reqs.empty()) return true;
  FCache* last = nullptr;
  for (Req* r : reqs)
    if (r->fcache && r->fcache != last) {
      last = r->fcache;
      status = r->fcache->prefill(*eng, reqs);
      if (status) return true;
    }
  return false;
}
void GpuOp::await_suspend(std::coroutine_handle<> h) { eng->enqueue(reqs, h, this); }
int GpuOp::await_resume() const noexcept { return status; }

// ---------------------------------------------------------------- Engine
Engine::Engine(int device) : device_(device) {}

Engine::~Engine() {
  if (task_log_) std::fflush(task_log_);
  if (stream_) cudaStreamSynchronize(stream_);
  if (hblob_) cudaFreeHost(hblob_);
  if (hres_) cudaFreeHost(hres_);
  if (dblob_) cudaFree(dblob_);
  if (dres_) cudaFree(dres_);
  if (dwork_) cudaFree(dwork_);
  if (dcounter_) cudaFree(dcounter_);
  if (ev0_) cudaEventDestroy(ev0_);
  if (ev1_) cudaEventDestroy(ev1_);
  if (done_) cudaEventDestroy(done_);
  if (hgat_) cudaFreeHost(hgat_);
  if (dgat_) cudaFree(dgat_);
  if (stream_) cudaStreamDestroy(stream_);
}

#define CUDA_TRY(x)                                                             \
  do {                                                                          \
    cudaError_t _e = (x);                                                       \
    if (_e != cudaSuccess) return fail(TCI_ERR_CUDA, cudaGetErrorString(_e));   \
  } while (0)

int Engine::init() {
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return fail(TCI_ERR_CUDA, "no CUDA device available");
  if (device_ < 0 || device_ >= ndev) return fail(TCI_ERR_ARG, "invalid device index");
  CUDA_TRY(cudaSetDevice(device_));
  CUDA_TRY(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
  CUDA_TRY(cudaEventCreate(&ev0_));
  CUDA_TRY(cudaEventCreate(&ev1_));
  CUDA_TRY(cudaEventCreateWithFlags(&done_, cudaEventDisableTiming));
  CUDA_TRY(tci_k256::kernels.configure());
  CUDA_TRY(tci_k512::kernels.configure());
  // TCI_PLAN_SMEM=<bytes> plans RRLU and SITE tasks against a smaller
  // shared-memory budget (the kernel keeps its own), so that tests reach the
  // global-memory layouts with small matrices; results do not depend on the layout.
  if (const char* s = std::getenv("TCI_PLAN_SMEM")) plan_limit_ = (size_t)std::max(1024L, std::atol(s));
  CUDA_TRY(cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, device_));
  CUDA_TRY(cudaMalloc(&dcounter_, 64));
  cudaMemPool_t pool;
  CUDA_TRY(cudaDeviceGetDefaultMemPool(&pool, device_));
  uint64_t thr = UINT64_MAX;
  CUDA_TRY(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr));
  // Optional per-task trace (step kind m n r npivot cycles smem lut), for tuning.
  // One stream shared by every engine of the process (lines stay whole).
  static FILE* shared_log = [] {
    const char* path = std::getenv("TCI_TASK_LOG");
    return path ? std::fopen(path, "a") : (FILE*)nullptr;
  }();
  task_log_ = shared_log;
  return 0;
}

double* Engine::alloc_core(size_t elems) {
  if (elems == 0) elems = 1;
  if (dpool_) return (double*)dpool_->alloc(elems * sizeof(double));
  void* p = nullptr;
  if (cudaMallocAsync(&p, elems * sizeof(double), stream_) != cudaSuccess) return nullptr;
  return (double*)p;
}
void Engine::free_core(double* p) {
  if (!p) return;
  if (dpool_)
    dpool_->free(p);
  else
    cudaFreeAsync(p, stream_);
}
void Engine::release_solve(Solve& s) {
  release_cores(s);
  if (s.lut_dev) free_core(s.lut_dev);
  s.lut_dev = nullptr;
  if (s.fcache) s.fcache->release();
}
void Engine::release_cores(Solve& s) {
  for (auto& c : s.cores) {
    if (c.p) free_core(c.p);
    c = Core();
  }
  s.cores_valid = false;
}

void Engine::enqueue(std::vector<Req*>& reqs, std::coroutine_handle<> h, GpuOp* op) {
  Waiter w{h, op, pending_.size(), reqs.size()};
  for (Req* r : reqs) pending_.push_back(r);
  waiters_.push_back(w);
}

int Engine::ensure(size_t blob, size_t res, size_t work) {
  if (blob > hblob_cap_) {
    size_t cap = std::max(blob, hblob_cap_ * 2);
    if (hblob_) cudaFreeHost(hblob_);
    hblob_ = nullptr;
    CUDA_TRY(cudaHostAlloc(&hblob_, cap, cudaHostAllocDefault));
    hblob_cap_ = cap;
  }
  if (blob > dblob_cap_) {
    size_t cap = std::max(blob, dblob_cap_ * 2);
    if (dblob_) cudaFree(dblob_);
    dblob_ = nullptr;
    CUDA_TRY(cudaMalloc(&dblob_, cap));
    dblob_cap_ = cap;
  }
  if (res > hres_cap_) {
    size_t cap = std::max(res, hres_cap_ * 2);
    if (hres_) cudaFreeHost(hres_);
    hres_ = nullptr;
    CUDA_TRY(cudaHostAlloc(&hres_, cap, cudaHostAllocDefault));
    hres_cap_ = cap;
  }
  if (res > dres_cap_) {
    size_t cap = std::max(res, dres_cap_ * 2);
    if (dres_) cudaFree(dres_);
    dres_ = nullptr;
    CUDA_TRY(cudaMalloc(&dres_, cap));
    dres_cap_ = cap;
  }
  if (work > dwork_cap_) {
    size_t cap = std::max(work, dwork_cap_ * 2);
    if (dwork_) cudaFree(dwork_);
    dwork_ = nullptr;
    CUDA_TRY(cudaMalloc(&dwork_, cap * sizeof(double)));
    dwork_cap_ = cap;
  }
  return 0;
}

// Shared-memory plan of a task; mirrors the SmemCursor use in step_kernel.cu.
// has_input: the RRLU matrix is given (t.ain, or a host matrix packed later), so
// no f states are needed.  mat_limit caps the shared memory that RRLU and SITE
// plans may use (TCI_PLAN_SMEM).  Returns false if the task cannot run.
static bool plan_task(tci_task& t, size_t smem, size_t& work_elems, bool has_input, int threads,
                      size_t mat_limit = SIZE_MAX) {
  const size_t m = (size_t)t.m, n = (size_t)t.n;
  work_elems = 0;
  if (t.kind == TCI_TASK_RRLU || t.kind == TCI_TASK_SITE) smem = std::min(smem, mat_limit);
  // argmax keys pack (column << 16) | row
  if ((t.kind == TCI_TASK_RRLU && (m > 65535 || n > 65535)) || (t.kind == TCI_TASK_SITE && t.r > 65535))
    return false;
  switch (t.kind) {
    case TCI_TASK_RRLU: {
      const size_t perms = a16(m * 4) + a16(n * 4);
      const size_t states = has_input ? 0 : 2 * a16(m * 8) + 2 * a16(n * 8);
      if (a16(m * n * 8) + perms + states <= smem) {
        t.smem_mode = 1;
      } else if (perms + states <= smem) {
        t.smem_mode = 0;
      } else if (perms <= smem && !has_input) {
        t.smem_mode = 2;  // the f states beside the matrix in global scratch
      } else {
        return false;
      }
      work_elems = tci_work_elems(&t);
      return true;
    }
    case TCI_TASK_SITE: {
      const size_t r = (size_t)t.r;
      const size_t small = 2 * a16(r * 4) + 5 * a16(r * 8), rowstates = 2 * a16(m * 8);
      size_t want_rows = std::min<size_t>(std::max<size_t>(m, 1), 64);
      if (a16(r * r * 8) + small + rowstates + want_rows * (r * 8 + 8) <= smem) {
        t.smem_mode = 1;
      } else if (small + rowstates + (r * 8 + 8) <= smem) {
        t.smem_mode = 0;
      } else if (small + (r * 8 + 8) <= smem) {
        t.smem_mode = 2;  // the row f states beside P in global scratch
      } else {
        return false;
      }
      work_elems = tci_work_elems(&t);
      return true;
    }
    case TCI_TASK_CORE:
      t.smem_mode = 1;
      return 2 * a16(m * 8) + 2 * a16(n * 8) <= smem;
    case TCI_TASK_EVAL:
      t.smem_mode = 1;
      if (t.r <= TCI_EVAL_THREAD_RMAX) return (size_t)2 * TCI_EVAL_THREAD_RMAX * threads * 8 <= smem;
      return (size_t)(threads / 32) * 2 * (size_t)std::max(t.r, 1) * 8 <= smem;
    case TCI_TASK_SUM:
      t.smem_mode = 1;
      return 2 * (size_t)std::max(t.r, 1) * 8 <= smem;
    case TCI_TASK_TABLE:
      t.smem_mode = 1;
      return t.lut != nullptr;
    case TCI_TASK_SEARCH:  // t.n = sum of the left and right bond sizes; then the core table
      t.smem_mode = 1;
      return a16((size_t)3 * (t.L + 1) * 4) + a16((size_t)t.n * 8) + (size_t)t.L * sizeof(tci_core_ref) <= smem;
    default:
      return false;
  }
}

// Shared memory a planned task takes (plan_task's figure for the chosen mode), for
// the kinds whose inputs the resident kernel may stage into the free top of
// shared memory; 0 for the others (never staged).  A SITE task takes as many
// row blocks as fit, so it keeps room for its planned count.
static size_t staged_plan_bytes(const tci_task& t) {
  const size_t m = (size_t)t.m, n = (size_t)t.n;
  switch (t.kind) {
    case TCI_TASK_RRLU: {
      const size_t perms = a16(m * 4) + a16(n * 4);
      const size_t states = (t.ain || t.smem_mode == 2) ? 0 : 2 * a16(m * 8) + 2 * a16(n * 8);
      return t.smem_mode == 1 ? a16(m * n * 8) + perms + states : perms + states + a16((m + n) * 8);
    }
    case TCI_TASK_SITE: {
      const size_t r = (size_t)t.r;
      const size_t rest = 2 * a16(r * 4) + 5 * a16(r * 8) + (t.smem_mode == 2 ? 0 : 2 * a16(m * 8));
      const size_t want_rows = std::min<size_t>(std::max<size_t>(m, 1), 64);
      return t.smem_mode == 1 ? a16(r * r * 8) + rest + want_rows * (r * 8 + 8) : rest + 8 * (r * 8 + 8);
    }
    case TCI_TASK_CORE:
      return 2 * a16(m * 8) + 2 * a16(n * 8);
    case TCI_TASK_SEARCH:
      return a16((size_t)3 * (t.L + 1) * 4) + a16((size_t)t.n * 8) + a16((size_t)t.L * sizeof(tci_core_ref));
    default:
      return 0;
  }
}

// Inputs larger than this are read from the host record in place.
static constexpr size_t STAGE_MAX_BYTES = 64 * 1024;

static size_t result_bytes(const tci_task& t) {
  size_t h = sizeof(tci_result_head);
  switch (t.kind) {
    case TCI_TASK_RRLU:
    case TCI_TASK_SITE:
      return a16(h + 2 * a8((size_t)t.kcap * 4) + (size_t)t.kcap * 8);
    case TCI_TASK_EVAL:
    case TCI_TASK_SEARCH:
      return a16(h + 2 * (size_t)t.m * 8);
    default:
      return a16(h);
  }
}

static int64_t task_cost(const tci_task& t) {
  const int64_t m = t.m, n = t.n;
  switch (t.kind) {
    case TCI_TASK_RRLU:
      return m * n * (40 + 2 * std::min<int64_t>(t.kcap, 64));
    case TCI_TASK_SITE:
      return (int64_t)t.r * t.r * (40 + 2 * t.r) + m * t.r * (40 + 2 * t.r);
    case TCI_TASK_CORE:
      return m * n * 40;
    case TCI_TASK_EVAL:
      return m * (40 + (int64_t)t.L * t.r * t.r);
    case TCI_TASK_SEARCH:
      return (m + 2 * (int64_t)t.L) * (int64_t)t.r * t.r * 2 + m * 40;
    case TCI_TASK_TABLE:
      return ((int64_t)t.lutcap0 + t.lutcap1) * 40;
    default:
      return 1;
  }
}

int Engine::step() {
  int rc = launch();
  if (rc) return rc;
  return complete();
}

bool Engine::ready() const { return !inflight_ || cudaEventQuery(done_) != cudaErrorNotReady; }

namespace {
// Adds the lifetime of the object, in milliseconds, to a counter.
struct MsTimer {
  double& acc;
  std::chrono::steady_clock::time_point t0;
  explicit MsTimer(double& a) : acc(a), t0(std::chrono::steady_clock::now()) {}
  ~MsTimer() { acc += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count(); }
};
}  // namespace

int Engine::launch() {
  if (pending_.empty() || inflight_) return 0;
  MsTimer timer(stats.host_launch_ms);
  std::vector<Req*>& batch = fl_batch_;
  batch.clear();
  batch.swap(pending_);
  std::vector<Waiter>& waiters = fl_waiters_;
  waiters.clear();
  waiters.swap(waiters_);
  const size_t nt = batch.size();
  // fewer tasks than SMs: each gets a whole SM (latency variant); else two
  // task CTAs share an SM (throughput variant)
  ks_ = nt < (size_t)num_sms ? &tci_k512::kernels : &tci_k256::kernels;

  // ---- layout
  size_t off = a16(nt * sizeof(tci_task));
  const size_t off_order = off;
  off = a16(off + nt * sizeof(int));
  std::vector<size_t> o_params(nt), o_rows(nt), o_cols(nt), o_prows(nt), o_cores(nt), o_ain(nt);
  std::vector<size_t> o_res(nt);
  size_t res_total = 0, work_total = 0, cta_stride = 0;
  // Plan every task; a task that cannot run fails its own waiter only.
  std::vector<char> bad(nt, 0);
  std::vector<size_t> wel(nt, 0);
  bool anybad = false;
  for (size_t i = 0; i < nt; ++i) {
    apply_tuning(batch[i]->t);
    if (!plan_task(batch[i]->t, ks_->step_smem_bytes(), wel[i], batch[i]->t.ain || batch[i]->ain_host,
                   ks_->threads, plan_limit_)) {
      bad[i] = 1;
      anybad = true;
    }
  }
  if (anybad) {
    std::vector<Req*> good;
    std::vector<Waiter> goodw, badw;
    for (auto& w : waiters) {
      bool wb = false;
      for (size_t k = w.first; k < w.first + w.count; ++k) wb |= bad[k] != 0;
      if (wb) {
        badw.push_back(w);
      } else {
        Waiter g = w;
        g.first = good.size();
        for (size_t k = w.first; k < w.first + w.count; ++k) good.push_back(batch[k]);
        goodw.push_back(g);
      }
    }
    set_error(TCI_ERR_TOO_LARGE, "a matrix exceeds the step kernel's on-chip plan");
    batch.clear();
    waiters.clear();
    // pending_/waiters_ were emptied above: requeue the runnable tasks, then let
    // the failed solves continue (whatever they enqueue lands behind them)
    for (Req* r : good) pending_.push_back(r);
    for (auto& w : goodw) waiters_.push_back(w);
    for (auto& w : badw) {
      w.op->status = TCI_ERR_TOO_LARGE;
      w.h.resume();
    }
    return launch();
  }
  for (size_t i = 0; i < nt; ++i) {
    Req& r = *batch[i];
    const size_t we = wel[i];
    o_params[i] = off;
    off = a16(off + (size_t)r.t.nparams * 8);
    o_rows[i] = off;
    off = a16(off + r.rows_bytes);
    o_cols[i] = off;
    off = a16(off + r.cols_bytes);
    o_prows[i] = off;
    off = a16(off + r.prows_bytes);
    o_cores[i] = off;
    off = a16(off + (size_t)r.ncores * sizeof(tci_core_ref));
    o_ain[i] = off;
    if (r.ain_host) off = a16(off + (size_t)r.t.m * r.t.n * 8);
    o_res[i] = res_total;
    r.res_bytes = result_bytes(r.t);
    res_total += r.res_bytes;
    // global-memory scratch (a matrix too large for shared memory, per-task f
    // tables): one area per CTA, reused by the CTA's successive tasks, so the
    // scratch stays hot in L2 instead of a fresh region per task
    size_t need = we;
    if (r.t.lutcap0 > 0 && !r.t.lut_full) need += (size_t)r.t.lutcap0 + (size_t)std::max(r.t.lutcap1, 0);
    cta_stride = std::max(cta_stride, need);
  }
  const size_t blob_total = off;
  const int grid = std::max(1, std::min<int>((int)nt, num_sms * ks_->ctas_per_sm));
  cta_stride = (cta_stride + 31) / 32 * 32;  // 256-byte aligned areas
  work_total = cta_stride * (size_t)grid;
  int rc = ensure(blob_total, res_total, work_total);
  if (rc) {
    std::vector<Waiter> ws;
    ws.swap(waiters);
    batch.clear();
    for (auto& w : ws) w.op->status = rc;
    for (auto& w : ws) w.h.resume();
    return rc;
  }

  // ---- pack
  tci_task* tasks = (tci_task*)hblob_;
  for (size_t i = 0; i < nt; ++i) {
    Req& r = *batch[i];
    tci_task t = r.t;
    t.params = (int64_t)o_params[i];
    t.rows = (int64_t)o_rows[i];
    t.cols = (int64_t)o_cols[i];
    t.prows = (int64_t)o_prows[i];
    t.cores = r.ncores ? (int64_t)o_cores[i] : 0;
    t.res = (int64_t)o_res[i];
    t.work = nullptr;  // the kernel points it (and a per-task table) into its CTA's area
    if (!t.lut_full) t.lut = nullptr;
    if (r.ain_host) t.ain = (const double*)(dblob_ + o_ain[i]);
    t.cost = task_cost(t);
    tasks[i] = t;
    if (t.nparams) std::memcpy(hblob_ + o_params[i], r.params, (size_t)t.nparams * 8);
    if (r.rows_bytes) std::memcpy(hblob_ + o_rows[i], r.rows, r.rows_bytes);
    if (r.cols_bytes) std::memcpy(hblob_ + o_cols[i], r.cols, r.cols_bytes);
    if (r.prows_bytes) std::memcpy(hblob_ + o_prows[i], r.prows, r.prows_bytes);
    if (r.ncores) std::memcpy(hblob_ + o_cores[i], r.cores, (size_t)r.ncores * sizeof(tci_core_ref));
    if (r.ain_host) std::memcpy(hblob_ + o_ain[i], r.ain_host, (size_t)r.t.m * r.t.n * 8);
  }
  int* order = (int*)(hblob_ + off_order);
  std::iota(order, order + nt, 0);
  std::stable_sort(order, order + nt, [&](int a, int b) { return tasks[a].cost > tasks[b].cost; });

  // ---- upload, launch, download
  CUDA_TRY(cudaMemcpyAsync(dblob_, hblob_, blob_total, cudaMemcpyHostToDevice, stream_));
  if (timing) CUDA_TRY(cudaEventRecord(ev0_, stream_));
  CUDA_TRY(ks_->step_launch(dblob_, dres_, (const int*)(dblob_ + off_order), (int)nt, dcounter_, grid, dwork_,
                           cta_stride, stream_));
  if (timing) CUDA_TRY(cudaEventRecord(ev1_, stream_));
  CUDA_TRY(cudaMemcpyAsync(hres_, dres_, res_total, cudaMemcpyDeviceToHost, stream_));
  CUDA_TRY(cudaEventRecord(done_, stream_));
  inflight_ = true;
  fl_blob_ = blob_total;
  fl_res_ = res_total;
  fl_o_res_.swap(o_res);
  fl_smem_.resize(nt);
  for (size_t i = 0; i < nt; ++i) fl_smem_[i] = (char)tasks[i].smem_mode;
  return 0;
}

// Per-task statistics and the optional task trace.
void Engine::account(const Req& r, int smem_mode) {
  const tci_result_head* h = r.head();
  stats.task_cycles += h->cycles;
  if (task_log_) {
    std::fprintf(task_log_, "%lld %d %d %d %d %d %lld %d %d %d %d %d %d\n", (long long)stats.steps, r.t.kind,
                 r.t.m, r.t.n, r.t.r, h->npivot, (long long)h->cycles, smem_mode, h->lut_used, h->status,
                 r.t.nl, r.t.nr, r.t.lutcap0);
  }
  const tci_task& t = r.t;
  if (h->lut_used) {
    if (t.kind == TCI_TASK_RRLU || t.kind == TCI_TASK_CORE) stats.feval_tabulated += (int64_t)t.m * t.n;
    if (t.kind == TCI_TASK_SITE) stats.feval_tabulated += (int64_t)t.r * t.r + (int64_t)t.m * t.r;
  }
  switch (t.kind) {
    case TCI_TASK_RRLU: {
      if (!t.ain) stats.feval += (int64_t)t.m * t.n;
      int64_t K = h->npivot;
      for (int64_t k = 1; k < K; ++k) stats.lu_updates += (int64_t)(t.m - k) * (t.n - k);
    } break;
    case TCI_TASK_SITE:
      stats.feval += (int64_t)t.r * t.r + (int64_t)t.m * t.r;
      for (int64_t k = 1; k < t.r; ++k) stats.lu_updates += (int64_t)(t.r - k) * (t.r - k);
      // forward (unit lower) and backward substitution of every row
      if (!(h->status & TCI_ST_SINGULAR)) stats.dense_macs += (int64_t)t.m * t.r * (t.r - 1);
      break;
    case TCI_TASK_CORE:
      stats.feval += (int64_t)t.m * t.n;
      break;
    case TCI_TASK_EVAL:
    case TCI_TASK_SEARCH:
      stats.feval += t.m;
      if (r.cores) {
        int64_t chain = 0, items = 0;  // sum of r0 r1 over the sites; sum of d (r0 r1 + r1)
        for (int p = 0; p < r.ncores; ++p) {
          const int64_t r0 = r.cores[p].r0, d = r.cores[p].d, r1 = r.cores[p].r1;
          chain += r0 * r1;
          items += d * (r0 * r1 + r1);
        }
        // EVAL: one left-to-right product per point; SEARCH: the left and right
        // environments of the start point and the value at every one-site change
        stats.dense_macs += t.kind == TCI_TASK_EVAL ? (int64_t)t.m * chain : 2 * chain + items;
      }
      break;
    default:
      break;
  }
}

int Engine::complete() {
  if (!inflight_) return 0;
  {
    MsTimer timer(stats.host_wait_ms);
    CUDA_TRY(cudaEventSynchronize(done_));
  }
  MsTimer timer(stats.host_resume_ms);
  inflight_ = false;
  std::vector<Req*>& batch = fl_batch_;
  const size_t nt = batch.size();
  const size_t blob_total = fl_blob_, res_total = fl_res_;
  const std::vector<size_t>& o_res = fl_o_res_;
  if (timing) {
    float ms = 0;
    cudaEventElapsedTime(&ms, ev0_, ev1_);
    stats.kernel_ms += ms;
  }
  stats.steps += 1;
  stats.launches += 1;
  stats.tasks += (int64_t)nt;
  stats.h2d_bytes += (int64_t)blob_total;
  stats.d2h_bytes += (int64_t)res_total;

  for (size_t i = 0; i < nt; ++i) {
    Req& r = *batch[i];
    r.res = hres_ + o_res[i];
    account(r, fl_smem_[i]);
  }
  // Resuming lets each solve continue to its next task (enqueued for the next
  // launch); the Req records of this batch may be gone afterwards.
  std::vector<Waiter> ws;
  ws.swap(fl_waiters_);
  batch.clear();
  for (auto& w : ws) {
    w.op->status = 0;
    w.h.resume();
  }
  return 0;
}

// ---------------------------------------------------------------- pools
BlockPool::BlockPool(Kind kind, int device, bool locked) : kind_(kind), device_(device), locked_(locked) {
  free_.resize(64);
}

BlockPool::~BlockPool() {
  if (side_) cudaStreamSynchronize(side_);
  for (void* p : owned_) {
    if (kind_ == HOST)
      cudaFreeHost(p);
    else
      cudaFree(p);
  }
  if (side_) cudaStreamDestroy(side_);
}

void* BlockPool::backing(size_t bytes) {
  void* p = nullptr;
  if (kind_ == HOST) {
    if (cudaHostAlloc(&p, bytes, cudaHostAllocMapped | cudaHostAllocPortable) != cudaSuccess) return nullptr;
  } else {
    if (!side_ && cudaStreamCreateWithFlags(&side_, cudaStreamNonBlocking) != cudaSuccess) return nullptr;
    if (cudaMallocAsync(&p, bytes, side_) != cudaSuccess) return nullptr;
    if (cudaStreamSynchronize(side_) != cudaSuccess) return nullptr;
  }
  owned_.push_back(p);
  reserved_ += bytes;
  return p;
}

bool BlockPool::reserve_slab() {
  std::unique_lock<std::mutex> lk(mu_, std::defer_lock);
  if (locked_) lk.lock();
  char* p = (char*)backing((size_t)1 << SLAB_SHIFT);
  if (!p) return false;
  slab_ = p;
  slab_left_ = (size_t)1 << SLAB_SHIFT;
  return true;
}

void* BlockPool::alloc(size_t bytes) {
  int k = MIN_SHIFT;
  while (((size_t)1 << k) < bytes) ++k;
  std::unique_lock<std::mutex> lk(mu_, std::defer_lock);
  if (locked_) lk.lock();
  auto& fl = free_[k];
  if (!fl.empty()) {
    void* p = fl.back();
    fl.pop_back();
    return p;
  }
  const size_t sz = (size_t)1 << k;
  void* p = nullptr;
  if (k <= CARVE_MAX) {
    if (slab_left_ < sz) {
      slab_ = (char*)backing((size_t)1 << SLAB_SHIFT);
      slab_left_ = slab_ ? ((size_t)1 << SLAB_SHIFT) : 0;
      if (!slab_) return nullptr;
    }
    p = slab_;
    slab_ += sz;
    slab_left_ -= sz;
  } else {
    p = backing(sz);
    if (!p) return nullptr;
  }
  cls_[p] = k;
  return p;
}

void BlockPool::free(void* p) {
  if (!p) return;
  std::unique_lock<std::mutex> lk(mu_, std::defer_lock);
  if (locked_) lk.lock();
  auto it = cls_.find(p);
  if (it != cls_.end()) free_[it->second].push_back(p);
}

// ---------------------------------------------------------------- resident ring
int ResidentQueue::init(int dev, int num_sms, int idle_us) {
  device = dev;
  this->num_sms = num_sms;
  grid = num_sms * ks->ctas_per_sm;
  nslots = 1u << 15;
  mask = nslots - 1;
  CUDA_TRY(cudaSetDevice(dev));
  CUDA_TRY(cudaHostAlloc((void**)&slots, sizeof(tci_queue_slot) * nslots,
                         cudaHostAllocMapped | cudaHostAllocPortable));
  std::memset((void*)slots, 0, sizeof(tci_queue_slot) * nslots);
  CUDA_TRY(cudaHostAlloc((void**)&qc, sizeof(tci_queue_ctl), cudaHostAllocMapped | cudaHostAllocPortable));
  std::memset((void*)qc, 0, sizeof(tci_queue_ctl));
  qc->idle_us = idle_us;
  CUDA_TRY(cudaMalloc((void**)&st_dev, sizeof(tci_resident_state)));
  CUDA_TRY(cudaMemset(st_dev, 0, sizeof(tci_resident_state)));
  CUDA_TRY(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  CUDA_TRY(cudaEventCreate(&ev0));
  CUDA_TRY(cudaEventCreate(&ev1));
  CUDA_TRY(cudaDeviceSynchronize());
  return 0;
}

ResidentQueue::~ResidentQueue() {
  if (running) stop();
  if (stream) cudaStreamSynchronize(stream);
  if (ev0) cudaEventDestroy(ev0);
  if (ev1) cudaEventDestroy(ev1);
  if (stream) cudaStreamDestroy(stream);
  if (st_dev) cudaFree(st_dev);
  if (qc) cudaFreeHost(qc);
  if (slots) cudaFreeHost(slots);
}

int ResidentQueue::start(const tci_kernel_set* k) {
  std::lock_guard<std::mutex> lk(mu);
  if (running) return k == ks ? 0 : fail(TCI_ERR_GENERIC, "resident kernel already running in another variant");
  ks = k;
  grid = num_sms * ks->ctas_per_sm;
  std::atomic_ref<int32_t>(qc->stop).store(0, std::memory_order_release);
  CUDA_TRY(cudaEventRecord(ev0, stream));
  CUDA_TRY(ks->resident_launch(slots, mask, st_dev, qc, grid, wait_ns, stream));
  CUDA_TRY(cudaEventRecord(ev1, stream));
  running = true;
  ++launches;
  return 0;
}

int ResidentQueue::ensure_alive() {
  std::lock_guard<std::mutex> lk(mu);
  if (!running) return 0;
  cudaError_t q = cudaEventQuery(ev1);
  if (q == cudaErrorNotReady) return 0;
  if (q != cudaSuccess) return fail(TCI_ERR_CUDA, cudaGetErrorString(q));
  // every CTA has left: account the launch; if a wait ran out, report it
  // instead of starting again, else (the idle limit) start again
  float ms = 0;
  cudaEventElapsedTime(&ms, ev0, ev1);
  kernel_ms += ms;
  int32_t err = 0;
  CUDA_TRY(cudaMemcpy(&err, &st_dev->error, sizeof(err), cudaMemcpyDeviceToHost));
  if (err) {
    running = false;
    return fail(TCI_ERR_TIMEOUT, "resident kernel: a wait for a task hit its limit");
  }
  CUDA_TRY(cudaEventRecord(ev0, stream));
  CUDA_TRY(ks->resident_launch(slots, mask, st_dev, qc, grid, wait_ns, stream));
  CUDA_TRY(cudaEventRecord(ev1, stream));
  ++launches;
  return 0;
}

int ResidentQueue::stop() {
  std::lock_guard<std::mutex> lk(mu);
  if (!running) return 0;
  std::atomic_ref<int32_t>(qc->stop).store(1, std::memory_order_release);
  cudaError_t e = cudaEventSynchronize(ev1);
  running = false;
  std::atomic_ref<int32_t>(qc->stop).store(0, std::memory_order_release);
  if (e != cudaSuccess) return fail(TCI_ERR_CUDA, cudaGetErrorString(e));
  float ms = 0;
  cudaEventElapsedTime(&ms, ev0, ev1);
  kernel_ms += ms;
  int32_t err = 0;
  CUDA_TRY(cudaMemcpy(&err, &st_dev->error, sizeof(err), cudaMemcpyDeviceToHost));
  if (err) return fail(TCI_ERR_TIMEOUT, "resident kernel: a wait for a task hit its limit");
  return 0;
}

int ResidentQueue::publish(const tci_task& t, uint64_t& ticket) {
  ticket = tail.fetch_add(1, std::memory_order_relaxed);
  tci_queue_slot& sl = slots[ticket & mask];
  if (ticket >= nslots) {  // wait for the CTA that took this slot's previous ticket
    const uint64_t want = ticket - nslots + 1;
    auto t0 = std::chrono::steady_clock::now();
    for (long it = 0; std::atomic_ref<uint64_t>(sl.taken).load(std::memory_order_acquire) != want; ++it) {
      if ((it & 1023) == 1023) {
        int rc = ensure_alive();
        if (rc) return rc;
        if (std::chrono::steady_clock::now() - t0 > std::chrono::seconds(30))
          return fail(TCI_ERR_TIMEOUT, "resident queue: ring slot not released");
      }
      std::this_thread::yield();
    }
  }
  sl.t = t;
  sl.t.ticket = ticket;
  std::atomic_ref<uint64_t>(sl.seq).store(ticket + 1, std::memory_order_release);
  return 0;
}

// ---------------------------------------------------------------- resident engine
void Engine::set_resident(ResidentQueue* q, BlockPool* host_pool, BlockPool* scratch_pool) {
  rq_ = q;
  hpool_ = host_pool;
  spool_ = scratch_pool;
  res_smem_ = q ? q->ks->resident_smem_bytes() : 0;
  res_threads_ = q ? q->ks->threads : 0;
}

int Engine::submit() {
  if (pending_.empty()) return 0;
  MsTimer timer(stats.host_launch_ms);
  std::vector<Req*> batch;
  batch.swap(pending_);
  std::vector<Waiter> ws;
  ws.swap(waiters_);
  // Staging shortens one task's critical path by a host round trip per dependent
  // read; with many tasks in flight those reads already overlap other tasks'
  // work and the copy would only add to each task, so stage in latency mode only.
  const bool latency_mode = inflight_tasks_ + batch.size() < (size_t)num_sms;
  for (auto& w : ws) {
    Flight f;
    f.w = w;
    int rc = 0;
    for (size_t k = w.first; k < w.first + w.count && !rc; ++k) {
      Req& r = *batch[k];
      tci_task& t = r.t;
      size_t we = 0;
      apply_tuning(t);
      if (!plan_task(t, res_smem_, we, t.ain || r.ain_host, res_threads_, plan_limit_)) {
        rc = fail(TCI_ERR_TOO_LARGE, "a matrix exceeds the step kernel's on-chip plan");
        break;
      }
      // one host record: inputs, then the result record
      size_t off = 0;
      const size_t o_params = off;
      off = a16(off + (size_t)t.nparams * 8);
      const size_t o_rows = off;
      off = a16(off + r.rows_bytes);
      const size_t o_cols = off;
      off = a16(off + r.cols_bytes);
      const size_t o_prows = off;
      off = a16(off + r.prows_bytes);
      const size_t o_cores = off;
      off = a16(off + (size_t)r.ncores * sizeof(tci_core_ref));
      const size_t o_ain = off;
      if (r.ain_host) off = a16(off + (size_t)t.m * t.n * 8);
      const size_t o_res = off;
      r.res_bytes = result_bytes(t);
      off += r.res_bytes;
      char* rec = (char*)hpool_->alloc(off);
      if (!rec) {
        rc = fail(TCI_ERR_OOM, "pinned host memory for task records");
        break;
      }
      f.hblocks.push_back(rec);
      if (t.nparams) std::memcpy(rec + o_params, r.params, (size_t)t.nparams * 8);
      if (r.rows_bytes) std::memcpy(rec + o_rows, r.rows, r.rows_bytes);
      if (r.cols_bytes) std::memcpy(rec + o_cols, r.cols, r.cols_bytes);
      if (r.prows_bytes) std::memcpy(rec + o_prows, r.prows, r.prows_bytes);
      if (r.ncores) std::memcpy(rec + o_cores, r.cores, (size_t)r.ncores * sizeof(tci_core_ref));
      if (r.ain_host) std::memcpy(rec + o_ain, r.ain_host, (size_t)t.m * t.n * 8);
      t.params = (int64_t)(uintptr_t)(rec + o_params);
      t.rows = (int64_t)(uintptr_t)(rec + o_rows);
      t.cols = (int64_t)(uintptr_t)(rec + o_cols);
      t.prows = (int64_t)(uintptr_t)(rec + o_prows);
      t.cores = r.ncores ? (int64_t)(uintptr_t)(rec + o_cores) : 0;
      t.res = (int64_t)(uintptr_t)(rec + o_res);
      if (r.ain_host) t.ain = (const double*)(rec + o_ain);
      r.res = rec + o_res;
      // the block may hold anything from an earlier use: clear the done word so
      // that a stale value can never read as this task's completion
      ((tci_result_head*)r.res)->done = 0;
      const size_t lut = (t.lutcap0 > 0 && !t.lut_full) ? (size_t)t.lutcap0 + (size_t)std::max(t.lutcap1, 0) : 0;
      t.work = nullptr;
      if (!t.lut_full) t.lut = nullptr;
      if (we + lut > 0) {
        double* d = (double*)spool_->alloc((we + lut) * sizeof(double));
        if (!d) {
          rc = fail(TCI_ERR_OOM, "device scratch for a task");
          break;
        }
        f.dblocks.push_back(d);
        if (t.smem_mode != 1) t.work = d;
        if (lut) t.lut = d + we;
      }
      t.cost = task_cost(t);
      // small inputs are copied to shared memory in one parallel pass when the
      // task starts: the task code then reads them on chip instead of making
      // dependent round trips to host memory
      t.stage_bytes = 0;
      if (latency_mode && o_params == 0 && o_res > 0 && o_res <= STAGE_MAX_BYTES) {
        const size_t plan = staged_plan_bytes(t);
        if (plan > 0 && plan + o_res <= res_smem_) t.stage_bytes = (int32_t)o_res;
      }
      stats.h2d_bytes += (int64_t)o_res;
      stats.d2h_bytes += (int64_t)r.res_bytes;
      rc = rq_->publish(t, r.ticket);
      if (!rc) f.reqs.push_back(&r);
    }
    if (rc) {
      if (!f.reqs.empty()) {  // some tasks are out: keep the blocks until they finish, then fail
        f.w.op->status = rc;
        inflight_tasks_ += f.reqs.size();
        flights_.push_back(std::move(f));
        continue;
      }
      for (void* p : f.hblocks) hpool_->free(p);
      for (void* p : f.dblocks) spool_->free(p);
      w.op->status = rc;
      w.h.resume();  // whatever it enqueues is submitted on the next call
      continue;
    }
    inflight_tasks_ += f.reqs.size();
    flights_.push_back(std::move(f));
  }
  return 0;
}

void Engine::abandon() {
  for (auto& f : flights_) {
    for (void* p : f.hblocks) hpool_->free(p);
    for (void* p : f.dblocks) spool_->free(p);
  }
  flights_.clear();
  inflight_tasks_ = 0;
  pending_.clear();
  waiters_.clear();
}

int Engine::poll(bool& progressed) {
  MsTimer timer(stats.host_resume_ms);
  for (size_t i = 0; i < flights_.size();) {
    Flight& f = flights_[i];
    bool done = true;
    for (Req* r : f.reqs) {
      uint64_t* d = const_cast<uint64_t*>(&r->head()->done);
      if (std::atomic_ref<uint64_t>(*d).load(std::memory_order_acquire) != r->ticket + 1) {
        done = false;
        break;
      }
    }
    if (!done) {
      ++i;
      continue;
    }
    Flight g = std::move(f);
    if (i + 1 != flights_.size()) flights_[i] = std::move(flights_.back());
    flights_.pop_back();
    inflight_tasks_ -= g.reqs.size();
    stats.tasks += (int64_t)g.reqs.size();
    for (Req* r : g.reqs) account(*r, r->t.smem_mode);
    const int status = g.w.op->status;  // nonzero: a task of this op could not be submitted
    g.w.op->status = status;
    g.w.h.resume();  // the Req records of this op may be gone afterwards
    for (void* p : g.hblocks) hpool_->free(p);
    for (void* p : g.dblocks) spool_->free(p);
    progressed = true;
  }
  return 0;
}

// Gather straight into mapped pinned host memory (the kernel writes across the
// host link; no staging copy and no host memcpy).
int Engine::gather_to_pinned(const std::vector<const double*>& src, const std::vector<int64_t>& len,
                             double* pinned_out) {
  const size_t n = src.size();
  if (n == 0) return 0;
  size_t total = 0;
  std::vector<int64_t> off(n);
  for (size_t i = 0; i < n; ++i) {
    off[i] = (int64_t)total;
    total += (size_t)len[i];
  }
  const size_t table = a16(n * (sizeof(void*) + 2 * sizeof(int64_t)));
  if (table > hgat_cap_) {
    if (hgat_) cudaFreeHost(hgat_);
    hgat_ = nullptr;
    CUDA_TRY(cudaHostAlloc(&hgat_, table, cudaHostAllocDefault));
    hgat_cap_ = table;
  }
  if (table > dgat_cap_) {
    if (dgat_) cudaFree(dgat_);
    dgat_ = nullptr;
    CUDA_TRY(cudaMalloc(&dgat_, table));
    dgat_cap_ = table;
  }
  std::memcpy(hgat_, src.data(), n * sizeof(void*));
  std::memcpy(hgat_ + n * sizeof(void*), len.data(), n * sizeof(int64_t));
  std::memcpy(hgat_ + n * (sizeof(void*) + sizeof(int64_t)), off.data(), n * sizeof(int64_t));
  CUDA_TRY(cudaMemcpyAsync(dgat_, hgat_, table, cudaMemcpyHostToDevice, stream_));
  CUDA_TRY(tci_gather_launch(dgat_, (int)n, pinned_out, std::min<int>((int)n, 4 * num_sms), stream_));
  CUDA_TRY(cudaStreamSynchronize(stream_));
  stats.launches += 1;
  stats.h2d_bytes += (int64_t)table;
  stats.d2h_bytes += (int64_t)(total * sizeof(double));
  return 0;
}

int Engine::gather_to_host(const std::vector<const double*>& src, const std::vector<int64_t>& len,
                           double* host_out) {
  const size_t n = src.size();
  if (n == 0) return 0;
  size_t total = 0;
  std::vector<int64_t> off(n);
  for (size_t i = 0; i < n; ++i) {
    off[i] = (int64_t)total;
    total += (size_t)len[i];
  }
  const size_t table = a16(n * (sizeof(void*) + 2 * sizeof(int64_t)));
  const size_t need = table + total * sizeof(double);
  if (need > hgat_cap_) {
    if (hgat_) cudaFreeHost(hgat_);
    hgat_ = nullptr;
    CUDA_TRY(cudaHostAlloc(&hgat_, need, cudaHostAllocDefault));
    hgat_cap_ = need;
  }
  if (need > dgat_cap_) {
    if (dgat_) cudaFree(dgat_);
    dgat_ = nullptr;
    CUDA_TRY(cudaMalloc(&dgat_, need));
    dgat_cap_ = need;
  }
  std::memcpy(hgat_, src.data(), n * sizeof(void*));
  std::memcpy(hgat_ + n * sizeof(void*), len.data(), n * sizeof(int64_t));
  std::memcpy(hgat_ + n * (sizeof(void*) + sizeof(int64_t)), off.data(), n * sizeof(int64_t));
  CUDA_TRY(cudaMemcpyAsync(dgat_, hgat_, table, cudaMemcpyHostToDevice, stream_));
  CUDA_TRY(tci_gather_launch(dgat_, (int)n, (double*)(dgat_ + table), std::min<int>((int)n, 4 * num_sms),
                             stream_));
  CUDA_TRY(cudaMemcpyAsync(hgat_ + table, dgat_ + table, total * sizeof(double), cudaMemcpyDeviceToHost,
                           stream_));
  CUDA_TRY(cudaStreamSynchronize(stream_));
  // staging -> caller's (pageable) buffer: large copies in parallel, which also
  // spreads the first-touch page faults of a fresh buffer over the threads
  const char* src0 = hgat_ + table;
  char* dst0 = (char*)host_out;
  const size_t bytes = total * sizeof(double);
  const size_t nthr = bytes >= ((size_t)64 << 20) ? 8 : 1;
  if (nthr == 1) {
    std::memcpy(dst0, src0, bytes);
  } else {
    const size_t part = (bytes / nthr + 4095) & ~(size_t)4095;
    std::vector<std::thread> th;
    for (size_t q = 1; q < nthr; ++q) {
      const size_t b = q * part;
      if (b >= bytes) break;
      th.emplace_back([=] { std::memcpy(dst0 + b, src0 + b, std::min(part, bytes - b)); });
    }
    std::memcpy(dst0, src0, std::min(part, bytes));
    for (auto& t : th) t.join();
  }
  stats.launches += 1;
  stats.h2d_bytes += (int64_t)table;
  stats.d2h_bytes += (int64_t)(total * sizeof(double));
  return 0;
}

static CoTask co_tasks(Engine& e, std::vector<Req*> reqs) {
  GpuOp op{&e, reqs};
  co_await op;
  co_return op.status;
}

// A rank-revealing LU of a given matrix large enough to spread over every SM:
// the multi-CTA kernel instead of one CTA working out of global memory.
static bool big_eligible(const Req& r, bool resident, int grid) {
  const tci_task& t = r.t;
  return !resident && t.kind == TCI_TASK_RRLU && (t.ain || r.ain_host) &&
         (t.post == TCI_POST_FACTORS || t.post == TCI_POST_NONE) && (int64_t)t.m * t.n >= ((int64_t)1 << 18) &&
         tci_rrlu_big_fits(t.m, t.n, grid);
}

int Engine::run_big(Req& r) {
  tci_task& t = r.t;
  const int64_t m = t.m, n = t.n;
  const int grid = num_sms * tci_k256::kernels.ctas_per_sm;
  const size_t rb = result_bytes(t);
  const size_t scratch = tci_rrlu_big_scratch_bytes(grid, t.maxrank);
  // one device block: result record, scratch, input copy (if host), working matrix
  const size_t in_elems = r.ain_host ? (size_t)(m * n) : 0;
  const size_t fact_elems = t.post == TCI_POST_FACTORS ? 0 : (size_t)(m * n) + ((size_t)(m + n) * 4 + 7) / 8;
  const size_t head_bytes = a16(rb) + a16(scratch);
  const size_t total = head_bytes / 8 + in_elems + (size_t)(m * n) + fact_elems;
  double* blk = alloc_core(total);
  if (!blk) return fail(TCI_ERR_OOM, "device memory for the rrLU");
  char* res = (char*)blk;
  void* scr = (char*)blk + a16(rb);
  double* in = blk + head_bytes / 8;
  double* work = in + in_elems;
  double* fact = t.post == TCI_POST_FACTORS ? t.core_out : work + (size_t)(m * n);
  const double* ain = t.ain;
  int rc = 0;
  cudaError_t ce = cudaSuccess;
  if (r.ain_host) {
    ce = cudaMemcpyAsync(in, r.ain_host, (size_t)(m * n) * 8, cudaMemcpyHostToDevice, stream_);
    ain = in;
  }
  if (ce == cudaSuccess && timing) ce = cudaEventRecord(ev0_, stream_);
  if (ce == cudaSuccess)
    ce = tci_rrlu_big_launch(ain, work, fact, res, scr, (int)m, (int)n, t.maxrank, t.kcap, t.leftorth, t.reltol,
                             t.abstol, grid, stream_);
  if (ce == cudaSuccess && timing) ce = cudaEventRecord(ev1_, stream_);
  big_res_.resize(rb);
  if (ce == cudaSuccess) ce = cudaMemcpyAsync(big_res_.data(), res, rb, cudaMemcpyDeviceToHost, stream_);
  if (ce == cudaSuccess) ce = cudaStreamSynchronize(stream_);
  free_core(blk);
  if (ce != cudaSuccess) return fail(TCI_ERR_CUDA, cudaGetErrorString(ce));
  if (timing) {
    float ms = 0;
    cudaEventElapsedTime(&ms, ev0_, ev1_);
    stats.kernel_ms += ms;
  }
  r.res = big_res_.data();
  r.res_bytes = rb;
  stats.launches += 1;
  stats.tasks += 1;
  stats.h2d_bytes += (int64_t)(in_elems * 8);
  stats.d2h_bytes += (int64_t)rb;
  for (int64_t k = 1; k < r.head()->npivot; ++k) stats.lu_updates += (m - k) * (n - k);
  if (r.head()->status & TCI_ST_TOO_LARGE) rc = fail(TCI_ERR_TIMEOUT, "multi-CTA rrLU: a grid barrier hit its bound");
  return rc;
}

int Engine::run_tasks(std::vector<Req*>& reqs) {
  if (fc_callback_depth()) return reentry();
  if (reqs.size() == 1 && big_eligible(*reqs[0], resident(), num_sms * tci_k256::kernels.ctas_per_sm))
    return run_big(*reqs[0]);
  CoTask t = co_tasks(*this, reqs);
  return run(t, false);
}

int Engine::run_resident(CoTask& t) {
  int rc = att_rq_->start(&tci_k512::kernels);  // one solve: its tasks run one at a time
  if (rc) return rc;
  set_resident(att_rq_, att_h_, att_s_);
  t.h.resume();
  auto now = [] { return std::chrono::steady_clock::now(); };
  auto last_progress = now(), last_done = now();
  while (!t.h.done()) {
    rc = submit();
    if (rc) break;
    if (t.h.done()) break;  // a task that could not be submitted failed the solve
    bool progressed = false;
    rc = poll(progressed);
    if (rc) break;
    const auto tnow = now();
    if (progressed) {
      last_progress = last_done = tnow;
      continue;
    }
    if (!has_flights()) {
      if (idle()) {
        rc = fail(TCI_ERR_GENERIC, "engine stalled");
        break;
      }
      continue;
    }
    if (tnow - last_progress > std::chrono::milliseconds(2)) {  // the kernel may have left on its idle limit
      rc = att_rq_->ensure_alive();
      if (rc) break;
      last_progress = tnow;
    }
    if (tnow - last_done > std::chrono::seconds(120)) {
      rc = fail(TCI_ERR_TIMEOUT, "resident mode: no task finished for 120 s");
      break;
    }
  }
  const int src = att_rq_->stop();
  abandon();
  set_resident(nullptr, nullptr, nullptr);
  if (rc) return rc;
  if (src) return src;
  return t.h.promise().rc;
}

int Engine::run(CoTask& t, bool allow_resident) {
  if (fc_callback_depth()) return reentry();
  if (allow_resident && att_rq_ && !resident()) return run_resident(t);
  t.h.resume();
  while (!t.h.done()) {
    if (idle()) return fail(TCI_ERR_GENERIC, "engine stalled");
    int rc = step();
    if (rc && !t.h.done() && idle()) return rc;
  }
  return t.h.promise().rc;
}

// ---------------------------------------------------------------- TCI2 pieces
static void updatemaxsample(Solve& s, double maxabs) {
  // updatemaxsample!/maxabs (tensorci2.jl:397-399, util.jl:1-10)
  s.maxsample = jmax(std::fabs(s.maxsample), maxabs);
}

// updatebonderror!/updatepivoterror!/updateerrors! (tensorci2.jl:132-169)
static void updateerrors(Solve& s, int b, const double* diag, int K, double err) {
  s.bonderrors[b] = err;
  size_t ne = (size_t)K + 1;
  size_t n = std::max(s.pivoterrors.size(), ne);
  std::vector<double> out(n);
  for (size_t i = 0; i < n; ++i) {
    double a = i < s.pivoterrors.size() ? s.pivoterrors[i] : 0.0;
    double c = i < (size_t)K ? diag[i] : (i == (size_t)K ? err : 0.0);
    out[i] = jmax(a, c);
  }
  s.pivoterrors.swap(out);
}

static void fill_f(Req& r, const Solve& s) {
  r.t.fid = s.fid;
  r.t.nparams = (int32_t)s.params.size();
  r.t.L = s.L;
  r.params = s.params.data();
  r.t.lutcap0 = s.lutcap0;
  r.t.lutcap1 = s.lutcap1;
  r.fcache = s.fcache.get();
  if (s.lut_dev) {
    r.t.lut = s.lut_dev;
    r.t.lut_full = 1;
    r.t.lut_base0 = s.L;
  }
}

static int clamp_rank(i64 maxrank, size_t m, size_t n) {
  i64 k = std::min<i64>(maxrank, (i64)std::min(m, n));
  return (int)std::max<i64>(k, 0);
}

i64 solve_rank(const Solve& s) {
  i64 r = 0;
  for (int b = 1; b < s.L; ++b) r = std::max<i64>(r, (i64)s.Iset[b].n);
  return r;
}

// A solve whose f values come from the device value cache, filled by a
// caller-supplied fn or by the library's own evaluator.
static int init_cached(Solve& s, int L, const int64_t* localdims, tci_batch_fn fn, void* user,
                       std::shared_ptr<FEvaluator> ev) {
  if (L < 2) return fail(TCI_ERR_GENERIC, "localdims should have at least 2 elements!");
  s.L = L;
  s.d.assign(localdims, localdims + L);
  for (int x : s.d)
    if (x < 1 || x > 256) return fail(TCI_ERR_ARG, "local dimensions must be in 1..256");
  s.fid = TCI_FID_CACHE;
  s.params.assign(4 + (size_t)L, 0.0);
  s.fcache = std::make_shared<FCache>();
  int rc = s.fcache->init(L, s.d.data(), fn, user, s.params.data(), std::move(ev));
  if (rc) return rc;
  s.Iset.assign(L, IndexSet());
  s.Jset.assign(L, IndexSet());
  for (int b = 0; b < L; ++b) {
    s.Iset[b].len = b;
    s.Jset[b].len = L - 1 - b;
  }
  s.cores.assign(L, Core());
  s.bonderrors.assign(L - 1, 0.0);
  s.lutcap0 = s.lutcap1 = 0;
  s.pivoterrors.clear();
  return 0;
}

int solve_init_evaluator(Solve& s, int L, const int64_t* localdims, std::shared_ptr<FEvaluator> ev) {
  return init_cached(s, L, localdims, nullptr, nullptr, std::move(ev));
}

int solve_init(Solve& s, int L, const int64_t* localdims, int fid, const double* params,
               int64_t nparams, const int64_t*, int64_t) {
  if (L < 2) return fail(TCI_ERR_GENERIC, "localdims should have at least 2 elements!");
  if (fid >= TCI_F_USER) {  // caller-supplied f behind the device value cache
    tci_batch_fn fn = nullptr;
    void* user = nullptr;
    if (!user_fn(fid, &fn, &user)) return fail(TCI_ERR_ARG, "unknown function id");
    return init_cached(s, L, localdims, fn, user, nullptr);
  }
  if (fid < TCI_F_LORENTZ || fid > TCI_F_PRODUCT) return fail(TCI_ERR_ARG, "unknown function id");
  s.L = L;
  s.d.assign(localdims, localdims + L);
  for (int x : s.d)
    if (x < 1 || x > 256) return fail(TCI_ERR_ARG, "local dimensions must be in 1..256");
  if (fid == TCI_F_SERVED && nparams < 3 + L) return fail(TCI_ERR_ARG, "served f needs 3+L params");
  if (fid == TCI_F_QTT2D)
    for (int x : s.d)
      if (x != 4) return fail(TCI_ERR_ARG, "qtt2d needs local dimension 4");
  if (fid == TCI_F_QTT1D)
    for (int x : s.d)
      if (x != 2) return fail(TCI_ERR_ARG, "qtt1d needs local dimension 2");
  if (fid == TCI_F_PRODUCT) {
    if (nparams < 3 || (int)params[0] != L) return fail(TCI_ERR_ARG, "product f parameter block");
    const int D = (int)params[1];
    for (int x : s.d)
      if (x > D) return fail(TCI_ERR_ARG, "product f tables narrower than a local dimension");
    if (nparams < 3 + 2 * (int64_t)L * D) return fail(TCI_ERR_ARG, "product f tables too short");
  }
  if (fid == TCI_F_DENSE) {
    if (nparams < 1 + L || (int)params[0] != L) return fail(TCI_ERR_ARG, "dense f parameter block");
    int64_t total = 1;
    for (int x : s.d) total *= x;
    if (nparams < 1 + L + total) return fail(TCI_ERR_ARG, "dense f table too short");
  }
  s.fid = fid;
  s.params.assign(params, params + nparams);
  s.Iset.assign(L, IndexSet());
  s.Jset.assign(L, IndexSet());
  for (int b = 0; b < L; ++b) {
    s.Iset[b].len = b;
    s.Jset[b].len = L - 1 - b;
  }
  s.cores.assign(L, Core());
  s.bonderrors.assign(L - 1, 0.0);
  // table ranges of the factored functions: sum v^2 over [L, sum d^2] and
  // sum (v - c)^2 over [0, sum max((d - c)^2, (1 - c)^2)]
  s.lutcap0 = s.lutcap1 = 0;
  if (fid == TCI_F_LORENTZ || fid == TCI_F_SERVED) {
    int64_t hi0 = 0, hi1 = 0;
    for (int p = 0; p < L; ++p) {
      hi0 += (int64_t)s.d[p] * s.d[p];
      if (fid == TCI_F_SERVED) {
        int64_t c = (int64_t)params[3 + p];
        int64_t a = (int64_t)s.d[p] - c, b = 1 - c;
        hi1 += std::max(a * a, b * b);
      }
    }
    if (hi0 - L + 1 <= (1 << 20)) s.lutcap0 = (int)(hi0 - L + 1);
    if (fid == TCI_F_SERVED) {
      if (hi1 + 1 <= (1 << 20) && s.lutcap0 > 0)
        s.lutcap1 = (int)(hi1 + 1);
      else
        s.lutcap0 = 0;
    }
  }
  s.pivoterrors.clear();
  return 0;
}

// addglobalpivots! (tensorci2.jl:193-213); pivots are 0-based byte vectors.
int addglobalpivots(Solve& s, const std::vector<std::vector<uint8_t>>& pivots) {
  for (const auto& p : pivots)
    if ((int)p.size() != s.L)
      return fail(TCI_ERR_DIM, "Please specify a pivot as one index per leg of the MPS.");
  for (const auto& p : pivots)
    for (int b = 0; b < s.L; ++b) {
      s.Iset[b].push_unique(p.data());
      s.Jset[b].push_unique(p.data() + b + 1);
    }
  return 0;
}

static void invalidate(Engine& e, Solve& s) { e.release_cores(s); }

// TensorCI2{ValueType}(func, localdims, initialpivots) (tensorci2.jl:42-53)
CoTask co_construct(Engine& e, Solve& s, std::vector<std::vector<uint8_t>> pivots) {
  if (pivots.empty()) co_return fail(TCI_ERR_ARG, "initialpivots must not be empty");
  int rc = addglobalpivots(s, pivots);
  if (rc) co_return rc;
  std::vector<uint8_t> pts;
  for (const auto& p : pivots) pts.insert(pts.end(), p.begin(), p.end());
  // the solve's f tables, once: every later task of the solve looks f up
  if (s.lutcap0 > 0 && !s.lut_dev) s.lut_dev = e.alloc_core((size_t)s.lutcap0 + (size_t)std::max(s.lutcap1, 0));
  Req r, tab;
  r.t.kind = TCI_TASK_EVAL;
  fill_f(r, s);
  r.t.m = (int32_t)pivots.size();
  r.t.nl = s.L;
  r.rows = pts.data();
  r.rows_bytes = pts.size();
  std::vector<Req*> reqs{&r};
  if (s.lut_dev) {
    tab.t.kind = TCI_TASK_TABLE;
    fill_f(tab, s);
    reqs.push_back(&tab);
  }
  GpuOp op{&e, reqs};
  co_await op;
  if (op.status) co_return op.status;
  double ms = -std::numeric_limits<double>::infinity();
  for (int i = 0; i < r.t.m; ++i) ms = jmax(ms, std::fabs(r.fvals()[i]));
  s.nfeval += r.t.m;
  s.maxsample = ms;
  if (!(std::fabs(ms) > 0.0)) co_return fail(TCI_ERR_GENERIC, "maxsamplevalue is zero!");
  invalidate(e, s);
  co_return 0;
}

// updatepivots! with pivotsearch=:full (tensorci2.jl:510-551, 599-607).  The
// site tensors left(luci)/right(luci) of :601-604 are not formed: the next
// updatepivots! (:524) or fillsitetensors! replaces them before any use.
CoTask co_updatepivots(Engine& e, Solve& s, int b, bool leftorth, double reltol, double abstol,
                       i64 maxbonddim, const IndexSet* extraI, const IndexSet* extraJ) {
  invalidate(e, s);
  IndexSet emptyI, emptyJ;
  emptyI.len = b + 1;
  emptyJ.len = s.L - 1 - b;
  IndexSet Ic = set_union(kron_right(s.Iset[b], s.d[b]), extraI ? *extraI : emptyI);
  IndexSet Jc = set_union(kron_left(s.d[b + 1], s.Jset[b + 1]), extraJ ? *extraJ : emptyJ);
  Req r;
  r.t.kind = TCI_TASK_RRLU;
  fill_f(r, s);
  r.t.m = (int32_t)Ic.n;
  r.t.n = (int32_t)Jc.n;
  r.t.nl = Ic.len;
  r.t.nr = Jc.len;
  r.t.maxrank = clamp_rank(maxbonddim, Ic.n, Jc.n);
  r.t.kcap = r.t.maxrank;
  r.t.reltol = reltol;
  r.t.abstol = abstol;
  r.t.leftorth = leftorth ? 1 : 0;
  r.t.post = TCI_POST_NONE;
  r.rows = Ic.data.data();
  r.rows_bytes = Ic.data.size();
  r.cols = Jc.data.data();
  r.cols_bytes = Jc.data.size();
  GpuOp op{&e, {&r}};
  co_await op;
  if (op.status) co_return op.status;
  const tci_result_head* h = r.head();
  s.nfeval += (i64)Ic.n * (i64)Jc.n;
  updatemaxsample(s, h->maxabs);
  if (h->status & TCI_ST_NAN) {
    if (std::getenv("TCI_DEBUG_NAN")) {
      std::fprintf(stderr, "NaN task: b %d m %d n %d nl %d nr %d lutcap %d %d lut_used %d smem %d K %d maxabs %g "
                   "maxabs_nan %d cycles %lld fid %d nparams %d L %d resident %d\n", b, r.t.m, r.t.n, r.t.nl,
                   r.t.nr, r.t.lutcap0, r.t.lutcap1, h->lut_used, r.t.smem_mode, h->npivot, h->maxabs,
                   h->maxabs_nan, (long long)h->cycles, r.t.fid, r.t.nparams, s.L, (int)e.resident());
      for (int q = 0; q < (int)s.params.size(); ++q) std::fprintf(stderr, " %g", s.params[q]);
      std::fprintf(stderr, "\n");
    }
    co_return fail(TCI_ERR_NAN, "lu.L contains NaNs");
  }
  const int K = h->npivot;
  s.Iset[b + 1] = select(Ic, r.rowperm(), K);
  s.Jset[b] = select(Jc, r.colperm(), K);
  updateerrors(s, b, r.diag(), K, h->error);
  co_return 0;
}

bool forwardsweep(int strategy, i64 iter) { return strategy == 1 || (strategy == 0 && (iter % 2) == 1); }

// fillsitetensors! (globalsearch.jl:97-103) -> setsitetensor!(tci, f, b)
// (tensorci2.jl:367-394) for all b in one step.
CoTask co_fillsitetensors(Engine& e, Solve& s) {
  const int L = s.L;
  for (int b = 0; b < L - 1; ++b)
    if (s.Iset[b + 1].n != s.Jset[b].n)
      co_return fail(TCI_ERR_GENERIC, "Pivot matrix at bond " + std::to_string(b + 1) + " is not square!");
  invalidate(e, s);
  std::vector<IndexSet> Is(L);
  std::vector<Req> reqs(L);
  std::vector<Req*> ptrs;
  for (int b = 0; b < L; ++b) {
    Is[b] = kron_right(s.Iset[b], s.d[b]);
    Req& r = reqs[b];
    fill_f(r, s);
    r.t.m = (int32_t)Is[b].n;
    r.t.nl = Is[b].len;
    r.t.nr = s.Jset[b].len;
    r.rows = Is[b].data.data();
    r.rows_bytes = Is[b].data.size();
    r.cols = s.Jset[b].data.data();
    r.cols_bytes = s.Jset[b].data.size();
    Core& c = s.cores[b];
    c.d0 = (i64)s.Iset[b].n;
    c.d1 = s.d[b];
    if (b == L - 1) {
      r.t.kind = TCI_TASK_CORE;
      r.t.n = (int32_t)s.Jset[b].n;
      c.d2 = (i64)s.Jset[b].n;
    } else {
      r.t.kind = TCI_TASK_SITE;
      r.t.r = (int32_t)s.Jset[b].n;
      r.t.n = r.t.r;
      r.t.maxrank = r.t.r;
      r.t.kcap = r.t.r;
      r.t.leftorth = 1;
      r.prows = s.Iset[b + 1].data.data();
      r.prows_bytes = s.Iset[b + 1].data.size();
      c.d2 = (i64)s.Iset[b + 1].n;
    }
    c.p = e.alloc_core(c.elems());
    if (!c.p) co_return fail(TCI_ERR_OOM, "device memory for site tensors");
    r.t.core_out = c.p;
    ptrs.push_back(&r);
  }
  GpuOp op{&e, ptrs};
  co_await op;
  if (op.status) co_return op.status;
  for (int b = 0; b < L; ++b) {
    const tci_result_head* h = reqs[b].head();
    updatemaxsample(s, h->maxabs);
    s.nfeval += (i64)reqs[b].t.m * (reqs[b].t.kind == TCI_TASK_SITE ? reqs[b].t.r : reqs[b].t.n);
    if (h->status & TCI_ST_SINGULAR) co_return fail(TCI_ERR_SINGULAR, "SingularException in setsitetensor!");
    if (h->status & TCI_ST_NAN) co_return fail(TCI_ERR_NAN, "Error: NaN in tensor T[" + std::to_string(b + 1) + "]");
  }
  s.cores_valid = true;
  co_return 0;
}

// sweep2site! (tensorci2.jl:855-916)
CoTask co_sweep2site(Engine& e, Solve& s, int niter, int iter1, double abstol, i64 maxbonddim,
                     int strategy, bool strictlynested, bool fillsite) {
  invalidate(e, s);
  const int n = s.L;
  for (int iter = iter1; iter < iter1 + niter; ++iter) {
    std::vector<IndexSet> extraI, extraJ;
    bool use_extra = !strictlynested && s.has_hist;
    if (use_extra) {  // the snapshot is replaced right below, so take it
      extraI = std::move(s.Ihist);
      extraJ = std::move(s.Jhist);
    }
    s.Ihist = s.Iset;
    s.Jhist = s.Jset;
    s.has_hist = true;
    s.pivoterrors.clear();
    if (forwardsweep(strategy, iter)) {
      for (int b = 0; b < n - 1; ++b)
        CO_TRY(co_updatepivots(e, s, b, true, 1e-14, abstol, maxbonddim,
                               use_extra ? &extraI[b + 1] : nullptr, use_extra ? &extraJ[b] : nullptr));
    } else {
      for (int b = n - 2; b >= 0; --b)
        CO_TRY(co_updatepivots(e, s, b, false, 1e-14, abstol, maxbonddim,
                               use_extra ? &extraI[b + 1] : nullptr, use_extra ? &extraJ[b] : nullptr));
    }
  }
  if (fillsite) CO_TRY(co_fillsitetensors(e, s));
  co_return 0;
}

// sweep1site! (tensorci2.jl:402-461)
CoTask co_sweep1site(Engine& e, Solve& s, bool forward, double reltol, double abstol, i64 maxbonddim,
                     bool updatetensors) {
  s.pivoterrors.clear();
  invalidate(e, s);
  const int L = s.L;
  for (int step = 0; step < L - 1; ++step) {
    const int b = forward ? step : L - 1 - step;
    IndexSet Is = forward ? kron_right(s.Iset[b], s.d[b]) : s.Iset[b];
    IndexSet Js = forward ? s.Jset[b] : kron_left(s.d[b], s.Jset[b]);
    Req r;
    r.t.kind = TCI_TASK_RRLU;
    fill_f(r, s);
    r.t.m = (int32_t)Is.n;
    r.t.n = (int32_t)Js.n;
    r.t.nl = Is.len;
    r.t.nr = Js.len;
    r.t.maxrank = clamp_rank(maxbonddim, Is.n, Js.n);
    r.t.kcap = r.t.maxrank;
    r.t.reltol = reltol;
    r.t.abstol = abstol;
    r.t.leftorth = forward ? 1 : 0;
    r.t.post = updatetensors ? (forward ? TCI_POST_LEFT : TCI_POST_RIGHT) : TCI_POST_NONE;
    r.rows = Is.data.data();
    r.rows_bytes = Is.data.size();
    r.cols = Js.data.data();
    r.cols_bytes = Js.data.size();
    double* out = nullptr;
    size_t cap = 0;
    if (updatetensors) {
      cap = forward ? (size_t)Is.n * r.t.kcap : (size_t)r.t.kcap * Js.n;
      out = e.alloc_core(cap);
      if (!out) co_return fail(TCI_ERR_OOM, "device memory for site tensors");
      r.t.core_out = out;
    }
    GpuOp op{&e, {&r}};
    co_await op;
    if (op.status) co_return op.status;
    const tci_result_head* h = r.head();
    s.nfeval += (i64)Is.n * (i64)Js.n;
    updatemaxsample(s, h->maxabs);
    if (h->status & TCI_ST_NAN) {
      if (out) e.free_core(out);
      co_return fail(TCI_ERR_NAN, "lu.L contains NaNs");
    }
    const int K = h->npivot;
    if (forward) {
      s.Iset[b + 1] = select(Is, r.rowperm(), K);
      s.Jset[b] = select(Js, r.colperm(), K);
    } else {
      s.Iset[b] = select(Is, r.rowperm(), K);
      s.Jset[b - 1] = select(Js, r.colperm(), K);
    }
    if (updatetensors) {
      Core& c = s.cores[b];
      c.p = out;
      c.d0 = (i64)s.Iset[b].n;
      c.d1 = s.d[b];
      c.d2 = (i64)s.Jset[b].n;
    }
    updateerrors(s, forward ? b : b - 1, r.diag(), K, h->error);
  }
  if (updatetensors) {
    const int b = forward ? L - 1 : 0;
    IndexSet Is = kron_right(s.Iset[b], s.d[b]);
    Req r;
    r.t.kind = TCI_TASK_CORE;
    fill_f(r, s);
    r.t.m = (int32_t)Is.n;
    r.t.n = (int32_t)s.Jset[b].n;
    r.t.nl = Is.len;
    r.t.nr = s.Jset[b].len;
    r.rows = Is.data.data();
    r.rows_bytes = Is.data.size();
    r.cols = s.Jset[b].data.data();
    r.cols_bytes = s.Jset[b].data.size();
    Core& c = s.cores[b];
    c.d0 = (i64)s.Iset[b].n;
    c.d1 = s.d[b];
    c.d2 = (i64)s.Jset[b].n;
    c.p = e.alloc_core(c.elems());
    if (!c.p) co_return fail(TCI_ERR_OOM, "device memory for site tensors");
    r.t.core_out = c.p;
    GpuOp op{&e, {&r}};
    co_await op;
    if (op.status) co_return op.status;
    s.nfeval += (i64)Is.n * (i64)s.Jset[b].n;
    s.cores_valid = true;
  }
  co_return 0;
}

static void core_table(const Solve& s, std::vector<tci_core_ref>& tab, int& rmax) {
  tab.resize(s.L);
  rmax = 1;
  for (int b = 0; b < s.L; ++b) {
    const Core& c = s.cores[b];
    tab[b].p = c.p;
    tab[b].r0 = (int32_t)c.d0;
    tab[b].d = (int32_t)c.d1;
    tab[b].r1 = (int32_t)c.d2;
    tab[b].pad = 0;
    rmax = std::max<int>(rmax, (int)std::max(c.d0, c.d2));
  }
}

// f and the train at points (np x L, 0-based bytes).  ttout may be null.
CoTask co_evaluate(Engine& e, Solve& s, const uint8_t* pts, i64 np, double* fout,
                   double* ttout) {
  if (ttout && !s.cores_valid) co_return fail(TCI_ERR_GENERIC, "site tensors are not available");
  std::vector<tci_core_ref> tab;
  int rmax = 1;
  if (ttout) core_table(s, tab, rmax);
  // one EVAL task per chunk of points, all in one step, so every SM takes a share
  const i64 chunk = 4096;
  const i64 ntask = (np + chunk - 1) / chunk;
  std::vector<Req> reqs((size_t)ntask);
  std::vector<Req*> ptrs;
  for (i64 q = 0; q < ntask; ++q) {
    Req& r = reqs[(size_t)q];
    const i64 p0 = q * chunk, n = std::min(chunk, np - p0);
    r.t.kind = TCI_TASK_EVAL;
    fill_f(r, s);
    if (!fout) {  // train values only: no f
      r.t.fid = 0;
      r.fcache = nullptr;
    }
    r.t.m = (int32_t)n;
    r.t.nl = s.L;
    r.rows = pts + (size_t)p0 * s.L;
    r.rows_bytes = (size_t)n * s.L;
    if (ttout) {
      r.cores = tab.data();
      r.ncores = s.L;
      r.t.r = rmax;
    }
    ptrs.push_back(&r);
  }
  GpuOp op{&e, ptrs};
  co_await op;
  if (op.status) co_return op.status;
  for (i64 q = 0; q < ntask; ++q) {
    const Req& r = reqs[(size_t)q];
    const i64 p0 = q * chunk;
    if (fout) std::memcpy(fout + p0, r.fvals(), (size_t)r.t.m * 8);
    if (ttout) std::memcpy(ttout + p0, r.ttvals(), (size_t)r.t.m * 8);
  }
  co_return 0;
}

CoTask co_sum(Engine& e, Solve& s, double* out) {
  if (!s.cores_valid) co_return fail(TCI_ERR_GENERIC, "site tensors are not available");
  std::vector<tci_core_ref> tab;
  int rmax = 1;
  core_table(s, tab, rmax);
  Req r;
  r.t.kind = TCI_TASK_SUM;
  r.t.L = s.L;
  r.t.r = rmax;
  r.cores = tab.data();
  r.ncores = s.L;
  GpuOp op{&e, {&r}};
  co_await op;
  if (op.status) co_return op.status;
  *out = r.head()->error;
  co_return 0;
}

// DefaultGlobalPivotFinder (globalpivotfinder.jl:143-195): nsearch random start
// points, a line scan along every site, the point of largest |f - tt| kept when
// it exceeds abstol * tolmarginglobalsearch.  Each start point is one SEARCH
// task (train values through left/right environments of the start point).
CoTask co_globalpivots(Engine& e, Solve& s, double abstol, int nsearch, int maxnglobalpivot,
                       double tolmargin, std::vector<std::vector<uint8_t>>* found) {
  found->clear();
  if (nsearch <= 0) co_return 0;
  if (!s.cores_valid) co_return fail(TCI_ERR_GENERIC, "site tensors are not available");
  const int L = s.L;
  std::vector<std::vector<uint8_t>> starts(nsearch, std::vector<uint8_t>(L));
  for (int q = 0; q < nsearch; ++q)
    for (int p = 0; p < L; ++p) starts[q][p] = (uint8_t)(tci_rng_uniform1(&s.rng, (uint64_t)s.d[p]) - 1);
  i64 per = 0;
  for (int p = 0; p < L; ++p) per += s.d[p];
  std::vector<tci_core_ref> tab;
  int rmax = 1;
  core_table(s, tab, rmax);
  int envs = 0;
  for (int p = 0; p < L; ++p) envs += tab[p].r0 + tab[p].r1;
  std::vector<Req> reqs(nsearch);
  std::vector<Req*> ptrs;
  for (int q = 0; q < nsearch; ++q) {
    Req& r = reqs[q];
    r.t.kind = TCI_TASK_SEARCH;
    fill_f(r, s);
    r.t.m = (int32_t)per;
    r.t.n = envs;
    r.t.r = rmax;
    r.rows = starts[q].data();
    r.rows_bytes = (size_t)L;
    r.cores = tab.data();
    r.ncores = L;
    ptrs.push_back(&r);
  }
  GpuOp op{&e, ptrs};
  co_await op;
  if (op.status) co_return op.status;
  s.nfeval += per * nsearch;
  for (int q = 0; q < nsearch; ++q) {
    const double* fv = reqs[q].fvals();
    const double* tv = reqs[q].ttvals();
    double best_error = 0.0;
    int bp_site = -1, bp_val = 0;
    int k = 0;
    for (int p = 0; p < L; ++p)
      for (int v = 0; v < s.d[p]; ++v, ++k) {
        double err = std::fabs(fv[k] - tv[k]);
        if (err > best_error) {
          best_error = err;
          bp_site = p;
          bp_val = v;
        }
      }
    if (best_error > abstol * tolmargin) {
      std::vector<uint8_t> bp = starts[q];
      if (bp_site >= 0) bp[bp_site] = (uint8_t)bp_val;
      found->push_back(bp);
    }
  }
  if ((int)found->size() > maxnglobalpivot) found->resize(maxnglobalpivot);
  co_return 0;
}

// convergencecriterion (tensorci2.jl:609-628)
bool convergencecriterion(const std::vector<i64>& ranks, const std::vector<double>& errors,
                          const std::vector<i64>& ngp, double tolerance, i64 maxbonddim,
                          i64 ncheckhistory, bool checkconvglobalpivot) {
  if ((i64)errors.size() < ncheckhistory) return false;
  const i64 n = ncheckhistory;
  if (n <= 0) return false;
  bool allerr = true, allg = true, allmax = true;
  i64 mn = INT64_MAX;
  for (i64 i = (i64)ranks.size() - n; i < (i64)ranks.size(); ++i) {
    allmax &= ranks[i] >= maxbonddim;
    mn = std::min(mn, ranks[i]);
  }
  for (i64 i = (i64)errors.size() - n; i < (i64)errors.size(); ++i) allerr &= errors[i] < tolerance;
  for (i64 i = (i64)ngp.size() - n; i < (i64)ngp.size(); ++i) allg &= ngp[i] == 0;
  return (allerr && (checkconvglobalpivot ? allg : true) && mn == ranks.back()) || allmax;
}

// optimize! (tensorci2.jl:700-850) with DefaultGlobalPivotFinder.
CoTask co_optimize(Engine& e, Solve& s, tci_opts o) {
  const double tol = o.tolerance;
  const i64 maxbonddim = o.maxbonddim <= 0 ? TYPEMAX : o.maxbonddim;
  if (o.nsearchglobalpivot > 0 && o.nsearchglobalpivot < o.maxnglobalpivot)
    co_return fail(TCI_ERR_GENERIC, "nsearchglobalpivot < maxnglobalpivot!");
  if (maxbonddim >= TYPEMAX && tol <= 0)
    co_return fail(TCI_ERR_ARG,
                   "Specify either tolerance > 0 or some maxbonddim; otherwise, the convergence "
                   "criterion is not reachable!");
  tci_rng_seed(&s.rng, o.seed);
  s.opts = o;
  s.ranks.clear();
  s.errors.clear();
  s.nglobal.clear();
  std::vector<std::vector<uint8_t>> gp;
  for (i64 iter = 1; iter <= o.maxiter; ++iter) {
    double errnorm = o.normalizeerror ? s.maxsample : 1.0;
    double abstol = tol * errnorm;
    CO_TRY(co_sweep2site(e, s, 2, 1, abstol, maxbonddim, o.sweepstrategy, o.strictlynested != 0, true));
    double perr = *std::max_element(s.bonderrors.begin(), s.bonderrors.end());
    s.errors.push_back(perr);
    CO_TRY(co_globalpivots(e, s, abstol, o.nsearchglobalpivot, o.maxnglobalpivot, o.tolmarginglobalsearch,
                           &gp));
    int rc = addglobalpivots(s, gp);
    if (rc) co_return rc;
    if (!gp.empty()) invalidate(e, s);
    s.nglobal.push_back((i64)gp.size());
    s.ranks.push_back(solve_rank(s));
    if (convergencecriterion(s.ranks, s.errors, s.nglobal, abstol, maxbonddim, o.ncheckhistory,
                             o.checkconvglobalpivot != 0))
      break;
  }
  double errnorm = o.normalizeerror ? s.maxsample : 1.0;
  double abstol = tol * errnorm;
  CO_TRY(co_sweep1site(e, s, true, 1e-14, abstol, maxbonddim, true));
  for (int b = 0; b < s.L - 1; ++b)  // _sanitycheck (globalsearch.jl:106-112)
    if (s.Iset[b + 1].n != s.Jset[b].n)
      co_return fail(TCI_ERR_GENERIC, "Pivot matrix at bond " + std::to_string(b + 1) + " is not square!");
  for (auto& x : s.errors) x = x / errnorm;
  co_return 0;
}

// crossinterpolate2 (tensorci2.jl:943-953)
CoTask co_crossinterpolate2(Engine& e, Solve& s, std::vector<std::vector<uint8_t>> pivots, tci_opts o) {
  CO_TRY(co_construct(e, s, std::move(pivots)));
  const int rc = co_await co_optimize(e, s, o);
  // the f tables serve the sweeps only; a finished solve keeps just its cores
  // (later calls on it build per-task tables again)
  if (s.lut_dev) e.free_core(s.lut_dev);
  s.lut_dev = nullptr;
  co_return rc;
}

}  // namespace tci
