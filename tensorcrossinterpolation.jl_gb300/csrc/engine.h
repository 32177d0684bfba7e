// Host engine of the TCI2 sweep: solve state, index sets, the coroutine
// machinery that lets each solve be written as straight-line code, and the
// step loop that batches the GPU tasks of all live solves into one launch.
#pragma once
#include <cuda_runtime.h>

#include <atomic>
#include <coroutine>
#include <cstdio>
#include <cstdint>
#include <memory>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/tci_gb300.h"
#include "fcache.h"
#include "kernels.h"
#include "tci_rng.h"
#include "tci_tasks.h"

namespace tci {

using i64 = int64_t;
const i64 TYPEMAX = INT64_MAX;

// Error with the reference's exception message.
struct Error {
  int code = 0;
  std::string msg;
};
void set_error(int code, const std::string& msg);
int last_code();

// A set of multi-indices of equal length, stored flat (0-based uint8 values).
// Order of insertion is kept (the reference's Vector{MultiIndex}).
struct IndexSet {
  int len = 0;
  size_t n = 0;
  std::vector<uint8_t> data;
  const uint8_t* at(size_t i) const { return data.data() + i * (size_t)len; }
  void push(const uint8_t* v) {
    data.insert(data.end(), v, v + len);
    ++n;
  }
  bool contains(const uint8_t* v) const;
  void push_unique(const uint8_t* v) {
    if (!contains(v)) push(v);
  }
};
IndexSet kron_right(const IndexSet& I, int d);   // kronecker(Iset, d) (tensorci2.jl:315-320)
IndexSet kron_left(int d, const IndexSet& J);    // kronecker(d, Jset) (tensorci2.jl:322-327)
IndexSet set_union(const IndexSet& a, const IndexSet& b);  // Base.union
IndexSet select(const IndexSet& s, const int32_t* idx, int k);

// ------------------------------------------------------------ coroutines
struct CoTask {
  struct promise_type {
    std::coroutine_handle<> cont;
    int rc = 0;
    CoTask get_return_object() {
      return CoTask{std::coroutine_handle<promise_type>::from_promise(*this)};
    }
    std::suspend_always initial_suspend() noexcept { return {}; }
    struct Final {
      bool await_ready() noexcept { return false; }
      std::coroutine_handle<> await_suspend(std::coroutine_handle<promise_type> h) noexcept {
        auto c = h.promise().cont;
        return c ? c : std::noop_coroutine();
      }
      void await_resume() noexcept {}
    };
    Final final_suspend() noexcept { return {}; }
    void return_value(int v) { rc = v; }
    void unhandled_exception() { rc = TCI_ERR_GENERIC; }
  };
  std::coroutine_handle<promise_type> h;
  explicit CoTask(std::coroutine_handle<promise_type> hh) : h(hh) {}
  CoTask(CoTask&& o) noexcept : h(o.h) { o.h = {}; }
  CoTask(const CoTask&) = delete;
  ~CoTask() {
    if (h) h.destroy();
  }
  bool await_ready() { return false; }
  std::coroutine_handle<> await_suspend(std::coroutine_handle<> parent) {
    h.promise().cont = parent;
    return h;
  }
  int await_resume() { return h.promise().rc; }
};

#define CO_TRY(expr)              \
  do {                            \
    int _rc = co_await (expr);    \
    if (_rc) co_return _rc;       \
  } while (0)

// One GPU task as the host sees it.
struct Req {
  tci_task t{};
  const uint8_t* rows = nullptr;
  size_t rows_bytes = 0;
  const uint8_t* cols = nullptr;
  size_t cols_bytes = 0;
  const uint8_t* prows = nullptr;
  size_t prows_bytes = 0;
  const double* params = nullptr;
  const tci_core_ref* cores = nullptr;
  int ncores = 0;
  const double* ain_host = nullptr;  // packed into the upload blob
  const char* res = nullptr;         // host copy of the result record after the step
  size_t res_bytes = 0;
  uint64_t ticket = 0;               // resident mode: ring ticket of the task
  FCache* fcache = nullptr;          // caller-supplied f: values come from this cache
  const tci_result_head* head() const { return (const tci_result_head*)res; }
  const int32_t* rowperm() const { return (const int32_t*)(res + sizeof(tci_result_head)); }
  const int32_t* colperm() const {
    return (const int32_t*)(res + sizeof(tci_result_head) + ((size_t)t.kcap * 4 + 7) / 8 * 8);
  }
  const double* diag() const {
    return (const double*)(res + sizeof(tci_result_head) + 2 * (((size_t)t.kcap * 4 + 7) / 8 * 8));
  }
  const double* fvals() const { return (const double*)(res + sizeof(tci_result_head)); }
  const double* ttvals() const { return fvals() + t.m; }
};

class Engine;

// Power-of-two size-class pool.  Small blocks are carved from large slabs;
// every block is kept for reuse until the pool is destroyed, so allocation in
// steady state makes no CUDA call (a CUDA allocation while the resident kernel
// runs would serialise the device).  Device pools back the allocations with
// stream-ordered cudaMallocAsync on a private stream; host pools with mapped
// pinned memory that the device reads and writes directly.
class BlockPool {
 public:
  enum Kind { DEVICE, HOST };
  BlockPool(Kind kind, int device, bool locked);
  ~BlockPool();
  void* alloc(size_t bytes);  // nullptr when the backing allocation fails
  void free(void* p);
  // Back the next small-block allocations now (a pinned allocation while the
  // resident kernel runs would serialise the device).
  bool reserve_slab();
  size_t reserved() const { return reserved_; }

 private:
  static constexpr int MIN_SHIFT = 8;      // 256 B
  static constexpr int SLAB_SHIFT = 26;    // 64 MiB slabs
  static constexpr int CARVE_MAX = 22;     // blocks up to 4 MiB come from slabs
  void* backing(size_t bytes);
  Kind kind_;
  int device_;
  bool locked_;
  std::mutex mu_;
  cudaStream_t side_ = nullptr;
  std::vector<void*> owned_;
  std::vector<std::vector<void*>> free_;
  std::unordered_map<void*, int> cls_;
  char* slab_ = nullptr;
  size_t slab_left_ = 0;
  size_t reserved_ = 0;
};

// The ring of the resident kernel, shared by the engines of a context.
struct ResidentQueue {
  int device = 0;
  int grid = 0, num_sms = 0;
  const tci_kernel_set* ks = &tci_k256::kernels;  // the variant of the running (or last) launch
  uint32_t nslots = 0, mask = 0;
  tci_queue_slot* slots = nullptr;       // mapped pinned host memory
  tci_queue_ctl* qc = nullptr;           // mapped pinned host memory
  tci_resident_state* st_dev = nullptr;   // device memory
  std::atomic<uint64_t> tail{0};
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::mutex mu;
  bool running = false;
  double kernel_ms = 0;
  int64_t launches = 0;
  unsigned long long wait_ns = 60ull * 1000000000ull;  // a worker's longest wait for its ticket
  int init(int device, int num_sms, int idle_us);
  ~ResidentQueue();
  // launch the kernel unless it is running: the throughput variant (k256) for
  // batched and served solves, the latency variant (k512) for a single solve
  int start(const tci_kernel_set* k);
  int ensure_alive(); // relaunch it if every CTA has left (idle limit)
  int stop();         // ask the CTAs to leave once the ring is drained; wait
  int publish(const tci_task& t, uint64_t& ticket);
};

struct GpuOp {
  Engine* eng;
  std::vector<Req*> reqs;
  // Fills the value caches of caller-supplied f's first; a failure there
  // completes the operation with that status.
  bool await_ready();
  void await_suspend(std::coroutine_handle<> h);
  int await_resume() const noexcept;
  int status = 0;
};

// Device copy of one site tensor.
struct Core {
  double* p = nullptr;
  i64 d0 = 0, d1 = 0, d2 = 0;
  size_t elems() const { return (size_t)(d0 * d1 * d2); }
};
const char* last_message();

struct Solve {
  int L = 0;
  std::vector<int> d;
  int fid = 0;
  std::vector<double> params;
  std::vector<IndexSet> Iset, Jset;       // Iset[b]: length b; Jset[b]: length L-1-b
  std::vector<IndexSet> Ihist, Jhist;     // last snapshot pushed by sweep2site!
  bool has_hist = false;
  std::vector<Core> cores;
  bool cores_valid = false;
  std::vector<double> pivoterrors, bonderrors;
  double maxsample = 0.0;
  std::vector<i64> ranks, nglobal;
  std::vector<double> errors;
  i64 nfeval = 0;
  tci_rng rng;
  int lutcap0 = 0, lutcap1 = 0;  // capacities of the f tables (tci_f_tables)
  double* lut_dev = nullptr;     // the tables over the whole range (device pool), built once
  std::shared_ptr<FCache> fcache;  // caller-supplied f (fid TCI_F_CACHE)
  tci_opts opts{};
  // bookkeeping for serving
  int rc = 0;
  std::string msg;
  double t_arrival = 0, t_done = 0;
  i64 id = -1;
};

class Engine {
 public:
  explicit Engine(int device);
  ~Engine();
  int init();
  cudaStream_t stream() const { return stream_; }

  // Queue tasks for the next step and remember the coroutine to resume.
  void enqueue(std::vector<Req*>& reqs, std::coroutine_handle<> h, GpuOp* op);
  bool idle() const { return pending_.empty(); }
  // Run one batched step: pack, upload, launch, download, resume.
  int step();
  // The same split in two: launch() packs and enqueues the pending tasks on
  // the engine's stream (no-op while a batch is in flight); complete() waits
  // for it and resumes the solves.  ready(): the in-flight batch is done.
  int launch();
  int complete();
  bool ready() const;
  bool inflight() const { return inflight_; }
  // Drive a single coroutine (and any others already queued) to completion.
  // With a ring attached (attach_ring) it runs on the resident kernel, which is
  // started for the call and stopped at its end; otherwise by batched launches.
  int run(CoTask& t, bool allow_resident = true);
  void attach_ring(ResidentQueue* q, BlockPool* host_pool, BlockPool* scratch_pool) {
    att_rq_ = q;
    att_h_ = host_pool;
    att_s_ = scratch_pool;
  }

  // Resident mode: tasks go to the context's ring as soon as they are queued
  // (submit) and each solve resumes as soon as its own tasks are done (poll),
  // with no batch boundary.  The pools must outlive the engine.
  void set_resident(ResidentQueue* q, BlockPool* host_pool, BlockPool* scratch_pool);
  bool resident() const { return rq_ != nullptr; }
  int submit();
  int poll(bool& progressed);
  bool has_flights() const { return !flights_.empty(); }
  // Drop every queued and finished-but-unresumed task (after a fatal error,
  // with the device idle); their solves are not resumed.
  void abandon();
  void set_device_pool(BlockPool* p) { dpool_ = p; }

  // Device memory for site tensors (the context's device pool).
  double* alloc_core(size_t elems);
  void free_core(double* p);
  void release_cores(Solve& s);
  void release_solve(Solve& s);  // cores and the f tables: the solve is going away
  // Run a list of tasks outside any solve (rrLU entry points).  A single large
  // rrLU of a given matrix runs on the multi-CTA kernel (run_big).
  int run_tasks(std::vector<Req*>& reqs);
  int run_big(Req& r);
  // Copy many device arrays to one host buffer: gather on the device into a
  // contiguous staging buffer, then a single device-to-host copy.
  int gather_to_host(const std::vector<const double*>& src, const std::vector<int64_t>& len,
                     double* host_out);
  // The same into mapped pinned host memory, written by the gather kernel itself.
  int gather_to_pinned(const std::vector<const double*>& src, const std::vector<int64_t>& len,
                       double* pinned_out);

  tci_stats stats{};
  bool timing = true;
  const tci_kernel_set* ks_ = &tci_k256::kernels;  // the variant of the current / last batched launch
  int num_sms = 0;
  size_t hbm_budget = 0;
  // Autotuned rrLU parameter per (rows, cols) bucket: the trailing-block size
  // (elements) at which a factorization continues on one warp instead of the
  // whole CTA; 0 = the kernel's default.  Filled by tci_autotune_rrlu.
  static constexpr int TUNE_BUCKETS = 12;
  int32_t tail_table[TUNE_BUCKETS] = {0};
  static int tune_bucket(int64_t m, int64_t n) {
    const int64_t s = m < n ? m : n, l = m < n ? n : m;
    const int size = s <= 24 ? 0 : s <= 48 ? 1 : s <= 96 ? 2 : s <= 160 ? 3 : s <= 256 ? 4 : 5;
    return 2 * size + (l > 2 * s ? 1 : 0);
  }
  void apply_tuning(tci_task& t) const {
    if (t.kind == TCI_TASK_RRLU && t.tail_elems == 0) t.tail_elems = tail_table[tune_bucket(t.m, t.n)];
  }

 private:
  struct Waiter {
    std::coroutine_handle<> h;
    GpuOp* op;
    size_t first, count;
  };
  int ensure(size_t blob, size_t res, size_t work);
  void account(const Req& r, int smem_mode);
  int device_ = 0;
  // resident mode
  struct Flight {
    Waiter w;
    std::vector<Req*> reqs;
    std::vector<void*> hblocks, dblocks;
  };
  ResidentQueue* rq_ = nullptr;
  ResidentQueue* att_rq_ = nullptr;
  BlockPool *att_h_ = nullptr, *att_s_ = nullptr;
  int run_resident(CoTask& t);
  BlockPool* hpool_ = nullptr;
  BlockPool* spool_ = nullptr;  // device scratch of this engine's tasks (this thread only)
  BlockPool* dpool_ = nullptr;
  size_t res_smem_ = 0;
  int res_threads_ = 0;  // tasks are planned for this variant's budget (it fits the other one too)
  size_t plan_limit_ = SIZE_MAX;  // TCI_PLAN_SMEM
  std::vector<Flight> flights_;
  size_t inflight_tasks_ = 0;  // tasks of flights_
  std::vector<char> big_res_;  // host copy of the last multi-CTA rrLU's result record
  cudaStream_t stream_ = nullptr;
  cudaEvent_t ev0_ = nullptr, ev1_ = nullptr;
  std::vector<Req*> pending_;
  std::vector<Waiter> waiters_;
  char* hblob_ = nullptr;
  size_t hblob_cap_ = 0;
  char* dblob_ = nullptr;
  size_t dblob_cap_ = 0;
  char* hres_ = nullptr;
  size_t hres_cap_ = 0;
  char* dres_ = nullptr;
  size_t dres_cap_ = 0;
  double* dwork_ = nullptr;
  size_t dwork_cap_ = 0;
  int* dcounter_ = nullptr;
  FILE* task_log_ = nullptr;
  // gather staging
  char* hgat_ = nullptr;
  size_t hgat_cap_ = 0;
  char* dgat_ = nullptr;
  size_t dgat_cap_ = 0;
  // the batch in flight
  bool inflight_ = false;
  cudaEvent_t done_ = nullptr;
  std::vector<Req*> fl_batch_;
  std::vector<Waiter> fl_waiters_;
  size_t fl_blob_ = 0, fl_res_ = 0;
  std::vector<size_t> fl_o_res_;
  std::vector<char> fl_smem_;
};

// ------------------------------------------------------------ TCI2 algorithm
// A solve whose f is the library's own evaluator (values through the device cache).
int solve_init_evaluator(Solve& s, int L, const int64_t* localdims, std::shared_ptr<FEvaluator> ev);
int solve_init(Solve& s, int L, const int64_t* localdims, int fid, const double* params,
               int64_t nparams, const int64_t* pivots, int64_t np);
CoTask co_construct(Engine& e, Solve& s, std::vector<std::vector<uint8_t>> pivots);
CoTask co_optimize(Engine& e, Solve& s, tci_opts o);
CoTask co_crossinterpolate2(Engine& e, Solve& s, std::vector<std::vector<uint8_t>> pivots, tci_opts o);
CoTask co_updatepivots(Engine& e, Solve& s, int b, bool leftorth, double reltol, double abstol,
                       i64 maxbonddim, const IndexSet* extraI, const IndexSet* extraJ);
CoTask co_sweep2site(Engine& e, Solve& s, int niter, int iter1, double abstol, i64 maxbonddim,
                     int strategy, bool strictlynested, bool fillsite);
CoTask co_sweep1site(Engine& e, Solve& s, bool forward, double reltol, double abstol, i64 maxbonddim,
                     bool updatetensors);
CoTask co_fillsitetensors(Engine& e, Solve& s);
CoTask co_evaluate(Engine& e, Solve& s, const uint8_t* pts, i64 np, double* fout,
                   double* ttout);
// optfirstpivot (util.jl:78-108) for several starts (0-based) in lockstep;
// valf gets |f| at the final pivots.
CoTask co_optfirstpivots(Engine& e, Solve& s, std::vector<std::vector<uint8_t>>* piv, std::vector<double>* valf,
                         int maxsweep);
// estimatetrueerror (globalsearch.jl:19-96) with the solve's f and site tensors.
CoTask co_estimatetrueerror(Engine& e, Solve& s, std::vector<std::vector<uint8_t>> starts,
                            std::vector<std::pair<std::vector<uint8_t>, double>>* out);
int addglobalpivots(Solve& s, const std::vector<std::vector<uint8_t>>& pivots);
i64 solve_rank(const Solve& s);
bool convergencecriterion(const std::vector<i64>& ranks, const std::vector<double>& errors,
                          const std::vector<i64>& ngp, double tolerance, i64 maxbonddim,
                          i64 ncheckhistory, bool checkconvglobalpivot);
CoTask co_sum(Engine& e, Solve& s, double* out);

}  // namespace tci
