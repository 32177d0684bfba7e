/*
 * tci_gb300.h -- C ABI of the GB300-native TCI2 two-site sweep library
 * (libtci_gpu.so).
 *
 * Drop-in boundary for TensorCrossInterpolation.jl's TCI2 path: a Julia host
 * binds these entry points with ccall; Python tests bind them with ctypes.
 * Conventions:
 *   - multi-indices are 1-based local indices, as in the reference
 *     (MultiIndex = Vector{Int}, abstracttensortrain.jl:6-7), passed as
 *     row-major int64 arrays (one multi-index per row);
 *   - matrices and site tensors are column-major (Julia layout);
 *   - host buffers are owned by the caller; device state lives behind opaque
 *     handles owned by the library;
 *   - every entry point returns 0 or a TCI_ERR_* code; tci_last_error() gives
 *     the message of the last failure on the calling thread.  The codes map to
 *     the exceptions the reference throws (ArgumentError, DimensionMismatch,
 *     ErrorException).
 * There is no CPU fallback: without a usable CUDA device every entry point
 * that computes returns TCI_ERR_CUDA.
 */
#ifndef TCI_GB300_H
#define TCI_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Error codes. */
enum {
  TCI_OK = 0,
  TCI_ERR_ARG = 1,       /* ArgumentError (e.g. tensorci2.jl:750-754, :197-199 family) */
  TCI_ERR_DIM = 2,       /* DimensionMismatch (tensorci2.jl:197-199) */
  TCI_ERR_NAN = 3,       /* ErrorException("lu.L contains NaNs") (matrixlu.jl:164-169),
                            "NaN in tensor T[b]" (tensorci2.jl:439-441) */
  TCI_ERR_SINGULAR = 4,  /* singular pivot matrix in setsitetensor! (tensorci2.jl:391) */
  TCI_ERR_GENERIC = 5,   /* other ErrorException (e.g. "maxsamplevalue is zero!") */
  TCI_ERR_CUDA = 6,      /* CUDA runtime failure or no device */
  TCI_ERR_OOM = 7,       /* device memory budget exceeded */
  TCI_ERR_TIMEOUT = 8,   /* a bounded device wait gave up */
  TCI_ERR_TOO_LARGE = 9  /* a matrix exceeds the kernel's on-chip plan */
};

/* Registered device functions f (tci_f_lookup names). */
enum {
  TCI_F_LORENTZ = 1, /* "lorentz": coeff / (1 + sum v^2)          params [coeff]            */
  TCI_F_SERVED = 2,  /* "served" : 1/(1+a v.v) + b exp(-g|v-c|^2)  params [a, b, g, c_1..c_L] */
  TCI_F_QTT1D = 3,   /* "qtt1d"  : quantics 1-D                    params [kind]             */
  TCI_F_QTT2D = 4,   /* "qtt2d"  : quantics 2-D, d = 4             params []                 */
  TCI_F_DENSE = 5,   /* "dense"  : table lookup                    params [L, strides, data] */
  TCI_F_PRODUCT = 6  /* "product": C prod_n t[n, v_n] (integrate)  params [L, D, C, log|t|, t<0] */
};

/* Precision of evaluation, site contractions and matrix products: FP64 (the
 * fixed-order kernels, bitwise equal to the oracle) or TF32x3 -- each FP64
 * operand split into TF32 hi + lo, hi*hi + hi*lo + lo*hi on the tensor cores
 * with FP32 accumulation (about 2^-21 relative error per product term;
 * operands must lie in the FP32 range). */
enum { TCI_PREC_FP64 = 0, TCI_PREC_TF32X3 = 1 };

/* Sweep strategies (sweepstrategies.jl:1-6). */
enum { TCI_SWEEP_BACKANDFORTH = 0, TCI_SWEEP_FORWARD = 1, TCI_SWEEP_BACKWARD = 2 };

/* Keyword arguments of optimize! (tensorci2.jl:700-720).  maxbonddim <= 0
 * means typemax(Int).  `seed` seeds the host RNG that replaces
 * Random.default_rng() in DefaultGlobalPivotFinder (globalpivotfinder.jl:156). */
typedef struct tci_opts {
  double tolerance;            /* :703, default 1e-8 */
  int64_t maxbonddim;          /* :705 */
  int64_t maxiter;             /* :706, default 20 */
  int32_t sweepstrategy;       /* :707 */
  int32_t normalizeerror;      /* :711 */
  int32_t ncheckhistory;       /* :712 */
  int32_t maxnglobalpivot;     /* :714 */
  int32_t nsearchglobalpivot;  /* :715 */
  int32_t strictlynested;      /* :717 */
  int32_t checkconvglobalpivot;/* :719 */
  int32_t pad_;
  double tolmarginglobalsearch;/* :716 */
  uint64_t seed;
} tci_opts;

typedef struct tci_ctx tci_ctx;
typedef struct tci_solve tci_solve;
typedef struct tci_server tci_server;

/* Fill `o` with the reference's defaults (tensorci2.jl:700-720). */
void tci_opts_default(tci_opts* o);

/* Library / device set-up.  hbm_budget = 0: no limit beyond the device. */
int tci_ctx_create(int device, size_t hbm_budget, tci_ctx** out);
int tci_ctx_destroy(tci_ctx* ctx);
const char* tci_last_error(void);
/* Name -> id of a registered device function ("lorentz", "served", ...). */
int tci_f_lookup(const char* name, int* fid);

/* ---- Caller-supplied f ---------------------------------------------------
 * The BatchEvaluator plugin point (cachedtensortrain.jl:1, batcheval.jl:67-83)
 * for functions that are not registered on the device, with the value cache of
 * CachedFunction (cachedfunction.jl:8-184) kept in device memory.  The callback
 * fills values[k] = f(points[k, :]) for npoints multi-indices (npoints x L,
 * row-major, 1-based) and returns 0, or nonzero to make the library call that
 * asked for the values fail with TCI_ERR_GENERIC.  f must be a pure function of
 * the multi-index: each solve asks for every distinct point at most once and
 * serves repeats from its device hash table (keys are the mixed-radix number of
 * the multi-index, so prod(localdims) must stay below 2^104).  The callback runs
 * on the thread that made the library call, between device steps.
 * tci_f_register returns an id >= TCI_F_USER that the solve entry points
 * (tci_solve_create, tci_crossinterpolate2, tci_feval, tci_optfirstpivot) take
 * in place of a registered function's id; the batched and serving entry points
 * accept only registered device functions.  A finalizer run inside the callback
 * may destroy objects of the same context; entry points that compute fail with
 * TCI_ERR_GENERIC when called from inside it. */
typedef int (*tci_batch_fn)(void* user, int32_t L, int64_t npoints, const int64_t* points,
                            double* values);
#define TCI_F_USER 1024
int tci_f_register(tci_batch_fn fn, void* user, int32_t* fid);
int tci_f_unregister(int32_t fid);
/* Cache counters of a solve with a caller-supplied f: distinct points stored,
 * points passed to the callback, callback invocations. */
int tci_fcache_stats(const tci_solve* s, int64_t* entries, int64_t* evaluated, int64_t* calls);

/* ---- TensorCI2 (tensorci2.jl:6-72) ------------------------------------- */
/* TensorCI2{Float64}(f, localdims, initialpivots) (tensorci2.jl:42-53).
 * pivots: np x L row-major, 1-based. */
int tci_solve_create(tci_ctx* ctx, int32_t L, const int64_t* localdims, int32_t fid,
                     const double* fparams, int64_t nparams, const int64_t* pivots, int64_t np,
                     tci_solve** out);
int tci_solve_destroy(tci_solve* s);

/* crossinterpolate2(Float64, f, localdims, initialpivots; opts...)
 * (tensorci2.jl:943-953): constructor + optimize!. */
int tci_crossinterpolate2(tci_ctx* ctx, int32_t L, const int64_t* localdims, int32_t fid,
                          const double* fparams, int64_t nparams, const int64_t* pivots,
                          int64_t np, const tci_opts* opts, tci_solve** out);

/* optimize!(tci, f; opts...) (tensorci2.jl:700-850). */
int tci_optimize(tci_solve* s, const tci_opts* opts);

/* updatepivots!(tci, b, f, leftorthogonal; reltol, abstol, maxbonddim)
 * (tensorci2.jl:510-607), pivotsearch=:full, no extra index sets; b 1-based. */
int tci_updatepivots(tci_solve* s, int32_t b, int32_t leftorthogonal, double reltol,
                     double abstol, int64_t maxbonddim);

/* sweep2site!(tci, f, niter; iter1, abstol, maxbonddim, sweepstrategy,
 * strictlynested, fillsitetensors) (tensorci2.jl:855-916). */
int tci_sweep2site(tci_solve* s, int32_t niter, int32_t iter1, double abstol, int64_t maxbonddim,
                   int32_t sweepstrategy, int32_t strictlynested, int32_t fillsitetensors);

/* sweep1site!(tci, f, :forward/:backward; reltol, abstol, maxbonddim,
 * updatetensors) (tensorci2.jl:402-461). */
int tci_sweep1site(tci_solve* s, int32_t forward, double reltol, double abstol,
                   int64_t maxbonddim, int32_t updatetensors);

/* fillsitetensors!(tci, f) (globalsearch.jl:97-103). */
int tci_fillsitetensors(tci_solve* s);

/* addglobalpivots!(tci, pivots) (tensorci2.jl:193-213). */
int tci_addglobalpivots(tci_solve* s, const int64_t* pivots, int64_t np);

/* addglobalpivots1sitesweep!(tci, f, pivots; reltol, abstol, maxbonddim)
 * (tensorci2.jl:219-229). */
int tci_addglobalpivots1sitesweep(tci_solve* s, const int64_t* pivots, int64_t np, double reltol,
                                  double abstol, int64_t maxbonddim);

/* Accessors.  linkdims (tensorci2.jl:83-85): L-1 values. */
int tci_solve_length(const tci_solve* s, int32_t* L);
int tci_linkdims(const tci_solve* s, int64_t* out);
double tci_maxsamplevalue(const tci_solve* s);
/* Iset[b], Jset[b] for 1-based site b: I is nI x (b-1), J is nJ x (L-b), row-major,
 * 1-based.  Pass NULL arrays to query nI/nJ only. */
int tci_get_sets(const tci_solve* s, int32_t b, int64_t* I, int64_t* nI, int64_t* J, int64_t* nJ);
/* Replace Iset[b] / Jset[b] (1-based multi-indices, row-major); invalidates the
 * site tensors. */
int tci_set_sets(tci_solve* s, int32_t b, const int64_t* I, int64_t nI, const int64_t* J, int64_t nJ);
/* bonderrors (tensorci2.jl:132-139), L-1 doubles. */
int tci_bonderrors(const tci_solve* s, double* out);
/* Site tensor b (1-based), column-major r_{b-1} x d_b x r_b; dims[3] out.
 * Pass NULL `out` to query dims.  Fails if site tensors are invalidated. */
int tci_get_core(const tci_solve* s, int32_t b, double* out, int64_t* dims);
/* All site tensors of n solves in one device-to-host copy: solve i's tensors,
 * site by site (each column-major), start at out + out_offsets[i]; offsets must
 * be contiguous (offset[i+1] = offset[i] + sum of solve i's tensor sizes).
 * The TensorTrain(tci) conversion (tensortrain.jl:62-64) for a batch. */
/* The (r0, d, r1) of every site tensor of n solves, concatenated (3 * sum of
 * the lengths entries); one call instead of one tci_get_core per site. */
int tci_get_core_dims_batched(int64_t n, tci_solve* const* solves, int64_t* dims);
/* Every site tensor of n solves, concatenated in solve then site order, in a
 * pinned host buffer that the library allocates and its gather kernel writes
 * directly (no staging copy).  *total_elems doubles; the caller hands the
 * buffer back with tci_host_free (buffers are pooled and reused). */
int tci_get_cores_pinned(tci_ctx* ctx, int64_t n, tci_solve* const* solves, double** out, int64_t* total_elems);
int tci_host_free(tci_ctx* ctx, void* p);
int tci_get_cores_batched(tci_ctx* ctx, int64_t n, tci_solve* const* solves, double* out,
                          const int64_t* out_offsets);
/* pivoterrors (length *npe) and bonderrors (L-1) (tensorci2.jl:13-16). */
int tci_get_errors(const tci_solve* s, double* pivoterrors, int64_t* npe, double* bonderrors);
/* ranks, errors (normalised) and number of global pivots per iteration of the
 * last optimize! (tensorci2.jl:849). */
int tci_get_history(const tci_solve* s, int64_t* ranks, double* errors, int64_t* nglobal,
                    int64_t* niter);
/* Number of function evaluations performed on the device so far. */
int64_t tci_solve_nfeval(const tci_solve* s);

/* ---- TensorTrain (abstracttensortrain.jl:124-199) ---------------------- */
/* evaluate(tt, indexset) for np points (np x L, 1-based) of the solve's train, FP64. */
int tci_evaluate(tci_solve* s, const int64_t* points, int64_t np, double* out);
/* sum(tt) (abstracttensortrain.jl:191-199), FP64. */
int tci_sum(tci_solve* s, double* out);
/* evaluate(tt, indexset) in a precision (TCI_PREC_FP64 = tci_evaluate, or
 * TCI_PREC_TF32X3: the row vectors of 128-point tiles stay on chip as TF32
 * hi/lo and every site is a split-precision tensor-core product with FP32
 * accumulation; bonds up to 128).  *err_est (may be NULL): the largest
 * |split - fp64| / max |fp64| over the first min(np, 256) points, whose FP64
 * values are computed alongside. */
int tci_evaluate_prec(tci_solve* s, const int64_t* points, int64_t np, double* out, int32_t precision,
                      double* err_est);

/* optfirstpivot(f, localdims, firstpivot; maxsweep) (util.jl:78-108): coordinate
 * ascent of |f| from `pivot` (1-based, L entries, updated in place); each sweep
 * moves every site to the first value that raises |f|; stops when a sweep
 * changes nothing or after maxsweep sweeps (<= 0: 1000).  f is a registered
 * device function or a caller-supplied one (tci_f_register). */
int tci_optfirstpivot(tci_ctx* ctx, int32_t fid, const double* fparams, int64_t nparams, int32_t L,
                      const int64_t* localdims, int64_t* pivot, int32_t maxsweep);

/* estimatetrueerror(TensorTrain(tci), f; nsearch, initialpoints) (globalsearch.jl:1-96):
 * greedy searches for large |f - tt| with the solve's f and site tensors, from the
 * np initial points (np x L, 1-based) or, when np = 0, from nsearch random points
 * drawn from `seed`.  Writes up to cap (pivot, error) pairs, sorted by error
 * descending with repeats removed: pivots cap x L row-major 1-based; *nout is the
 * number of pairs found (may exceed cap). */
int tci_estimatetrueerror(tci_solve* s, int32_t nsearch, const int64_t* initialpoints, int64_t np, uint64_t seed,
                          int64_t cap, int64_t* pivots, double* errors, int64_t* nout);

/* Batch evaluation of a registered f at np points (np x L, 1-based) on the
 * device: the BatchEvaluator call of batcheval.jl:67-83 with M = L. */
int tci_feval(tci_ctx* ctx, int32_t fid, const double* fparams, int64_t nparams, int32_t L,
              const int64_t* localdims, const int64_t* points, int64_t np, double* out);

/* convergencecriterion (tensorci2.jl:609-628); host only, returns 1 or 0. */
int tci_convergencecriterion(const int64_t* ranks, const double* errors, const int64_t* nglobalpivots,
                             int64_t n, double tolerance, int64_t maxbonddim, int64_t ncheckhistory,
                             int32_t checkconvglobalpivot);

/* ---- batched solves and serving ---------------------------------------- */
/* One request of a batch: crossinterpolate2 with initial pivot all ones. */
typedef struct tci_request {
  int32_t L, fid;
  const int64_t* localdims;
  const double* fparams;
  int64_t nparams;
  tci_opts opts;
} tci_request;

/* Solve `n` requests together: every engine step batches the current sweep
 * stage of all live solves into one launch.  max_live caps concurrent solves
 * (0 = all).  out[i] receives solve i (caller destroys). */
int tci_crossinterpolate2_batched(tci_ctx* ctx, int64_t n, const tci_request* reqs,
                                  int64_t max_live, tci_solve** out);

/* Continuous-batching server over a request stream with arrival times
 * (seconds from start).  Requests are admitted as they arrive while live
 * solves and the HBM estimate allow (L*d^2*r_max^2 doubles per solve);
 * completed solves are released.  latency[i] = completion - arrival,
 * rank[i] = final rank.  Returns total wall seconds in *wall. */
int tci_serve_run(tci_ctx* ctx, int64_t n, const tci_request* reqs, const double* arrival,
                  int64_t max_live, double* latency, int64_t* rank, double* wall);

/* ---- rrLU (matrixlu.jl:194-225) ---------------------------------------- */
/* rrlu(A; maxrank, reltol, abstol, leftorthogonal) on a host matrix (m x n,
 * column-major; copied).  rowperm (m), colperm (n): full 1-based permutations;
 * L (m x npivot) and U (npivot x n) column-major with capacities m*min(m,n) and
 * min(m,n)*n; either may be NULL.  maxrank <= 0 means typemax(Int). */
int tci_rrlu(tci_ctx* ctx, const double* A, int64_t m, int64_t n, int64_t maxrank, double reltol,
             double abstol, int32_t leftorthogonal, int64_t* rowperm, int64_t* colperm, double* L,
             double* U, int64_t* npivot, double* error);

/* Many independent rrLUs (host buffers).  Matrix i is at A + offsets[i]
 * (column-major ms[i] x ns[i]).  Outputs: npivots[i], errors[i] and the first
 * npivot entries of the 1-based row/col pivot lists at piv + piv_offsets[i]
 * (rows then cols, 2*min(maxrank, m, n) capacity each matrix). */
int tci_rrlu_batched(tci_ctx* ctx, int64_t nmat, const double* A, const int64_t* offsets,
                     const int64_t* ms, const int64_t* ns, int64_t maxrank, double reltol,
                     double abstol, int32_t leftorthogonal, int64_t* piv, const int64_t* piv_offsets,
                     int64_t* npivots, double* errors);

/* rrlu on caller-owned device buffers, with no allocation by the library.
 * No counterpart in the reference.  It serves callers that cannot let a
 * library allocate device memory: hosts whose every device buffer comes from
 * their own allocator (a Julia GPU array pool, a framework's arena), where a
 * library's cudaMalloc would go around their accounting or fail against their
 * reservation, and latency-critical loops where a cudaMalloc/cudaFree would
 * synchronise the device.  Same arithmetic as tci_rrlu (bit-identical
 * permutations, npivot, error and factors), but all pointers are device
 * pointers: A_dev (m x n column-major, read only); rowperm_dev (m) and
 * colperm_dev (n) receive the full 0-based permutations, npivot_dev and
 * error_dev one value each, status_dev 0 or TCI_ERR_NAN when L or U holds a
 * NaN (where tci_rrlu returns TCI_ERR_NAN: the reference's ErrorException
 * "lu.L contains NaNs", matrixlu.jl:164-169), factors_dev (m x n, optional,
 * may be NULL) the factored matrix (L below the diagonal, U on and above,
 * unit diagonal implied on the side leftorthogonal selects).  Work goes to
 * `stream`; the call returns after enqueueing, so the outputs, status_dev
 * included, are valid once the stream has reached them.
 * Limits: 1 <= m, n <= 16384 and m*n <= 524288 (larger sizes return
 * TCI_ERR_ARG).  The working storage is one fixed device array of the library
 * (about 8.6 MB on every GPU that loads it, kept until the process exits),
 * shared by all calls: calls that overlap on the GPU race on it, calls on one
 * stream are ordered.  Every element a call reads from that array is written
 * earlier in the same call.  The first call on a device looks up that array's
 * device address and sets the kernel's shared-memory limit with the device
 * current; make it before any stream capture.  The address is kept per device
 * for the life of the process: a device reset after the first call is not
 * supported.  A CUDA error already pending on the calling thread makes the
 * call return TCI_ERR_CUDA without launching and without clearing it. */
int tci_rrlu_noalloc(const double* A_dev, int64_t m, int64_t n, int64_t maxrank, double reltol,
                     double abstol, int32_t leftorthogonal, int32_t* rowperm_dev, int32_t* colperm_dev,
                     int32_t* npivot_dev, double* error_dev, int32_t* status_dev, double* factors_dev,
                     uintptr_t stream);

/* ---- autotuner (no reference counterpart) -------------------------------
 * The rank-revealing LU of a step-kernel task runs on the whole CTA until its
 * trailing block has at most T elements and finishes on one warp (no CTA
 * barriers per pivot).  tci_autotune_rrlu picks T per (rows, cols) bucket
 * (12 buckets: the smaller dimension in <= 24, <= 48, <= 96, <= 160, <= 256,
 * > 256, times square-ish or more than 2:1) by timing the candidates
 * {1, 96, 192, 384, 768, 1536} with CUDA events around the step kernel on a
 * seeded set of each bucket: about three matrices per CTA (at most 24 M
 * elements), half low rank (U diag(10^(-k/4)) V^T + 1e-12 noise) and half
 * graded full rank (pivots reaching reltol 1e-10 near 0.9 min(m, n)), one
 * warm-up launch, then reps launches per candidate, interleaved.  A candidate
 * replaces the default (T = 192) only if it is 2 % faster on that set and again
 * on a fresh validation set of the bucket; every later rrLU and TCI task of the
 * context uses the table.  *speedup = the sum of the default's times over the
 * sum of the chosen ones (validation times where the choice changed);
 * ms_default / ms_tuned those sums (any may be NULL).  Pivots do not depend
 * on T. */
int tci_autotune_rrlu(tci_ctx* ctx, int32_t reps, double* speedup, double* ms_default, double* ms_tuned);
/* Read (set = 0) or write (set = 1) the tuned table: nbuckets entries (0 = the
 * kernel's default); *nbuckets receives the count (pass table = NULL to query). */
int tci_autotune_table(tci_ctx* ctx, int32_t* table, int32_t* nbuckets, int32_t set);

/* ---- context utilities --------------------------------------------------- */
/* cudaStream_t of the context, as an integer. */
uintptr_t tci_ctx_stream(tci_ctx* ctx);
int tci_ctx_synchronize(tci_ctx* ctx);
/* Engine counters since the last reset: steps, kernel launches, tasks, kernel
 * milliseconds (CUDA events around each step kernel on the context stream),
 * function evaluations and rank-1 update elements. */
typedef struct tci_stats {
  int64_t steps, launches, tasks;
  double kernel_ms;
  int64_t feval, lu_updates;
  int64_t h2d_bytes, d2h_bytes;
  /* host milliseconds spent packing/launching steps, waiting for them, and
   * resuming the solves after them (summed over the engines' threads) */
  double host_launch_ms, host_wait_ms, host_resume_ms;
  /* SM clock cycles spent inside tasks, summed over all tasks (each task runs
   * on one CTA; one or two task CTAs per SM): divided by task CTAs x clock x
   * wall time it gives the fraction of the task slots kept busy */
  int64_t task_cycles;
  /* elements of feval computed from tables of the factored f parts (one FP64
   * operation each) rather than by evaluating f */
  int64_t feval_tabulated;
  /* split-precision tensor-core work: device milliseconds of its kernels
   * (CUDA events; operand packing included) and the product FLOPs they did,
   * counted as 2 M N K per split product (each one is 3 tensor-core products) */
  double tc_ms, tc_flops;
  /* most solves live at once in a batched or serving run (admission by the
   * live cap and the HBM budget) */
  int64_t peak_live;
  /* FP64 multiply-add (or multiply-subtract) pairs outside the rank-1 updates:
   * the triangular solves of setsitetensor! (m r (r - 1) per SITE task) and the
   * train contractions of the global pivot search and of evaluate */
  int64_t dense_macs;
} tci_stats;
int tci_ctx_stats(tci_ctx* ctx, tci_stats* out, int32_t reset);
/* Bounds of the resident kernel's waits (no reference counterpart): it leaves
 * after idle_us with nothing published (default 20000; the host relaunches it
 * on demand), and a worker CTA waits at most wait_us for its task ticket
 * (default 60 s); a wait that runs out stops the kernel and the call in
 * progress returns TCI_ERR_TIMEOUT.  Tasks of that call that were published
 * but not run are abandoned: after TCI_ERR_TIMEOUT destroy the context.  Takes
 * effect at the next launch of the kernel. */
int tci_ctx_set_resident_limits(tci_ctx* ctx, int32_t idle_us, int64_t wait_us);

/* evaluate / sum (abstracttensortrain.jl:124-199) of a tensor train the caller
 * gives: cores[b] is r0 x d x r1 column-major, dims[3*b + 0..2] its sizes;
 * points np x L, 1-based, row-major. */
int tci_tt_evaluate(tci_ctx* ctx, int32_t L, const int64_t* dims, const double* const* cores, const int64_t* points,
                    int64_t np, double* out);
int tci_tt_sum(tci_ctx* ctx, int32_t L, const int64_t* dims, const double* const* cores, double* out);
/* tci_tt_evaluate in a precision, as tci_evaluate_prec. */
int tci_tt_evaluate_prec(tci_ctx* ctx, int32_t L, const int64_t* dims, const double* const* cores,
                         const int64_t* points, int64_t np, double* out, int32_t precision, double* err_est);

/* ---- incremental server: requests are submitted one at a time while the
 * context serves them with continuous batching (host threads + the resident
 * kernel); completed requests are polled.  The server owns the context until
 * tci_serve_stop returns (other calls on the context wait). */
typedef struct tci_server tci_server;
int tci_serve_start(tci_ctx* ctx, int64_t max_live, tci_server** out);
/* Copies the request's arrays; *id = 0, 1, 2, ... in submission order. */
int tci_serve_submit(tci_server* s, const tci_request* req, int64_t* id);
/* Up to cap completed requests since the last poll (waits up to timeout_ms
 * for the first): id, status (0 or a TCI_ERR_* code), rank (max bond
 * dimension, -1 on error), latency from submit to completion in seconds. */
int tci_serve_poll(tci_server* s, int64_t cap, int64_t* ids, int32_t* status, int64_t* ranks, double* latency,
                   int64_t* n, int32_t timeout_ms);
/* Finishes every submitted request, then stops; results not polled are dropped. */
int tci_serve_stop(tci_server* s);

/* ---- tensor trains with 4-leg cores (link, s_in, s_out, link'), column-major,
 * and their contraction (contraction.jl) and recompression (tensortrain.jl).
 * dims[4*b + q] is the size of leg q of core b; cores[b] points to its values.
 * Results stay on the device behind a tci_tt4 handle. */
typedef struct tci_tt4 tci_tt4;
enum { TCI_CONTRACT_NAIVE = 1, TCI_CONTRACT_ZIPUP = 2 };
/* Factorization of _factorize (tensortrain.jl:94-137): rrlu's left/right, or
 * MatrixLUCI's (matrixluci.jl:40-84). */
enum { TCI_FACTORIZE_LU = 0, TCI_FACTORIZE_CI = 1 };
/* contract(A, B; algorithm, tolerance, maxbonddim) (contraction.jl:515-560) for
 * algorithm = :naive (contract_naive, :351-372) and :zipup (contract_zipup,
 * :442-486) with method = :LU or :CI.  A's s_out leg contracts with B's s_in leg.
 * Deviations from the reference, which factorizes with LinearAlgebra.svd by
 * default: :naive with tolerance > 0 or maxbonddim > 0 recompresses with
 * compress!(method), and :zipup factorizes with rrlu / MatrixLUCI
 * (leftorthogonal = false, reltol = tolerance); method = :SVD is not on the
 * device.  maxbonddim <= 0 means typemax(Int).  Errors as the reference:
 * different lengths -> TCI_ERR_ARG, unmatched site index -> TCI_ERR_GENERIC. */
int tci_tt4_contract(tci_ctx* ctx, int32_t L, const int64_t* a_dims, const double* const* a_cores,
                     const int64_t* b_dims, const double* const* b_cores, int32_t algorithm, int32_t method,
                     double tolerance, int64_t maxbonddim, tci_tt4** out);
/* compress!(tt, method; tolerance, maxbonddim, normalizeerror) (tensortrain.jl:149-183)
 * with method = :LU or :CI. */
int tci_tt4_compress(tci_ctx* ctx, int32_t L, const int64_t* dims, const double* const* cores, int32_t method,
                     double tolerance, int64_t maxbonddim, int32_t normalizeerror, tci_tt4** out);
/* contract(A, B; algorithm = :TCI, tolerance, maxbonddim, f, initialpivots, kwargs...)
 * (contraction.jl:399-434, 515-545): crossinterpolate2 of the Contraction evaluator
 * (contraction.jl:5-62, 103-335), which runs on the device with its left/right
 * environment caches; f values are cached per point.  Local indices of the
 * interpolated function fuse A's s_in and B's s_out (A's fastest, at most 256).
 * initialpivots: np x L fused, 1-based; np = 0 draws ninitialpivots random starts
 * from opts->seed and improves each with optfirstpivot (util.jl:78-108).  f, if
 * not NULL, maps values in place (values[k] = f(values[k])).  opts carries the
 * crossinterpolate2 keywords (tolerance, maxbonddim, ...).  Errors as the
 * reference: different lengths or site dimensions -> TCI_ERR_ARG, no pivot with
 * a nonzero value -> TCI_ERR_GENERIC. */
typedef int (*tci_value_fn)(void* user, int64_t n, double* values);
int tci_tt4_contract_tci(tci_ctx* ctx, int32_t L, const int64_t* a_dims, const double* const* a_cores,
                         const int64_t* b_dims, const double* const* b_cores, const int64_t* initialpivots,
                         int64_t np, int32_t ninitialpivots, tci_value_fn f, void* user, const tci_opts* opts,
                         tci_tt4** out);
/* tci_tt4_contract with a precision: TCI_PREC_TF32X3 (algorithm = :zipup)
 * runs both site contractions of contract_zipup (contraction.jl:458-469) as
 * split-precision tensor-core products; the rank-revealing factorizations stay
 * FP64.  *err_est (may be NULL) receives the largest relative error of any of
 * those products against FP64, measured at sampled entries
 * (max |C - C_fp64| / max |C_fp64|). */
int tci_tt4_contract_prec(tci_ctx* ctx, int32_t L, const int64_t* a_dims, const double* const* a_cores,
                          const int64_t* b_dims, const double* const* b_cores, int32_t algorithm, int32_t method,
                          double tolerance, int64_t maxbonddim, int32_t precision, double* err_est, tci_tt4** out);
/* C = A * B for host column-major A (M x K), B (K x N), C (M x N) -- the
 * Matrix product of contraction.jl:92 -- in the given precision; *err_est as
 * above (0 for FP64). */
int tci_matmul(tci_ctx* ctx, int64_t M, int64_t N, int64_t K, const double* A, const double* B, double* C,
               int32_t precision, double* err_est);
int32_t tci_tt4_length(const tci_tt4* t);
int tci_tt4_dims(const tci_tt4* t, int64_t* dims);
int tci_tt4_get_core(const tci_tt4* t, int32_t b, double* out); /* b is 1-based */
int tci_tt4_destroy(tci_tt4* t);

/* Measured FP64 throughput of the current device (operations per second) for
 * separate multiply+subtract and for fused multiply-add; the roofline
 * denominator of the FP64-bound kernels.  No reference counterpart. */
int tci_fp64_peak(uintptr_t stream, double* ops_separate, double* ops_fused);

#ifdef __cplusplus
}
#endif
#endif /* TCI_GB300_H */
