// Task records shared by the host engine and the step kernel.
//
// Batch mode: one engine step uploads a blob [tci_task array | params | uint8
// index lists | core tables | input matrices] and one result area.  The step
// kernel pulls tasks from an atomic queue, one CTA per task, and writes one
// result record per task.  All offsets are byte offsets from the start of the
// blob (inputs) or of the result area (outputs).
//
// Resident mode: host threads publish tasks into a ring of tci_queue_slot in
// mapped pinned host memory while the resident kernel runs.  One warp of the
// kernel (the dispatcher) moves published descriptors into a ring in device
// memory; the other CTAs claim device tickets with one atomic each, read the
// task inputs from host memory and write the result record there, then set the
// record's `done` word.  The offsets are then absolute addresses (the base
// pointers passed to the kernel are zero).
#pragma once
#include <stddef.h>
#include <stdint.h>

enum {
  TCI_TASK_RRLU = 1,  // Pi = f(rows x cols) or a given matrix -> full-pivot rrLU
  TCI_TASK_SITE = 2,  // setsitetensor!(tci, f, b): T = Pi1 * inv(P)
  TCI_TASK_CORE = 3,  // core = Pi1 (last site of fillsitetensors!/sweep1site!)
  TCI_TASK_EVAL = 4,  // f and the tensor train at a list of points
  TCI_TASK_SUM = 5,   // sum of the tensor train over all sites
  TCI_TASK_SEARCH = 6, // line scans of the global pivot search from one start point
  TCI_TASK_TABLE = 7   // a solve's f parts tabulated over the whole range of its integer sums
};

enum {
  TCI_POST_NONE = 0,   // pivots, pivot errors, error only
  TCI_POST_LEFT = 1,   // + left(MatrixLUCI) (colstimespivotinv or colmatrix) into core_out
  TCI_POST_RIGHT = 2,  // + right(MatrixLUCI) (rowmatrix or pivotinvtimesrows) into core_out
  TCI_POST_FACTORS = 3 // + the factored m x n matrix (L below, U on/above the diagonal)
};

enum {
  TCI_ST_NAN = 1,        // NaN in L or U (matrixlu.jl:164-169) or in a site tensor
  TCI_ST_TOO_LARGE = 2,  // task does not fit the kernel's shared-memory plan
  TCI_ST_SINGULAR = 4,   // exact zero pivot in the pivot-matrix solve
};

typedef struct tci_core_ref {
  const double* p;  // column-major r0 x d x r1
  int32_t r0, d, r1, pad;
} tci_core_ref;

typedef struct tci_task {
  int32_t kind, fid, nparams, L;
  int32_t m, n;          // matrix rows / cols (EVAL: m = number of points)
  int32_t nl, nr;        // lengths of the row / column multi-indices
  int32_t maxrank, leftorth, post, r;  // r: size of the pivot matrix P for SITE
  double reltol, abstol;
  int64_t rows, cols, prows;  // uint8 0-based multi-index lists (row-major)
  int64_t params;             // double parameters of f
  int64_t res;                // result record
  int64_t cores;              // EVAL: tci_core_ref[L]
  const double* ain;          // RRLU: input matrix (column-major, lda = m) instead of f
  double* core_out;           // LEFT/RIGHT/FACTORS, SITE and CORE output
  double* work;               // global scratch (matrix too large for shared memory)
  int64_t cost;               // scheduling weight
  int32_t smem_mode;           // 1: matrix held in shared memory; 0: matrix in `work`; 2: matrix
                               // and the row / column f states in `work` (tci_work_elems)
  int32_t kcap;                // pivot capacity of the result record
  double* lut;                 // scratch for tabulated f parts (lutcap0 + lutcap1 doubles)
  int32_t lutcap0, lutcap1;    // table capacities (0: evaluate f directly)
  uint64_t ticket;             // resident mode: host-ring ticket (the record's done word = ticket + 1)
  int32_t lut_full;            // lut holds the solve's tables over the whole range (no per-task build)
  int32_t lut_base0;           // the integer sum at table0[0] (table1 starts at 0)
  int32_t tail_elems;          // RRLU: trailing blocks of at most this many elements finish on one
                               // warp (0: the kernel's default); set from the autotuned table
  int32_t stage_bytes;         // resident mode: the first stage_bytes of the task's host record (its
                               // inputs, starting at params) are copied to the top of shared memory
                               // before the task runs (0: read in place)
} tci_task;

// Doubles of global scratch a planned task uses at `work` (its f tables follow).
#ifdef __CUDACC__
__host__ __device__
#endif
static inline size_t tci_work_elems(const tci_task* t) {
  const size_t m = (size_t)t->m, n = (size_t)t->n, r = (size_t)t->r;
  if (t->smem_mode == 1) return 0;
  if (t->kind == TCI_TASK_RRLU) return m * n + (t->smem_mode == 2 ? 2 * (m + n) : 0);
  if (t->kind == TCI_TASK_SITE) return r * r + (t->smem_mode == 2 ? 2 * m : 0);
  return 0;
}

// Result record: fixed header followed by per-task arrays.
typedef struct tci_result_head {
  int32_t status, npivot;
  double error;
  double maxabs;      // max |value| over the filled matrix (updatemaxsample!)
  int32_t maxabs_nan, lut_used;
  int64_t cycles;     // SM clock cycles the CTA spent on the task
  uint64_t done;      // resident mode: ticket + 1 once the record is complete
} tci_result_head;
// RRLU/SITE: head, int32 rowperm[kcap], int32 colperm[kcap], double diag[kcap]
//            (each array padded to 8 bytes)
// EVAL: head, double f[m], double tt[m]
// SEARCH: head, double f[m], double tt[m], m = sum of the local dimensions; item
//         (p, v) (site-major) is the start point with site p set to v
// SUM : head with the sum in `error`

// One ring slot of the resident queue.  seq = ticket + 1 once the host has
// written `t` for that ticket; taken = ticket + 1 once a CTA has copied `t` out
// (the slot may then be reused for ticket + ring size).
typedef struct tci_queue_slot {
  tci_task t;
  uint64_t seq;
  uint64_t taken;
} tci_queue_slot;

// Control words of the resident kernel (mapped pinned host memory).
typedef struct tci_queue_ctl {
  int32_t stop;        // host sets 1: the kernel leaves once every published task is dispatched
  int32_t idle_us;     // the kernel leaves after this long with nothing published
  int32_t pad[2];
} tci_queue_ctl;

// Device-memory state of the resident kernel.  host_pos persists across
// launches; everything from `count` on is cleared before every launch.
#define TCI_DRING 4096
typedef struct tci_resident_state {
  unsigned long long host_pos;  // next host-ring ticket to dispatch
  unsigned long long pad0[15];
  unsigned long long count;     // device tickets dispatched in this launch
  unsigned long long pad1[15];
  unsigned long long head;      // device tickets claimed in this launch
  unsigned long long pad2[15];
  int32_t stop;                 // dispatcher has left: no ticket beyond `count` will come
  int32_t error;                // a worker's wait hit its limit
  int32_t pad3[30];
  tci_queue_slot ring[TCI_DRING];
} tci_resident_state;

// EVAL tasks whose bonds are at most this run one thread per point, the running
// vector in 2 x TCI_EVAL_THREAD_RMAX x (task CTA threads) doubles of shared memory.
#define TCI_EVAL_THREAD_RMAX 16
