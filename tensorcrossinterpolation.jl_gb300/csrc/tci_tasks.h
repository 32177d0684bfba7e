// Task records shared by the host engine and the step kernel.
//
// One engine step uploads a blob [tci_task array | params | uint8 index lists |
// core tables | input matrices] and one result area.  The step kernel pulls
// tasks from an atomic queue, one CTA per task, and writes one result record
// per task.  All offsets are byte offsets from the start of the blob (inputs)
// or of the result area (outputs).
#pragma once
#include <stdint.h>

enum {
  TCI_TASK_RRLU = 1,  // Pi = f(rows x cols) or a given matrix -> full-pivot rrLU
  TCI_TASK_SITE = 2,  // setsitetensor!(tci, f, b): T = Pi1 * inv(P)
  TCI_TASK_CORE = 3,  // core = Pi1 (last site of fillsitetensors!/sweep1site!)
  TCI_TASK_EVAL = 4,  // f and the tensor train at a list of points
  TCI_TASK_SUM = 5,   // sum of the tensor train over all sites
  TCI_TASK_SEARCH = 6 // line scans of the global pivot search from one start point
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
  int32_t smem_mode;           // 1: matrix held in shared memory
  int32_t kcap;                // pivot capacity of the result record
  double* lut;                 // scratch for tabulated f parts (lutcap0 + lutcap1 doubles)
  int32_t lutcap0, lutcap1;    // table capacities (0: evaluate f directly)
} tci_task;

// Result record: fixed header followed by per-task arrays.
typedef struct tci_result_head {
  int32_t status, npivot;
  double error;
  double maxabs;      // max |value| over the filled matrix (updatemaxsample!)
  int32_t maxabs_nan, lut_used;
  int64_t cycles;     // SM clock cycles the CTA spent on the task
} tci_result_head;
// RRLU/SITE: head, int32 rowperm[kcap], int32 colperm[kcap], double diag[kcap]
//            (each array padded to 8 bytes)
// EVAL: head, double f[m], double tt[m]
// SEARCH: head, double f[m], double tt[m], m = sum of the local dimensions; item
//         (p, v) (site-major) is the start point with site p set to v
// SUM : head with the sum in `error`

#define TCI_STEP_THREADS 512
