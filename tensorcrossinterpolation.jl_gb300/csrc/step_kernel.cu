// The TCI2 sweep step kernel (sm_103a): batched evaluation of f over Pi,
// full-pivot rank-revealing LU, and the per-bond post-processing, fused so that
// a Pi matrix that fits in shared memory never leaves the SM.
//
// One CTA takes one task at a time from an atomic queue (tasks are ordered
// largest first on the host).  Task kinds (tci_tasks.h):
//   RRLU : Pi[i,j] = f(rows[i] ++ cols[j]) (filltensor, tensorci2.jl:290-312,
//          batcheval.jl:32-61) or a given matrix, then rrLU exactly as
//          _optimizerrlu!/addpivot! (matrixlu.jl:98-181), then optionally
//          left/right of MatrixLUCI (matrixluci.jl:40-84).
//   SITE : setsitetensor!(tci, f, b) (tensorci2.jl:367-394): the pivot matrix P
//          is factored with partial pivoting in LAPACK's order and
//          T = Pi1 * inv(P) is solved row by row.
//   CORE : core = Pi1 (tensorci2.jl:379-383, :449-459).
//   EVAL : f and the tensor train at points (globalpivotfinder.jl:167-177,
//          abstracttensortrain.jl:124-132).
//
// Bit-exactness of the pivots: the rank-1 update is a separate IEEE multiply and
// subtract (__dmul_rn/__dsub_rn, as the reference's loop at matrixlu.jl:128-134
// is compiled without FMA), scaling is an IEEE division (matrixlu.jl:119-123),
// and the argmax compares abs2 = v*v with strict '>' and breaks ties towards the
// first element in column-major order of the physically permuted matrix
// (matrixlu.jl:16-31).  The comparison of v*v is skipped for elements whose |v|
// is more than 16 ulps below the running maximum, where v*v is provably smaller.
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <limits.h>
#include <stddef.h>
#include <stdint.h>

#include "kernels.h"
#include "tci_functions.h"
#include "tci_tasks.h"

// The variant this translation unit builds (kernels.h): the threads of one task
// CTA and the task CTAs per SM, and the namespace of its kernels and launchers.
#ifndef TCI_KNS
#define TCI_KNS tci_k256
#define TCI_STEP_THREADS 256
#define TCI_CTAS_PER_SM 2
#endif

// Optional per-phase timing hook (defined by an instrumented build; no-op here).
#ifndef TCI_PHASE
#define TCI_PHASE(id) ((void)0)
#endif

namespace TCI_KNS {
namespace {

constexpr int NT = TCI_STEP_THREADS;
constexpr int NW = NT / 32;
constexpr unsigned FULL = 0xffffffffu;
constexpr uint64_t NAN_FLOOR = 0x7ff0000000000000ULL;  // bits above this are NaN
constexpr uint64_t SQ_SMALL = (uint64_t)(1023 - 500) << 52;  // below: squares may be subnormal
constexpr uint64_t SQ_BIG = (uint64_t)(1023 + 500) << 52;    // above: squares may overflow

template <int W>
struct CtlT {
  int task;
  int r, c, K, stop, kmax, need_exact, bar_err;
  int status;
  double piv, maxerror, err;
  double red_s[W + 1];
  int red_k[W + 1];
  unsigned long long red_u[W + 1];
  unsigned long long red_b[W + 1];
  unsigned red_p[W + 1];
  long long red4[4][W + 1];
};
using Ctl = CtlT<NW>;
// The multi-CTA rrLU runs one 512-thread CTA per SM whatever the task CTAs are.
constexpr int BIG_NT = 512;
constexpr int BIG_NW = BIG_NT / 32;
using BigCtl = CtlT<BIG_NW>;

__device__ __forceinline__ double jmax(double a, double b) {
  if (a != a || b != b) return __longlong_as_double(0x7ff8000000000000LL);
  return a > b ? a : b;
}

// Bit pattern of |v| computed on the integer pipe.  Written as a register move
// plus integer AND so that it cannot be lowered to an FP64 absolute-value
// instruction: on this GPU the FP64 pipe is 1/64 of the FP32 rate and is the
// bottleneck of the rank-1 update.
__device__ __forceinline__ uint64_t abs_bits(double v) {
  unsigned lo, hi;
  asm("mov.b64 {%0, %1}, %2;" : "=r"(lo), "=r"(hi) : "d"(v));
  return ((uint64_t)(hi & 0x7fffffffu) << 32) | (uint64_t)lo;
}
// v is NaN, tested on the integer pipe (an FP64 self-comparison would take the
// slow FP64 pipe).
__device__ __forceinline__ bool is_nan_bits(double v) { return abs_bits(v) > 0x7ff0000000000000ULL; }

// Argmax of abs2 with first-in-column-major tie breaking, without squaring on
// the FP64 pipe in the common case: while updating, each thread tracks the
// largest |v| bit pattern, its first key and the next smaller pattern (integer
// ops, NaN excluded); one block reduction gives the winner unless another
// element lies within 16 ulps of the largest |v| (where v*v can tie with the
// largest square) or the magnitude is below 2^-500 or above 2^500 (squares can
// underflow or overflow).  Then a read-only pass squares the elements near the
// maximum and picks the largest square, ties to the smallest key.
// Element keys are (column << 16) | row: ordered like the column-major position
// (matrices have at most 65535 rows and columns).
__device__ __forceinline__ uint32_t pack_key(int i, int j) { return ((uint32_t)j << 16) | (uint32_t)i; }

// One thread's running argmax of |v| in key order, integer pipe only: A = the
// largest |v| bit pattern + 1, k = its first key, B = the largest bit pattern
// + 1 below A (0 = none).  NaN never wins (the reference's scan starts from
// typemin and compares with '>').
struct ArgTrack {
  uint64_t A, B;
  uint32_t k;
  __device__ __forceinline__ void init() {
    A = B = 0;
    k = 0xffffffffu;
  }
  __device__ __forceinline__ void push(double v, uint32_t key) {
    uint64_t b = abs_bits(v);
    if (b > NAN_FLOOR) return;
    b += 1;
    if (b > A) {
      B = A;
      A = b;
      k = key;
    } else if (b < A && b > B) {
      B = b;
    }
  }
};
__device__ __forceinline__ void track_combine(uint64_t& A, uint32_t& k, uint64_t& B, uint64_t A2, uint32_t k2,
                                              uint64_t B2) {
  if (A2 > A) {
    B = B2 > A ? B2 : A;
    A = A2;
    k = k2;
  } else if (A2 == A) {
    B = B2 > B ? B2 : B;
    k = k2 < k ? k2 : k;
  } else if (A2 > B) {
    B = A2;
  }
}

// Warp-wide versions with the hardware reductions (redux.sync) instead of a
// shuffle tree; every lane gets the result.  warp_track gives what folding
// track_combine over the lanes gives in any order: the largest A, the smallest
// key among the lanes that hold it, and B = the largest value below A held
// anywhere (a lane below the maximum offers its A, a lane at it its B).
__device__ __forceinline__ uint64_t warp_max_u64(uint64_t x) {
  const unsigned hi = __reduce_max_sync(FULL, (unsigned)(x >> 32));
  const unsigned lo = __reduce_max_sync(FULL, (unsigned)(x >> 32) == hi ? (unsigned)x : 0u);
  return ((uint64_t)hi << 32) | lo;
}
__device__ __forceinline__ void warp_track(uint64_t& A, uint32_t& k, uint64_t& B) {
  const uint64_t Am = warp_max_u64(A);
  const uint32_t km = __reduce_min_sync(FULL, A == Am ? k : 0xffffffffu);
  B = warp_max_u64(A == Am ? B : A);
  A = Am;
  k = km;
}
// The largest s and the smallest key among the lanes that hold it.
__device__ __forceinline__ void warp_best(uint64_t& s, uint32_t& key) {
  const uint64_t sm = warp_max_u64(s);
  key = __reduce_min_sync(FULL, s == sm ? key : 0xffffffffu);
  s = sm;
}

// Exact candidate of the second pass: abs2 = v*v (never NaN here, >= +0), so
// its bit pattern orders like its value; ties go to the smaller key.
struct ArgBest {
  uint64_t s;  // abs2 bits + 1, 0 = none
  uint32_t key;
  double val;  // the element at key
  __device__ __forceinline__ void init() {
    s = 0;
    key = 0xffffffffu;
    val = 0.0;
  }
  __device__ __forceinline__ void consider(double v, uint32_t k) {
    const uint64_t q = (uint64_t)__double_as_longlong(__dmul_rn(v, v)) + 1;
    if (q > s || (q == s && k < key)) {
      s = q;
      key = k;
      val = v;
    }
  }
};
__device__ __forceinline__ bool near_max(uint64_t b, uint64_t Mstar) {
  return b <= NAN_FLOOR && (b + 16 >= Mstar || Mstar < SQ_SMALL || Mstar >= SQ_BIG);
}

// Block-wide exact argmax; every thread gets (abs2 bits + 1, key).  Ends with a barrier.
__device__ void block_argmax(const ArgBest& a, Ctl& ctl, uint64_t& out_s, uint32_t& out_key) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint64_t s = a.s;
  uint32_t key = a.key;
  warp_best(s, key);
  if (lane == 0) {
    ctl.red_u[warp] = s;
    ctl.red_k[warp] = (int)key;
  }
  __syncthreads();
  if (warp == 0) {
    s = lane < NW ? ctl.red_u[lane] : 0ULL;
    key = lane < NW ? (uint32_t)ctl.red_k[lane] : 0xffffffffu;
    warp_best(s, key);
    if (lane == 0) {
      ctl.red_u[NW] = s;
      ctl.red_k[NW] = (int)key;
    }
  }
  __syncthreads();
  out_s = ctl.red_u[NW];
  out_key = (uint32_t)ctl.red_k[NW];
  __syncthreads();
}

// Block-wide max of unsigned 64-bit values (|v| bit patterns: NaN sorts above Inf).
__device__ unsigned long long block_max_u64(unsigned long long v, Ctl& ctl) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    unsigned long long o = __shfl_down_sync(FULL, v, off);
    v = o > v ? o : v;
  }
  if (lane == 0) ctl.red_u[warp] = v;
  __syncthreads();
  if (warp == 0) {
    v = lane < NW ? ctl.red_u[lane] : 0ULL;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      unsigned long long o = __shfl_down_sync(FULL, v, off);
      v = o > v ? o : v;
    }
    if (lane == 0) ctl.red_u[NW] = v;
  }
  __syncthreads();
  unsigned long long r = ctl.red_u[NW];
  __syncthreads();
  return r;
}


// Second argmax pass over the block A[r0:r0+rows, c0:c0+cols]: squares only
// the elements near the largest |v| (Mstar).  Every thread gets the result;
// s == 0 means no element qualified (all NaN).
__device__ void exact_argmax(const double* A, int lda, int r0, int rows, int c0, int cols, uint64_t Mstar,
                             Ctl& ctl, uint64_t& s, uint32_t& key) {
  ArgBest ab;
  ab.init();
  if (rows > 0 && cols > 0) {
    const long long total = (long long)rows * cols;
    const int sq = NT / rows, sr = NT % rows;
    int jj = threadIdx.x / rows, ii = threadIdx.x % rows;
    for (long long e = threadIdx.x; e < total; e += NT) {
      const int i = r0 + ii, j = c0 + jj;
      const double v = A[i + (size_t)j * lda];
      if (near_max(abs_bits(v), Mstar)) ab.consider(v, pack_key(i, j));
      ii += sr;
      jj += sq;
      if (ii >= rows) {
        ii -= rows;
        jj += 1;
      }
    }
  }
  block_argmax(ab, ctl, s, key);
}

// The pivot of the next step (submatrixargmax of abs2, matrixlu.jl:1-32) from
// every thread's ArgTrack over the block A[r0:, c0:]; sets ctl.r / ctl.c and
// ends with a barrier.  One integer reduction decides it unless some element
// other than the largest |v| lies within 16 ulps of it (its square could tie)
// or the magnitude is where squares underflow or overflow; then the exact
// second pass runs.  `decide` runs on the one thread that sets ctl.r / ctl.c,
// before the final barrier (the next pivot's decision without a barrier of its own).
struct NoDecide {
  __device__ void operator()() const {}
};
template <class Decide = NoDecide>
__device__ void argmax_resolve(const ArgTrack& t, const double* A, int lda, int r0, int rows, int c0, int cols,
                               Ctl& ctl, const Decide& decide = Decide()) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint64_t a = t.A, b = t.B;
  uint32_t k = t.k;
  warp_track(a, k, b);
  if (lane == 0) {
    ctl.red_u[warp] = a;
    ctl.red_b[warp] = b;
    ctl.red_k[warp] = (int)k;
  }
  __syncthreads();
  if (warp == 0) {
    a = lane < NW ? ctl.red_u[lane] : 0ULL;
    b = lane < NW ? ctl.red_b[lane] : 0ULL;
    k = lane < NW ? (uint32_t)ctl.red_k[lane] : 0xffffffffu;
    warp_track(a, k, b);
    if (lane == 0) {
      const uint64_t Mstar = a ? a - 1 : 0;
      const bool safe = Mstar >= SQ_SMALL && Mstar < SQ_BIG;
      const bool close = b != 0 && (b - 1) + 16 >= Mstar;
      if (a == 0) {  // every element NaN: the scan keeps its start
        ctl.r = r0;
        ctl.c = c0;
        ctl.need_exact = 0;
        decide();
      } else if (safe && !close) {
        ctl.r = (int)(k & 0xffffu);
        ctl.c = (int)(k >> 16);
        ctl.need_exact = 0;
        decide();
      } else {
        ctl.need_exact = 1;
      }
      ctl.red_u[NW] = Mstar;
    }
  }
  __syncthreads();
  if (ctl.need_exact) {
    const uint64_t Mstar = ctl.red_u[NW];
    uint64_t s;
    uint32_t key;
    exact_argmax(A, lda, r0, rows, c0, cols, Mstar, ctl, s, key);
    if (threadIdx.x == 0) {
      ctl.r = s ? (int)(key & 0xffffu) : r0;
      ctl.c = s ? (int)(key >> 16) : c0;
      decide();
    }
    __syncthreads();
  }
}

__device__ int block_or(int v, Ctl& ctl) {
  int r = __syncthreads_or(v);
  return r;
}

__device__ __forceinline__ size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// base + offset as integer arithmetic: in resident mode the base is zero and
// the offsets are absolute addresses.
__device__ __forceinline__ const char* at(const char* base, int64_t off) {
  return (const char*)((uintptr_t)base + (uintptr_t)off);
}
__device__ __forceinline__ char* atw(char* base, int64_t off) { return (char*)((uintptr_t)base + (uintptr_t)off); }

// Row / column partial sums of the registered f (tci_functions.h).  For a
// task that may tabulate f (int_states), the sums are exact integers and are
// stored as long long in the same 8-byte slots; make_filler turns them back
// into doubles if it decides against tables.
__device__ __forceinline__ bool int_states(const tci_task& T) {
  return tci_f_tables(T.fid) > 0 && T.lut != nullptr && T.lutcap0 > 0;
}
__device__ void compute_states(const tci_task& T, const double* params, const uint8_t* idx, int count, int len,
                               int site0, double* s0, double* s1) {
  if (int_states(T)) {
    long long* q0 = (long long*)s0;
    long long* q1 = (long long*)s1;
    for (int i = threadIdx.x; i < count; i += NT) {
      long long a0 = 0, a1 = 0;
      const uint8_t* v = idx + (size_t)i * len;
      for (int p = 0; p < len; ++p) tci_f_term_int(T.fid, params, site0 + p, v[p], &a0, &a1);
      q0[i] = a0;
      q1[i] = a1;
    }
    return;
  }
  for (int i = threadIdx.x; i < count; i += NT) {
    double a0 = 0.0, a1 = 0.0;
    const uint8_t* v = idx + (size_t)i * len;
    for (int p = 0; p < len; ++p) tci_f_term(T.fid, params, site0 + p, v[p], &a0, &a1);
    s0[i] = a0;
    s1[i] = a1;
  }
}

// Element generator of a registered f from row/column partial sums.  When f
// factors through exact integer sums (tci_f_tables), the distinct values of
// part0 and of scale1(part1) over the task's range are computed once into
// T.lut and each element is combine_scaled(table0[s0], table1[s1]) -- one FP64
// operation; the direct path computes the same functions, so the bits are
// identical.
struct Filler {
  int fid, nparams;
  const double* prm;
  const double* lut0;
  const double* lut1;
  int lo0, lo1;
  // element (i, j) from row states r0/r1 and column states c0/c1
  __device__ __forceinline__ double val(const double* r0, const double* r1, int i, const double* c0,
                                        const double* c1, int j) const {
    if (lut0) {
      const double p0 = lut0[(int)(((const long long*)r0)[i] + ((const long long*)c0)[j]) - lo0];
      if (!lut1) return p0;
      const double q1 = lut1[(int)(((const long long*)r1)[i] + ((const long long*)c1)[j]) - lo1];
      return tci_f_combine_scaled(fid, p0, q1);
    }
    return tci_f_finish(fid, prm, nparams, r0[i] + c0[j], r1[i] + c1[j]);
  }
};

// Block-wide max of four signed 64-bit integers (pass -x for a minimum).
__device__ void block_max4_i64(long long v[4], Ctl& ctl) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < 4; ++q) {
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
      const long long o = __shfl_down_sync(FULL, v[q], off);
      v[q] = o > v[q] ? o : v[q];
    }
    if (lane == 0) ctl.red4[q][warp] = v[q];
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      long long x = lane < NW ? ctl.red4[q][lane] : LLONG_MIN;
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        const long long o = __shfl_down_sync(FULL, x, off);
        x = o > x ? o : x;
      }
      if (lane == 0) ctl.red4[q][NW] = x;
    }
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < 4; ++q) v[q] = ctl.red4[q][NW];
  __syncthreads();
}

// Decide on tabulation for a task whose elements are sums rs[i] + cs[j] over
// the given row-state groups, and fill the tables.  Ends with a barrier.
__device__ Filler make_filler(const tci_task& T, const double* prm, double* const* rs0, double* const* rs1,
                              const int* rcount, int ngroups, double* cs0, double* cs1, int n, int64_t elems,
                              Ctl& ctl) {
  Filler F;
  F.fid = T.fid;
  F.nparams = T.nparams;
  F.prm = prm;
  F.lut0 = F.lut1 = nullptr;
  F.lo0 = F.lo1 = 0;
  if (!int_states(T)) return F;
  const int tables = tci_f_tables(T.fid);
  if (T.lut_full) {  // the solve's tables, built once by its TABLE task
    F.lut0 = T.lut;
    F.lut1 = tables > 1 ? T.lut + T.lutcap0 : nullptr;
    F.lo0 = T.lut_base0;
    F.lo1 = 0;
    return F;
  }
  // max / -min of the row and column sums
  long long v[4] = {LLONG_MIN, LLONG_MIN, LLONG_MIN, LLONG_MIN};  // max r0, max r1, -min r0, -min r1
  long long w[4] = {LLONG_MIN, LLONG_MIN, LLONG_MIN, LLONG_MIN};
  for (int g = 0; g < ngroups; ++g) {
    const long long* a0 = (const long long*)rs0[g];
    const long long* a1 = (const long long*)rs1[g];
    for (int i = threadIdx.x; i < rcount[g]; i += NT) {
      v[0] = max(v[0], a0[i]);
      v[1] = max(v[1], a1[i]);
      v[2] = max(v[2], -a0[i]);
      v[3] = max(v[3], -a1[i]);
    }
  }
  {
    const long long* b0 = (const long long*)cs0;
    const long long* b1 = (const long long*)cs1;
    for (int j = threadIdx.x; j < n; j += NT) {
      w[0] = max(w[0], b0[j]);
      w[1] = max(w[1], b1[j]);
      w[2] = max(w[2], -b0[j]);
      w[3] = max(w[3], -b1[j]);
    }
  }
  block_max4_i64(v, ctl);
  block_max4_i64(w, ctl);
  bool use = v[0] != LLONG_MIN && w[0] != LLONG_MIN;  // rows and columns exist
  long long lo0 = 0, lo1 = 0, n0 = 0, n1 = 0;
  if (use) {
    lo0 = -v[2] - w[2];
    lo1 = -v[3] - w[3];
    n0 = v[0] + w[0] - lo0 + 1;
    n1 = tables > 1 ? v[1] + w[1] - lo1 + 1 : 0;
    use = n0 <= T.lutcap0 && (tables == 1 || n1 <= T.lutcap1) &&
          n0 + n1 <= elems;  // tabulating must cost less than it saves
  }
  if (!use) {  // direct evaluation: the sums become doubles (exact)
    for (int g = 0; g < ngroups; ++g)
      for (int i = threadIdx.x; i < rcount[g]; i += NT) {
        rs0[g][i] = (double)((const long long*)rs0[g])[i];
        rs1[g][i] = (double)((const long long*)rs1[g])[i];
      }
    for (int j = threadIdx.x; j < n; j += NT) {
      cs0[j] = (double)((const long long*)cs0)[j];
      cs1[j] = (double)((const long long*)cs1)[j];
    }
    __syncthreads();
    return F;
  }
  double* t0 = T.lut;
  double* t1 = T.lut + T.lutcap0;
  for (int k = threadIdx.x; k < (int)n0; k += NT) t0[k] = tci_f_part0(T.fid, prm, T.nparams, (double)(lo0 + k));
  for (int k = threadIdx.x; k < (int)n1; k += NT)
    t1[k] = tci_f_scale1(T.fid, prm, tci_f_part1(T.fid, prm, (double)(lo1 + k)));
  __syncthreads();
  F.lut0 = t0;
  F.lut1 = tables > 1 ? t1 : nullptr;
  F.lo0 = (int)lo0;
  F.lo1 = (int)lo1;
  return F;
}

// Result record pointers.
struct ResPtrs {
  tci_result_head* head;
  int* rowp;
  int* colp;
  double* diag;
};
__device__ ResPtrs res_ptrs(char* resb, const tci_task& T) {
  ResPtrs p;
  char* base = atw(resb, T.res);
  p.head = (tci_result_head*)base;
  const int kcap = T.kcap;
  size_t off = sizeof(tci_result_head);
  p.rowp = (int*)(base + off);
  off += align_up((size_t)kcap * 4, 8);
  p.colp = (int*)(base + off);
  off += align_up((size_t)kcap * 4, 8);
  p.diag = (double*)(base + off);
  return p;
}

// Pivot decision of _optimizerrlu! (matrixlu.jl:150-158) for the pivot at
// (ctl.r, ctl.c): lu.error, the stopping rule, and the permutation bookkeeping of
// addpivot!.  One thread.
__device__ void rr_decide(Ctl& ctl, const double* A, int lda, int K, double reltol, double abstol, double* diag_out,
                          int* rowperm, int* colperm) {
  const int r = ctl.r, c = ctl.c;
  const double piv = A[r + (size_t)c * lda];
  const double e = fabs(piv);
  ctl.err = e;
  const int stop = ((e < reltol * ctl.maxerror || e < abstol) && K > 0) ? 1 : 0;
  ctl.stop = stop;
  if (!stop) {
    ctl.maxerror = jmax(ctl.maxerror, e);
    ctl.piv = piv;
    diag_out[K] = e;
    int t = rowperm[K];
    rowperm[K] = rowperm[r];
    rowperm[r] = t;
    t = colperm[K];
    colperm[K] = colperm[c];
    colperm[c] = t;
  }
}

// swaprow!(K, R), swapcol!(K, C) and the scaling of addpivot! (matrixlu.jl:98-124)
// in one pass: new(i, j) = old(pr(i), pc(j)) with pr, pc the two transpositions,
// divided by the pivot in column K below the diagonal (leftorthogonal) or in row
// K right of it.  The moved elements form disjoint pairs -- rows K/R outside
// columns K/C, columns K/C outside rows K/R, and the corners -- and each pair is
// read and written by one thread.  Ends with a barrier.
// The body for threads t = 0, stride, ... of a group (no barrier).
// nan: set when an entry of the new row K (columns >= K) or of the new column K
// (rows >= K) is NaN -- the entries that join U and L at this pivot.  Every
// other entry of L and U joined at an earlier pivot (swaps only move them), so
// the flags of all pivots cover the NaN check of L and U (matrixlu.jl:162-169).
__device__ __forceinline__ void swap_scale_body(double* A, int lda, int m, int n, int K, int R, int C, double piv,
                                                bool leftorth, int t, int stride, bool& nan) {
  for (int w = t; w < n + m + 1; w += stride) {
    if (w < n) {  // row pair (K, j) <-> (R, j)
      const int j = w;
      if (j == K || j == C) continue;
      double* col = A + (size_t)j * lda;
      if (R != K) {
        const double a = col[K], b = col[R];
        const double v = (!leftorth && j > K) ? __ddiv_rn(b, piv) : b;
        col[K] = v;
        col[R] = a;
        if (j > K && is_nan_bits(v)) nan = true;
      } else if (j > K) {
        const double v = !leftorth ? __ddiv_rn(col[K], piv) : col[K];
        col[K] = v;
        if (is_nan_bits(v)) nan = true;
      }
    } else if (w < n + m) {  // column pair (i, K) <-> (i, C)
      const int i = w - n;
      if (i == K || i == R) continue;
      double* ck = A + (size_t)K * lda;
      if (C != K) {
        double* cc = A + (size_t)C * lda;
        const double a = ck[i], b = cc[i];
        const double v = (leftorth && i > K) ? __ddiv_rn(b, piv) : b;
        ck[i] = v;
        cc[i] = a;
        if (i > K && is_nan_bits(v)) nan = true;
      } else if (i > K) {
        const double v = leftorth ? __ddiv_rn(ck[i], piv) : ck[i];
        ck[i] = v;
        if (is_nan_bits(v)) nan = true;
      }
    } else {  // the corners (K, K), (K, C), (R, K), (R, C)
      const int rows[2] = {K, R}, cols[2] = {K, C};
      const int nr = R != K ? 2 : 1, nc = C != K ? 2 : 1;
      double old[2][2];
      for (int p = 0; p < nr; ++p)
        for (int q = 0; q < nc; ++q) old[p][q] = A[rows[p] + (size_t)cols[q] * lda];
      for (int p = 0; p < nr; ++p)
        for (int q = 0; q < nc; ++q) {
          // source of (rows[p], cols[q]) is (rows[p^1], cols[q^1]) where swapped
          const int sp = nr == 2 ? 1 - p : p, sq = nc == 2 ? 1 - q : q;
          double v = old[sp][sq];
          const int i = rows[p], j = cols[q];
          if ((leftorth && j == K && i > K) || (!leftorth && i == K && j > K)) v = __ddiv_rn(v, piv);
          A[i + (size_t)j * lda] = v;
          if ((i == K || j == K) && is_nan_bits(v)) nan = true;
        }
    }
  }
}
__device__ void swap_scale(double* A, int lda, int m, int n, int K, int R, int C, double piv, bool leftorth,
                           bool& nan) {
  swap_scale_body(A, lda, m, n, K, R, C, piv, leftorth, threadIdx.x, NT, nan);
  __syncthreads();
}

// Trailing blocks of at most this many elements are finished by warp 0 alone:
// with one warp no CTA barrier is needed per pivot.  Measured: up to ~6 elements
// per lane one warp beats the barriers of the whole CTA.
constexpr int WARP_TAIL_RRLU = 192;

// rrlu_loop from pivot K on (decision for K already taken, not stopped), warp 0
// only; same arithmetic and argmax as the CTA path.  Returns the final K on
// every lane of warp 0.
__device__ int rrlu_warp_tail(double* A, int lda, int m, int n, int K, int kmax, double reltol, double abstol,
                              bool leftorth, int* rowperm, int* colperm, double* diag_out, Ctl& ctl, bool& nan) {
  const int lane = threadIdx.x & 31;
  while (true) {
    swap_scale_body(A, lda, m, n, K, ctl.r, ctl.c, ctl.piv, leftorth, lane, 32, nan);
    __syncwarp();
    ++K;
    if (K == kmax) break;
    ArgTrack at;
    at.init();
    {
      const double* x = A + (size_t)(K - 1) * lda;
      const int rows = m - K;
      const int total = rows * (n - K);
      const int sq = 32 / rows, sr = 32 % rows;
      int jj = lane / rows, ii = lane % rows;
      for (int e = lane; e < total; e += 32) {
        const int i = K + ii, j = K + jj;
        double* col = A + (size_t)j * lda;
        const double v = __dsub_rn(col[i], __dmul_rn(x[i], col[K - 1]));
        col[i] = v;
        at.push(v, pack_key(i, j));
        ii += sr;
        jj += sq;
        if (ii >= rows) {
          ii -= rows;
          jj += 1;
        }
      }
    }
    uint64_t a = at.A, b = at.B;
    uint32_t k = at.k;
    warp_track(a, k, b);
    __syncwarp();  // every lane's update is in place before the exact pass / decision
    const uint64_t Mstar = a ? a - 1 : 0;
    const bool safe = Mstar >= SQ_SMALL && Mstar < SQ_BIG;
    const bool close = b != 0 && (b - 1) + 16 >= Mstar;
    int r, c;
    if (a == 0) {
      r = K;
      c = K;
    } else if (safe && !close) {
      r = (int)(k & 0xffffu);
      c = (int)(k >> 16);
    } else {  // squares of the elements near the maximum
      ArgBest ab;
      ab.init();
      const int rows = m - K, total = rows * (n - K);
      for (int e = lane; e < total; e += 32) {
        const int i = K + e % rows, j = K + e / rows;
        const double v = A[i + (size_t)j * lda];
        if (near_max(abs_bits(v), Mstar)) ab.consider(v, pack_key(i, j));
      }
      uint64_t sv = ab.s;
      uint32_t key = ab.key;
      warp_best(sv, key);
      r = sv ? (int)(key & 0xffffu) : K;
      c = sv ? (int)(key >> 16) : K;
    }
    if (lane == 0) {
      ctl.r = r;
      ctl.c = c;
      rr_decide(ctl, A, lda, K, reltol, abstol, diag_out, rowperm, colperm);
    }
    __syncwarp();
    if (ctl.stop) break;
  }
  return K;
}

// The rrLU main loop (matrixlu.jl:141-181) on A (m x n, leading dim lda) with the
// first argmax already in ctl.r/ctl.c.  rowperm/colperm are full permutations.
// Per pivot: one swap/scale pass, the rank-1 update fused with the next argmax,
// whose resolving thread also takes the next decision -- three barriers.
// xy: optional shared-memory copy (m + n doubles) of the pivot column and row
// for a matrix in global memory, so that each element of the update costs one
// load and one store.  Returns this thread's part of the NaN check of L and U
// (an OR over the CTA gives it).
__device__ bool rrlu_loop(double* A, int lda, int m, int n, int maxrank, double reltol, double abstol,
                          bool leftorth, int* rowperm, int* colperm, double* diag_out, Ctl& ctl,
                          double* xy = nullptr, int warp_tail = WARP_TAIL_RRLU) {
  const int tid = threadIdx.x;
  const int kmax = min(maxrank, min(m, n));
  bool nan = false;
  if (tid == 0) {
    ctl.K = 0;
    ctl.maxerror = 0.0;
    ctl.err = __longlong_as_double(0x7ff8000000000000LL);
    ctl.kmax = kmax;
    ctl.stop = 1;
    if (kmax > 0) rr_decide(ctl, A, lda, 0, reltol, abstol, diag_out, rowperm, colperm);
  }
  __syncthreads();
  int K = 0;
  bool tail = false;
  while (!ctl.stop) {
    TCI_PHASE(1);
    if ((m - K) * (n - K) <= warp_tail) {
      tail = true;
      break;
    }
    swap_scale(A, lda, m, n, K, ctl.r, ctl.c, ctl.piv, leftorth, nan);
    TCI_PHASE(3);
    ++K;
    if (K == kmax) break;  // the trailing update after the last pivot is not observable
    // A[K:, K:] -= x * y^T fused with the argmax of abs2 for the next pivot.
    // The trailing block is walked as one column-major sequence so that every
    // lane of every warp has an element (no half-empty warps at column ends).
    ArgTrack at;
    at.init();
    const int rows = m - K;
    const long long total = (long long)rows * (n - K);
    const int sq = NT / rows, sr = NT % rows;  // stride NT as (columns, rows)
    if (xy) {
      // x = A[K:, K-1] and y = A[K-1, K:] on chip, indexed from K
      double* xs = xy;
      double* ys = xy + m;
      for (int i = K + tid; i < m; i += NT) xs[i] = A[i + (size_t)(K - 1) * lda];
      for (int j = K + tid; j < n; j += NT) ys[j] = A[(K - 1) + (size_t)j * lda];
      __syncthreads();
      int jj = tid / rows, ii = tid % rows;
      long long e = tid;
      // four elements per step with their global loads issued first; the keys
      // still reach the tracker in increasing order
      for (; e + 3LL * NT < total; e += 4LL * NT) {
        int i4[4], j4[4];
        double a4[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          i4[q] = K + ii;
          j4[q] = K + jj;
          ii += sr;
          jj += sq;
          if (ii >= rows) {
            ii -= rows;
            jj += 1;
          }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) a4[q] = A[i4[q] + (size_t)j4[q] * lda];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const double v = __dsub_rn(a4[q], __dmul_rn(xs[i4[q]], ys[j4[q]]));
          A[i4[q] + (size_t)j4[q] * lda] = v;
          at.push(v, pack_key(i4[q], j4[q]));
        }
      }
      for (; e < total; e += NT) {
        const int i = K + ii, j = K + jj;
        double* col = A + (size_t)j * lda;
        const double v = __dsub_rn(col[i], __dmul_rn(xs[i], ys[j]));
        col[i] = v;
        at.push(v, pack_key(i, j));
        ii += sr;
        jj += sq;
        if (ii >= rows) {
          ii -= rows;
          jj += 1;
        }
      }
    } else {
      const double* x = A + (size_t)(K - 1) * lda;
      int jj = tid / rows, ii = tid % rows;
      for (long long e = tid; e < total; e += NT) {
        const int i = K + ii, j = K + jj;
        double* col = A + (size_t)j * lda;
        double v = __dsub_rn(col[i], __dmul_rn(x[i], col[K - 1]));
        col[i] = v;
        at.push(v, pack_key(i, j));
        ii += sr;
        jj += sq;
        if (ii >= rows) {
          ii -= rows;
          jj += 1;
        }
      }
    }
    TCI_PHASE(4);
    const int Kc = K;
    argmax_resolve(at, A, lda, K, m - K, K, n - K, ctl,
                   [&] { rr_decide(ctl, A, lda, Kc, reltol, abstol, diag_out, rowperm, colperm); });
    TCI_PHASE(6);
  }
  if (tail && tid < 32) K = rrlu_warp_tail(A, lda, m, n, K, kmax, reltol, abstol, leftorth, rowperm, colperm,
                                           diag_out, ctl, nan);
  if (tid == 0) {
    ctl.K = K;
    if (K >= min(m, n)) ctl.err = 0.0;
  }
  __syncthreads();
  return nan;
}

// left(MatrixLUCI) for leftorthogonal (colstimespivotinv, matrixluci.jl:48-57):
// rows K.. of L solved against the unit-lower L11, rows scattered by rowperm.
// For !leftorthogonal: colmatrix = left(lu) * U[:, 1:K] (matrixluci.jl:40-42).
__device__ void post_left(double* A, int lda, int m, int n, int K, bool leftorth, const int* rowperm,
                          double* out) {
  const int tid = threadIdx.x;
  if (leftorth) {
    // X * L11 = L21 with unit-lower L11, one thread per row of L21, in the
    // oracle's order: X[p, q] = L21[p, q] - sum over t = q+1 .. K-1 (ascending)
    // of X[p, t] * L11[t, q], for q from K-1 down to 0 (the division by the
    // unit diagonal is exact and omitted).
    for (int p = K + tid; p < m; p += NT) {
      for (int q = K - 1; q >= 0; --q) {
        double s = A[p + (size_t)q * lda];
        for (int t = q + 1; t < K; ++t) s = s - A[p + (size_t)t * lda] * A[t + (size_t)q * lda];
        A[p + (size_t)q * lda] = s;
      }
    }
    __syncthreads();
    for (int q = 0; q < K; ++q)
      for (int p = tid; p < m; p += NT) {
        double v = p < K ? (p == q ? 1.0 : 0.0) : A[p + (size_t)q * lda];
        out[rowperm[p] + (size_t)q * m] = v;
      }
  } else {
    // colmatrix: (L with rows scattered) * U11, U11 unit upper; L keeps its diagonal
    for (int p = tid; p < m; p += NT)
      for (int q = 0; q < K; ++q) {
        double s = 0.0;
        const int tmax = min(p, q);
        for (int t = 0; t <= tmax; ++t) {
          double l = A[p + (size_t)t * lda];
          double u = (t == q) ? 1.0 : A[t + (size_t)q * lda];
          s = s + l * u;
        }
        out[rowperm[p] + (size_t)q * m] = s;
      }
  }
  __syncthreads();
}

// right(MatrixLUCI): for leftorthogonal rowmatrix = L11 * right(lu)
// (matrixluci.jl:44-46); otherwise pivotinvtimesrows (matrixluci.jl:59-68).
__device__ void post_right(double* A, int lda, int m, int n, int K, bool leftorth, const int* colperm,
                           double* out) {
  const int tid = threadIdx.x;
  if (leftorth) {
    for (int j = tid; j < n; j += NT)
      for (int q = 0; q < K; ++q) {
        double s = 0.0;
        for (int t = 0; t <= q; ++t) {
          double l = (t == q) ? 1.0 : A[q + (size_t)t * lda];
          double u = (t <= j) ? A[t + (size_t)j * lda] : 0.0;
          s = s + l * u;
        }
        out[q + (size_t)colperm[j] * K] = s;
      }
  } else {
    // U11 X = U12 with unit-upper U11, one thread per column of U12, in the
    // oracle's order: X[q, j] = U12[q, j] - sum over p = q+1 .. K-1 (ascending)
    // of U11[q, p] * X[p, j], for q from K-1 down to 0.
    for (int j = K + tid; j < n; j += NT) {
      double* col = A + (size_t)j * lda;
      for (int q = K - 1; q >= 0; --q) {
        double s = col[q];
        for (int p = q + 1; p < K; ++p) s = s - A[q + (size_t)p * lda] * col[p];
        col[q] = s;
      }
    }
    __syncthreads();
    for (int j = tid; j < n; j += NT)
      for (int q = 0; q < K; ++q) {
        double v = j < K ? (q == j ? 1.0 : 0.0) : A[q + (size_t)j * lda];
        out[q + (size_t)colperm[j] * K] = v;
      }
  }
  __syncthreads();
}

struct SmemCursor {
  char* p;
  __device__ char* take(size_t bytes) {
    char* r = p;
    p += align_up(bytes, 16);
    return r;
  }
};

// ---------------------------------------------------------------- RRLU task
__device__ void task_rrlu(const tci_task& T, const char* blob, char* resb, char* smem, Ctl& ctl, size_t smem_bytes) {
  const int m = T.m, n = T.n, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  ResPtrs rp = res_ptrs(resb, T);
  SmemCursor cur{smem};
  double* A = T.smem_mode == 1 ? (double*)cur.take((size_t)m * n * 8) : T.work;
  const int lda = m;
  int* rowperm = (int*)cur.take((size_t)m * 4);
  int* colperm = (int*)cur.take((size_t)n * 4);
  for (int i = tid; i < m; i += NT) rowperm[i] = i;
  for (int j = tid; j < n; j += NT) colperm[j] = j;
  int lut_used = 0;
  ArgTrack am;
  am.init();
  unsigned long long mx = 0;
  if (T.ain) {
    // the input is read once: evict-first loads keep it from pushing the
    // working matrices (re-read every pivot) out of L2
    for (int j = warp; j < n; j += NW) {
      const double* src = T.ain + (size_t)j * m;
      double* dst = A + (size_t)j * lda;
      for (int i = lane; i < m; i += 32) {
        double v = __ldcs(src + i);
        dst[i] = v;
        am.push(v, pack_key(i, j));
        unsigned long long b = abs_bits(v);
        mx = b > mx ? b : mx;
      }
    }
  } else {
    const double* prm = (const double*)at(blob, T.params);
    // the row / column f states: on chip, or after the matrix in global scratch
    double* const st = T.smem_mode == 2 ? T.work + (size_t)m * n : nullptr;
    double* rs0 = st ? st : (double*)cur.take((size_t)m * 8);
    double* rs1 = st ? st + m : (double*)cur.take((size_t)m * 8);
    double* cs0 = st ? st + 2 * (size_t)m : (double*)cur.take((size_t)n * 8);
    double* cs1 = st ? st + 2 * (size_t)m + n : (double*)cur.take((size_t)n * 8);
    compute_states(T, prm, (const uint8_t*)at(blob, T.rows), m, T.nl, 0, rs0, rs1);
    compute_states(T, prm, (const uint8_t*)at(blob, T.cols), n, T.nr, T.nl, cs0, cs1);
    __syncthreads();
    double* const rg0[1] = {rs0};
    double* const rg1[1] = {rs1};
    const int rc[1] = {m};
    const Filler F = make_filler(T, prm, rg0, rg1, rc, 1, cs0, cs1, n, (int64_t)m * n, ctl);
    lut_used = F.lut0 != nullptr;
    for (int j = warp; j < n; j += NW) {
      double* dst = A + (size_t)j * lda;
      for (int i = lane; i < m; i += 32) {
        double v = F.val(rs0, rs1, i, cs0, cs1, j);
        dst[i] = v;
        am.push(v, pack_key(i, j));
        unsigned long long b = abs_bits(v);
        mx = b > mx ? b : mx;
      }
    }
  }
  __syncthreads();
  unsigned long long mxall = block_max_u64(mx, ctl);
  if (tid == 0) ctl.status = 0;
  argmax_resolve(am, A, lda, 0, m, 0, n, ctl);
  const bool leftorth = T.leftorth != 0;
  double* xy = nullptr;
  if (T.smem_mode != 1 && (size_t)(cur.p - smem) + (size_t)(m + n) * 8 <= smem_bytes) xy = (double*)cur.take((size_t)(m + n) * 8);
  const bool nan_part = rrlu_loop(A, lda, m, n, T.maxrank, T.reltol, T.abstol, leftorth, rowperm, colperm, rp.diag,
                                  ctl, xy, T.tail_elems > 0 ? T.tail_elems : WARP_TAIL_RRLU);
  const int K = ctl.K;
  // NaN check of L = tril(A[:, 1:K]) and U = triu(A[1:K, :]) (matrixlu.jl:162-169),
  // gathered while the pivots were taken
  int nan = block_or(nan_part ? 1 : 0, ctl);
  if (T.post == TCI_POST_LEFT && !nan) post_left(A, lda, m, n, K, leftorth, rowperm, T.core_out);
  if (T.post == TCI_POST_RIGHT && !nan) post_right(A, lda, m, n, K, leftorth, colperm, T.core_out);
  if (T.post == TCI_POST_FACTORS)
    for (int j = warp; j < n; j += NW)
      for (int i = lane; i < m; i += 32) T.core_out[i + (size_t)j * m] = A[i + (size_t)j * lda];
  if (tid == 0) {
    rp.head->status = nan ? TCI_ST_NAN : 0;
    rp.head->npivot = K;
    rp.head->error = ctl.err;
    rp.head->maxabs = __longlong_as_double((long long)mxall);
    rp.head->maxabs_nan = mxall > NAN_FLOOR ? 1 : 0;
    rp.head->lut_used = lut_used;
  }
  if (T.post == TCI_POST_FACTORS) {
    // full permutations go after the factors: rowperm (m) then colperm (n)
    int* fr = (int*)(T.core_out + (size_t)m * n);
    for (int i = tid; i < m; i += NT) fr[i] = rowperm[i];
    for (int j = tid; j < n; j += NT) fr[m + j] = colperm[j];
  }
  for (int k = tid; k < K; k += NT) {
    rp.rowp[k] = rowperm[k];
    rp.colp[k] = colperm[k];
  }
  __syncthreads();
}

// ---------------------------------------------------------------- SITE task
// Warp-wide pivot search of column j of A (lda = r) over rows j .. r-1 with the
// rule of LAPACK's partial pivoting as the oracle states it: start from |A[j,j]|
// and take the first row whose |a| is strictly larger than the running best
// (NaN never wins; a NaN diagonal keeps row j).  Bit patterns of |a| order like
// the values, so the search runs on the integer pipe.  Every lane gets the row.
__device__ int site_col_pivot(const double* col, int j, int r) {
  const int lane = threadIdx.x & 31;
  uint64_t s = 0;  // |a| bits + 1 of this lane's first maximum, 0 = none
  int si = INT_MAX;
  for (int i = j + 1 + lane; i < r; i += 32) {
    const uint64_t b = abs_bits(col[i]);
    if (b <= NAN_FLOOR && b + 1 > s) {
      s = b + 1;
      si = i;
    }
  }
#pragma unroll
  for (int off = 16; off > 0; off >>= 1) {
    const uint64_t os = __shfl_xor_sync(FULL, s, off);
    const int oi = __shfl_xor_sync(FULL, si, off);
    if (os > s || (os == s && oi < si)) {
      s = os;
      si = oi;
    }
  }
  const uint64_t d = abs_bits(col[j]);
  if (d > NAN_FLOOR) return j;
  return s > d + 1 ? si : j;
}

// getrf with partial pivoting of the r x r matrix A (lda = r), in the oracle's
// order: per column j, the pivot row p (site_col_pivot), a whole-row swap of
// rows j and p, the column below the diagonal times the IEEE reciprocal of the
// pivot, then the rank-1 update of the trailing block as a separate multiply
// and subtract.  ipiv[j] = p.  Returns (to every thread) 1 when a pivot is
// exactly zero -- the reference's SingularException -- else 0.
// Two block barriers per column: (swap + scale) and (update + next pivot
// search); warp 0 owns the column being scaled and the next column, whose
// update it fuses with the search.  Matrices of at most 32 rows run on warp 0
// alone with warp-level synchronisation.
__device__ int site_getrf(double* A, int r, int* ipiv, Ctl& ctl) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  if (r <= 32) {
    if (warp == 0) {
      int sing = 0;
      for (int j = 0; j < r; ++j) {
        const int p = site_col_pivot(A + (size_t)j * r, j, r);
        const double piv = A[p + (size_t)j * r];
        if (piv == 0.0) {
          sing = 1;
          break;
        }
        if (lane == 0) ipiv[j] = p;
        __syncwarp();
        if (p != j && lane < r) {
          const double a = A[j + (size_t)lane * r], b = A[p + (size_t)lane * r];
          A[j + (size_t)lane * r] = b;
          A[p + (size_t)lane * r] = a;
        }
        __syncwarp();
        const double rcp = 1.0 / A[j + (size_t)j * r];
        if (lane > j && lane < r) A[lane + (size_t)j * r] = A[lane + (size_t)j * r] * rcp;
        __syncwarp();
        if (lane > j && lane < r)
          for (int c = j + 1; c < r; ++c)
            A[lane + (size_t)c * r] = A[lane + (size_t)c * r] - A[lane + (size_t)j * r] * A[j + (size_t)c * r];
        __syncwarp();
      }
      if (lane == 0) ctl.status = sing;
    }
    __syncthreads();
    const int s = ctl.status;
    __syncthreads();
    return s;
  }
  if (warp == 0) {
    const int p = site_col_pivot(A, 0, r);
    if (lane == 0) {
      ctl.r = p;
      ctl.piv = A[p];
    }
  }
  __syncthreads();
  for (int j = 0; j < r; ++j) {
    const int p = ctl.r;
    const double piv = ctl.piv;
    if (piv == 0.0) {
      __syncthreads();
      return 1;
    }
    // swap rows j and p (warp 0 takes column j and scales it)
    if (warp == 0) {
      double* cj = A + (size_t)j * r;
      const double djj = cj[j];
      __syncwarp();
      const double rcp = 1.0 / piv;
      for (int i = j + 1 + lane; i < r; i += 32) {
        const double v = i == p ? djj : cj[i];
        cj[i] = v * rcp;
      }
      if (lane == 0) {
        cj[j] = piv;
        ipiv[j] = p;
      }
    } else if (p != j) {
      for (int c = tid - 32; c < r; c += NT - 32) {
        if (c == j) continue;
        const double a = A[j + (size_t)c * r], b = A[p + (size_t)c * r];
        A[j + (size_t)c * r] = b;
        A[p + (size_t)c * r] = a;
      }
    }
    __syncthreads();
    // trailing update; warp 0 updates column j+1 and searches its pivot
    const double* lj = A + (size_t)j * r;
    if (warp == 0) {
      if (j + 1 < r) {
        double* c1 = A + (size_t)(j + 1) * r;
        const double y = c1[j];
        for (int i = j + 1 + lane; i < r; i += 32) c1[i] = c1[i] - lj[i] * y;
        __syncwarp();
        const int pn = site_col_pivot(c1, j + 1, r);
        if (lane == 0) {
          ctl.r = pn;
          ctl.piv = c1[pn];
        }
      }
    } else {
      for (int c = j + 2 + (warp - 1); c < r; c += NW - 1) {
        double* cc = A + (size_t)c * r;
        const double y = cc[j];
        for (int i = j + 1 + lane; i < r; i += 32) cc[i] = cc[i] - lj[i] * y;
      }
    }
    __syncthreads();
  }
  return 0;
}

// setsitetensor!(tci, f, b) (tensorci2.jl:367-394): P (r x r) = f(prows x cols),
// Pi1 (m x r) = f(rows x cols), T = Pi1 * inv(P) from transpose(P) \ transpose(Pi1)
// (:391), i.e. getrf of A = P^T with partial pivoting and, per row of Pi1, the
// row interchanges, the unit-lower forward substitution and the upper back
// substitution (division by the diagonal) -- the order of the oracle's LAPACK
// restatement, so the tensor equals the oracle's bit for bit.
__device__ void task_site(const tci_task& T, const char* blob, char* resb, char* smem, Ctl& ctl,
                          size_t smem_bytes) {
  const int r = T.r, m = T.m, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  ResPtrs rp = res_ptrs(resb, T);
  const double* prm = (const double*)at(blob, T.params);
  SmemCursor cur{smem};
  double* A = T.smem_mode == 1 ? (double*)cur.take((size_t)r * r * 8) : T.work;
  int* ipiv = (int*)cur.take((size_t)r * 4);
  (void)cur.take((size_t)r * 4);  // unused slot (keeps the host's shared-memory plan)
  double* ps0 = (double*)cur.take((size_t)r * 8);
  double* ps1 = (double*)cur.take((size_t)r * 8);
  double* cs0 = (double*)cur.take((size_t)r * 8);
  double* cs1 = (double*)cur.take((size_t)r * 8);
  // the row f states: on chip, or after P in global scratch
  double* rs0 = T.smem_mode == 2 ? T.work + (size_t)r * r : (double*)cur.take((size_t)m * 8);
  double* rs1 = T.smem_mode == 2 ? T.work + (size_t)r * r + m : (double*)cur.take((size_t)m * 8);
  compute_states(T, prm, (const uint8_t*)at(blob, T.prows), r, T.nl, 0, ps0, ps1);
  compute_states(T, prm, (const uint8_t*)at(blob, T.cols), r, T.nr, T.nl, cs0, cs1);
  compute_states(T, prm, (const uint8_t*)at(blob, T.rows), m, T.nl, 0, rs0, rs1);
  __syncthreads();
  double* const rg0[2] = {ps0, rs0};
  double* const rg1[2] = {ps1, rs1};
  const int rc[2] = {r, m};
  const Filler F = make_filler(T, prm, rg0, rg1, rc, 2, cs0, cs1, r, (int64_t)(r + m) * r, ctl);
  // A[i, j] = P[j, i] = f(prows[j] ++ cols[i])
  for (int j = warp; j < r; j += NW)
    for (int i = lane; i < r; i += 32) A[i + (size_t)j * r] = F.val(ps0, ps1, j, cs0, cs1, i);
  __syncthreads();
  const int singular = site_getrf(A, r, ipiv, ctl);
  (void)cur.take((size_t)r * 8);  // unused slot (keeps the host's shared-memory plan)
  size_t used = (size_t)(cur.p - smem);
  int RB = (int)((smem_bytes > used ? smem_bytes - used : 0) / ((size_t)r * 8 + 8));
  RB = RB > NT ? NT : RB;
  RB = RB < 1 ? 1 : RB;
  double* W = (double*)cur.take((size_t)RB * r * 8);
  unsigned long long mx = 0;
  int nanflag = 0;
  for (int base = 0; base < m; base += RB) {
    const int rows_here = min(RB, m - base);
    for (int e = tid; e < rows_here * r; e += NT) {
      int rr = e % rows_here, q = e / rows_here;
      double v = F.val(rs0, rs1, base + rr, cs0, cs1, q);
      W[rr + (size_t)q * RB] = v;
      unsigned long long b = abs_bits(v);
      mx = b > mx ? b : mx;
    }
    __syncthreads();
    if (!singular) {
      for (int rr = tid; rr < rows_here; rr += NT) {
        double* w = W + rr;
        for (int j = 0; j < r; ++j) {
          const int p = ipiv[j];
          if (p != j) {
            const double a = w[(size_t)j * RB];
            w[(size_t)j * RB] = w[(size_t)p * RB];
            w[(size_t)p * RB] = a;
          }
        }
        for (int j = 0; j < r; ++j) {
          const double bj = w[(size_t)j * RB];
          for (int i = j + 1; i < r; ++i) w[(size_t)i * RB] = w[(size_t)i * RB] - A[i + (size_t)j * r] * bj;
        }
        for (int j = r - 1; j >= 0; --j) {
          const double bj = w[(size_t)j * RB] / A[j + (size_t)j * r];
          w[(size_t)j * RB] = bj;
          for (int i = 0; i < j; ++i) w[(size_t)i * RB] = w[(size_t)i * RB] - A[i + (size_t)j * r] * bj;
        }
      }
    }
    __syncthreads();
    for (int e = tid; e < rows_here * r; e += NT) {
      int rr = e % rows_here, q = e / rows_here;
      double v = W[rr + (size_t)q * RB];
      if (is_nan_bits(v)) nanflag = 1;
      T.core_out[(base + rr) + (size_t)q * m] = v;
    }
    __syncthreads();
  }
  unsigned long long mxall = block_max_u64(mx, ctl);
  int nan = block_or(nanflag, ctl);
  if (tid == 0) {
    rp.head->status = (singular ? TCI_ST_SINGULAR : 0) | (nan ? TCI_ST_NAN : 0);
    rp.head->npivot = singular ? 0 : r;
    rp.head->error = 0.0;
    rp.head->maxabs = __longlong_as_double((long long)mxall);
    rp.head->maxabs_nan = mxall > NAN_FLOOR ? 1 : 0;
    rp.head->lut_used = F.lut0 != nullptr;
  }
  __syncthreads();
}

// ---------------------------------------------------------------- CORE task
__device__ void task_core(const tci_task& T, const char* blob, char* resb, char* smem, Ctl& ctl) {
  const int m = T.m, n = T.n, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const double* prm = (const double*)at(blob, T.params);
  SmemCursor cur{smem};
  double* rs0 = (double*)cur.take((size_t)m * 8);
  double* rs1 = (double*)cur.take((size_t)m * 8);
  double* cs0 = (double*)cur.take((size_t)n * 8);
  double* cs1 = (double*)cur.take((size_t)n * 8);
  compute_states(T, prm, (const uint8_t*)at(blob, T.rows), m, T.nl, 0, rs0, rs1);
  compute_states(T, prm, (const uint8_t*)at(blob, T.cols), n, T.nr, T.nl, cs0, cs1);
  __syncthreads();
  double* const rg0[1] = {rs0};
  double* const rg1[1] = {rs1};
  const int rc[1] = {m};
  const Filler F = make_filler(T, prm, rg0, rg1, rc, 1, cs0, cs1, n, (int64_t)m * n, ctl);
  unsigned long long mx = 0;
  for (int j = warp; j < n; j += NW)
    for (int i = lane; i < m; i += 32) {
      double v = F.val(rs0, rs1, i, cs0, cs1, j);
      T.core_out[i + (size_t)j * m] = v;
      unsigned long long b = abs_bits(v);
      mx = b > mx ? b : mx;
    }
  unsigned long long mxall = block_max_u64(mx, ctl);
  if (tid == 0) {
    tci_result_head* h = (tci_result_head*)(atw(resb, T.res));
    h->status = 0;
    h->npivot = 0;
    h->error = 0.0;
    h->maxabs = __longlong_as_double((long long)mxall);
    h->maxabs_nan = mxall > NAN_FLOOR ? 1 : 0;
    h->lut_used = F.lut0 != nullptr;
  }
  __syncthreads();
}

// ---------------------------------------------------------------- EVAL task
constexpr int EVAL_THREAD_RMAX = TCI_EVAL_THREAD_RMAX;  // largest bond of the thread-per-point path

// f and the tensor train at T.m points (rows, L sites each).  The train: one
// thread per point for bonds up to EVAL_THREAD_RMAX, else one warp per point;
// out[q] = sum_p v[p] * core[p, i, q], summed in order of p with separate
// multiply and add, as the oracle's loop.
__device__ void task_eval(const tci_task& T, const char* blob, char* resb, char* smem, Ctl& ctl) {
  const int np = T.m, L = T.L, tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const double* prm = (const double*)at(blob, T.params);
  const uint8_t* pts = (const uint8_t*)at(blob, T.rows);
  char* base = atw(resb, T.res);
  double* fout = (double*)(base + sizeof(tci_result_head));
  double* tout = fout + np;
  for (int p = tid; p < np; p += NT) {
    double a0 = 0.0, a1 = 0.0;
    for (int s = 0; s < L; ++s) tci_f_term(T.fid, prm, s, pts[(size_t)p * L + s], &a0, &a1);
    fout[p] = tci_f_finish(T.fid, prm, T.nparams, a0, a1);
  }
  if (T.cores && T.r <= EVAL_THREAD_RMAX) {
    // bonds up to EVAL_THREAD_RMAX: one thread per point (a warp per point would
    // leave most lanes idle), the running vector in the thread's own column of
    // shared memory (2 x EVAL_THREAD_RMAX x NT doubles, within the step's plan)
    const tci_core_ref* cr = (const tci_core_ref*)at(blob, T.cores);
    double* vs = (double*)smem;
    double* ws = vs + (size_t)EVAL_THREAD_RMAX * NT;
    for (int p = tid; p < np; p += NT) {
      double* v = vs;
      double* w = ws;
      v[tid] = 1.0;
      for (int s = 0; s < L; ++s) {
        const tci_core_ref c = cr[s];
        const int i = pts[(size_t)p * L + s];
        for (int q = 0; q < c.r1; ++q) {
          const double* col = c.p + (size_t)c.r0 * (i + (size_t)c.d * q);
          double acc = 0.0;
          for (int t = 0; t < c.r0; ++t) acc = __dadd_rn(acc, __dmul_rn(v[(size_t)t * NT + tid], col[t]));
          w[(size_t)q * NT + tid] = acc;
        }
        double* tmp = v;
        v = w;
        w = tmp;
      }
      tout[p] = v[tid];
    }
  } else if (T.cores) {
    const tci_core_ref* cr = (const tci_core_ref*)at(blob, T.cores);
    const int rmax = T.r;
    double* va = (double*)smem + (size_t)warp * 2 * rmax;
    double* vb = va + rmax;
    for (int p = warp; p < np; p += NW) {
      if (lane == 0) va[0] = 1.0;
      __syncwarp();
      double* v = va;
      double* w = vb;
      for (int s = 0; s < L; ++s) {
        const tci_core_ref c = cr[s];
        const int i = pts[(size_t)p * L + s];
        for (int q = lane; q < c.r1; q += 32) {
          double acc = 0.0;
          const double* col = c.p + (size_t)c.r0 * (i + (size_t)c.d * q);
          for (int t = 0; t < c.r0; ++t) acc = __dadd_rn(acc, __dmul_rn(v[t], col[t]));
          w[q] = acc;
        }
        __syncwarp();
        double* tmp = v;
        v = w;
        w = tmp;
      }
      if (lane == 0) tout[p] = v[0];
      __syncwarp();
    }
  } else {
    for (int p = tid; p < np; p += NT) tout[p] = 0.0;
  }
  if (tid == 0) {
    tci_result_head* h = (tci_result_head*)base;
    h->status = 0;
    h->npivot = 0;
  }
  __syncthreads();
}

// ---------------------------------------------------------------- SEARCH task
// One start point of DefaultGlobalPivotFinder (globalpivotfinder.jl:160-177):
// f and the train at every point that differs from the start in one site.  The
// train values use left environments Le_p = C_0[i_0] ... C_{p-1}[i_{p-1}] and
// right environments Re_p = C_{p+1}[i_{p+1}] ... C_{L-1}[i_{L-1}] of the start,
// value(p, v) = sum_b (sum_a Le_p[a] C_p[a, v, b]) Re_p[b], every sum in index
// order with separate multiply and add (the oracle uses the same order).
__device__ void task_search(const tci_task& T, const char* blob, char* resb, char* smem) {
  const int L = T.L, tid = threadIdx.x;
  const double* prm = (const double*)at(blob, T.params);
  const uint8_t* st = (const uint8_t*)at(blob, T.rows);
  char* base = atw(resb, T.res);
  double* fout = (double*)(base + sizeof(tci_result_head));
  double* tout = fout + T.m;
  // environment offsets: Le_p has r0(p) entries, Re_p has r1(p) entries
  int* loff = (int*)smem;
  int* roff = loff + (L + 1);
  int* ioff = roff + (L + 1);  // first item of site p
  double* env = (double*)(smem + align_up((size_t)(3 * (L + 1)) * 4, 16));
  // the core table on chip: every site step below reads it, and in resident
  // mode the task's copy is in host memory (one round trip here instead of one
  // per read)
  tci_core_ref* cr = (tci_core_ref*)(smem + align_up((size_t)(3 * (L + 1)) * 4, 16) +
                                     align_up((size_t)T.n * 8, 16));
  {
    const tci_core_ref* src = (const tci_core_ref*)at(blob, T.cores);
    for (int p = tid; p < L; p += NT) cr[p] = src[p];
  }
  __syncthreads();
  if (tid == 0) {
    int a = 0, b = 0, c = 0;
    for (int p = 0; p < L; ++p) {
      loff[p] = a;
      a += cr[p].r0;
      ioff[p] = c;
      c += cr[p].d;
    }
    for (int p = 0; p < L; ++p) {
      roff[p] = a + b;
      b += cr[p].r1;
    }
    ioff[L] = c;
  }
  __syncthreads();
  // left environments
  if (tid == 0) env[loff[0]] = 1.0;
  __syncthreads();
  for (int p = 0; p + 1 < L; ++p) {
    const tci_core_ref c = cr[p];
    const int i = st[p];
    const double* le = env + loff[p];
    double* nx = env + loff[p + 1];
    for (int b = tid; b < c.r1; b += NT) {
      double acc = 0.0;
      const double* col = c.p + (size_t)c.r0 * (i + (size_t)c.d * b);
      for (int a = 0; a < c.r0; ++a) acc = __dadd_rn(acc, __dmul_rn(le[a], col[a]));
      nx[b] = acc;
    }
    __syncthreads();
  }
  // right environments
  if (tid == 0) env[roff[L - 1]] = 1.0;
  __syncthreads();
  for (int p = L - 1; p > 0; --p) {
    const tci_core_ref c = cr[p];
    const int i = st[p];
    const double* re = env + roff[p];
    double* nx = env + roff[p - 1];
    for (int a = tid; a < c.r0; a += NT) {
      double acc = 0.0;
      for (int b = 0; b < c.r1; ++b)
        acc = __dadd_rn(acc, __dmul_rn(c.p[a + (size_t)c.r0 * (i + (size_t)c.d * b)], re[b]));
      nx[a] = acc;
    }
    __syncthreads();
  }
  // every (p, v)
  const int nitems = ioff[L];
  for (int it = tid; it < nitems; it += NT) {
    int p = 0;
    while (ioff[p + 1] <= it) ++p;
    const int v = it - ioff[p];
    const tci_core_ref c = cr[p];
    const double* le = env + loff[p];
    const double* re = env + roff[p];
    double val = 0.0;
    for (int b = 0; b < c.r1; ++b) {
      const double* col = c.p + (size_t)c.r0 * (v + (size_t)c.d * b);
      double w = 0.0;
      for (int a = 0; a < c.r0; ++a) w = __dadd_rn(w, __dmul_rn(le[a], col[a]));
      val = __dadd_rn(val, __dmul_rn(w, re[b]));
    }
    tout[it] = val;
    double a0 = 0.0, a1 = 0.0;
    for (int s = 0; s < L; ++s) tci_f_term(T.fid, prm, s, s == p ? v : st[s], &a0, &a1);
    fout[it] = tci_f_finish(T.fid, prm, T.nparams, a0, a1);
  }
  if (tid == 0) {
    tci_result_head* h = (tci_result_head*)base;
    h->status = 0;
    h->npivot = 0;
    h->lut_used = 0;
  }
  __syncthreads();
}

// ---------------------------------------------------------------- SUM task
// sum(tt) (abstracttensortrain.jl:164-199): v <- v * (sum over the local index
// of core b), left to right; one thread per output bond index.
__device__ void task_sum(const tci_task& T, const char* blob, char* resb, char* smem) {
  const int L = T.L, tid = threadIdx.x;
  const tci_core_ref* cr = (const tci_core_ref*)at(blob, T.cores);
  double* v = (double*)smem;
  double* w = v + T.r;
  if (tid == 0) v[0] = 1.0;
  __syncthreads();
  for (int s = 0; s < L; ++s) {
    const tci_core_ref c = cr[s];
    for (int q = tid; q < c.r1; q += NT) {
      double acc = 0.0;
      for (int p = 0; p < c.r0; ++p) {
        double sm = 0.0;
        for (int i = 0; i < c.d; ++i) sm = __dadd_rn(sm, c.p[p + (size_t)c.r0 * (i + (size_t)c.d * q)]);
        acc = __dadd_rn(acc, __dmul_rn(v[p], sm));
      }
      w[q] = acc;
    }
    __syncthreads();
    double* t = v;
    v = w;
    w = t;
  }
  if (tid == 0) {
    tci_result_head* h = (tci_result_head*)(atw(resb, T.res));
    h->status = 0;
    h->npivot = 0;
    h->error = v[0];
  }
  __syncthreads();
}

// TABLE task: part0 over [lut_base0, lut_base0 + lutcap0) and scale1(part1)
// over [0, lutcap1) of the solve's f into T.lut -- the same functions the
// per-element path calls, so table entries equal direct evaluation bit for bit.
__device__ void task_table(const tci_task& T, const char* blob, char* resb) {
  const double* prm = (const double*)at(blob, T.params);
  for (int k = threadIdx.x; k < T.lutcap0; k += NT)
    T.lut[k] = tci_f_part0(T.fid, prm, T.nparams, (double)(T.lut_base0 + k));
  if (tci_f_tables(T.fid) > 1)
    for (int k = threadIdx.x; k < T.lutcap1; k += NT)
      T.lut[T.lutcap0 + k] = tci_f_scale1(T.fid, prm, tci_f_part1(T.fid, prm, (double)k));
  if (threadIdx.x == 0) {
    tci_result_head* h = (tci_result_head*)(atw(resb, T.res));
    h->status = 0;
    h->npivot = 0;
    h->lut_used = 1;
  }
  __syncthreads();
}

__device__ void run_task(const tci_task& T, const char* blob, char* resb, char* smem, Ctl& ctl,
                         size_t smem_bytes) {
  switch (T.kind) {
    case TCI_TASK_RRLU: task_rrlu(T, blob, resb, smem, ctl, smem_bytes); break;
    case TCI_TASK_SITE: task_site(T, blob, resb, smem, ctl, smem_bytes); break;
    case TCI_TASK_CORE: task_core(T, blob, resb, smem, ctl); break;
    case TCI_TASK_EVAL: task_eval(T, blob, resb, smem, ctl); break;
    case TCI_TASK_SUM: task_sum(T, blob, resb, smem); break;
    case TCI_TASK_SEARCH: task_search(T, blob, resb, smem); break;
    case TCI_TASK_TABLE: task_table(T, blob, resb); break;
    default: break;
  }
}

// cta_area: the global scratch of each CTA (cta_stride doubles apiece), reused
// by the CTA's successive tasks: the working matrix of a task too large for
// shared memory, then its per-task f tables (the host sized the stride for the
// largest task).
__global__ void __launch_bounds__(NT, TCI_CTAS_PER_SM)
    tci_step_kernel(const char* __restrict__ blob, char* __restrict__ resb, const int* __restrict__ order,
                    int ntasks, int* counter, size_t smem_bytes, double* cta_area, size_t cta_stride) {
  extern __shared__ __align__(16) char smem[];
  __shared__ Ctl ctl;
  const tci_task* tasks = (const tci_task*)blob;
  double* const area = cta_area + (size_t)blockIdx.x * cta_stride;
  for (;;) {
    if (threadIdx.x == 0) ctl.task = atomicAdd(counter, 1);
    __syncthreads();
    const int ti = ctl.task;
    __syncthreads();
    if (ti >= ntasks) break;
    tci_task T = tasks[order[ti]];
    size_t we = 0;
    if (T.smem_mode != 1) {
      we = tci_work_elems(&T);
      T.work = area;
    }
    if (!T.lut_full) T.lut = T.lutcap0 > 0 ? area + we : nullptr;
    const long long t0 = clock64();
    run_task(T, blob, resb, smem, ctl, smem_bytes);
    if (threadIdx.x == 0) ((tci_result_head*)(atw(resb, T.res)))->cycles = clock64() - t0;
  }
}

// ------------------------------------------------------------ resident kernel
// System-scope acquire / release on mapped host memory.
__device__ __forceinline__ uint64_t ld_acquire_sys(const uint64_t* p) {
  uint64_t v;
  asm volatile("ld.acquire.sys.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_sys(uint64_t* p, uint64_t v) {
  asm volatile("st.release.sys.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ uint64_t ld_acquire_gpu(const uint64_t* p) {
  uint64_t v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ int ld_acquire_gpu_s32(const int32_t* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void st_release_gpu(uint64_t* p, uint64_t v) {
  asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ void st_release_gpu_s32(int32_t* p, int v) {
  asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

constexpr int RES_MAX_PARAMS = 64;                          // params copied to shared memory
constexpr long long RES_MAX_POLLS = 1LL << 31;  // a worker's most polls of one ticket
constexpr int TASK_WORDS = (int)(sizeof(tci_task) / 8);
static_assert(sizeof(tci_task) % 8 == 0, "task record is a whole number of words");

// Warp 0 of CTA 0: move published host-ring descriptors, 32 at a time, into
// the device ring (in ticket order, while the device ring has room), mark the
// host slots free, publish the device tickets.  Leaves -- and tells the
// workers -- when the host asks to stop and nothing published is left, after
// qc->idle_us with nothing published, when a worker has reported a failed
// wait, or after wait_ns without room in the device ring.
__device__ void resident_dispatch(tci_queue_slot* __restrict__ hs, uint32_t hmask, tci_resident_state* st,
                                  tci_queue_ctl* qc, uint64_t wait_ns) {
  const int lane = threadIdx.x;
  unsigned long long pos = *(volatile unsigned long long*)&st->host_pos;
  unsigned long long k = 0;
  const uint64_t idle_ns = (uint64_t)(*(volatile int32_t*)&qc->idle_us) * 1000ull;
  uint64_t t_idle = global_ns();
  unsigned sleep_ns = 32;
  for (;;) {
    const unsigned long long hp = pos + lane, dk = k + lane;
    tci_queue_slot* h = &hs[hp & hmask];
    tci_queue_slot* d = &st->ring[dk & (TCI_DRING - 1)];
    const bool pub = ld_acquire_sys(&h->seq) == hp + 1;
    const bool room = dk < TCI_DRING || ld_acquire_gpu(&d->taken) == dk - TCI_DRING + 1;
    const unsigned okm = __ballot_sync(FULL, pub && room);
    const int p = okm == FULL ? 32 : __ffs(~okm) - 1;
    if (p > 0) {
      if (lane < p) {
        // all loads first (independent, uncached: one trip over the host link),
        // then the stores; ordered after this lane's acquire of `seq`
        const unsigned long long* src = (const unsigned long long*)&h->t;
        unsigned long long* dst = (unsigned long long*)&d->t;
        unsigned long long w[TASK_WORDS];
#pragma unroll
        for (int q = 0; q < TASK_WORDS; ++q) w[q] = __ldcv(src + q);
#pragma unroll
        for (int q = 0; q < TASK_WORDS; ++q) dst[q] = w[q];
        st_release_sys(&h->taken, hp + 1);
        st_release_gpu(&d->seq, dk + 1);
      }
      pos += p;
      k += p;
      if (lane == 0) *(volatile unsigned long long*)&st->host_pos = pos;
      t_idle = global_ns();
      sleep_ns = 32;
      continue;
    }
    int leave = 0;
    if (lane == 0) {
      const uint64_t waited = global_ns() - t_idle;
      if (!pub)  // nothing published: the host is done, quiet for too long, or a worker failed
        leave = (*(volatile int32_t*)&qc->stop != 0) || waited > idle_ns || (*(volatile int32_t*)&st->error != 0);
      else       // published but no room: the workers must free slots; they may have failed
        leave = (*(volatile int32_t*)&st->error != 0) || waited > wait_ns;
    }
    if (__shfl_sync(FULL, leave, 0)) break;
    __nanosleep(sleep_ns);
    sleep_ns = sleep_ns < 512 ? sleep_ns * 2 : 512;
  }
  __syncwarp();
  if (lane == 0) {
    *(volatile unsigned long long*)&st->count = k;
    st_release_gpu_s32(&st->stop, 1);
  }
}

// Persistent kernel of the resident mode (cooperative launch, one CTA per SM).
// CTA 0 hosts the dispatcher; every other CTA claims the next device ticket
// with one atomic, waits until it is dispatched (or the dispatcher has left:
// tickets past the last dispatched one are never used), runs the task and
// publishes the result record to the host.  A worker waits at most wait_ns for
// its ticket; then it sets st->error and every CTA leaves.
__global__ void __launch_bounds__(NT, TCI_CTAS_PER_SM)
    tci_resident_kernel(tci_queue_slot* __restrict__ hslots, uint32_t hmask, tci_resident_state* st,
                        tci_queue_ctl* qc, size_t smem_bytes, unsigned long long wait_ns) {
  if (blockIdx.x == 0) {
    if (threadIdx.x < 32) resident_dispatch(hslots, hmask, st, qc, wait_ns);
    return;
  }
  extern __shared__ __align__(16) char smem[];
  __shared__ Ctl ctl;
  __shared__ __align__(16) tci_task Ts;
  __shared__ double s_params[RES_MAX_PARAMS];
  __shared__ long long s_ticket;
  const int tid = threadIdx.x;
  for (;;) {
    if (tid == 0) {
      long long got = -1;
      const unsigned long long t = atomicAdd(&st->head, 1ull);
      tci_queue_slot* d = &st->ring[t & (TCI_DRING - 1)];
      const uint64_t t_begin = global_ns();
      unsigned sleep_ns = 32;
      for (long long it = 0;; ++it) {
        if (ld_acquire_gpu(&d->seq) == t + 1) {
          got = (long long)t;
          break;
        }
        if (ld_acquire_gpu_s32(&st->stop)) {  // every dispatch happened before the stop flag
          if (ld_acquire_gpu(&d->seq) == t + 1) got = (long long)t;
          break;
        }
        if (it >= RES_MAX_POLLS || global_ns() - t_begin > wait_ns) {
          atomicExch(&st->error, 1);
          break;
        }
        if (*(volatile int32_t*)&st->error) break;  // another wait has failed: leave too
        __nanosleep(sleep_ns);
        sleep_ns = sleep_ns < 256 ? sleep_ns * 2 : 256;
      }
      s_ticket = got;
    }
    __syncthreads();
    const long long ticket = s_ticket;
    if (ticket < 0) break;
    tci_queue_slot* d = &st->ring[(unsigned long long)ticket & (TCI_DRING - 1)];
    if (tid < TASK_WORDS) ((uint64_t*)&Ts)[tid] = ((const volatile uint64_t*)&d->t)[tid];
    __syncthreads();
    if (tid == 0) st_release_gpu(&d->taken, (uint64_t)ticket + 1);
    const long long t0 = clock64();
    size_t task_smem = smem_bytes;
    if (Ts.stage_bytes > 0) {
      // The record's input part (params, index lists, core table; 16-byte
      // multiple, 256-byte aligned block) to the top of shared memory, with
      // every thread's loads issued before its stores; pointers into it are
      // moved to the copy.
      const size_t sb = (size_t)Ts.stage_bytes;
      const char* base = (const char*)(uintptr_t)Ts.params;
      char* dst = smem + (smem_bytes - sb);
      const uint4* s4 = (const uint4*)base;
      uint4* d4 = (uint4*)dst;
      const int n4 = (int)(sb / 16);
      for (int k0 = tid; k0 < n4; k0 += 4 * NT) {
        uint4 v[4];
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (k0 + q * NT < n4) v[q] = s4[k0 + q * NT];
#pragma unroll
        for (int q = 0; q < 4; ++q)
          if (k0 + q * NT < n4) d4[k0 + q * NT] = v[q];
      }
      __syncthreads();
      if (tid == 0) {
        const uintptr_t lo = (uintptr_t)base, hi = lo + sb;
        auto move = [&](int64_t p) -> int64_t {
          const uintptr_t q = (uintptr_t)p;
          return (q >= lo && q < hi) ? (int64_t)(uintptr_t)(dst + (q - lo)) : p;
        };
        Ts.params = move(Ts.params);
        Ts.rows = move(Ts.rows);
        Ts.cols = move(Ts.cols);
        Ts.prows = move(Ts.prows);
        Ts.cores = move(Ts.cores);
        Ts.ain = (const double*)(uintptr_t)move((int64_t)(uintptr_t)Ts.ain);
      }
      task_smem = smem_bytes - sb;
      __syncthreads();
    }
    if (Ts.nparams <= RES_MAX_PARAMS) {  // f parameters are read per element: keep them on chip
      const double* src = (const double*)(uintptr_t)Ts.params;
      for (int k = tid; k < Ts.nparams; k += NT) s_params[k] = src[k];
    }
    __syncthreads();
    if (tid == 0 && Ts.nparams <= RES_MAX_PARAMS) Ts.params = (int64_t)(uintptr_t)s_params;
    __syncthreads();
    run_task(Ts, nullptr, nullptr, smem, ctl, task_smem);
    __syncthreads();
    if (tid == 0) {
      tci_result_head* h = (tci_result_head*)(uintptr_t)Ts.res;
      h->cycles = clock64() - t0;
      __threadfence_system();
      st_release_sys(&h->done, Ts.ticket + 1);
    }
  }
}

// ------------------------------------------------------------ multi-CTA rrLU
// One rank-revealing LU spread over every SM (cooperative launch) for matrices
// far larger than shared memory.  The CTAs form a Pr x Pc grid; CTA (p, q) owns
// the row block p x column block q of the working matrix.  Nothing moves: the
// row and column swaps of swaprow!/swapcol! (matrixlu.jl:98-112) are tracked as
// permutations (pos: physical -> logical position, stor: logical -> physical),
// and the argmax key of an element is (logical column << 16) | logical row, so
// ties break exactly as in the physically permuted matrix.  The scaling of
// addpivot! (matrixlu.jl:114-124) is applied where it is needed with the same
// operands: the update of step k uses x_i = A[i, C] / piv (leftorthogonal) or
// y_j = A[R, j] / piv, each CTA dividing the entries of its own rows / columns
// (the pivot row R and column C are stable after the barrier: they leave the
// trailing block), and the stored factors are divided the same way when they
// are written out.  Per pivot: every CTA reduces the G partial argmaxes (same
// result everywhere), takes the decision, forms its x and y slices, updates its
// block of the trailing matrix fused with its partial argmax, and meets the
// others at ONE grid barrier.  The arithmetic per element is the same
// __dmul_rn/__dsub_rn/__ddiv_rn sequence as rrlu_loop, so the factors are
// bit-identical.

struct BigBar {
  unsigned int count, gen;
  int error;
  unsigned int arrived;  // partials published so far (G per pivot step; never reset)
};
struct BigPartial {
  unsigned long long A, B;
  unsigned int k, ph;  // key and physical position (row | column << 16) of the maximum
  double v;            // the element at key k (the next pivot's value)
  unsigned int nan, pad;
};

// Running argmax of |v| with the value and physical position at its key (push
// in any key order).
struct BigTrack {
  uint64_t A, B;
  uint32_t k, ph;
  double v;
  __device__ __forceinline__ void init() {
    A = B = 0;
    k = 0xffffffffu;
    ph = 0;
    v = 0.0;
  }
  __device__ __forceinline__ void push(double x, uint32_t key, uint32_t phys) {
    uint64_t b = abs_bits(x);
    if (b > NAN_FLOOR) return;
    b += 1;
    if (b > A) {
      B = A;
      A = b;
      k = key;
      ph = phys;
      v = x;
    } else if (b == A) {
      if (key < k) {
        k = key;
        ph = phys;
        v = x;
      }
    } else if (b > B) {
      B = b;
    }
  }
};
__device__ __forceinline__ void big_combine(uint64_t& A, uint32_t& k, uint32_t& ph, uint64_t& B, double& v,
                                            uint64_t A2, uint32_t k2, uint32_t ph2, uint64_t B2, double v2) {
  if (A2 > A) {
    B = B2 > A ? B2 : A;
    A = A2;
    k = k2;
    ph = ph2;
    v = v2;
  } else if (A2 == A) {
    B = B2 > B ? B2 : B;
    if (k2 < k) {
      k = k2;
      ph = ph2;
      v = v2;
    }
  } else if (A2 > B) {
    B = A2;
  }
}

// warp_track with the winner's physical position and value (from the first lane
// that holds the winning key); every lane gets the result.  Same result as
// folding big_combine over the lanes.
__device__ __forceinline__ void warp_track5(uint64_t& A, uint32_t& k, uint32_t& ph, uint64_t& B, double& v) {
  const uint64_t Am = warp_max_u64(A);
  const uint32_t km = __reduce_min_sync(FULL, A == Am ? k : 0xffffffffu);
  const int src = __ffs(__ballot_sync(FULL, A == Am && k == km)) - 1;
  B = warp_max_u64(A == Am ? B : A);
  ph = __shfl_sync(FULL, ph, src);
  v = __shfl_sync(FULL, v, src);
  A = Am;
  k = km;
}

__device__ __forceinline__ unsigned ld_acquire_gpu_u32(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void red_release_gpu_add_u32(unsigned* p, unsigned v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

constexpr long long BIG_BAR_POLLS = 1LL << 24;  // bounded wait of one grid barrier (a few seconds)

// Grid-wide barrier (sense by generation).  Returns false once any CTA has hit
// the wait bound; every CTA then leaves the factorization.
__device__ bool big_barrier(BigBar* bar, unsigned nblocks, unsigned& gen, BigCtl& ctl) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned g = gen;
    if (atomicAdd(&bar->count, 1u) == nblocks - 1) {
      atomicExch(&bar->count, 0u);
      __threadfence();
      atomicExch(&bar->gen, g + 1);
    } else {
      unsigned sleep_ns = 32;
      for (long long it = 0; ld_acquire_gpu_u32(&bar->gen) == g; ++it) {
        if (it > BIG_BAR_POLLS || *(volatile int*)&bar->error) {
          atomicExch(&bar->error, 1);
          break;
        }
        __nanosleep(sleep_ns);
        sleep_ns = sleep_ns < 128 ? sleep_ns * 2 : 128;
      }
    }
    gen = g + 1;
    ctl.bar_err = *(volatile int*)&bar->error;
  }
  __syncthreads();
  return ctl.bar_err == 0;
}

// Block reduction of every thread's BigTrack; every thread gets the result.
// Ends with a barrier.
__device__ void block_track(BigTrack& t, BigCtl& ctl) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint64_t a = t.A, b = t.B;
  uint32_t kk = t.k, ph = t.ph;
  double v = t.v;
  warp_track5(a, kk, ph, b, v);
  if (lane == 0) {
    ctl.red_u[warp] = a;
    ctl.red_b[warp] = b;
    ctl.red_k[warp] = (int)kk;
    ctl.red_p[warp] = ph;
    ctl.red_s[warp] = v;
  }
  __syncthreads();
  if (warp == 0) {
    a = lane < BIG_NW ? ctl.red_u[lane] : 0ULL;
    b = lane < BIG_NW ? ctl.red_b[lane] : 0ULL;
    kk = lane < BIG_NW ? (uint32_t)ctl.red_k[lane] : 0xffffffffu;
    ph = lane < BIG_NW ? ctl.red_p[lane] : 0u;
    v = lane < BIG_NW ? ctl.red_s[lane] : 0.0;
    warp_track5(a, kk, ph, b, v);
    if (lane == 0) {
      ctl.red_u[BIG_NW] = a;
      ctl.red_b[BIG_NW] = b;
      ctl.red_k[BIG_NW] = (int)kk;
      ctl.red_p[BIG_NW] = ph;
      ctl.red_s[BIG_NW] = v;
    }
  }
  __syncthreads();
  t.A = ctl.red_u[BIG_NW];
  t.B = ctl.red_b[BIG_NW];
  t.k = (uint32_t)ctl.red_k[BIG_NW];
  t.ph = ctl.red_p[BIG_NW];
  t.v = ctl.red_s[BIG_NW];
  __syncthreads();
}

// Block reduction of every thread's BigTrack into thread 0's (the others keep
// partial values).  One CTA barrier; the caller's next barrier orders the reuse
// of the staging slots.
__device__ void block_track_to0(BigTrack& t, BigCtl& ctl) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint64_t a = t.A, b = t.B;
  uint32_t kk = t.k, ph = t.ph;
  double v = t.v;
  warp_track5(a, kk, ph, b, v);
  if (lane == 0) {
    ctl.red_u[warp] = a;
    ctl.red_b[warp] = b;
    ctl.red_k[warp] = (int)kk;
    ctl.red_p[warp] = ph;
    ctl.red_s[warp] = v;
  }
  __syncthreads();
  if (warp == 0) {
    a = lane < BIG_NW ? ctl.red_u[lane] : 0ULL;
    b = lane < BIG_NW ? ctl.red_b[lane] : 0ULL;
    kk = lane < BIG_NW ? (uint32_t)ctl.red_k[lane] : 0xffffffffu;
    ph = lane < BIG_NW ? ctl.red_p[lane] : 0u;
    v = lane < BIG_NW ? ctl.red_s[lane] : 0.0;
    warp_track5(a, kk, ph, b, v);
    t.A = a;
    t.B = b;
    t.k = kk;
    t.ph = ph;
    t.v = v;
  }
}

// Publish this CTA's partial (one thread, after a CTA barrier that follows the
// CTA's update): the fields, then one arrival on the grid's counter with release
// semantics (cumulative: it also covers the other threads' update writes, which
// the CTA barrier ordered before it), so that a CTA that sees the count with
// acquire also sees the partial and the update.  The arrival is a reduction (no
// round trip).
__device__ __forceinline__ void big_publish(BigPartial& o, const BigTrack& t, BigBar* bar) {
  o.A = t.A;
  o.B = t.B;
  o.k = t.k;
  o.ph = t.ph;
  o.v = t.v;
  red_release_gpu_add_u32(&bar->arrived, 1u);
}

// Partials one lane of the gathering warp loads at once, and the most it handles
// (grids of up to 320 CTAs).
constexpr int BIG_GATHER_Q = 5;
constexpr int BIG_GATHER_MAX = 2 * BIG_GATHER_Q;

// Warp 0: wait until `target` partials have arrived in all (lane 0 polls the
// counter, bounded), then combine the G partials of this step, every lane
// loading its share at once; every lane gets the result.  This wait is the pivot
// step's only grid-wide synchronisation: a CTA publishes after its update, so
// once all G are in, every update of the step is done and visible.  Returns
// false if the wait hit its bound or another CTA has flagged an error (the flag
// is then set).
__device__ bool big_gather(const BigPartial* cur, int G, unsigned target, BigBar* bar, BigTrack& g) {
  const int lane = threadIdx.x & 31;
  g.init();
  int ok = 1;
  if (lane == 0) {
    unsigned sleep_ns = 16;
    for (long long it = 0; ld_acquire_gpu_u32(&bar->arrived) < target; ++it) {
      if (it > BIG_BAR_POLLS || *(volatile int*)&bar->error) {
        atomicExch(&bar->error, 1);
        ok = 0;
        break;
      }
      __nanosleep(sleep_ns);
      sleep_ns = sleep_ns < 64 ? sleep_ns * 2 : 64;
    }
  }
  ok = __shfl_sync(FULL, ok, 0);
  __syncwarp();  // lane 0's acquire orders the warp's loads below
  for (int base = 0; ok && base < G; base += 32 * BIG_GATHER_Q) {
    uint64_t qa[BIG_GATHER_Q], qb[BIG_GATHER_Q];
    uint32_t qk[BIG_GATHER_Q], qp[BIG_GATHER_Q];
    double qv[BIG_GATHER_Q];
#pragma unroll
    for (int q = 0; q < BIG_GATHER_Q; ++q) {
      if (base + lane + 32 * q < G) {
        const BigPartial* p = cur + base + lane + 32 * q;
        qa[q] = __ldcg(&p->A);
        qb[q] = __ldcg(&p->B);
        qk[q] = __ldcg(&p->k);
        qp[q] = __ldcg(&p->ph);
        qv[q] = __ldcg(&p->v);
      }
    }
#pragma unroll
    for (int q = 0; q < BIG_GATHER_Q; ++q)
      if (base + lane + 32 * q < G) big_combine(g.A, g.k, g.ph, g.B, g.v, qa[q], qk[q], qp[q], qb[q], qv[q]);
  }
  uint64_t a = g.A, b = g.B;
  uint32_t kk = g.k, ph = g.ph;
  double v = g.v;
  warp_track5(a, kk, ph, b, v);
  g.A = __shfl_sync(FULL, a, 0);
  g.B = __shfl_sync(FULL, b, 0);
  g.k = __shfl_sync(FULL, kk, 0);
  g.ph = __shfl_sync(FULL, ph, 0);
  g.v = __shfl_sync(FULL, v, 0);
  return ok != 0;
}

struct BigArgs {
  const double* ain;      // m x n input (column-major)
  double* A;              // m x n working copy (physical positions never change)
  double* fact;           // m x n factors in logical order, then int32 rowperm[m], colperm[n]
  char* res;              // result record (tci_result_head, rowp[kcap], colp[kcap], diag[kcap])
  BigPartial* parts;      // 2 x gridDim.x partials (double-buffered by pivot parity)
  double* pivs;           // signed pivot of every step (kmax)
  BigBar* bar;
  int m, n, kmax, kcap, leftorth;
  int pr, pc, mb, nb;     // CTA grid and block sizes
  double reltol, abstol;
};

__global__ void __launch_bounds__(BIG_NT, 1) rrlu_big_kernel(BigArgs P) {
  extern __shared__ __align__(16) char smem[];
  __shared__ BigCtl ctl;
  const int tid = threadIdx.x, G = gridDim.x, b = blockIdx.x, m = P.m, n = P.n;
  const bool leftorth = P.leftorth != 0;
  const int r0 = (b / P.pc) * P.mb, c0 = (b % P.pc) * P.nb;
  const int r1 = min(m, r0 + P.mb), c1 = min(n, c0 + P.nb);
  const int nrb = max(0, r1 - r0), ncb = max(0, c1 - c0);  // block extent
  double* xs = (double*)smem;          // x of the active rows (mb)
  double* ys = xs + P.mb;              // y of the active columns (nb)
  int* pos_r = (int*)(ys + P.nb);      // physical row -> logical (m)
  int* stor_r = pos_r + m;             // logical row -> physical (m)
  int* pos_c = stor_r + m;             // (n)
  int* stor_c = pos_c + n;             // (n)
  int* act_r = stor_c + n;             // active rows of the block, and the slot of each (mb each)
  int* slot_r = act_r + P.mb;
  int* act_c = slot_r + P.mb;          // (nb each)
  int* slot_c = act_c + P.nb;
  unsigned gen = 0;
  for (int i = tid; i < m; i += BIG_NT) pos_r[i] = stor_r[i] = i;
  for (int j = tid; j < n; j += BIG_NT) pos_c[j] = stor_c[j] = j;
  for (int t = tid; t < nrb; t += BIG_NT) act_r[t] = slot_r[t] = t;  // local indices
  for (int u = tid; u < ncb; u += BIG_NT) act_c[u] = slot_c[u] = u;
  if (tid == 0) {
    ctl.maxerror = 0.0;
    ctl.err = __longlong_as_double(0x7ff8000000000000LL);
    ctl.stop = 0;
    ctl.r = nrb;  // active row / column counts
    ctl.c = ncb;
  }
  // copy own block, first argmax
  BigTrack bt;
  bt.init();
  {
    const long long tot = (long long)nrb * ncb;
    for (long long e = tid; e < tot; e += BIG_NT) {
      const int i = r0 + (int)(e % nrb), j = c0 + (int)(e / nrb);
      const double v = P.ain[i + (size_t)j * m];
      P.A[i + (size_t)j * m] = v;
      bt.push(v, pack_key(i, j), pack_key(i, j));
    }
  }
  block_track(bt, ctl);
  if (tid == 0) big_publish(P.parts[b], bt, P.bar);  // buffer 0: read at pivot 0
  bool ok = true;
  int K = 0;
  tci_result_head* head = (tci_result_head*)P.res;
  const int kcap = P.kcap;
  int* rowp = (int*)(P.res + sizeof(tci_result_head));
  int* colp = (int*)(P.res + sizeof(tci_result_head) + align_up((size_t)kcap * 4, 8));
  double* diag = (double*)(P.res + sizeof(tci_result_head) + 2 * align_up((size_t)kcap * 4, 8));
  // Decision of pivot step K (every CTA takes the same one), by one thread: the
  // error, the stopping rule, swaprow!(K, rl) / swapcol!(K, cl) on the maps, and
  // the pivot row and column leaving this block's active sets.
  auto decide = [&]() {
    const unsigned key = (unsigned)ctl.K, ph = (unsigned)ctl.kmax;
    const int rl = (int)(key & 0xffffu), cl = (int)(key >> 16);
    const int R = (int)(ph & 0xffffu), Cc = (int)(ph >> 16);
    const double piv = ctl.piv;
    const double e = fabs(piv);
    ctl.err = e;
    ctl.stop = ((e < P.reltol * ctl.maxerror || e < P.abstol) && K > 0) ? 1 : 0;
    if (!ctl.stop) {
      ctl.maxerror = jmax(ctl.maxerror, e);
      if (b == 0) {
        diag[K] = e;
        P.pivs[K] = piv;
      }
      // swaprow!(K, rl), swapcol!(K, cl) on the maps
      const int sr = stor_r[K];
      stor_r[K] = R;
      stor_r[rl] = sr;
      pos_r[R] = K;
      pos_r[sr] = rl;
      const int sc = stor_c[K];
      stor_c[K] = Cc;
      stor_c[cl] = sc;
      pos_c[Cc] = K;
      pos_c[sc] = cl;
      // the pivot row and column leave this block's active sets
      if (R >= r0 && R < r1) {
        const int s = slot_r[R - r0], last = act_r[ctl.r - 1];
        act_r[s] = last;
        slot_r[last] = s;
        ctl.r -= 1;
      }
      if (Cc >= c0 && Cc < c1) {
        const int s = slot_c[Cc - c0], last = act_c[ctl.c - 1];
        act_c[s] = last;
        slot_c[last] = s;
        ctl.c -= 1;
      }
    }
  };
  while (ok) {
    // the partials of pivot K are in buffer K & 1: a CTA writes the next set to
    // the other buffer, so a fast CTA never overwrites what a slow one reads
    BigPartial* const cur = P.parts + (size_t)(K & 1) * G;
    // ---- the pivot: argmax of abs2 over the trailing block, from the G partials
    // (warp 0 waits for them); unless the exact pass is needed, lane 0 also takes
    // the decision
    if (tid < 32) {
      BigTrack g;
      const bool got = big_gather(cur, G, (unsigned)(K + 1) * (unsigned)G, P.bar, g);
      if (tid == 0) {
        ctl.bar_err = got ? 0 : 1;
        if (got) {
          const uint64_t Mstar = g.A ? g.A - 1 : 0;
          const bool safe = Mstar >= SQ_SMALL && Mstar < SQ_BIG;
          const bool close = g.B != 0 && (g.B - 1) + 16 >= Mstar;
          ctl.red_u[BIG_NW] = Mstar;
          ctl.need_exact = (g.A != 0 && !(safe && !close)) ? 1 : 0;
          if (g.A == 0) {  // every element NaN: the scan keeps its start
            ctl.kmax = (int)(((unsigned)stor_c[K] << 16) | (unsigned)stor_r[K]);
            ctl.K = (K << 16) | K;
            ctl.piv = __ldcg(&P.A[stor_r[K] + (size_t)stor_c[K] * m]);
          } else {
            ctl.kmax = (int)g.ph;
            ctl.K = (int)g.k;
            ctl.piv = g.v;
          }
          if (!ctl.need_exact) decide();
        }
      }
    }
    __syncthreads();
    if (ctl.bar_err) {
      ok = false;
      break;
    }
    if (ctl.need_exact) {  // squares of the elements near the maximum (rare)
      const uint64_t Mstar = ctl.red_u[BIG_NW];
      const int nr = ctl.r, nc = ctl.c;
      ArgBest ab;
      ab.init();
      uint32_t abph = 0;
      for (long long e = tid; e < (long long)nr * nc; e += BIG_NT) {
        const int i = r0 + act_r[(int)(e % nr)], j = c0 + act_c[(int)(e / nr)];
        const double v = P.A[i + (size_t)j * m];
        if (near_max(abs_bits(v), Mstar)) {
          const uint32_t key = pack_key(pos_r[i], pos_c[j]);
          const uint64_t q = (uint64_t)__double_as_longlong(__dmul_rn(v, v)) + 1;
          if (q > ab.s || (q == ab.s && key < ab.key)) {
            ab.s = q;
            ab.key = key;
            ab.val = v;
            abph = pack_key(i, j);
          }
        }
      }
      BigTrack et;
      et.A = ab.s;
      et.B = 0;
      et.k = ab.key;
      et.ph = abph;
      et.v = ab.val;
      ok = big_barrier(P.bar, G, gen, ctl);  // everyone has read the partials
      if (!ok) break;
      block_track(et, ctl);
      if (tid == 0) {
        BigPartial& o = cur[b];
        o.A = et.A;
        o.B = 0;
        o.k = et.k;
        o.ph = et.ph;
        o.v = et.v;
      }
      ok = big_barrier(P.bar, G, gen, ctl);
      if (!ok) break;
      BigTrack g;
      g.init();
      for (int t = tid; t < G; t += BIG_NT) {
        const BigPartial* q = cur + t;
        big_combine(g.A, g.k, g.ph, g.B, g.v, __ldcg(&q->A), __ldcg(&q->k), __ldcg(&q->ph), __ldcg(&q->B),
                    __ldcg(&q->v));
      }
      block_track(g, ctl);
      if (tid == 0) {
        if (g.A) {
          ctl.kmax = (int)g.ph;
          ctl.K = (int)g.k;
          ctl.piv = g.v;
        }
        decide();
      }
      __syncthreads();
    }
    const int R = (int)((unsigned)ctl.kmax & 0xffffu), Cc = (int)((unsigned)ctl.kmax >> 16);
    const double piv = ctl.piv;
    if (ctl.stop) break;
    ++K;
    if (K == P.kmax) break;  // the trailing update after the last pivot is not observable
    // ---- x (pivot column) for the active rows, y (pivot row) for the active columns
    // (one element per thread: the x and y entries on different threads)
    const int nr = ctl.r, nc = ctl.c;
    for (int t = tid; t < nr + nc; t += BIG_NT) {
      if (t < nr) {
        const double v = __ldcg(&P.A[r0 + act_r[t] + (size_t)Cc * m]);
        xs[t] = leftorth ? __ddiv_rn(v, piv) : v;
      } else {
        const int u = t - nr;
        const double v = __ldcg(&P.A[R + (size_t)(c0 + act_c[u]) * m]);
        ys[u] = leftorth ? v : __ddiv_rn(v, piv);
      }
    }
    __syncthreads();
    // ---- rank-1 update of the block's active part, fused with its argmax.
    // Four elements per step with their loads issued first (four L2 reads in
    // flight per thread); the columns are walked in reverse on odd pivots, so
    // the part of the block the last pass touched last is still in L1.
    bt.init();
    if (nr > 0 && nc > 0) {
      const long long tot = (long long)nr * nc;
      const int sq = BIG_NT / nr, sr = BIG_NT % nr;
      const bool rev = (K & 1) != 0;
      int tt = tid % nr, uu = tid / nr;
      long long e = tid;
      for (; e + 3LL * BIG_NT < tot; e += 4LL * BIG_NT) {
        int ti[4], ui[4];
        double* ap[4];
        double av[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          ti[q] = tt;
          ui[q] = rev ? nc - 1 - uu : uu;
          ap[q] = P.A + (r0 + act_r[ti[q]]) + (size_t)(c0 + act_c[ui[q]]) * m;
          tt += sr;
          uu += sq;
          if (tt >= nr) {
            tt -= nr;
            uu += 1;
          }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) av[q] = *ap[q];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
          const double v = __dsub_rn(av[q], __dmul_rn(xs[ti[q]], ys[ui[q]]));
          *ap[q] = v;
          const int i = r0 + act_r[ti[q]], j = c0 + act_c[ui[q]];
          bt.push(v, pack_key(pos_r[i], pos_c[j]), pack_key(i, j));
        }
      }
      for (; e < tot; e += BIG_NT) {
        const int u = rev ? nc - 1 - uu : uu;
        const int i = r0 + act_r[tt], j = c0 + act_c[u];
        double* a = P.A + i + (size_t)j * m;
        const double v = __dsub_rn(*a, __dmul_rn(xs[tt], ys[u]));
        *a = v;
        bt.push(v, pack_key(pos_r[i], pos_c[j]), pack_key(i, j));
        tt += sr;
        uu += sq;
        if (tt >= nr) {
          tt -= nr;
          uu += 1;
        }
      }
    }
    block_track_to0(bt, ctl);
    // read at pivot K (already incremented); no grid barrier: the next gather
    // waits for every CTA's partial
    if (tid == 0) big_publish(P.parts[(size_t)(K & 1) * G + b], bt, P.bar);
  }
  if (ok) ok = big_barrier(P.bar, G, gen, ctl);  // every pivot value is recorded
  if (!ok) {
    if (b == 0 && tid == 0) head->status = TCI_ST_TOO_LARGE;
    return;
  }
  // ---- the factors in logical order, with the deferred scaling of addpivot!,
  // and the NaN scan of L and U (matrixlu.jl:162-169)
  int bad = 0;
  {
    const long long tot = (long long)nrb * ncb;
    for (long long e = tid; e < tot; e += BIG_NT) {
      const int i = r0 + (int)(e % nrb), j = c0 + (int)(e / nrb);
      const int lr = pos_r[i], lc = pos_c[j];
      double v = P.A[i + (size_t)j * m];
      if (leftorth && lc < K && lr > lc) v = __ddiv_rn(v, __ldcg(&P.pivs[lc]));
      if (!leftorth && lr < K && lc > lr) v = __ddiv_rn(v, __ldcg(&P.pivs[lr]));
      const bool inL = lc < K && lr >= lc;
      const bool inU = lr < K && lr <= lc;
      if ((inL || inU) && is_nan_bits(v)) bad = 1;
      P.fact[lr + (size_t)lc * m] = v;
    }
  }
  bad = __syncthreads_or(bad);
  if (tid == 0) P.parts[b].nan = bad;
  ok = big_barrier(P.bar, G, gen, ctl);
  if (!ok) {
    if (b == 0 && tid == 0) head->status = TCI_ST_TOO_LARGE;
    return;
  }
  if (b == 0) {
    int nan = 0;
    for (int t = tid; t < G; t += BIG_NT) nan |= (int)__ldcg(&P.parts[t].nan);
    nan = __syncthreads_or(nan);
    int* fr = (int*)(P.fact + (size_t)m * n);
    for (int i = tid; i < m; i += BIG_NT) fr[i] = stor_r[i];
    for (int j = tid; j < n; j += BIG_NT) fr[m + j] = stor_c[j];
    for (int q = tid; q < K; q += BIG_NT) {
      rowp[q] = stor_r[q];
      colp[q] = stor_c[q];
    }
    if (tid == 0) {
      head->status = nan ? TCI_ST_NAN : 0;
      head->npivot = K;
      head->error = K >= min(m, n) ? 0.0 : ctl.err;
      head->maxabs = 0.0;
      head->maxabs_nan = 0;
      head->lut_used = 0;
    }
  }
}

}  // namespace

// Shared-memory budget of one CTA of the step kernel.
size_t tci_step_smem_bytes() {
  // 228 KB per SM, 1 KB reserved per CTA, ~2 KB of static shared memory per CTA
  return (size_t)(228 * 1024) / TCI_CTAS_PER_SM - 3 * 1024 - 1024 * (TCI_CTAS_PER_SM - 1);
}

// Dynamic shared memory of the resident kernel (its static shared memory holds
// the task record and the f parameters as well).
size_t tci_resident_smem_bytes() { return tci_step_smem_bytes(); }

// Dynamic shared memory of one multi-CTA rrLU CTA (one per SM).
size_t tci_big_smem_limit() { return (size_t)(228 * 1024) - 3 * 1024; }

cudaError_t tci_step_configure() {
  cudaError_t e = cudaFuncSetAttribute(tci_step_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)tci_step_smem_bytes());
  if (e != cudaSuccess) return e;
  e = cudaFuncSetAttribute(tci_resident_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)tci_resident_smem_bytes());
  if (e != cudaSuccess) return e;
  return cudaFuncSetAttribute(rrlu_big_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              (int)tci_big_smem_limit());
}

// Multi-CTA rrLU (rrlu_big_kernel).  The CTA grid: pr x pc <= G CTAs with the
// largest count, then the most square blocks.  Shared memory per CTA: both
// permutation maps (8 (m + n) bytes) and, per block row / column, x or y, the
// active list and the slot map (16 bytes each).
namespace {
struct BigGrid {
  int pr, pc, mb, nb;
};
// G: the task kernels' grid (TCI_CTAS_PER_SM per SM); the multi-CTA rrLU runs
// one CTA per SM.
BigGrid big_grid(int64_t m, int64_t n, int G) {
  G = std::max(1, G / TCI_CTAS_PER_SM);
  G = std::min(G, 32 * BIG_GATHER_MAX);  // one gathering warp reads every partial
  BigGrid best{1, 1, (int)m, (int)n};
  double best_score = -1.0;
  for (int pr = 1; pr <= G; ++pr) {
    const int pc = G / pr;
    if (pr > m || pc > n || pc < 1) continue;
    const int mb = (int)((m + pr - 1) / pr), nb = (int)((n + pc - 1) / pc);
    const double aspect = (double)mb / nb;
    const double score = (double)pr * pc - 1e-3 * std::fabs(std::log(aspect));
    if (score > best_score) {
      best_score = score;
      best = BigGrid{pr, pc, mb, nb};
    }
  }
  return best;
}
}  // namespace
size_t tci_rrlu_big_smem(int64_t m, int64_t n, int G) {
  const BigGrid g = big_grid(m, n, G);
  return (size_t)(8 * (m + n) + 16 * ((int64_t)g.mb + g.nb) + 64);
}
bool tci_rrlu_big_fits(int64_t m, int64_t n, int G) {
  return m >= 1 && n >= 1 && m <= 65535 && n <= 65535 && tci_rrlu_big_smem(m, n, G) <= tci_big_smem_limit();
}
size_t tci_rrlu_big_scratch_bytes(int grid, int kmax) {
  return 64 + 2 * (size_t)grid * sizeof(BigPartial) + (size_t)std::max(kmax, 1) * sizeof(double);
}

// Launch on up to `grid` CTAs (all co-resident: cooperative launch).  scratch
// holds the grid barrier, the partials and the pivot values
// (tci_rrlu_big_scratch_bytes); it is cleared here.  res is a device result
// record with room for kcap pivots.
cudaError_t tci_rrlu_big_launch(const double* ain, double* work, double* fact, char* res, void* scratch, int m,
                                int n, int kmax, int kcap, int leftorth, double reltol, double abstol, int grid,
                                cudaStream_t stream) {
  cudaError_t e = cudaMemsetAsync(scratch, 0, tci_rrlu_big_scratch_bytes(grid, kmax), stream);
  if (e != cudaSuccess) return e;
  const BigGrid g = big_grid(m, n, grid);
  BigArgs a;
  a.ain = ain;
  a.A = work;
  a.fact = fact;
  a.res = res;
  a.bar = (BigBar*)scratch;
  a.parts = (BigPartial*)((char*)scratch + 64);
  a.pivs = (double*)((char*)scratch + 64 + 2 * (size_t)grid * sizeof(BigPartial));
  a.m = m;
  a.n = n;
  a.kmax = kmax;
  a.kcap = kcap;
  a.leftorth = leftorth;
  a.pr = g.pr;
  a.pc = g.pc;
  a.mb = g.mb;
  a.nb = g.nb;
  a.reltol = reltol;
  a.abstol = abstol;
  // Most of the SM's on-chip memory as L1 (the CTA's block of the working matrix
  // is re-read every pivot), but enough shared memory for the CTAs that share
  // an SM: the carveout is what the occupancy of a cooperative launch is
  // computed with.
  const size_t smem = tci_rrlu_big_smem(m, n, grid);
  const int nsm = std::max(1, grid / TCI_CTAS_PER_SM);
  const int per_sm = (g.pr * g.pc + nsm - 1) / nsm;
  const double need = (double)per_sm * (double)(smem + 3 * 1024) / (228.0 * 1024.0);
  const int pct = std::min(100, std::max(25, (int)std::ceil(100.0 * need)));
  static int carve = -1;
  if (pct != carve) {
    e = cudaFuncSetAttribute((const void*)rrlu_big_kernel, cudaFuncAttributePreferredSharedMemoryCarveout, pct);
    if (e != cudaSuccess) return e;
    carve = pct;
  }
  void* args[] = {(void*)&a};
  return cudaLaunchCooperativeKernel((const void*)rrlu_big_kernel, dim3(g.pr * g.pc), dim3(BIG_NT), args, smem,
                                     stream);
}

// Launch the resident kernel: one CTA per SM, all resident at once
// (cooperative launch), after clearing the per-launch part of its state.
// slots/qc are mapped pinned host memory, st device memory.
cudaError_t tci_resident_launch(tci_queue_slot* slots, uint32_t mask, tci_resident_state* st, tci_queue_ctl* qc,
                                int grid, unsigned long long wait_ns, cudaStream_t stream) {
  const size_t off = offsetof(tci_resident_state, count);
  cudaError_t e = cudaMemsetAsync((char*)st + off, 0, sizeof(tci_resident_state) - off, stream);
  if (e != cudaSuccess) return e;
  size_t smem = tci_resident_smem_bytes();
  void* args[] = {(void*)&slots, (void*)&mask, (void*)&st, (void*)&qc, (void*)&smem, (void*)&wait_ns};
  return cudaLaunchCooperativeKernel((const void*)tci_resident_kernel, dim3(grid), dim3(NT), args, smem, stream);
}

// Launch one step.  counter must be zero (the launcher clears it on the stream).
cudaError_t tci_step_launch(const char* blob_dev, char* res_dev, const int* order_dev, int ntasks,
                            int* counter_dev, int grid, double* cta_area, size_t cta_stride, cudaStream_t stream) {
  cudaError_t e = cudaMemsetAsync(counter_dev, 0, sizeof(int), stream);
  if (e != cudaSuccess) return e;
  tci_step_kernel<<<grid, NT, tci_step_smem_bytes(), stream>>>(blob_dev, res_dev, order_dev, ntasks,
                                                              counter_dev, tci_step_smem_bytes(), cta_area,
                                                              cta_stride);
  return cudaGetLastError();
}

extern const tci_kernel_set kernels = {TCI_STEP_THREADS, TCI_CTAS_PER_SM, tci_step_smem_bytes,
                                       tci_resident_smem_bytes, tci_step_configure, tci_step_launch,
                                       tci_resident_launch};

}  // namespace TCI_KNS

// The entry point without allocation is built once (in the throughput variant).
#ifndef TCI_SECONDARY

// ===================================================================== rrLU
// without allocation (tci_rrlu_noalloc; no counterpart in the reference).
//
// Some callers cannot let the library allocate device memory: latency-critical
// serving loops where a cudaMalloc/cudaFree would stall the device, and hosts
// that own every device buffer through their own allocator (a Julia GPU array
// pool, a framework arena).  This entry point runs the same rank-revealing LU as the
// step kernel's RRLU task on caller-owned device buffers and keeps its working
// copy of the matrix, the factors and the result record in the fixed array
// below.  The array lives in every GPU that loads the library until the
// process exits.  Calls share it, so two calls that overlap on the GPU (on
// different streams, or interleaved with no ordering) race on it; calls issued
// on one stream are ordered and safe.  Nothing in it needs clearing between
// calls: every element a call reads is written earlier in the same call.
#include <mutex>
#include <string>

// error codes of include/tci_gb300.h (that header's function ids clash with
// tci_functions.h, so it is not included here)
#define TCI_ERR_ARG 1
#define TCI_ERR_NAN 3
#define TCI_ERR_CUDA 6

namespace tci {
void set_error(int code, const std::string& msg);
}

namespace TCI_KNS {
namespace {

constexpr int64_t NOALLOC_MAX_ELEMS = (int64_t)1 << 19;  // m * n
constexpr int64_t NOALLOC_MAX_DIM = 16384;               // m and n
// working matrix | factors + full permutations | result record
constexpr int64_t NOALLOC_FACT_DOUBLES = NOALLOC_MAX_ELEMS + NOALLOC_MAX_DIM;
constexpr int64_t NOALLOC_RES_DOUBLES = 16 + 2 * NOALLOC_MAX_DIM;
constexpr int64_t NOALLOC_SCRATCH_DOUBLES = NOALLOC_MAX_ELEMS + NOALLOC_FACT_DOUBLES + NOALLOC_RES_DOUBLES;

static __device__ __align__(256) double g_noalloc_scratch[NOALLOC_SCRATCH_DOUBLES];

__global__ void __launch_bounds__(NT, TCI_CTAS_PER_SM) rrlu_noalloc_kernel(const tci_task T, char* resb) {
  extern __shared__ __align__(16) char smem[];
  __shared__ Ctl ctl;
  task_rrlu(T, nullptr, resb, smem, ctl, 0);
}

// Copies the result record and the factors from the scratch array to the
// caller's buffers; *status = TCI_ERR_NAN when L or U holds a NaN (the
// reference's ErrorException "lu.L contains NaNs", matrixlu.jl:164-169), else 0.
__global__ void rrlu_noalloc_epilogue(const double* fact, const char* resb, int m, int n, int32_t* rowperm,
                                      int32_t* colperm, int32_t* npivot, double* error, int32_t* status,
                                      double* factors_out) {
  const tci_result_head* h = (const tci_result_head*)resb;
  const int32_t* perms = (const int32_t*)(fact + (size_t)m * n);
  const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
  for (int i = tid; i < m; i += nth) rowperm[i] = perms[i];
  for (int j = tid; j < n; j += nth) colperm[j] = perms[m + j];
  if (factors_out)
    for (int64_t e = tid; e < (int64_t)m * n; e += nth) factors_out[e] = fact[e];
  if (tid == 0) {
    *npivot = h->npivot;
    *error = h->error;
    *status = (h->status & TCI_ST_NAN) ? TCI_ERR_NAN : 0;
  }
}

struct NoallocDevice {
  bool ready = false;
  double* scratch = nullptr;  // device address of g_noalloc_scratch
};

}  // namespace
}  // namespace TCI_KNS

// See include/tci_gb300.h.  The first call on a device resolves the device
// address of the scratch array (cudaGetSymbolAddress) and raises the kernel's
// shared-memory limit, with that device current; make that first call before
// any stream capture.  Later calls only launch two kernels on `stream_u`.  The
// address is cached per device for the life of the process, so a device reset
// (cudaDeviceReset) after the first call is not supported.
extern "C" int tci_rrlu_noalloc(const double* A_dev, int64_t m, int64_t n, int64_t maxrank, double reltol,
                                double abstol, int32_t leftorthogonal, int32_t* rowperm_dev, int32_t* colperm_dev,
                                int32_t* npivot_dev, double* error_dev, int32_t* status_dev, double* factors_dev,
                                uintptr_t stream_u) {
  using namespace TCI_KNS;
  static std::mutex mu;
  static NoallocDevice devs[64];
  if (m < 1 || n < 1 || m > NOALLOC_MAX_DIM || n > NOALLOC_MAX_DIM || m * n > NOALLOC_MAX_ELEMS) {
    tci::set_error(TCI_ERR_ARG, "tci_rrlu_noalloc: matrix must satisfy 1 <= m, n <= " +
                                            std::to_string(NOALLOC_MAX_DIM) + " and m*n <= " +
                                            std::to_string(NOALLOC_MAX_ELEMS) + " (got " + std::to_string(m) +
                                            " x " + std::to_string(n) + ")");
    return TCI_ERR_ARG;
  }
  if (!A_dev || !rowperm_dev || !colperm_dev || !npivot_dev || !error_dev || !status_dev) {
    tci::set_error(TCI_ERR_ARG, "tci_rrlu_noalloc: null input or output pointer");
    return TCI_ERR_ARG;
  }
  // A launch error left pending by earlier work on this thread is reported,
  // not cleared: the caller's own error check still sees it.
  cudaError_t ce = cudaPeekAtLastError();
  if (ce != cudaSuccess) {
    tci::set_error(TCI_ERR_CUDA, std::string("tci_rrlu_noalloc: a CUDA error was pending before the call: ") +
                                     cudaGetErrorString(ce));
    return TCI_ERR_CUDA;
  }
  int dev = 0;
  ce = cudaGetDevice(&dev);
  if (ce != cudaSuccess || dev < 0 || dev >= 64) {
    tci::set_error(TCI_ERR_CUDA,std::string("tci_rrlu_noalloc: ") + cudaGetErrorString(ce));
    return TCI_ERR_CUDA;
  }
  NoallocDevice& D = devs[dev];
  {
    std::lock_guard<std::mutex> lk(mu);
    if (!D.ready) {
      void* p = nullptr;
      ce = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (ce == cudaSuccess)
        ce = cudaFuncSetAttribute(rrlu_noalloc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)tci_step_smem_bytes());
      if (ce != cudaSuccess) {
        tci::set_error(TCI_ERR_CUDA,std::string("tci_rrlu_noalloc set-up: ") + cudaGetErrorString(ce));
        return TCI_ERR_CUDA;
      }
      D.scratch = (double*)p;
      D.ready = true;
    }
  }
  double* work = D.scratch;
  double* fact = D.scratch + NOALLOC_MAX_ELEMS;
  char* resb = (char*)(D.scratch + NOALLOC_MAX_ELEMS + NOALLOC_FACT_DOUBLES);
  tci_task T;
  memset(&T, 0, sizeof(T));
  T.kind = TCI_TASK_RRLU;
  T.m = (int32_t)m;
  T.n = (int32_t)n;
  int64_t kmax = maxrank <= 0 ? (m < n ? m : n) : maxrank;
  if (kmax > m) kmax = m;
  if (kmax > n) kmax = n;
  T.maxrank = (int32_t)kmax;
  T.kcap = (int32_t)kmax;
  T.reltol = reltol;
  T.abstol = abstol;
  T.leftorth = leftorthogonal ? 1 : 0;
  T.post = TCI_POST_FACTORS;
  T.ain = A_dev;
  T.core_out = fact;
  T.res = 0;
  const size_t smem = tci_step_smem_bytes();
  auto a16 = [](size_t x) { return (x + 15) / 16 * 16; };
  const size_t perms = a16((size_t)m * 4) + a16((size_t)n * 4);
  T.smem_mode = a16((size_t)m * n * 8) + perms <= smem ? 1 : 0;
  T.work = T.smem_mode ? nullptr : work;
  cudaStream_t stream = (cudaStream_t)stream_u;
  rrlu_noalloc_kernel<<<1, NT, smem, stream>>>(T, resb);
  rrlu_noalloc_epilogue<<<64, 256, 0, stream>>>(fact, resb, (int)m, (int)n, rowperm_dev, colperm_dev, npivot_dev,
                                                error_dev, status_dev, factors_dev);
  ce = cudaGetLastError();
  if (ce != cudaSuccess) {
    tci::set_error(TCI_ERR_CUDA,std::string("tci_rrlu_noalloc: ") + cudaGetErrorString(ce));
    return TCI_ERR_CUDA;
  }
  return 0;
}
#endif  // TCI_SECONDARY
