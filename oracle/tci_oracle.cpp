// CPU ORACLE -- test infrastructure only.
//
// A plain C++ restatement of the reference's TCI2 two-site sweep path
// (TensorCrossInterpolation.jl v0.9.19).  Only tests/, the smoke check and the
// CPU-baseline legs of bench.py load this library, and only as the checker or
// the timed CPU baseline; the product library never links or calls it.
//
// Every function cites the reference file:line it follows.  Arithmetic is kept
// in the reference's order: the rank-revealing LU multiplies and subtracts
// separately (no FMA; build with -ffp-contract=off), divides (never multiplies
// by a reciprocal), picks the first maximum of abs2 in column-major order and
// swaps rows and columns physically, exactly as matrixlu.jl does.  Where the
// reference calls LAPACK/BLAS (the partial-pivot solve of tensorci2.jl:391, the
// trsm of matrixluci.jl:53,64, gemm in matrixluci.jl:41,45 and the products in
// abstracttensortrain.jl:131), the oracle uses plain loops; those results are
// compared to a tolerance, never bitwise, as the reference's own tests do.
//
// The registered functions f are written here independently from the device
// library (full multi-index in, value out); they share only the deterministic
// exp/cos of tci_math.h so that GPU and oracle function values are identical.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <memory>
#include <unordered_map>
#include <string>
#include <thread>
#include <unordered_set>
#include <vector>

#include "../tensorcrossinterpolation.jl_gb300/csrc/tci_math.h"
#include "../tensorcrossinterpolation.jl_gb300/csrc/tci_rng.h"

namespace {

using i64 = int64_t;
using MultiIndex = std::vector<int>;  // 1-based local indices (abstracttensortrain.jl:6-7)
const i64 TYPEMAX = std::numeric_limits<i64>::max();
const double NaN = std::numeric_limits<double>::quiet_NaN();

enum { ORC_OK = 0, ORC_ARG = 1, ORC_DIM = 2, ORC_NAN = 3, ORC_SINGULAR = 4, ORC_ERR = 5 };

thread_local std::string g_err;
int fail(int code, const std::string& msg) { g_err = msg; return code; }

// Julia's max for Float64: NaN propagates (Base.max).
double jmax(double a, double b) {
  if (a != a || b != b) return NaN;
  return a > b ? a : b;
}

// ---------------------------------------------------------------- functions
enum { F_LORENTZ = 1, F_SERVED = 2, F_QTT1D = 3, F_QTT2D = 4, F_DENSE = 5, F_PRODUCT = 6 };

// A caller-supplied f (the BatchEvaluator plugin point, batcheval.jl:67-83):
// values[k] = f(points[k, :]) for npoints row-major 1-based multi-indices.
typedef int (*orc_batch_fn)(void* user, int32_t L, int64_t npoints, const int64_t* points, double* values);
constexpr int F_USER = 1024;

struct OrcContraction;  // the Contraction evaluator of contract(algorithm = :TCI), below
double contraction_point(OrcContraction& c, const MultiIndex& v);

struct Func {
  int fid = 0;
  std::vector<double> params;
  orc_batch_fn cb = nullptr;
  void* user = nullptr;
  std::shared_ptr<OrcContraction> ctr;
  // values at many points through one evaluator call (filltensor on a
  // BatchEvaluator, batcheval.jl:67-83); NaN everywhere if the evaluator fails
  void batch(int L, int64_t np, const int64_t* pts, double* out) const {
    if (cb(user, L, np, pts, out) != 0)
      for (int64_t k = 0; k < np; ++k) out[k] = NaN;
  }
  double operator()(const MultiIndex& v) const {
    const int L = (int)v.size();
    if (ctr) return contraction_point(*ctr, v);
    if (cb) {
      std::vector<int64_t> p(v.begin(), v.end());
      double out = NaN;
      batch(L, 1, p.data(), &out);
      return out;
    }
    switch (fid) {
      case F_LORENTZ: {  // coeff ./ (sum(v .^ 2) + 1), test_tensorci2.jl:249
        i64 s = 0;
        for (int p = 0; p < L; ++p) s += (i64)v[p] * v[p];
        double coeff = params.empty() ? 1.0 : params[0];
        return coeff / (double)(s + 1);
      }
      case F_SERVED: {  // 1/(1+a v.v) + b exp(-g |v-c|^2), v and c on the 1-based lattice
        i64 s1 = 0, s2 = 0;
        for (int p = 0; p < L; ++p) {
          s1 += (i64)v[p] * v[p];
          i64 dv = (i64)v[p] - (i64)params[3 + p];
          s2 += dv * dv;
        }
        double a = 1.0 / (1.0 + params[0] * (double)s1);
        double e = tci_exp(-(params[2] * (double)s2));
        return a + params[1] * e;
      }
      case F_QTT1D: {  // x = sum_i b_i 2^-i, b_i = v_i - 1
        double x = 0.0;
        for (int p = 0; p < L; ++p)
          if (v[p] == 2) x = x + std::ldexp(1.0, -(p + 1));
        int kind = params.empty() ? 0 : (int)params[0];
        if (kind == 1) return tci_exp(-x);
        if (kind == 2) return tci_exp(-x) + 1e-4 * tci_exp(-(2.0 * x));
        double t1 = tci_exp(-x);
        double t2 = tci_cos(6283.185307179587 * x);
        double dx = x - 0.3;
        double t3 = tci_exp(-(dx * dx) / 1e-4);
        return t1 * t2 + 0.5 * t3;
      }
      case F_QTT2D: {  // site value s = v-1 in 0..3: x bit = s & 1, y bit = s >> 1
        double x = 0.0, y = 0.0;
        for (int p = 0; p < L; ++p) {
          int s = v[p] - 1;
          if (s & 1) x = x + std::ldexp(1.0, -(p + 1));
          if (s & 2) y = y + std::ldexp(1.0, -(p + 1));
        }
        double dx = x - 0.5, dy = y - 0.5;
        double g = tci_exp(-(dx * dx + dy * dy) / 0.01);
        return g * tci_cos(1256.6370614359173 * (x + y));
      }
      case F_PRODUCT: {  // C (-1)^(sum neg) exp(sum q); q are multiples of 2^-40, sums exact
        const i64 D = (i64)params[1];
        double q = 0.0, ng = 0.0;
        for (int p = 0; p < L; ++p) {
          q = q + params[3 + p * D + (v[p] - 1)];
          ng = ng + params[3 + L * D + p * D + (v[p] - 1)];
        }
        const double e = params[2] * tci_exp(q);
        return (((long long)ng) & 1) ? -e : e;
      }
      case F_DENSE: {  // params = [L, strides..., values...]
        i64 off = 0;
        for (int p = 0; p < L; ++p) off += (i64)(v[p] - 1) * (i64)params[1 + p];
        return params[1 + L + off];
      }
      default:
        return NaN;
    }
  }
};

// ---------------------------------------------------------------- rrLU
// mutable struct rrLU (matrixlu.jl:71-96); permutations kept 0-based here.
struct RRLU {
  i64 m = 0, n = 0;
  std::vector<i64> rowperm, colperm;
  std::vector<double> L;  // m x npivot, column-major
  std::vector<double> U;  // npivot x n, column-major
  bool leftorth = true;
  i64 npivot = 0;
  double error = NaN;
};

// submatrixargmax(abs2, A, k) (matrixlu.jl:1-32, 63-65): column-major scan of the
// trailing block, strict '>' so the first maximum wins; starts from typemin.
void submatrixargmax_abs2(const double* A, i64 m, i64 n, i64 k, i64& mr, i64& mc) {
  double mval = -std::numeric_limits<double>::infinity();
  mr = k;
  mc = k;
  for (i64 c = k; c < n; ++c)
    for (i64 r = k; r < m; ++r) {
      double a = A[r + c * m];
      double v = a * a;
      if (v > mval) {
        mval = v;
        mr = r;
        mc = c;
      }
    }
}

// swaprow!/swapcol!/addpivot! (matrixlu.jl:98-136)
void addpivot(RRLU& lu, double* A, i64 r, i64 c) {
  const i64 m = lu.m, n = lu.n;
  i64 k = lu.npivot;
  lu.npivot += 1;
  std::swap(lu.rowperm[k], lu.rowperm[r]);
  for (i64 j = 0; j < n; ++j) std::swap(A[k + j * m], A[r + j * m]);
  std::swap(lu.colperm[k], lu.colperm[c]);
  for (i64 i = 0; i < m; ++i) std::swap(A[i + k * m], A[i + c * m]);
  const double piv = A[k + k * m];
  if (lu.leftorth) {
    for (i64 i = k + 1; i < m; ++i) A[i + k * m] = A[i + k * m] / piv;
  } else {
    for (i64 j = k + 1; j < n; ++j) A[k + j * m] = A[k + j * m] / piv;
  }
  for (i64 j = k + 1; j < n; ++j) {
    const double y = A[k + j * m];
    double* col = A + j * m;
    const double* x = A + k * m;
    for (i64 i = k + 1; i < m; ++i) {
      double p = x[i] * y;
      col[i] = col[i] - p;
    }
  }
}

// _optimizerrlu! (matrixlu.jl:141-181) on an rrLU initialised as in :92-95.
int optimizerrlu(RRLU& lu, double* A, i64 maxrank, double reltol, double abstol) {
  const i64 m = lu.m, n = lu.n;
  maxrank = std::min(maxrank, std::min(m, n));
  double maxerror = 0.0;
  while (lu.npivot < maxrank) {
    i64 k = lu.npivot, r, c;
    submatrixargmax_abs2(A, m, n, k, r, c);
    lu.error = std::fabs(A[r + c * m]);
    if ((std::fabs(lu.error) < reltol * maxerror || std::fabs(lu.error) < abstol) && lu.npivot > 0)
      break;
    maxerror = jmax(maxerror, lu.error);
    addpivot(lu, A, r, c);
  }
  const i64 K = lu.npivot;
  lu.L.assign((size_t)(m * K), 0.0);
  lu.U.assign((size_t)(K * n), 0.0);
  bool nan = false;
  for (i64 j = 0; j < K; ++j)
    for (i64 i = j; i < m; ++i) {
      double v = A[i + j * m];
      nan |= (v != v);
      lu.L[i + j * m] = v;
    }
  for (i64 j = 0; j < n; ++j)
    for (i64 i = 0; i < K && i <= j; ++i) {
      double v = A[i + j * m];
      nan |= (v != v);
      lu.U[i + j * K] = v;
    }
  if (nan) return fail(ORC_NAN, "lu.L contains NaNs");
  if (lu.leftorth)
    for (i64 k = 0; k < K; ++k) lu.L[k + k * m] = 1.0;
  else
    for (i64 k = 0; k < K; ++k) lu.U[k + k * K] = 1.0;
  if (lu.npivot >= std::min(m, n)) lu.error = 0.0;
  return ORC_OK;
}

// rrlu(A; maxrank, reltol, abstol, leftorthogonal) (matrixlu.jl:217-225) -- copies A.
int rrlu(const double* A0, i64 m, i64 n, i64 maxrank, double reltol, double abstol, bool leftorth,
         RRLU& lu) {
  std::vector<double> A(A0, A0 + m * n);
  lu = RRLU();
  lu.m = m;
  lu.n = n;
  lu.leftorth = leftorth;
  lu.rowperm.resize(m);
  lu.colperm.resize(n);
  for (i64 i = 0; i < m; ++i) lu.rowperm[i] = i;
  for (i64 j = 0; j < n; ++j) lu.colperm[j] = j;
  return optimizerrlu(lu, A.data(), maxrank, reltol, abstol);
}

// pivoterrors(lu) = vcat(abs.(diag(lu)), lu.error) (matrixlu.jl:409-411, :395-401)
std::vector<double> pivoterrors(const RRLU& lu) {
  std::vector<double> e;
  for (i64 k = 0; k < lu.npivot; ++k)
    e.push_back(std::fabs(lu.leftorth ? lu.U[k + k * lu.npivot] : lu.L[k + k * lu.m]));
  e.push_back(lu.error);
  return e;
}

// MatrixLUCI left/right (matrixluci.jl:40-84).  Results column-major.
// colstimespivotinv: rows K.. of L solved against LowerTriangular(L[1:K,:]), rows scattered.
std::vector<double> luci_left(const RRLU& lu) {
  const i64 m = lu.m, n = lu.n, K = lu.npivot;
  std::vector<double> res((size_t)(m * K), 0.0);
  if (lu.leftorth) {
    std::vector<double> t((size_t)(m * K), 0.0);
    for (i64 k = 0; k < K; ++k) t[k + k * m] = 1.0;
    for (i64 i = K; i < m; ++i)
      for (i64 q = K - 1; q >= 0; --q) {
        double s = lu.L[i + q * m];
        for (i64 p = q + 1; p < K; ++p) s = s - t[i + p * m] * lu.L[p + q * m];
        t[i + q * m] = s / lu.L[q + q * m];
      }
    for (i64 i = 0; i < m; ++i)
      for (i64 q = 0; q < K; ++q) res[lu.rowperm[i] + q * m] = t[i + q * m];
  } else {
    // colmatrix: left(lu) * right(lu, permute=false)[:, 1:K]
    for (i64 i = 0; i < m; ++i)
      for (i64 q = 0; q < K; ++q) {
        double s = 0.0;
        for (i64 p = 0; p <= q; ++p) s = s + lu.L[i + p * m] * lu.U[p + q * K];
        res[lu.rowperm[i] + q * m] = s;
      }
  }
  (void)n;
  return res;
}

std::vector<double> luci_right(const RRLU& lu) {
  const i64 m = lu.m, n = lu.n, K = lu.npivot;
  std::vector<double> res((size_t)(K * n), 0.0);
  if (lu.leftorth) {
    // rowmatrix: left(lu, permute=false)[1:K, :] * right(lu)
    for (i64 j = 0; j < n; ++j)
      for (i64 q = 0; q < K; ++q) {
        double s = 0.0;
        for (i64 p = 0; p <= q; ++p) s = s + lu.L[q + p * m] * lu.U[p + j * K];
        res[q + lu.colperm[j] * K] = s;
      }
  } else {
    // pivotinvtimesrows: UpperTriangular(U[:, 1:K]) \ U[:, K+1:end], columns scattered
    std::vector<double> t((size_t)(K * n), 0.0);
    for (i64 k = 0; k < K; ++k) t[k + k * K] = 1.0;
    for (i64 j = K; j < n; ++j)
      for (i64 q = K - 1; q >= 0; --q) {
        double s = lu.U[q + j * K];
        for (i64 p = q + 1; p < K; ++p) s = s - lu.U[q + p * K] * t[p + j * K];
        t[q + j * K] = s / lu.U[q + q * K];
      }
    for (i64 j = 0; j < n; ++j)
      for (i64 q = 0; q < K; ++q) res[q + lu.colperm[j] * K] = t[q + j * K];
  }
  return res;
}

// ---------------------------------------------------------------- dense LU solve
// transpose(P) \ transpose(Pi1) (tensorci2.jl:391): Julia calls LAPACK getrf
// (partial pivoting, first max |a| per column, reciprocal scaling) and getrs.
// Returns T = Pi1 * inv(P) (rows x r), column-major.
int lapack_style_solve(const std::vector<double>& P, i64 r, const std::vector<double>& Pi1, i64 rows,
                       std::vector<double>& T) {
  // A = P^T (r x r)
  std::vector<double> A((size_t)(r * r));
  for (i64 i = 0; i < r; ++i)
    for (i64 j = 0; j < r; ++j) A[i + j * r] = P[j + i * r];
  std::vector<i64> ipiv(r);
  for (i64 j = 0; j < r; ++j) {
    i64 p = j;
    double best = std::fabs(A[j + j * r]);
    for (i64 i = j + 1; i < r; ++i)
      if (std::fabs(A[i + j * r]) > best) {
        best = std::fabs(A[i + j * r]);
        p = i;
      }
    ipiv[j] = p;
    if (A[p + j * r] == 0.0) return fail(ORC_SINGULAR, "SingularException in setsitetensor!");
    if (p != j)
      for (i64 c = 0; c < r; ++c) std::swap(A[j + c * r], A[p + c * r]);
    double rcp = 1.0 / A[j + j * r];
    for (i64 i = j + 1; i < r; ++i) A[i + j * r] = A[i + j * r] * rcp;
    for (i64 c = j + 1; c < r; ++c) {
      double y = A[j + c * r];
      for (i64 i = j + 1; i < r; ++i) A[i + c * r] = A[i + c * r] - A[i + j * r] * y;
    }
  }
  // B = Pi1^T (r x rows); solve A X = B
  std::vector<double> B((size_t)(r * rows));
  for (i64 i = 0; i < rows; ++i)
    for (i64 j = 0; j < r; ++j) B[j + i * r] = Pi1[i + j * rows];
  for (i64 col = 0; col < rows; ++col) {
    double* b = B.data() + col * r;
    for (i64 j = 0; j < r; ++j)
      if (ipiv[j] != j) std::swap(b[j], b[ipiv[j]]);
    for (i64 j = 0; j < r; ++j)
      for (i64 i = j + 1; i < r; ++i) b[i] = b[i] - A[i + j * r] * b[j];
    for (i64 j = r - 1; j >= 0; --j) {
      b[j] = b[j] / A[j + j * r];
      for (i64 i = 0; i < j; ++i) b[i] = b[i] - A[i + j * r] * b[j];
    }
  }
  T.assign((size_t)(rows * r), 0.0);
  for (i64 i = 0; i < rows; ++i)
    for (i64 j = 0; j < r; ++j) T[i + j * rows] = B[j + i * r];
  return ORC_OK;
}

// ---------------------------------------------------------------- index sets
struct MIHash {
  size_t operator()(const MultiIndex& v) const {
    uint64_t h = 1469598103934665603ULL;
    for (int x : v) h = (h ^ (uint64_t)(uint32_t)x) * 1099511628211ULL;
    return (size_t)h;
  }
};

// pushunique! (util.jl:16-20)
void pushunique(std::vector<MultiIndex>& coll, const MultiIndex& item) {
  for (const auto& c : coll)
    if (c == item) return;
  coll.push_back(item);
}

// kronecker(Iset, d) (tensorci2.jl:315-320): Iset index fastest, then local index.
std::vector<MultiIndex> kron_right(const std::vector<MultiIndex>& I, int d) {
  std::vector<MultiIndex> out;
  out.reserve(I.size() * d);
  for (int j = 1; j <= d; ++j)
    for (const auto& is : I) {
      MultiIndex v = is;
      v.push_back(j);
      out.push_back(std::move(v));
    }
  return out;
}
// kronecker(d, Jset) (tensorci2.jl:322-327): local index fastest, then Jset index.
std::vector<MultiIndex> kron_left(int d, const std::vector<MultiIndex>& J) {
  std::vector<MultiIndex> out;
  out.reserve(J.size() * d);
  for (const auto& js : J)
    for (int i = 1; i <= d; ++i) {
      MultiIndex v;
      v.reserve(js.size() + 1);
      v.push_back(i);
      v.insert(v.end(), js.begin(), js.end());
      out.push_back(std::move(v));
    }
  return out;
}
// Base.union(a, b): unique elements in order of first appearance.
std::vector<MultiIndex> vunion(const std::vector<MultiIndex>& a, const std::vector<MultiIndex>& b) {
  std::unordered_set<MultiIndex, MIHash> seen;
  std::vector<MultiIndex> out;
  for (const auto* src : {&a, &b})
    for (const auto& v : *src)
      if (seen.insert(v).second) out.push_back(v);
  return out;
}

struct Tensor3 {
  i64 d0 = 0, d1 = 0, d2 = 0;
  std::vector<double> v;  // column-major
};

// ---------------------------------------------------------------- TensorCI2
struct Opts {
  double tolerance;
  int64_t maxbonddim;
  int64_t maxiter;
  int32_t sweepstrategy;  // 0 backandforth, 1 forward, 2 backward
  int32_t normalizeerror;
  int32_t ncheckhistory;
  int32_t maxnglobalpivot;
  int32_t nsearchglobalpivot;
  int32_t strictlynested;
  int32_t checkconvglobalpivot;
  int32_t pad_;
  double tolmarginglobalsearch;
  uint64_t seed;
};

struct TCI2 {
  int L = 0;
  std::vector<int> localdims;
  Func f;
  std::vector<std::vector<MultiIndex>> Iset, Jset;  // Iset[b] entries length b, Jset[b] length L-1-b
  std::vector<Tensor3> sitetensors;
  std::vector<double> pivoterrors, bonderrors;
  double maxsamplevalue = 0.0;
  std::vector<std::vector<std::vector<MultiIndex>>> Ihist, Jhist;
  std::vector<i64> ranks;
  std::vector<double> errors;
  std::vector<i64> nglobal;
  i64 nfeval = 0;
  double t_fill = 0, t_lu = 0;
};

// filltensor(..., Val(0)) over explicit row/col multi-index lists (tensorci2.jl:290-312,
// batcheval.jl:32-61).  Column-major |I| x |J|.
void contraction_fill(OrcContraction& c, const std::vector<MultiIndex>& I, const std::vector<MultiIndex>& J,
                      std::vector<double>& out);

std::vector<double> fill(TCI2& t, const std::vector<MultiIndex>& I, const std::vector<MultiIndex>& J) {
  std::vector<double> out(I.size() * J.size());
  if (t.f.ctr) {
    contraction_fill(*t.f.ctr, I, J, out);
    t.nfeval += (i64)out.size();
    return out;
  }
  if (t.f.cb) {  // one evaluator call for the whole block, column-major
    std::vector<int64_t> pts;
    pts.reserve(out.size() * (size_t)t.L);
    for (size_t j = 0; j < J.size(); ++j)
      for (size_t i = 0; i < I.size(); ++i) {
        pts.insert(pts.end(), I[i].begin(), I[i].end());
        pts.insert(pts.end(), J[j].begin(), J[j].end());
      }
    if (!out.empty()) t.f.batch(t.L, (int64_t)out.size(), pts.data(), out.data());
    t.nfeval += (i64)out.size();
    return out;
  }
  MultiIndex v(t.L);
  for (size_t j = 0; j < J.size(); ++j)
    for (size_t i = 0; i < I.size(); ++i) {
      std::copy(I[i].begin(), I[i].end(), v.begin());
      std::copy(J[j].begin(), J[j].end(), v.begin() + I[i].size());
      out[i + j * I.size()] = t.f(v);
    }
  t.nfeval += (i64)out.size();
  return out;
}

// updatemaxsample!/maxabs (tensorci2.jl:397-399, util.jl:1-10)
void updatemaxsample(TCI2& t, const std::vector<double>& s) {
  double m = t.maxsamplevalue;
  for (double x : s) m = jmax(std::fabs(m), std::fabs(x));
  t.maxsamplevalue = m;
}

void invalidate(TCI2& t) {
  for (auto& s : t.sitetensors) s = Tensor3();
}

// updatepivoterror!/updatebonderror!/updateerrors! (tensorci2.jl:132-169)
void updateerrors(TCI2& t, int b, const std::vector<double>& e) {
  t.bonderrors[b] = e.back();
  size_t n = std::max(t.pivoterrors.size(), e.size());
  std::vector<double> out(n);
  for (size_t i = 0; i < n; ++i) {
    double a = i < t.pivoterrors.size() ? t.pivoterrors[i] : 0.0;
    double c = i < e.size() ? e[i] : 0.0;
    out[i] = jmax(a, c);
  }
  t.pivoterrors = out;
}

void setsitetensor(TCI2& t, int b, const std::vector<double>& T) {
  Tensor3& s = t.sitetensors[b];
  s.d0 = (i64)t.Iset[b].size();
  s.d1 = t.localdims[b];
  s.d2 = (i64)t.Jset[b].size();
  s.v = T;
}

// addglobalpivots! (tensorci2.jl:193-213)
int addglobalpivots(TCI2& t, const std::vector<MultiIndex>& pivots) {
  for (const auto& p : pivots)
    if ((int)p.size() != t.L)
      return fail(ORC_DIM, "Please specify a pivot as one index per leg of the MPS.");
  for (const auto& p : pivots)
    for (int b = 0; b < t.L; ++b) {
      pushunique(t.Iset[b], MultiIndex(p.begin(), p.begin() + b));
      pushunique(t.Jset[b], MultiIndex(p.begin() + b + 1, p.end()));
    }
  if (!pivots.empty()) invalidate(t);
  return ORC_OK;
}

// TensorCI2{ValueType}(func, localdims, initialpivots) (tensorci2.jl:23-53)
int tci_new(TCI2& t, const std::vector<int>& localdims, const Func& f,
            const std::vector<MultiIndex>& initialpivots) {
  if (localdims.size() < 2) return fail(ORC_ERR, "localdims should have at least 2 elements!");
  t = TCI2();
  t.L = (int)localdims.size();
  t.localdims = localdims;
  t.f = f;
  t.Iset.assign(t.L, {});
  t.Jset.assign(t.L, {});
  t.sitetensors.assign(t.L, Tensor3());
  t.bonderrors.assign(t.L - 1, 0.0);
  if (initialpivots.empty()) return fail(ORC_ARG, "initialpivots must not be empty");
  int rc = addglobalpivots(t, initialpivots);
  if (rc) return rc;
  double m = -std::numeric_limits<double>::infinity();
  for (const auto& p : initialpivots) m = jmax(m, std::fabs(f(p)));
  t.maxsamplevalue = m;
  if (!(std::fabs(t.maxsamplevalue) > 0.0)) return fail(ORC_ERR, "maxsamplevalue is zero!");
  invalidate(t);
  return ORC_OK;
}

int luci(TCI2& t, const std::vector<double>& Pi, i64 m, i64 n, double reltol, double abstol,
         i64 maxrank, bool leftorth, RRLU& lu) {
  return rrlu(Pi.data(), m, n, maxrank, reltol, abstol, leftorth, lu);
}

// updatepivots! with pivotsearch=:full (tensorci2.jl:510-551, 599-607)
int updatepivots(TCI2& t, int b, bool leftorth, double reltol, double abstol, i64 maxbonddim,
                 const std::vector<MultiIndex>& extraI, const std::vector<MultiIndex>& extraJ) {
  invalidate(t);
  auto Ic = vunion(kron_right(t.Iset[b], t.localdims[b]), extraI);
  auto Jc = vunion(kron_left(t.localdims[b + 1], t.Jset[b + 1]), extraJ);
  auto Pi = fill(t, Ic, Jc);
  updatemaxsample(t, Pi);
  RRLU lu;
  int rc = luci(t, Pi, (i64)Ic.size(), (i64)Jc.size(), reltol, abstol, maxbonddim, leftorth, lu);
  if (rc) return rc;
  std::vector<MultiIndex> In, Jn;
  for (i64 k = 0; k < lu.npivot; ++k) {
    In.push_back(Ic[lu.rowperm[k]]);
    Jn.push_back(Jc[lu.colperm[k]]);
  }
  t.Iset[b + 1] = In;
  t.Jset[b] = Jn;
  if (extraI.empty() && extraJ.empty()) {
    setsitetensor(t, b, luci_left(lu));
    setsitetensor(t, b + 1, luci_right(lu));
  }
  updateerrors(t, b, pivoterrors(lu));
  return ORC_OK;
}

// setsitetensor!(tci, f, b) (tensorci2.jl:367-394), leftorthogonal=true
int setsitetensor_f(TCI2& t, int b) {
  auto Is = kron_right(t.Iset[b], t.localdims[b]);
  const auto& Js = t.Jset[b];
  auto Pi1 = fill(t, Is, Js);
  updatemaxsample(t, Pi1);
  if (b == t.L - 1) {
    setsitetensor(t, b, Pi1);
    return ORC_OK;
  }
  auto P = fill(t, t.Iset[b + 1], t.Jset[b]);
  if (t.Iset[b + 1].size() != t.Jset[b].size())
    return fail(ORC_ERR, "Pivot matrix at bond " + std::to_string(b + 1) + " is not square!");
  std::vector<double> T;
  int rc = lapack_style_solve(P, (i64)t.Jset[b].size(), Pi1, (i64)Is.size(), T);
  if (rc) return rc;
  Tensor3& s = t.sitetensors[b];
  s.d0 = (i64)t.Iset[b].size();
  s.d1 = t.localdims[b];
  s.d2 = (i64)t.Iset[b + 1].size();
  s.v = T;
  return ORC_OK;
}

// fillsitetensors! (globalsearch.jl:97-103)
int fillsitetensors(TCI2& t) {
  for (int b = 0; b < t.L; ++b) {
    int rc = setsitetensor_f(t, b);
    if (rc) return rc;
  }
  return ORC_OK;
}

// sweep1site! (tensorci2.jl:402-461)
int sweep1site(TCI2& t, bool forward, double reltol, double abstol, i64 maxbonddim, bool updatetensors) {
  t.pivoterrors.clear();
  invalidate(t);
  const int L = t.L;
  for (int step = 0; step < L - 1; ++step) {
    int b = forward ? step : L - 1 - step;
    std::vector<MultiIndex> Is, Js;
    if (forward) {
      Is = kron_right(t.Iset[b], t.localdims[b]);
      Js = t.Jset[b];
    } else {
      Is = t.Iset[b];
      Js = kron_left(t.localdims[b], t.Jset[b]);
    }
    auto Pi = fill(t, Is, Js);
    updatemaxsample(t, Pi);
    RRLU lu;
    int rc = luci(t, Pi, (i64)Is.size(), (i64)Js.size(), reltol, abstol, maxbonddim, forward, lu);
    if (rc) return rc;
    std::vector<MultiIndex> In, Jn;
    for (i64 k = 0; k < lu.npivot; ++k) {
      In.push_back(Is[lu.rowperm[k]]);
      Jn.push_back(Js[lu.colperm[k]]);
    }
    if (forward) {
      t.Iset[b + 1] = In;
      t.Jset[b] = Jn;
    } else {
      t.Iset[b] = In;
      t.Jset[b - 1] = Jn;
    }
    if (updatetensors) {
      auto T = forward ? luci_left(lu) : luci_right(lu);
      setsitetensor(t, b, T);
      for (double x : T)
        if (x != x) return fail(ORC_NAN, "Error: NaN in tensor T[" + std::to_string(b + 1) + "]");
    }
    updateerrors(t, forward ? b : b - 1, pivoterrors(lu));
  }
  if (updatetensors) {
    int b = forward ? L - 1 : 0;
    auto Is = kron_right(t.Iset[b], t.localdims[b]);
    auto T = fill(t, Is, t.Jset[b]);
    setsitetensor(t, b, T);
  }
  return ORC_OK;
}

// makecanonical! (tensorci2.jl:463-474)
int makecanonical(TCI2& t, double reltol, double abstol, i64 maxbonddim) {
  int rc = sweep1site(t, true, 0.0, 0.0, TYPEMAX, false);
  if (!rc) rc = sweep1site(t, false, reltol, abstol, maxbonddim, false);
  if (!rc) rc = sweep1site(t, true, reltol, abstol, maxbonddim, true);
  return rc;
}

// forwardsweep (sweepstrategies.jl:1-6); strategy 0 backandforth, 1 forward, 2 backward
bool forwardsweep(int strategy, i64 iter) { return strategy == 1 || (strategy == 0 && (iter % 2) == 1); }

// sweep2site! (tensorci2.jl:855-916)
int sweep2site(TCI2& t, int niter, int iter1, double abstol, i64 maxbonddim, int strategy,
               bool strictlynested, bool fillsite) {
  invalidate(t);
  const int n = t.L;
  for (int iter = iter1; iter < iter1 + niter; ++iter) {
    std::vector<std::vector<MultiIndex>> extraI(n), extraJ(n);
    if (!strictlynested && !t.Ihist.empty()) {
      extraI = t.Ihist.back();
      extraJ = t.Jhist.back();
    }
    t.Ihist.push_back(t.Iset);
    t.Jhist.push_back(t.Jset);
    t.pivoterrors.clear();
    if (forwardsweep(strategy, iter)) {
      for (int b = 0; b < n - 1; ++b) {
        int rc = updatepivots(t, b, true, 1e-14, abstol, maxbonddim, extraI[b + 1], extraJ[b]);
        if (rc) return rc;
      }
    } else {
      for (int b = n - 2; b >= 0; --b) {
        int rc = updatepivots(t, b, false, 1e-14, abstol, maxbonddim, extraI[b + 1], extraJ[b]);
        if (rc) return rc;
      }
    }
  }
  if (fillsite) return fillsitetensors(t);
  return ORC_OK;
}

// evaluate (abstracttensortrain.jl:124-132): left-to-right chain of T[:, i, :].
double tt_evaluate(const std::vector<Tensor3>& tt, const MultiIndex& idx) {
  std::vector<double> v(1, 1.0), w;
  for (size_t s = 0; s < tt.size(); ++s) {
    const Tensor3& T = tt[s];
    const i64 i = idx[s] - 1;
    w.assign((size_t)T.d2, 0.0);
    for (i64 q = 0; q < T.d2; ++q) {
      double acc = 0.0;
      for (i64 p = 0; p < T.d0; ++p) acc = acc + v[p] * T.v[p + T.d0 * (i + T.d1 * q)];
      w[q] = acc;
    }
    v.swap(w);
  }
  return v.empty() ? NaN : v[0];
}

// sum / _sum (abstracttensortrain.jl:164-199) over all sites.
double tt_sum(const std::vector<Tensor3>& tt) {
  std::vector<double> v(1, 1.0), w;
  for (const Tensor3& T : tt) {
    w.assign((size_t)T.d2, 0.0);
    for (i64 q = 0; q < T.d2; ++q) {
      double acc = 0.0;
      for (i64 p = 0; p < T.d0; ++p) {
        double s = 0.0;
        for (i64 i = 0; i < T.d1; ++i) s = s + T.v[p + T.d0 * (i + T.d1 * q)];
        acc = acc + v[p] * s;
      }
      w[q] = acc;
    }
    v.swap(w);
  }
  return v.empty() ? NaN : v[0];
}

// DefaultGlobalPivotFinder (globalpivotfinder.jl:143-195) with the shared host RNG.
std::vector<MultiIndex> default_global_pivots(TCI2& t, double abstol, int nsearch, int maxnglobalpivot,
                                              double tolmargin, tci_rng* rng) {
  const int L = t.L;
  std::vector<MultiIndex> starts;
  for (int s = 0; s < nsearch; ++s) {
    MultiIndex p(L);
    for (int q = 0; q < L; ++q) p[q] = (int)tci_rng_uniform1(rng, (uint64_t)t.localdims[q]);
    starts.push_back(p);
  }
  std::vector<MultiIndex> found;
  const auto& C = t.sitetensors;
  for (const auto& point : starts) {
    // The train at the start point with site q changed is the product
    // Le_q * C_q[:, v, :] * Re_q of the start's left and right environments
    // (the same matrix products as evaluate(), associated around site q).
    std::vector<std::vector<double>> Le(L), Re(L);
    Le[0].assign(1, 1.0);
    for (int q = 0; q + 1 < L; ++q) {
      const Tensor3& T = C[q];
      const i64 i = point[q] - 1;
      Le[q + 1].assign((size_t)T.d2, 0.0);
      for (i64 b = 0; b < T.d2; ++b) {
        double acc = 0.0;
        for (i64 a = 0; a < T.d0; ++a) acc = acc + Le[q][a] * T.v[a + T.d0 * (i + T.d1 * b)];
        Le[q + 1][b] = acc;
      }
    }
    Re[L - 1].assign(1, 1.0);
    for (int q = L - 1; q > 0; --q) {
      const Tensor3& T = C[q];
      const i64 i = point[q] - 1;
      Re[q - 1].assign((size_t)T.d0, 0.0);
      for (i64 a = 0; a < T.d0; ++a) {
        double acc = 0.0;
        for (i64 b = 0; b < T.d2; ++b) acc = acc + T.v[a + T.d0 * (i + T.d1 * b)] * Re[q][b];
        Re[q - 1][a] = acc;
      }
    }
    MultiIndex cur = point, best = point;
    double best_error = 0.0;
    for (int q = 0; q < L; ++q) {
      const Tensor3& T = C[q];
      for (int v = 1; v <= t.localdims[q]; ++v) {
        cur[q] = v;
        double val = 0.0;
        for (i64 b = 0; b < T.d2; ++b) {
          double w = 0.0;
          for (i64 a = 0; a < T.d0; ++a) w = w + Le[q][a] * T.v[a + T.d0 * ((v - 1) + T.d1 * b)];
          val = val + w * Re[q][b];
        }
        double err = std::fabs(t.f(cur) - val);
        t.nfeval += 1;
        if (err > best_error) {
          best_error = err;
          best = cur;
        }
      }
      cur[q] = point[q];
    }
    if (best_error > abstol * tolmargin) found.push_back(best);
  }
  if ((int)found.size() > maxnglobalpivot) found.resize(maxnglobalpivot);
  return found;
}

i64 tci_rank(const TCI2& t) {
  i64 r = 0;
  for (int b = 1; b < t.L; ++b) r = std::max(r, (i64)t.Iset[b].size());
  return r;
}

// convergencecriterion (tensorci2.jl:609-628)
bool convergencecriterion(const std::vector<i64>& ranks, const std::vector<double>& errors,
                          const std::vector<i64>& ngp, double tolerance, i64 maxbonddim,
                          i64 ncheckhistory, bool checkconvglobalpivot) {
  if ((i64)errors.size() < ncheckhistory) return false;
  const i64 n = ncheckhistory;
  auto lastr = std::vector<i64>(ranks.end() - n, ranks.end());
  auto lastg = std::vector<i64>(ngp.end() - n, ngp.end());
  auto laste = std::vector<double>(errors.end() - n, errors.end());
  bool allerr = true, allg = true, allmax = true;
  for (double e : laste) allerr &= (e < tolerance);
  for (i64 g : lastg) allg &= (g == 0);
  for (i64 r : lastr) allmax &= (r >= maxbonddim);
  i64 mn = *std::min_element(lastr.begin(), lastr.end());
  return (allerr && (checkconvglobalpivot ? allg : true) && mn == lastr.back()) || allmax;
}

// optimize! (tensorci2.jl:700-850) with the default global pivot finder.
int optimize(TCI2& t, const Opts& o) {
  const double tol = o.tolerance;
  const i64 maxbonddim = o.maxbonddim <= 0 ? TYPEMAX : o.maxbonddim;
  if (o.nsearchglobalpivot > 0 && o.nsearchglobalpivot < o.maxnglobalpivot)
    return fail(ORC_ERR, "nsearchglobalpivot < maxnglobalpivot!");
  if (maxbonddim >= TYPEMAX && tol <= 0)
    return fail(ORC_ARG,
                "Specify either tolerance > 0 or some maxbonddim; otherwise, the convergence "
                "criterion is not reachable!");
  tci_rng rng;
  tci_rng_seed(&rng, o.seed);
  t.ranks.clear();
  t.errors.clear();
  t.nglobal.clear();
  for (i64 iter = 1; iter <= o.maxiter; ++iter) {
    double errnorm = o.normalizeerror ? t.maxsamplevalue : 1.0;
    double abstol = tol * errnorm;
    int rc = sweep2site(t, 2, 1, abstol, maxbonddim, o.sweepstrategy, o.strictlynested != 0, true);
    if (rc) return rc;
    double perr = *std::max_element(t.bonderrors.begin(), t.bonderrors.end());
    t.errors.push_back(perr);
    auto gp = default_global_pivots(t, abstol, o.nsearchglobalpivot, o.maxnglobalpivot,
                                    o.tolmarginglobalsearch, &rng);
    rc = addglobalpivots(t, gp);
    if (rc) return rc;
    t.nglobal.push_back((i64)gp.size());
    t.ranks.push_back(tci_rank(t));
    if (convergencecriterion(t.ranks, t.errors, t.nglobal, abstol, maxbonddim, o.ncheckhistory,
                             o.checkconvglobalpivot != 0))
      break;
  }
  double errnorm = o.normalizeerror ? t.maxsamplevalue : 1.0;
  double abstol = tol * errnorm;
  int rc = sweep1site(t, true, 1e-14, abstol, maxbonddim, true);
  if (rc) return rc;
  for (int b = 0; b < t.L - 1; ++b)  // _sanitycheck (globalsearch.jl:106-112)
    if (t.Iset[b + 1].size() != t.Jset[b].size())
      return fail(ORC_ERR, "Pivot matrix at bond " + std::to_string(b + 1) + " is not square!");
  for (auto& e : t.errors) e = e / errnorm;
  return ORC_OK;
}

std::vector<std::pair<orc_batch_fn, void*>> user_fns;  // id F_USER + k

Func make_func(int fid, const double* params, i64 nparams) {
  Func f;
  f.fid = fid;
  if (params) f.params.assign(params, params + nparams);
  const i64 k = (i64)fid - F_USER;
  if (k >= 0 && k < (i64)user_fns.size()) {
    f.cb = user_fns[(size_t)k].first;
    f.user = user_fns[(size_t)k].second;
  }
  return f;
}

std::vector<MultiIndex> read_pivots(const int64_t* piv, i64 np, int L) {
  std::vector<MultiIndex> out;
  for (i64 p = 0; p < np; ++p) {
    MultiIndex v(L);
    for (int q = 0; q < L; ++q) v[q] = (int)piv[p * L + q];
    out.push_back(v);
  }
  return out;
}

// ---------------------------------------------------------------- tensor-train contraction
// Cores with 4 legs (link, s_in, s_out, link'), column-major.  Every contracted
// element is a sum in ascending order of the contracted (fused) index with a
// separate multiply and add -- the reference leaves that order to BLAS
// (contraction.jl:71-93); fixing it makes the device results reproducible.
struct Core4 {
  i64 d[4] = {1, 1, 1, 1};
  std::vector<double> v;
  i64 size() const { return d[0] * d[1] * d[2] * d[3]; }
};
using TT4 = std::vector<Core4>;

// left(lu) / right(lu) (matrixlu.jl:374-392): rows / columns put back in place.
void lu_left(const RRLU& lu, std::vector<double>& out) {
  const i64 m = lu.m, K = lu.npivot;
  out.assign((size_t)(m * K), 0.0);
  for (i64 k = 0; k < K; ++k)
    for (i64 i = 0; i < m; ++i) out[lu.rowperm[i] + m * k] = lu.L[i + m * k];
}
void lu_right(const RRLU& lu, std::vector<double>& out) {
  const i64 n = lu.n, K = lu.npivot;
  out.assign((size_t)(K * n), 0.0);
  for (i64 j = 0; j < n; ++j)
    for (i64 k = 0; k < K; ++k) out[k + K * lu.colperm[j]] = lu.U[k + K * j];
}

// _contractsitetensors (contraction.jl:333-349)
Core4 naive_site(const Core4& a, const Core4& b) {
  Core4 c;
  c.d[0] = a.d[0] * b.d[0];
  c.d[1] = a.d[1];
  c.d[2] = b.d[2];
  c.d[3] = a.d[3] * b.d[3];
  c.v.assign((size_t)c.size(), 0.0);
  const i64 ra = a.d[0], s1 = a.d[1], s2 = a.d[2], ra2 = a.d[3], rb = b.d[0], s3 = b.d[2], rb2 = b.d[3];
  i64 e = 0;
  for (i64 jb = 0; jb < rb2; ++jb)
    for (i64 ja = 0; ja < ra2; ++ja)
      for (i64 i3 = 0; i3 < s3; ++i3)
        for (i64 i1 = 0; i1 < s1; ++i1)
          for (i64 ib = 0; ib < rb; ++ib)
            for (i64 ia = 0; ia < ra; ++ia, ++e) {
              double acc = 0.0;
              for (i64 k = 0; k < s2; ++k)
                acc = acc + a.v[ia + ra * (i1 + s1 * (k + s2 * ja))] * b.v[ib + rb * (k + s2 * (i3 + s3 * jb))];
              c.v[e] = acc;
            }
  return c;
}

// C = A (M x K) * B (K x N), column-major.
void matmul(const double* A, i64 lda, const double* B, i64 ldb, double* C, i64 ldc, i64 M, i64 N, i64 K) {
  for (i64 j = 0; j < N; ++j)
    for (i64 i = 0; i < M; ++i) {
      double acc = 0.0;
      for (i64 k = 0; k < K; ++k) acc = acc + A[i + lda * k] * B[k + ldb * j];
      C[i + ldc * j] = acc;
    }
}

// _factorize(A, :LU; tolerance, maxbonddim, leftorthogonal, normalizeerror)
// (tensortrain.jl:95-110)
// _factorize(A, :LU or :CI; tolerance, maxbonddim, leftorthogonal, normalizeerror)
// (tensortrain.jl:94-110): left/right of the rrLU, or of MatrixLUCI over it.
int factorize_lu(const std::vector<double>& A, i64 m, i64 n, double tolerance, i64 maxbonddim, bool leftorth,
                 bool normalizeerror, std::vector<double>& left, std::vector<double>& right, i64& K,
                 bool ci = false) {
  const double reltol = normalizeerror ? tolerance : 1e-14;
  const double abstol = normalizeerror ? 0.0 : tolerance;
  RRLU lu;
  int rc = rrlu(A.data(), m, n, maxbonddim, reltol, abstol, leftorth, lu);
  if (rc) return rc;
  if (ci) {
    left = luci_left(lu);
    right = luci_right(lu);
  } else {
    lu_left(lu, left);
    lu_right(lu, right);
  }
  K = lu.npivot;
  return ORC_OK;
}

// contract_zipup(A, B; tolerance, method=:LU, maxbonddim) (contraction.jl:442-486)
int contract_zipup_lu(const TT4& A, const TT4& B, double tolerance, i64 maxbonddim, TT4& out, bool ci = false) {
  out.clear();
  const size_t L = A.size();
  std::vector<double> R(1, 1.0);  // (link_ab, link_an, link_bn)
  i64 nab = 1, rna = 1, rnb = 1;
  for (size_t n = 0; n < L; ++n) {
    const Core4 &a = A[n], &b = B[n];
    const i64 s = a.d[1], sp = a.d[2], an2 = a.d[3], spp = b.d[2], bn2 = b.d[3];
    // RA[ab, bn, s, s', an'] = sum_an R[ab, an, bn] A[an, s, s', an']
    std::vector<double> RA((size_t)(nab * rnb * s * sp * an2));
    const i64 ncol = s * sp * an2;
    for (i64 col = 0; col < ncol; ++col)
      for (i64 bn = 0; bn < rnb; ++bn)
        for (i64 ab = 0; ab < nab; ++ab) {
          double acc = 0.0;
          for (i64 k = 0; k < rna; ++k) acc = acc + R[ab + nab * (k + rna * bn)] * a.v[k + rna * col];
          RA[ab + nab * (bn + rnb * col)] = acc;
        }
    // C[ab, s, s'', an', bn'] = sum_{s', bn} RA[ab, bn, s, s', an'] B[bn, s', s'', bn']
    const i64 rows = nab * s * spp, cols = an2 * bn2;
    std::vector<double> C((size_t)(rows * cols));
    i64 e = 0;
    for (i64 b2 = 0; b2 < bn2; ++b2)
      for (i64 a2 = 0; a2 < an2; ++a2)
        for (i64 ipp = 0; ipp < spp; ++ipp)
          for (i64 i = 0; i < s; ++i)
            for (i64 ab = 0; ab < nab; ++ab, ++e) {
              double acc = 0.0;
              for (i64 q = 0; q < sp; ++q)
                for (i64 bn = 0; bn < rnb; ++bn)
                  acc = acc + RA[ab + nab * (bn + rnb * (i + s * (q + sp * a2)))] *
                                  b.v[bn + rnb * (q + sp * (ipp + spp * b2))];
              C[e] = acc;
            }
    Core4 core;
    core.d[0] = nab;
    core.d[1] = s;
    core.d[2] = spp;
    if (n + 1 == L) {
      core.d[3] = cols;
      core.v.swap(C);
      out.push_back(core);
      break;
    }
    std::vector<double> left, right;
    i64 K = 0;
    int rc = factorize_lu(C, rows, cols, tolerance, maxbonddim, false, true, left, right, K, ci);
    if (rc) return rc;
    core.d[3] = K;
    core.v.swap(left);
    out.push_back(core);
    R.swap(right);
    nab = K;
    rna = an2;
    rnb = bn2;
  }
  return ORC_OK;
}

// compress!(tt, :LU; tolerance, maxbonddim, normalizeerror) (tensortrain.jl:149-183)
int compress_lu(TT4& tt, double tolerance, i64 maxbonddim, bool normalizeerror, bool ci = false) {
  const size_t L = tt.size();
  for (size_t l = 0; l + 1 < L; ++l) {
    Core4 &c = tt[l], &nx = tt[l + 1];
    const i64 m = c.d[0] * c.d[1] * c.d[2], ncol = c.d[3];
    std::vector<double> left, right;
    i64 K = 0;
    int rc = factorize_lu(c.v, m, ncol, 0.0, TYPEMAX, true, true, left, right, K, ci);
    if (rc) return rc;
    const i64 nrest = nx.d[1] * nx.d[2] * nx.d[3];
    std::vector<double> nt((size_t)(K * nrest));
    matmul(right.data(), K, nx.v.data(), nx.d[0], nt.data(), K, K, nrest, nx.d[0]);
    c.v.swap(left);
    c.d[3] = K;
    nx.v.swap(nt);
    nx.d[0] = K;
  }
  for (size_t l = L - 1; L >= 2 && l >= 1; --l) {
    Core4 &c = tt[l], &pv = tt[l - 1];
    const i64 mrow = c.d[0], ncol = c.d[1] * c.d[2] * c.d[3];
    std::vector<double> left, right;
    i64 K = 0;
    int rc = factorize_lu(c.v, mrow, ncol, tolerance, maxbonddim, false, normalizeerror, left, right, K, ci);
    if (rc) return rc;
    const i64 prow = pv.d[0] * pv.d[1] * pv.d[2];
    std::vector<double> nt((size_t)(prow * K));
    matmul(pv.v.data(), prow, left.data(), mrow, nt.data(), prow, prow, K, mrow);
    c.v.swap(right);
    c.d[0] = K;
    pv.v.swap(nt);
    pv.d[3] = K;
  }
  return ORC_OK;
}

TT4 read_tt4(int L, const int64_t* dims, const double* values) {
  TT4 t((size_t)L);
  i64 off = 0;
  for (int b = 0; b < L; ++b) {
    for (int q = 0; q < 4; ++q) t[b].d[q] = dims[4 * b + q];
    t[b].v.assign(values + off, values + off + t[b].size());
    off += t[b].size();
  }
  return t;
}

// ---------------------------------------------------------------- Contraction
// The Contraction batch evaluator (contraction.jl:5-62, 103-335) over two trains
// of 4-leg cores, for contract(algorithm = :TCI).  Fused local index v (0-based)
// = i + s_in(A) * j (_unfuse_idx, :95-97).  Environments follow _extend_cache
// (:103-109): left  tmp[b, t, a'] = sum_a P[a, b] A[a, i, t, a'],
// E[a', b'] = sum over (b, t), b fastest, of tmp[b, t, a'] B[b, t, j, b'];
// right the same with the cores' link legs swapped (:165-169).  A Pi element is
// sum over (a, b), a fastest, of Lenv[a, b] Renv[a, b] (:325-329); a single point
// is its full left environment.  Values are cached per point, the first request
// fixing the value (the device evaluator sits behind a value cache).
typedef int (*orc_value_fn)(void* user, int64_t n, double* values);

struct OrcContraction {
  TT4 a, b;
  int L = 0;
  orc_value_fn vf = nullptr;
  void* vuser = nullptr;
  std::unordered_map<std::string, std::vector<double>> left, right;
  std::unordered_map<std::string, double> values;
};

std::string key_of(const MultiIndex& v, size_t from, size_t to) {
  std::string k;
  for (size_t q = from; q < to; ++q) k.push_back((char)(uint8_t)(v[q] - 1));
  return k;
}

const std::vector<double>& env_left(OrcContraction& c, const std::string& k) {
  auto it = c.left.find(k);
  if (it != c.left.end()) return it->second;
  std::vector<double> E;
  if (k.empty()) {
    E.assign(1, 1.0);
  } else {
    const std::vector<double> P = env_left(c, k.substr(0, k.size() - 1));
    const int site = (int)k.size() - 1;
    const Core4 &A = c.a[(size_t)site], &B = c.b[(size_t)site];
    const i64 ra = A.d[0], s = A.d[1], S = A.d[2], ra2 = A.d[3], rb = B.d[0], s2 = B.d[2], rb2 = B.d[3];
    const int v = (uint8_t)k.back();
    const i64 i = v % s, j = v / s;
    std::vector<double> tmp((size_t)(rb * S * ra2));
    for (i64 a2 = 0; a2 < ra2; ++a2)
      for (i64 t = 0; t < S; ++t)
        for (i64 bb = 0; bb < rb; ++bb) {
          double acc = 0.0;
          for (i64 aa = 0; aa < ra; ++aa) acc = acc + P[aa + ra * bb] * A.v[aa + ra * (i + s * (t + S * a2))];
          tmp[bb + rb * (t + S * a2)] = acc;
        }
    E.assign((size_t)(ra2 * rb2), 0.0);
    for (i64 b2 = 0; b2 < rb2; ++b2)
      for (i64 a2 = 0; a2 < ra2; ++a2) {
        double acc = 0.0;
        for (i64 t = 0; t < S; ++t)
          for (i64 bb = 0; bb < rb; ++bb)
            acc = acc + tmp[bb + rb * (t + S * a2)] * B.v[bb + rb * (t + S * (j + s2 * b2))];
        E[a2 + ra2 * b2] = acc;
      }
  }
  return c.left.emplace(k, std::move(E)).first->second;
}

const std::vector<double>& env_right(OrcContraction& c, const std::string& k) {
  auto it = c.right.find(k);
  if (it != c.right.end()) return it->second;
  std::vector<double> E;
  if (k.empty()) {
    E.assign(1, 1.0);
  } else {
    const std::vector<double> P = env_right(c, k.substr(1));
    const int site = c.L - (int)k.size();
    const Core4 &A = c.a[(size_t)site], &B = c.b[(size_t)site];
    const i64 ra = A.d[0], s = A.d[1], S = A.d[2], ra2 = A.d[3], rb = B.d[0], s2 = B.d[2], rb2 = B.d[3];
    const int v = (uint8_t)k[0];
    const i64 i = v % s, j = v / s;
    std::vector<double> tmp((size_t)(rb2 * S * ra));
    for (i64 aa = 0; aa < ra; ++aa)
      for (i64 t = 0; t < S; ++t)
        for (i64 b2 = 0; b2 < rb2; ++b2) {
          double acc = 0.0;
          for (i64 a2 = 0; a2 < ra2; ++a2) acc = acc + P[a2 + ra2 * b2] * A.v[aa + ra * (i + s * (t + S * a2))];
          tmp[b2 + rb2 * (t + S * aa)] = acc;
        }
    E.assign((size_t)(ra * rb), 0.0);
    for (i64 bb = 0; bb < rb; ++bb)
      for (i64 aa = 0; aa < ra; ++aa) {
        double acc = 0.0;
        for (i64 t = 0; t < S; ++t)
          for (i64 b2 = 0; b2 < rb2; ++b2)
            acc = acc + tmp[b2 + rb2 * (t + S * aa)] * B.v[bb + rb * (t + S * (j + s2 * b2))];
        E[aa + ra * bb] = acc;
      }
  }
  return c.right.emplace(k, std::move(E)).first->second;
}

double contraction_value(OrcContraction& c, const std::string& lk, const std::string& rk) {
  const std::vector<double>& Lv = env_left(c, lk);
  const std::vector<double>& Rv = env_right(c, rk);
  double acc = 0.0;
  for (size_t q = 0; q < Lv.size(); ++q) acc = acc + Lv[q] * Rv[q];
  if (c.vf) c.vf(c.vuser, 1, &acc);
  return acc;
}

double contraction_point(OrcContraction& c, const MultiIndex& v) {
  const std::string k = key_of(v, 0, v.size());
  auto it = c.values.find(k);
  if (it != c.values.end()) return it->second;
  const double x = contraction_value(c, k, std::string());
  c.values.emplace(k, x);
  return x;
}

void contraction_fill(OrcContraction& c, const std::vector<MultiIndex>& I, const std::vector<MultiIndex>& J,
                      std::vector<double>& out) {
  for (size_t j = 0; j < J.size(); ++j)
    for (size_t i = 0; i < I.size(); ++i) {
      const std::string lk = key_of(I[i], 0, I[i].size()), rk = key_of(J[j], 0, J[j].size());
      const std::string k = lk + rk;
      auto it = c.values.find(k);
      if (it != c.values.end()) {
        out[i + j * I.size()] = it->second;
        continue;
      }
      const double x = contraction_value(c, lk, rk);
      c.values.emplace(k, x);
      out[i + j * I.size()] = x;
    }
}

// _findinitialpivots + optfirstpivot (contraction.jl:385-397, util.jl:78-108);
// random starts from tci_rng seeded with `seed`.
std::vector<MultiIndex> findinitialpivots(const Func& f, const std::vector<int>& d, int nmax, uint64_t seed) {
  const int L = (int)d.size();
  tci_rng rng;
  tci_rng_seed(&rng, seed);
  std::vector<MultiIndex> starts((size_t)nmax, MultiIndex((size_t)L));
  for (auto& p : starts)
    for (int q = 0; q < L; ++q) p[(size_t)q] = (int)tci_rng_uniform1(&rng, (uint64_t)d[(size_t)q]);
  std::vector<MultiIndex> out;
  for (auto& pivot : starts) {
    double valf = std::fabs(f(pivot));
    for (int sweep = 0; sweep < 1000; ++sweep) {
      const double prev = valf;
      for (int q = 0; q < L; ++q)
        for (int x = 1; x <= d[(size_t)q]; ++x) {
          const int bak = pivot[(size_t)q];
          pivot[(size_t)q] = x;
          const double nv = std::fabs(f(pivot));
          if (nv > valf)
            valf = nv;
          else
            pivot[(size_t)q] = bak;
        }
      if (prev == valf) break;
    }
    if (std::fabs(f(pivot)) == 0.0) continue;
    out.push_back(pivot);
  }
  return out;
}

}  // namespace

// ======================================================================== C ABI
extern "C" {

typedef Opts orc_opts;

const char* orc_last_error(void) { return g_err.c_str(); }

// rrlu (matrixlu.jl:217-225).  rowperm/colperm are 0-based full permutations;
// L is m x npivot and U is npivot x n (column-major), capacities m*min(m,n) and
// min(m,n)*n.  Returns 0, or ORC_NAN with the reference's message.
int orc_rrlu(const double* A, int64_t m, int64_t n, int64_t maxrank, double reltol, double abstol,
             int leftorth, int64_t* rowperm, int64_t* colperm, double* L, double* U,
             int64_t* npivot, double* err) {
  RRLU lu;
  int rc = rrlu(A, m, n, maxrank <= 0 ? TYPEMAX : maxrank, reltol, abstol, leftorth != 0, lu);
  if (rowperm) std::copy(lu.rowperm.begin(), lu.rowperm.end(), rowperm);
  if (colperm) std::copy(lu.colperm.begin(), lu.colperm.end(), colperm);
  if (L) std::copy(lu.L.begin(), lu.L.end(), L);
  if (U) std::copy(lu.U.begin(), lu.U.end(), U);
  if (npivot) *npivot = lu.npivot;
  if (err) *err = lu.error;
  return rc;
}

// MatrixLUCI left/right on the same inputs (matrixluci.jl:70-84).
int orc_luci(const double* A, int64_t m, int64_t n, int64_t maxrank, double reltol, double abstol,
             int leftorth, double* left, double* right, int64_t* npivot) {
  RRLU lu;
  int rc = rrlu(A, m, n, maxrank <= 0 ? TYPEMAX : maxrank, reltol, abstol, leftorth != 0, lu);
  if (rc) return rc;
  auto l = luci_left(lu);
  auto r = luci_right(lu);
  if (left) std::copy(l.begin(), l.end(), left);
  if (right) std::copy(r.begin(), r.end(), right);
  if (npivot) *npivot = lu.npivot;
  return 0;
}

// Many independent rrLUs (matrices packed back to back, column-major), split over
// `nthreads` host threads.  Outputs per matrix: npivot, error, and the first
// min(m,n) entries of the row/col permutations at the given offsets.
int orc_rrlu_batched(int64_t nmat, const double* A, const int64_t* offsets, const int64_t* ms,
                     const int64_t* ns, int64_t maxrank, double reltol, double abstol, int leftorth,
                     int64_t* perm_out, const int64_t* perm_offsets, int64_t* npivots, double* errs,
                     int nthreads) {
  std::atomic<int64_t> next(0);
  std::atomic<int> bad(0);
  auto worker = [&]() {
    for (;;) {
      int64_t i = next.fetch_add(1);
      if (i >= nmat) break;
      RRLU lu;
      int rc = rrlu(A + offsets[i], ms[i], ns[i], maxrank <= 0 ? TYPEMAX : maxrank, reltol, abstol,
                    leftorth != 0, lu);
      if (rc) bad = rc;
      npivots[i] = lu.npivot;
      errs[i] = lu.error;
      if (perm_out) {
        int64_t* o = perm_out + perm_offsets[i];
        for (int64_t k = 0; k < lu.npivot; ++k) {
          o[2 * k] = lu.rowperm[k];
          o[2 * k + 1] = lu.colperm[k];
        }
      }
    }
  };
  nthreads = std::max(1, nthreads);
  std::vector<std::thread> th;
  for (int t = 1; t < nthreads; ++t) th.emplace_back(worker);
  worker();
  for (auto& x : th) x.join();
  return bad.load();
}

// Caller-supplied f under id F_USER + k (k = 0, 1, ... in order of registration).
int orc_register_fn(orc_batch_fn fn, void* user) {
  user_fns.emplace_back(fn, user);
  return F_USER + (int)user_fns.size() - 1;
}

// Function values at points (row-major np x L, 1-based).
int orc_feval(int fid, const double* params, int64_t nparams, int L, const int64_t* pts, int64_t np,
              double* out) {
  Func f = make_func(fid, params, nparams);
  if (f.cb) {
    if (np > 0) f.batch(L, np, pts, out);
    return 0;
  }
  MultiIndex v(L);
  for (int64_t p = 0; p < np; ++p) {
    for (int q = 0; q < L; ++q) v[q] = (int)pts[p * L + q];
    out[p] = f(v);
  }
  return 0;
}

// TensorCI2 handle ---------------------------------------------------------
void* orc_tci_new(int L, const int64_t* localdims, int fid, const double* params, int64_t nparams,
                  const int64_t* pivots, int64_t npiv, int* rc) {
  auto* t = new TCI2();
  std::vector<int> d(localdims, localdims + L);
  *rc = tci_new(*t, d, make_func(fid, params, nparams), read_pivots(pivots, npiv, L));
  return t;
}
void orc_tci_free(void* h) { delete (TCI2*)h; }

// crossinterpolate2 (tensorci2.jl:943-953) = constructor + optimize!
void* orc_crossinterpolate2(int L, const int64_t* localdims, int fid, const double* params,
                            int64_t nparams, const int64_t* pivots, int64_t npiv, const orc_opts* o,
                            int* rc) {
  void* h = orc_tci_new(L, localdims, fid, params, nparams, pivots, npiv, rc);
  if (*rc) return h;
  *rc = optimize(*(TCI2*)h, *o);
  return h;
}

int orc_tci_optimize(void* h, const orc_opts* o) { return optimize(*(TCI2*)h, *o); }

int orc_tci_updatepivots(void* h, int b1, int leftorth, double reltol, double abstol,
                         int64_t maxbonddim) {
  TCI2& t = *(TCI2*)h;
  if (b1 < 1 || b1 > t.L - 1) return fail(ORC_ARG, "bond out of range");
  return updatepivots(t, b1 - 1, leftorth != 0, reltol, abstol, maxbonddim <= 0 ? TYPEMAX : maxbonddim,
                      {}, {});
}

int orc_tci_sweep2site(void* h, int niter, int iter1, double abstol, int64_t maxbonddim, int strategy,
                       int strictlynested, int fillsite) {
  return sweep2site(*(TCI2*)h, niter, iter1, abstol, maxbonddim <= 0 ? TYPEMAX : maxbonddim, strategy,
                    strictlynested != 0, fillsite != 0);
}

int orc_tci_sweep1site(void* h, int forward, double reltol, double abstol, int64_t maxbonddim,
                       int updatetensors) {
  return sweep1site(*(TCI2*)h, forward != 0, reltol, abstol, maxbonddim <= 0 ? TYPEMAX : maxbonddim,
                    updatetensors != 0);
}

int orc_tci_fillsitetensors(void* h) { return fillsitetensors(*(TCI2*)h); }

int orc_tci_addglobalpivots(void* h, const int64_t* pivots, int64_t npiv) {
  TCI2& t = *(TCI2*)h;
  return addglobalpivots(t, read_pivots(pivots, npiv, t.L));
}

// addglobalpivots1sitesweep! (tensorci2.jl:219-229)
int orc_tci_addglobalpivots1sitesweep(void* h, const int64_t* pivots, int64_t npiv, double reltol,
                                      double abstol, int64_t maxbonddim) {
  TCI2& t = *(TCI2*)h;
  int rc = addglobalpivots(t, read_pivots(pivots, npiv, t.L));
  if (rc) return rc;
  return makecanonical(t, reltol, abstol, maxbonddim <= 0 ? TYPEMAX : maxbonddim);
}

int orc_tci_L(void* h) { return ((TCI2*)h)->L; }
double orc_tci_maxsample(void* h) { return ((TCI2*)h)->maxsamplevalue; }
int64_t orc_tci_nfeval(void* h) { return ((TCI2*)h)->nfeval; }

// linkdims (tensorci2.jl:83-85)
int orc_tci_linkdims(void* h, int64_t* out) {
  TCI2& t = *(TCI2*)h;
  for (int b = 0; b < t.L - 1; ++b) out[b] = (int64_t)t.Iset[b + 1].size();
  return 0;
}

// Iset[b]/Jset[b] (b 1-based) as row-major arrays of 1-based indices.  Pass null
// buffers to query the counts only.
int orc_tci_sets(void* h, int b1, int64_t* I, int64_t* nI, int64_t* J, int64_t* nJ) {
  TCI2& t = *(TCI2*)h;
  int b = b1 - 1;
  *nI = (int64_t)t.Iset[b].size();
  *nJ = (int64_t)t.Jset[b].size();
  if (I)
    for (size_t i = 0; i < t.Iset[b].size(); ++i)
      for (int q = 0; q < b; ++q) I[i * b + q] = t.Iset[b][i][q];
  int nr = t.L - 1 - b;
  if (J)
    for (size_t j = 0; j < t.Jset[b].size(); ++j)
      for (int q = 0; q < nr; ++q) J[j * nr + q] = t.Jset[b][j][q];
  return 0;
}

int orc_tci_core(void* h, int b1, double* out, int64_t* dims) {
  TCI2& t = *(TCI2*)h;
  const Tensor3& s = t.sitetensors[b1 - 1];
  dims[0] = s.d0;
  dims[1] = s.d1;
  dims[2] = s.d2;
  if (out) std::copy(s.v.begin(), s.v.end(), out);
  return 0;
}

int orc_tci_errors(void* h, double* pivoterrors, int64_t* npe, double* bonderrors) {
  TCI2& t = *(TCI2*)h;
  *npe = (int64_t)t.pivoterrors.size();
  if (pivoterrors) std::copy(t.pivoterrors.begin(), t.pivoterrors.end(), pivoterrors);
  if (bonderrors) std::copy(t.bonderrors.begin(), t.bonderrors.end(), bonderrors);
  return 0;
}

int orc_tci_history(void* h, int64_t* ranks, double* errors, int64_t* nglobal, int64_t* niter) {
  TCI2& t = *(TCI2*)h;
  *niter = (int64_t)t.ranks.size();
  if (ranks) std::copy(t.ranks.begin(), t.ranks.end(), ranks);
  if (errors) std::copy(t.errors.begin(), t.errors.end(), errors);
  if (nglobal) std::copy(t.nglobal.begin(), t.nglobal.end(), nglobal);
  return 0;
}

int orc_tci_evaluate(void* h, const int64_t* pts, int64_t np, double* out) {
  TCI2& t = *(TCI2*)h;
  MultiIndex v(t.L);
  for (int64_t p = 0; p < np; ++p) {
    for (int q = 0; q < t.L; ++q) v[q] = (int)pts[p * t.L + q];
    out[p] = tt_evaluate(t.sitetensors, v);
  }
  return 0;
}

double orc_tci_sum(void* h) { return tt_sum(((TCI2*)h)->sitetensors); }

// TT given as packed cores (site by site, column-major r_{b-1} x d_b x r_b).
int orc_tt_evaluate(int L, const int64_t* linkdims /*L+1*/, const int64_t* localdims,
                    const double* cores, const int64_t* pts, int64_t np, double* out) {
  std::vector<Tensor3> tt(L);
  const double* c = cores;
  for (int b = 0; b < L; ++b) {
    tt[b].d0 = linkdims[b];
    tt[b].d1 = localdims[b];
    tt[b].d2 = linkdims[b + 1];
    size_t sz = (size_t)(tt[b].d0 * tt[b].d1 * tt[b].d2);
    tt[b].v.assign(c, c + sz);
    c += sz;
  }
  MultiIndex v(L);
  for (int64_t p = 0; p < np; ++p) {
    for (int q = 0; q < L; ++q) v[q] = (int)pts[p * L + q];
    out[p] = tt_evaluate(tt, v);
  }
  return 0;
}

// optfirstpivot(f, localdims, firstpivot; maxsweep) (util.jl:78-108), pivot 1-based, in place.
int orc_optfirstpivot(int fid, const double* params, int64_t nparams, int L, const int64_t* localdims,
                      int64_t* pivot, int maxsweep) {
  Func f = make_func(fid, params, nparams);
  MultiIndex p(L);
  for (int q = 0; q < L; ++q) p[q] = (int)pivot[q];
  double valf = std::fabs(f(p));
  for (int sweep = 0; sweep < maxsweep; ++sweep) {
    const double prev = valf;
    for (int i = 0; i < L; ++i)
      for (int d = 1; d <= localdims[i]; ++d) {
        const int bak = p[i];
        p[i] = d;
        const double nv = std::fabs(f(p));
        if (nv > valf)
          valf = nv;
        else
          p[i] = bak;
      }
    if (prev == valf) break;
  }
  for (int q = 0; q < L; ++q) pivot[q] = p[q];
  return 0;
}

// estimatetrueerror(tt, f; initialpoints) (globalsearch.jl:19-96) for the train
// given as in orc_tt_evaluate and np start points (1-based); writes the (pivot,
// error) pairs sorted by error descending (stable), repeats removed.
int orc_estimatetrueerror(int fid, const double* params, int64_t nparams, int L, const int64_t* linkdims,
                          const int64_t* localdims, const double* cores, const int64_t* starts, int64_t np,
                          int64_t* pivots, double* errors, int64_t* nout) {
  Func f = make_func(fid, params, nparams);
  std::vector<Tensor3> tt(L);
  const double* c = cores;
  for (int b = 0; b < L; ++b) {
    tt[b].d0 = linkdims[b];
    tt[b].d1 = localdims[b];
    tt[b].d2 = linkdims[b + 1];
    size_t sz = (size_t)(tt[b].d0 * tt[b].d1 * tt[b].d2);
    tt[b].v.assign(c, c + sz);
    c += sz;
  }
  std::vector<std::pair<MultiIndex, double>> res;
  for (int64_t k = 0; k < np; ++k) {  // _floatingzone (:48-96)
    MultiIndex p(L);
    for (int q = 0; q < L; ++q) p[q] = (int)starts[k * L + q];
    double maxerror = std::fabs(f(p) - tt_evaluate(tt, p));
    for (;;) {
      const double prev = maxerror;
      for (int ipos = 0; ipos < L; ++ipos) {
        double best = -1.0;
        int arg = 1;
        for (int v = 1; v <= localdims[ipos]; ++v) {
          MultiIndex x = p;
          x[ipos] = v;
          const double err = std::fabs(f(x) - tt_evaluate(tt, x));
          if (err > best) {
            best = err;
            arg = v;
          }
        }
        p[ipos] = arg;
        maxerror = std::max(best, maxerror);
      }
      if (maxerror == prev) break;
    }
    res.emplace_back(p, maxerror);
  }
  std::vector<size_t> order(res.size());
  for (size_t k = 0; k < order.size(); ++k) order[k] = k;
  std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return res[a].second > res[b].second; });
  std::vector<std::pair<MultiIndex, double>> uniq;
  for (size_t k : order)
    if (std::find(uniq.begin(), uniq.end(), res[k]) == uniq.end()) uniq.push_back(res[k]);
  *nout = (int64_t)uniq.size();
  for (size_t k = 0; k < uniq.size(); ++k) {
    for (int q = 0; q < L; ++q) pivots[k * L + q] = uniq[k].first[q];
    errors[k] = uniq[k].second;
  }
  return 0;
}

double orc_tt_sum(int L, const int64_t* linkdims, const int64_t* localdims, const double* cores) {
  std::vector<Tensor3> tt(L);
  const double* c = cores;
  for (int b = 0; b < L; ++b) {
    tt[b].d0 = linkdims[b];
    tt[b].d1 = localdims[b];
    tt[b].d2 = linkdims[b + 1];
    size_t sz = (size_t)(tt[b].d0 * tt[b].d1 * tt[b].d2);
    tt[b].v.assign(c, c + sz);
    c += sz;
  }
  return tt_sum(tt);
}

int orc_convergencecriterion(const int64_t* ranks, const double* errors, const int64_t* ngp, int64_t n,
                             double tolerance, int64_t maxbonddim, int64_t ncheckhistory,
                             int checkconvglobalpivot) {
  std::vector<i64> r(ranks, ranks + n), g(ngp, ngp + n);
  std::vector<double> e(errors, errors + n);
  return convergencecriterion(r, e, g, tolerance, maxbonddim, ncheckhistory, checkconvglobalpivot != 0)
             ? 1
             : 0;
}

// A stream of independent crossinterpolate2 solves split over host threads
// (the CPU baseline for batches of solves).  Request q: sites L[q], local dims
// at dims + doff[q], function fid[q] with params at params + poff[q] (np[q]
// values), tolerance tol[q], maxbonddim mbd[q]; initial pivot all ones.
// Writes per-request rank and wall seconds.
int orc_solve_batch(int64_t nreq, const int32_t* Ls, const int64_t* dims, const int64_t* doff,
                    const int32_t* fids, const double* params, const int64_t* poff, const int64_t* np,
                    const double* tol, const int64_t* mbd, const orc_opts* base, int64_t* rank_out,
                    double* secs_out, int nthreads) {
  std::atomic<int64_t> next(0);
  std::atomic<int> bad(0);
  auto worker = [&]() {
    for (;;) {
      int64_t q = next.fetch_add(1);
      if (q >= nreq) break;
      auto t0 = std::chrono::steady_clock::now();
      Opts o = *base;
      o.tolerance = tol[q];
      o.maxbonddim = mbd[q];
      std::vector<int64_t> piv(Ls[q], 1);
      int rc = 0;
      void* h = orc_crossinterpolate2(Ls[q], dims + doff[q], fids[q], params + poff[q], np[q],
                                      piv.data(), 1, &o, &rc);
      if (rc) bad = rc;
      rank_out[q] = tci_rank(*(TCI2*)h);
      delete (TCI2*)h;
      secs_out[q] =
          std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
  };
  nthreads = std::max(1, nthreads);
  std::vector<std::thread> th;
  for (int t = 1; t < nthreads; ++t) th.emplace_back(worker);
  worker();
  for (auto& x : th) x.join();
  return bad.load();
}

// Tensor-train contraction.  Cores are concatenated in `values` (core b's
// column-major values after core b-1's); dims[4*b + q] is the size of leg q of
// core b.  algorithm: 1 naive (recompressed with compress!(:LU) when tolerance
// > 0 or maxbonddim > 0), 2 zipup with rrLU.  Returns a handle to read with
// orc_tt4_* and free with orc_tt4_free.  method: 0 = :LU, 1 = :CI factorization.
void* orc_tt4_contract(int L, const int64_t* a_dims, const double* a_values, const int64_t* b_dims,
                       const double* b_values, int algorithm, int method, double tolerance, int64_t maxbonddim,
                       int* rc) {
  TT4 a = read_tt4(L, a_dims, a_values), b = read_tt4(L, b_dims, b_values);
  auto* out = new TT4();
  *rc = ORC_OK;
  const bool ci = method == 1;
  if (algorithm == 1) {
    for (int n = 0; n < L; ++n) out->push_back(naive_site(a[n], b[n]));
    if (tolerance > 0 || maxbonddim > 0)
      *rc = compress_lu(*out, tolerance, maxbonddim > 0 ? maxbonddim : TYPEMAX, true, ci);
  } else {
    *rc = contract_zipup_lu(a, b, tolerance, maxbonddim > 0 ? maxbonddim : TYPEMAX, *out, ci);
  }
  return out;
}

// compress!(tt, method) with method 0 = :LU, 1 = :CI.
void* orc_tt4_compress(int L, const int64_t* dims, const double* values, int method, double tolerance,
                       int64_t maxbonddim, int normalizeerror, int* rc) {
  auto* out = new TT4(read_tt4(L, dims, values));
  *rc = compress_lu(*out, tolerance, maxbonddim > 0 ? maxbonddim : TYPEMAX, normalizeerror != 0, method == 1);
  return out;
}

// contract(A, B; algorithm = :TCI, f, initialpivots, kwargs...) (contraction.jl:399-434):
// pivots np x L fused and 1-based, or np = 0 for ninit random starts.  Returns a
// TT4 handle with the legs split.
void* orc_tt4_contract_tci(int L, const int64_t* a_dims, const double* a_values, const int64_t* b_dims,
                           const double* b_values, const int64_t* pivots, int64_t np, int ninit, orc_value_fn vf,
                           void* vuser, const orc_opts* o, int* rc) {
  auto c = std::make_shared<OrcContraction>();
  c->a = read_tt4(L, a_dims, a_values);
  c->b = read_tt4(L, b_dims, b_values);
  c->L = L;
  c->vf = vf;
  c->vuser = vuser;
  auto* out = new TT4();
  *rc = ORC_OK;
  std::vector<int> d((size_t)L);
  for (int n = 0; n < L; ++n) {
    if (c->a[(size_t)n].d[2] != c->b[(size_t)n].d[1]) {
      *rc = fail(ORC_ARG, "Cannot contract tensor trains with non-matching site dimensions.");
      return out;
    }
    d[(size_t)n] = (int)(c->a[(size_t)n].d[1] * c->b[(size_t)n].d[2]);
  }
  Func f;
  f.fid = -1;
  f.ctr = c;
  std::vector<MultiIndex> piv = np > 0 ? read_pivots(pivots, np, L) : findinitialpivots(f, d, ninit, o->seed);
  if (piv.empty()) {
    *rc = fail(ORC_ERR, "No initial pivots found.");
    return out;
  }
  TCI2 t;
  *rc = tci_new(t, d, f, piv);
  if (!*rc) *rc = optimize(t, *o);
  if (*rc) return out;
  for (int n = 0; n < L; ++n) {
    const Tensor3& T = t.sitetensors[(size_t)n];
    Core4 k;
    k.d[0] = T.d0;
    k.d[1] = c->a[(size_t)n].d[1];
    k.d[2] = c->b[(size_t)n].d[2];
    k.d[3] = T.d2;
    k.v = T.v;
    out->push_back(k);
  }
  return out;
}

int orc_tt4_length(void* h) { return (int)((TT4*)h)->size(); }
void orc_tt4_dims(void* h, int64_t* dims) {
  const TT4& t = *(TT4*)h;
  for (size_t b = 0; b < t.size(); ++b)
    for (int q = 0; q < 4; ++q) dims[4 * b + q] = t[b].d[q];
}
void orc_tt4_core(void* h, int b, double* out) {
  const Core4& c = (*(TT4*)h)[(size_t)b];
  std::memcpy(out, c.v.data(), c.v.size() * sizeof(double));
}
void orc_tt4_free(void* h) { delete (TT4*)h; }

}  // extern "C"
