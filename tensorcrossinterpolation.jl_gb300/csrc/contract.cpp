// Tensor-train contraction on the device: contract_naive (contraction.jl:351-372),
// contract_zipup with rrLU factorization (contraction.jl:442-486 with
// _factorize(:LU) or _factorize(:CI), tensortrain.jl:94-110) and compress!(:LU / :CI)
// (tensortrain.jl:149-183).  The rank-revealing LUs are RRLU tasks of the step
// kernel (bit-exact pivots); the contractions are the fixed-order kernels of
// contract.cu, so every result equals the CPU oracle's bit for bit.
#include "contract.h"

#include <algorithm>
#include <climits>
#include <cstring>
#include <string>

#include "tc_gemm.h"

cudaError_t tci_naive_site_launch(const double* a, const double* b, double* out, int ra, int s1, int s2, int ra2,
                                  int rb, int s3, int rb2, cudaStream_t st);
cudaError_t tci_zip_ra_launch(const double* R, const double* A, double* RA, int nab, int nan_, int nbn, int s,
                              int sp, int nan2, cudaStream_t st);
cudaError_t tci_zip_c_launch(const double* RA, const double* B, double* C, int nab, int nbn, int s, int sp, int nan2,
                             int spp, int nbn2, cudaStream_t st);
cudaError_t tci_lu_left_right_launch(const double* F, const int32_t* rowperm, const int32_t* colperm, int m, int n,
                                     int K, int leftorth, double* left, double* right, cudaStream_t st);
cudaError_t tci_luci_left_right_launch(const double* F, const int32_t* rowperm, const int32_t* colperm, int m,
                                       int n, int K, int leftorth, double* left, double* right, cudaStream_t st);
cudaError_t tci_gemm_launch(const double* A, int64_t lda, const double* B, int64_t ldb, double* C, int64_t ldc,
                            int M, int N, int K, cudaStream_t st);

namespace tci {

namespace {

int fail(int code, const std::string& msg) {
  set_error(code, msg);
  return code;
}

#define CT_TRY(x)                                                              \
  do {                                                                         \
    cudaError_t _e = (x);                                                      \
    if (_e != cudaSuccess) return fail(TCI_ERR_CUDA, cudaGetErrorString(_e));  \
  } while (0)

bool fits_int(int64_t v) { return v >= 0 && v <= INT_MAX; }

// Device buffer from the engine's pool, released on scope exit unless taken.
struct Buf {
  Engine& e;
  double* p = nullptr;
  Buf(Engine& eng, size_t elems) : e(eng) { p = e.alloc_core(elems); }
  ~Buf() {
    if (p) e.free_core(p);
  }
  double* take() {
    double* q = p;
    p = nullptr;
    return q;
  }
};

// One split-precision product on the engine stream, then its FP64 error at
// split->samples hashed entries (waits for the stream).
int split_product(Engine& e, SplitRun* split, int64_t M, int64_t N, int64_t K, const double* A, tci_map3 a_row,
                  tci_map3 a_k, int a_kfast, const double* B, tci_map3 b_row, tci_map3 b_k, int b_kfast, double* C,
                  tci_map3 c_row, tci_map3 c_col) {
  if (M == 0 || N == 0) return 0;
  const size_t ws = tci_tc_gemm_workspace(M, N, K);
  Buf W(e, ws / sizeof(double) + 1), S(e, 4);
  if (!W.p || !S.p) return fail(TCI_ERR_OOM, "device memory for the split-precision product");
  CT_TRY(cudaMemsetAsync(S.p, 0, 4 * sizeof(double), e.stream()));
  int* err = (int*)(S.p + 2);
  cudaEvent_t ev[2];
  CT_TRY(cudaEventCreate(&ev[0]));
  CT_TRY(cudaEventCreate(&ev[1]));
  struct EvGuard {
    cudaEvent_t* ev;
    ~EvGuard() {
      cudaEventDestroy(ev[0]);
      cudaEventDestroy(ev[1]);
    }
  } evg{ev};
  CT_TRY(cudaEventRecord(ev[0], e.stream()));
  CT_TRY(tci_tc_gemm_split(M, N, K, A, a_row, a_k, a_kfast, B, b_row, b_k, b_kfast, C, c_row, c_col, W.p, err,
                           e.stream()));
  CT_TRY(cudaEventRecord(ev[1], e.stream()));
  CT_TRY(tci_tc_gemm_sample_error(M, N, K, A, a_row, a_k, B, b_row, b_k, C, c_row, c_col, split->samples,
                                  0x5eedULL + (uint64_t)split->products, (unsigned long long*)S.p, e.stream()));
  double h[4];
  CT_TRY(cudaMemcpyAsync(h, S.p, sizeof(h), cudaMemcpyDeviceToHost, e.stream()));
  CT_TRY(cudaStreamSynchronize(e.stream()));
  int code;
  std::memcpy(&code, &h[2], sizeof(int));
  if (code) return fail(TCI_ERR_TIMEOUT, "tensor-core product: a bounded wait ran out (code " + std::to_string(code) + ")");
  const double rel = h[1] > 0 ? h[0] / h[1] : h[0];
  split->max_rel_err = std::max(split->max_rel_err, rel);
  split->products += 1;
  split->flops += 2.0 * (double)M * (double)N * (double)K;
  float ms = 0.f;
  if (cudaEventElapsedTime(&ms, ev[0], ev[1]) == cudaSuccess) e.stats.tc_ms += ms;
  e.stats.tc_flops += 2.0 * (double)M * (double)N * (double)K;
  return 0;
}

}  // namespace

int device_matmul(Engine& e, const double* A, const double* B, double* C, int64_t M, int64_t N, int64_t K,
                  SplitRun* split) {
  if (M == 0 || N == 0) return 0;
  if (!split) {
    if (!fits_int(M) || !fits_int(N) || !fits_int(K)) return fail(TCI_ERR_TOO_LARGE, "matrix too large");
    CT_TRY(tci_gemm_launch(A, M, B, K, C, M, (int)M, (int)N, (int)K, e.stream()));
    CT_TRY(cudaStreamSynchronize(e.stream()));
    return 0;
  }
  // C[m, n] = sum_k A[m + M k] * B[k + K n]: A rows unit stride, B "rows" (n) stride K
  return split_product(e, split, M, N, K, A, tci_map_stride(1), tci_map_stride(M), M == 1, B, tci_map_stride(K),
                       tci_map_stride(1), 1, C, tci_map_stride(1), tci_map_stride(M));
}

void TT4::release(Engine& e) {
  for (auto& c : cores) {
    if (c.p) e.free_core(c.p);
    c.p = nullptr;
  }
  cores.clear();
}

// rrlu(A; maxrank, reltol, abstol, leftorthogonal) on a device matrix, then
// left (m x K) and right (K x n) into new device arrays: those of the rrLU
// (matrixlu.jl:374-392), or with ci those of MatrixLUCI (matrixluci.jl:40-84).
int device_rrlu_left_right(Engine& e, const double* A, int64_t m, int64_t n, int64_t maxrank, double reltol,
                           double abstol, bool leftorth, double** left, double** right, int64_t* npivot,
                           bool ci) {
  *left = *right = nullptr;
  if (m > 65535 || n > 65535 || m * n > INT_MAX)
    return fail(TCI_ERR_TOO_LARGE, "matrix too large for the rrLU kernel");
  const int64_t kmax = std::min<int64_t>(maxrank <= 0 ? INT64_MAX : maxrank, std::min(m, n));
  Req r;
  r.t.kind = TCI_TASK_RRLU;
  r.t.m = (int32_t)m;
  r.t.n = (int32_t)n;
  r.t.maxrank = (int32_t)kmax;
  r.t.kcap = (int32_t)std::max<int64_t>(kmax, 1);
  r.t.reltol = reltol;
  r.t.abstol = abstol;
  r.t.leftorth = leftorth ? 1 : 0;
  r.t.post = TCI_POST_FACTORS;
  r.t.ain = A;
  const size_t fact = (size_t)(m * n) + ((size_t)(m + n) * 4 + 7) / 8;
  Buf F(e, fact);
  if (!F.p) return fail(TCI_ERR_OOM, "device memory for the factors");
  r.t.core_out = F.p;
  std::vector<Req*> reqs{&r};
  int rc = e.run_tasks(reqs);
  if (rc) return rc;
  const tci_result_head* h = r.head();
  if (h->status & TCI_ST_NAN) return fail(TCI_ERR_NAN, "lu.L contains NaNs");
  const int64_t K = h->npivot;
  Buf L(e, (size_t)std::max<int64_t>(m * K, 1)), U(e, (size_t)std::max<int64_t>(K * n, 1));
  if (!L.p || !U.p) return fail(TCI_ERR_OOM, "device memory for the factors");
  const int32_t* perms = (const int32_t*)(F.p + m * n);
  if (ci)
    CT_TRY(tci_luci_left_right_launch(F.p, perms, perms + m, (int)m, (int)n, (int)K, leftorth ? 1 : 0, L.p, U.p,
                                      e.stream()));
  else
    CT_TRY(tci_lu_left_right_launch(F.p, perms, perms + m, (int)m, (int)n, (int)K, leftorth ? 1 : 0, L.p, U.p,
                                    e.stream()));
  CT_TRY(cudaStreamSynchronize(e.stream()));  // F goes back to the pool below
  *left = L.take();
  *right = U.take();
  *npivot = K;
  return 0;
}

static int check_tt(const TT4& t, const char* name) {
  for (size_t n = 0; n < t.cores.size(); ++n) {
    const Tensor4& c = t.cores[n];
    for (int q = 0; q < 4; ++q)
      if (!fits_int(c.d[q]) || c.d[q] < 1) return fail(TCI_ERR_DIM, std::string(name) + ": bad core dimensions");
    if (n > 0 && t.cores[n - 1].d[3] != c.d[0])
      return fail(TCI_ERR_DIM, std::string(name) + ": bond dimensions of neighbouring cores differ");
  }
  if (!t.cores.empty() && (t.cores.front().d[0] != 1 || t.cores.back().d[3] != 1))
    return fail(TCI_ERR_DIM, std::string(name) + ": outer bonds must be 1");
  return 0;
}

// contract_naive without recompression (contraction.jl:351-372, :333-349).
int tt4_contract_naive(Engine& e, const TT4& a, const TT4& b, TT4& out) {
  out.cores.clear();
  const size_t L = a.cores.size();
  for (size_t n = 0; n < L; ++n) {
    const Tensor4 &x = a.cores[n], &y = b.cores[n];
    Tensor4 c;
    c.d[0] = x.d[0] * y.d[0];
    c.d[1] = x.d[1];
    c.d[2] = y.d[2];
    c.d[3] = x.d[3] * y.d[3];
    for (int q = 0; q < 4; ++q)
      if (!fits_int(c.d[q])) return fail(TCI_ERR_TOO_LARGE, "contracted core too large");
    c.p = e.alloc_core(c.elems());
    if (!c.p) {
      out.release(e);
      return fail(TCI_ERR_OOM, "device memory for the contracted cores");
    }
    out.cores.push_back(c);
    CT_TRY(tci_naive_site_launch(x.p, y.p, c.p, (int)x.d[0], (int)x.d[1], (int)x.d[2], (int)x.d[3], (int)y.d[0],
                                 (int)y.d[2], (int)y.d[3], e.stream()));
  }
  CT_TRY(cudaStreamSynchronize(e.stream()));
  return 0;
}

// contract_zipup(A, B; tolerance, method=:LU, maxbonddim) (contraction.jl:442-486).
int tt4_contract_zipup(Engine& e, const TT4& a, const TT4& b, double tolerance, int64_t maxbonddim, TT4& out,
                       bool ci, SplitRun* split) {
  out.cores.clear();
  const size_t L = a.cores.size();
  // R: (link_ab, link_an, link_bn), starts as ones(1, 1, 1)
  int64_t nab = 1, rna = 1, rnb = 1;
  Buf R(e, 1);
  if (!R.p) return fail(TCI_ERR_OOM, "device memory");
  const double one = 1.0;
  CT_TRY(cudaMemcpyAsync(R.p, &one, sizeof(double), cudaMemcpyHostToDevice, e.stream()));
  CT_TRY(cudaStreamSynchronize(e.stream()));
  for (size_t n = 0; n < L; ++n) {
    const Tensor4 &A = a.cores[n], &B = b.cores[n];
    const int64_t s = A.d[1], sp = A.d[2], an2 = A.d[3], spp = B.d[2], bn2 = B.d[3];
    const int64_t ra_elems = nab * rnb * s * sp * an2;
    const int64_t c_rows = nab * s * spp, c_cols = an2 * bn2;
    if (!fits_int(ra_elems) || !fits_int(c_rows * c_cols)) return fail(TCI_ERR_TOO_LARGE, "zipup block too large");
    Buf RA(e, (size_t)ra_elems), C(e, (size_t)(c_rows * c_cols));
    if (!RA.p || !C.p) {
      out.release(e);
      return fail(TCI_ERR_OOM, "device memory for the zipup blocks");
    }
    if (!split) {
      CT_TRY(tci_zip_ra_launch(R.p, A.p, RA.p, (int)nab, (int)rna, (int)rnb, (int)s, (int)sp, (int)an2, e.stream()));
      CT_TRY(tci_zip_c_launch(RA.p, B.p, C.p, (int)nab, (int)rnb, (int)s, (int)sp, (int)an2, (int)spp, (int)bn2,
                              e.stream()));
    } else {
      // RA[ab, bn, (s, s', an')] = sum_an R[ab, an, bn] A[an, (s, s', an')]: rows (ab, bn)
      int rc = split_product(e, split, nab * rnb, s * sp * an2, rna, R.p, tci_map_2(nab, 1, nab * rna),
                             tci_map_stride(nab), nab == 1, A.p, tci_map_stride(rna), tci_map_stride(1), 1, RA.p,
                             tci_map_stride(1), tci_map_stride(nab * rnb));
      // C[ab, s, s'', an', bn'] = sum_(bn, s') RA[ab, bn, s, s', an'] B[bn, s', s'', bn']:
      // rows (ab, s, an'), contracted (bn, s'), columns (s'', bn')
      if (!rc)
        rc = split_product(e, split, nab * s * an2, spp * bn2, rnb * sp, RA.p,
                           tci_map_3(nab, s, 1, nab * rnb, nab * rnb * s * sp), tci_map_2(rnb, nab, nab * rnb * s),
                           nab == 1, B.p, tci_map_stride(rnb * sp), tci_map_stride(1), 1, C.p,
                           tci_map_3(nab, s, 1, nab, nab * s * spp), tci_map_2(spp, nab * s, nab * s * spp * an2));
      if (rc) {
        out.release(e);
        return rc;
      }
    }
    Tensor4 core;
    core.d[0] = nab;
    core.d[1] = s;
    core.d[2] = spp;
    if (n + 1 == L) {  // reshape(C, size(C)[1:3]..., 1)
      CT_TRY(cudaStreamSynchronize(e.stream()));
      core.d[3] = c_cols;  // 1 x 1 for a closed train
      core.p = C.take();
      out.cores.push_back(core);
      break;
    }
    double *left = nullptr, *right = nullptr;
    int64_t K = 0;
    CT_TRY(cudaStreamSynchronize(e.stream()));
    // _factorize(Cmat, :LU; tolerance, maxbonddim): reltol = tolerance, leftorthogonal = false
    int rc =
        device_rrlu_left_right(e, C.p, c_rows, c_cols, maxbonddim, tolerance, 0.0, false, &left, &right, &K, ci);
    if (rc) {
      out.release(e);
      return rc;
    }
    core.d[3] = K;
    core.p = left;
    out.cores.push_back(core);
    e.free_core(R.take());
    R.p = right;  // R = reshape(right, K, an', bn')
    nab = K;
    rna = an2;
    rnb = bn2;
  }
  return 0;
}

// compress!(tt, :LU or :CI; tolerance, maxbonddim, normalizeerror) (tensortrain.jl:149-183).
int tt4_compress(Engine& e, TT4& tt, double tolerance, int64_t maxbonddim, bool normalizeerror, bool ci) {
  const size_t L = tt.cores.size();
  auto rest = [](const Tensor4& c) { return c.d[1] * c.d[2]; };
  // left to right, no truncation, left-orthogonal
  for (size_t l = 0; l + 1 < L; ++l) {
    Tensor4& c = tt.cores[l];
    Tensor4& nx = tt.cores[l + 1];
    const int64_t m = c.d[0] * rest(c), ncol = c.d[3];
    double *left = nullptr, *right = nullptr;
    int64_t K = 0;
    int rc = device_rrlu_left_right(e, c.p, m, ncol, 0, 0.0, 0.0, true, &left, &right, &K, ci);
    if (rc) return rc;
    const int64_t nrest = rest(nx) * nx.d[3];
    double* nt = e.alloc_core((size_t)std::max<int64_t>(K * nrest, 1));
    if (!nt) {
      e.free_core(left);
      e.free_core(right);
      return fail(TCI_ERR_OOM, "device memory");
    }
    // nexttensor = right (K x r) * reshape(next, r, rest)
    CT_TRY(tci_gemm_launch(right, K, nx.p, nx.d[0], nt, K, (int)K, (int)nrest, (int)nx.d[0], e.stream()));
    CT_TRY(cudaStreamSynchronize(e.stream()));
    e.free_core(right);
    e.free_core(c.p);
    e.free_core(nx.p);
    c.p = left;
    c.d[3] = K;
    nx.p = nt;
    nx.d[0] = K;
  }
  if (L < 2) return 0;
  // right to left, truncating, right factor kept
  for (size_t l = L - 1; l >= 1; --l) {
    Tensor4& c = tt.cores[l];
    Tensor4& pv = tt.cores[l - 1];
    const int64_t mrow = c.d[0], ncol = rest(c) * c.d[3];
    double *left = nullptr, *right = nullptr;
    int64_t K = 0;
    const double reltol = normalizeerror ? tolerance : 1e-14;
    const double abstol = normalizeerror ? 0.0 : tolerance;
    int rc =
        device_rrlu_left_right(e, c.p, mrow, ncol, maxbonddim, reltol, abstol, false, &left, &right, &K, ci);
    if (rc) return rc;
    const int64_t prow = pv.d[0] * rest(pv);
    double* nt = e.alloc_core((size_t)std::max<int64_t>(prow * K, 1));
    if (!nt) {
      e.free_core(left);
      e.free_core(right);
      return fail(TCI_ERR_OOM, "device memory");
    }
    // nexttensor = reshape(prev, prow, r) * left (r x K)
    CT_TRY(tci_gemm_launch(pv.p, prow, left, mrow, nt, prow, (int)prow, (int)K, (int)mrow, e.stream()));
    CT_TRY(cudaStreamSynchronize(e.stream()));
    e.free_core(left);
    e.free_core(c.p);
    e.free_core(pv.p);
    c.p = right;
    c.d[0] = K;
    pv.p = nt;
    pv.d[3] = K;
  }
  return 0;
}

int tt4_check_pair(const TT4& a, const TT4& b, bool sites_must_match) {
  if (a.cores.size() != b.cores.size())
    return fail(TCI_ERR_ARG, "Cannot contract tensor trains with different length.");
  int rc = check_tt(a, "A");
  if (!rc) rc = check_tt(b, "B");
  if (rc) return rc;
  if (sites_must_match)
    for (size_t n = 0; n < a.cores.size(); ++n)
      if (a.cores[n].d[2] != b.cores[n].d[1])
        return fail(TCI_ERR_GENERIC, "Tensor trains must share the identical index at n=" + std::to_string(n + 1) + "!");
  return 0;
}

int tt4_check(const TT4& t) { return check_tt(t, "tensor train"); }

}  // namespace tci
