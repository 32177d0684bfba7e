// Tensor-train contraction kernels (contraction.jl): the site contractions of
// contract_naive (:333-349) and contract_zipup (:442-486), the left/right
// factors of an rrLU (matrixlu.jl:374-392) and the small matrix products of
// compress! (tensortrain.jl:149-183).
//
// Every output element is one thread's sum over the contracted index in a fixed
// ascending order with separate IEEE multiply and add (the file is compiled
// without FMA contraction), so the results are reproducible and equal, bit for
// bit, to the CPU oracle's loops.  The reference contracts through BLAS, whose
// summation order is unspecified, so against the reference itself these are
// tolerance-level results (as its own tests compare them).
//
// Layouts are column-major.  A 4-leg core is (link, s_in, s_out, link').
#include <cuda_runtime.h>
#include <stdint.h>

namespace {

constexpr int CT = 256;

__device__ __forceinline__ int64_t gtid() { return (int64_t)blockIdx.x * blockDim.x + threadIdx.x; }
__device__ __forceinline__ int64_t gstride() { return (int64_t)gridDim.x * blockDim.x; }

// _contractsitetensors (contraction.jl:333-349):
// out[(ia, ib), s1, s3, (ja, jb)] = sum_k a[ia, s1, k, ja] * b[ib, k, s3, jb],
// (ia, ib) and (ja, jb) fused with the a index fastest.
__global__ void naive_site_kernel(const double* __restrict__ a, const double* __restrict__ b, double* __restrict__ out,
                                  int ra, int s1, int s2, int ra2, int rb, int s3, int rb2) {
  const int64_t total = (int64_t)ra * rb * s1 * s3 * ra2 * rb2;
  for (int64_t e = gtid(); e < total; e += gstride()) {
    int64_t t = e;
    const int ia = (int)(t % ra); t /= ra;
    const int ib = (int)(t % rb); t /= rb;
    const int i1 = (int)(t % s1); t /= s1;
    const int i3 = (int)(t % s3); t /= s3;
    const int ja = (int)(t % ra2); t /= ra2;
    const int jb = (int)t;
    double acc = 0.0;
    for (int k = 0; k < s2; ++k) {
      const double x = a[ia + (int64_t)ra * (i1 + (int64_t)s1 * (k + (int64_t)s2 * ja))];
      const double y = b[ib + (int64_t)rb * (k + (int64_t)s2 * (i3 + (int64_t)s3 * jb))];
      acc = __dadd_rn(acc, __dmul_rn(x, y));
    }
    out[e] = acc;
  }
}

// Zipup, first product (contraction.jl:461-463): RA[ab, bn, s, s', an'] =
// sum_an R[ab, an, bn] * A[an, s, s', an'].
__global__ void zip_ra_kernel(const double* __restrict__ R, const double* __restrict__ A, double* __restrict__ RA,
                              int nab, int nan_, int nbn, int s, int sp, int nan2) {
  const int64_t total = (int64_t)nab * nbn * s * sp * nan2;
  for (int64_t e = gtid(); e < total; e += gstride()) {
    int64_t t = e;
    const int ab = (int)(t % nab); t /= nab;
    const int bn = (int)(t % nbn); t /= nbn;
    const int col = (int)t;  // (s, s', an') fused
    double acc = 0.0;
    for (int k = 0; k < nan_; ++k) {
      const double x = R[ab + (int64_t)nab * (k + (int64_t)nan_ * bn)];
      const double y = A[k + (int64_t)nan_ * col];
      acc = __dadd_rn(acc, __dmul_rn(x, y));
    }
    RA[e] = acc;
  }
}

// Zipup, second product (contraction.jl:464-469): C[ab, s, s'', an', bn'] =
// sum_{s'} sum_{bn} RA[ab, bn, s, s', an'] * B[bn, s', s'', bn'], the fused
// contracted index (bn, s') ascending with bn fastest.
__global__ void zip_c_kernel(const double* __restrict__ RA, const double* __restrict__ B, double* __restrict__ C,
                             int nab, int nbn, int s, int sp, int nan2, int spp, int nbn2) {
  const int64_t total = (int64_t)nab * s * spp * nan2 * nbn2;
  for (int64_t e = gtid(); e < total; e += gstride()) {
    int64_t t = e;
    const int ab = (int)(t % nab); t /= nab;
    const int i = (int)(t % s); t /= s;
    const int ipp = (int)(t % spp); t /= spp;
    const int a2 = (int)(t % nan2); t /= nan2;
    const int b2 = (int)t;
    double acc = 0.0;
    for (int q = 0; q < sp; ++q)
      for (int bn = 0; bn < nbn; ++bn) {
        const double x = RA[ab + (int64_t)nab * (bn + (int64_t)nbn * (i + (int64_t)s * (q + (int64_t)sp * a2)))];
        const double y = B[bn + (int64_t)nbn * (q + (int64_t)sp * (ipp + (int64_t)spp * b2))];
        acc = __dadd_rn(acc, __dmul_rn(x, y));
      }
    C[e] = acc;
  }
}

// left(lu) and right(lu) (matrixlu.jl:374-392) from the factored m x n matrix F
// (L below the diagonal, U on and above; unit diagonal on L when leftorth,
// else on U) and the full 0-based permutations:
// left[rowperm[i], k] = L[i, k] (m x K), right[k, colperm[j]] = U[k, j] (K x n).
__global__ void lu_left_right_kernel(const double* __restrict__ F, const int32_t* __restrict__ rowperm,
                                     const int32_t* __restrict__ colperm, int m, int n, int K, int leftorth,
                                     double* __restrict__ left, double* __restrict__ right) {
  const int64_t nl = left ? (int64_t)m * K : 0, nr = right ? (int64_t)K * n : 0;
  for (int64_t e = gtid(); e < nl + nr; e += gstride()) {
    if (e < nl) {
      const int i = (int)(e % m), k = (int)(e / m);
      const double v = i < k ? 0.0 : (i == k && leftorth ? 1.0 : F[i + (int64_t)m * k]);
      left[rowperm[i] + (int64_t)m * k] = v;
    } else {
      const int64_t f = e - nl;
      const int k = (int)(f % K), j = (int)(f / K);
      const double v = k > j ? 0.0 : (k == j && !leftorth ? 1.0 : F[k + (int64_t)m * j]);
      right[k + (int64_t)K * colperm[j]] = v;
    }
  }
}

// MatrixLUCI left/right (matrixluci.jl:40-84) from the factored matrix F as
// above: one thread per row of left (m threads), then one per column of right
// (n threads), each in the order of the oracle's loops (separate multiply,
// add/subtract and divide).
//   leftorth:  left = colstimespivotinv (rows K.. of L against LowerTriangular(L11),
//              rows scattered by rowperm), right = rowmatrix = L[1:K, :] * right(lu)
//   !leftorth: left = colmatrix = left(lu) * U[:, 1:K], right = pivotinvtimesrows
//              (UpperTriangular(U11) \ U12, columns scattered by colperm)
__device__ __forceinline__ double f_L(const double* F, int m, int i, int p, int leftorth) {
  return i < p ? 0.0 : (i == p && leftorth ? 1.0 : F[i + (int64_t)m * p]);
}
__device__ __forceinline__ double f_U(const double* F, int m, int p, int j, int leftorth) {
  return p > j ? 0.0 : (p == j && !leftorth ? 1.0 : F[p + (int64_t)m * j]);
}

__global__ void luci_left_right_kernel(const double* __restrict__ F, const int32_t* __restrict__ rowperm,
                                       const int32_t* __restrict__ colperm, int m, int n, int K, int leftorth,
                                       double* __restrict__ left, double* __restrict__ right) {
  for (int64_t e = gtid(); e < (int64_t)m + n; e += gstride()) {
    if (e < m) {
      const int i = (int)e;
      double* out = left + rowperm[i];  // out[q * m] = entry (rowperm[i], q)
      if (leftorth) {
        if (i < K) {
          for (int q = 0; q < K; ++q) out[(int64_t)m * q] = i == q ? 1.0 : 0.0;
        } else {
          for (int q = K - 1; q >= 0; --q) {
            double s = f_L(F, m, i, q, 1);
            for (int p = q + 1; p < K; ++p) s = __dsub_rn(s, __dmul_rn(out[(int64_t)m * p], f_L(F, m, p, q, 1)));
            out[(int64_t)m * q] = __ddiv_rn(s, f_L(F, m, q, q, 1));
          }
        }
      } else {
        for (int q = 0; q < K; ++q) {
          double s = 0.0;
          for (int p = 0; p <= q; ++p) s = __dadd_rn(s, __dmul_rn(f_L(F, m, i, p, 0), f_U(F, m, p, q, 0)));
          out[(int64_t)m * q] = s;
        }
      }
    } else {
      const int j = (int)(e - m);
      double* out = right + (int64_t)K * colperm[j];  // out[q] = entry (q, colperm[j])
      if (leftorth) {
        for (int q = 0; q < K; ++q) {
          double s = 0.0;
          for (int p = 0; p <= q; ++p) s = __dadd_rn(s, __dmul_rn(f_L(F, m, q, p, 1), f_U(F, m, p, j, 1)));
          out[q] = s;
        }
      } else if (j < K) {
        for (int q = 0; q < K; ++q) out[q] = j == q ? 1.0 : 0.0;
      } else {
        for (int q = K - 1; q >= 0; --q) {
          double s = f_U(F, m, q, j, 0);
          for (int p = q + 1; p < K; ++p) s = __dsub_rn(s, __dmul_rn(f_U(F, m, q, p, 0), out[p]));
          out[q] = __ddiv_rn(s, f_U(F, m, q, q, 0));
        }
      }
    }
  }
}

// C (M x N) = A (M x K) * B (K x N), column-major with leading dimensions.
__global__ void gemm_kernel(const double* __restrict__ A, int64_t lda, const double* __restrict__ B, int64_t ldb,
                            double* __restrict__ C, int64_t ldc, int M, int N, int K) {
  const int64_t total = (int64_t)M * N;
  for (int64_t e = gtid(); e < total; e += gstride()) {
    const int i = (int)(e % M), j = (int)(e / M);
    double acc = 0.0;
    for (int k = 0; k < K; ++k) acc = __dadd_rn(acc, __dmul_rn(A[i + lda * k], B[k + ldb * j]));
    C[i + ldc * j] = acc;
  }
}

// ---- environments of the Contraction evaluator (contraction.jl:103-176) ----
// One level of new environments: entry e extends parent[e] (ra x rb) by site
// value (ii[e], jj[e]) of A (ra x s x S x ra2) and B (rb x S x s2 x rb2).
//   left:  tmp[b, t, a'] = sum_a P[a, b] A[a, i, t, a']
//          E[a', b']     = sum_(b, t), b fastest, tmp[b, t, a'] B[b, t, j, b']
//   right: tmp[b2, t, a] = sum_a2 P[a2, b2] A[a, i, t, a2]     (P is ra2 x rb2)
//          E[a, b]       = sum_(b2, t), b2 fastest, tmp[b2, t, a] B[b, t, j, b2]
// (_extend_cache, contraction.jl:103-109, with the permuted cores of :165-169).
struct EnvLevel {
  const double* A;
  const double* B;
  int ra, s, S, ra2, rb, s2, rb2;
  int right;
  int n;  // entries
  const double* const* parent;
  double* const* out;
  double* const* tmp;
  const int32_t* ii;
  const int32_t* jj;
};

__global__ void env_tmp_kernel(EnvLevel v) {
  // left: per entry rb * S * ra2 values; right: rb2 * S * ra values
  const int64_t per = v.right ? (int64_t)v.rb2 * v.S * v.ra : (int64_t)v.rb * v.S * v.ra2;
  for (int64_t g = gtid(); g < per * v.n; g += gstride()) {
    const int e = (int)(g / per);
    const int64_t x = g % per;
    const double* P = v.parent[e];
    const int i = v.ii[e];
    double acc = 0.0;
    if (!v.right) {
      const int b = (int)(x % v.rb), t = (int)((x / v.rb) % v.S), a2 = (int)(x / ((int64_t)v.rb * v.S));
      const double* Ac = v.A + (int64_t)v.ra * (i + (int64_t)v.s * (t + (int64_t)v.S * a2));
      for (int a = 0; a < v.ra; ++a) acc = __dadd_rn(acc, __dmul_rn(P[a + (int64_t)v.ra * b], Ac[a]));
    } else {
      const int b2 = (int)(x % v.rb2), t = (int)((x / v.rb2) % v.S), a = (int)(x / ((int64_t)v.rb2 * v.S));
      for (int a2 = 0; a2 < v.ra2; ++a2)
        acc = __dadd_rn(acc, __dmul_rn(P[a2 + (int64_t)v.ra2 * b2],
                                       v.A[a + (int64_t)v.ra * (i + (int64_t)v.s * (t + (int64_t)v.S * a2))]));
    }
    v.tmp[e][x] = acc;
  }
}

__global__ void env_out_kernel(EnvLevel v) {
  const int64_t per = v.right ? (int64_t)v.ra * v.rb : (int64_t)v.ra2 * v.rb2;
  for (int64_t g = gtid(); g < per * v.n; g += gstride()) {
    const int e = (int)(g / per);
    const int64_t x = g % per;
    const double* T = v.tmp[e];
    const int j = v.jj[e];
    double acc = 0.0;
    if (!v.right) {
      const int a2 = (int)(x % v.ra2), b2 = (int)(x / v.ra2);
      for (int t = 0; t < v.S; ++t) {
        const double* Tc = T + (int64_t)v.rb * (t + (int64_t)v.S * a2);
        const double* Bc = v.B + (int64_t)v.rb * (t + (int64_t)v.S * (j + (int64_t)v.s2 * b2));
        for (int b = 0; b < v.rb; ++b) acc = __dadd_rn(acc, __dmul_rn(Tc[b], Bc[b]));
      }
    } else {
      const int a = (int)(x % v.ra), b = (int)(x / v.ra);
      for (int t = 0; t < v.S; ++t) {
        const double* Tc = T + (int64_t)v.rb2 * (t + (int64_t)v.S * a);
        for (int b2 = 0; b2 < v.rb2; ++b2)
          acc = __dadd_rn(acc, __dmul_rn(Tc[b2], v.B[b + (int64_t)v.rb * (t + (int64_t)v.S * (j + (int64_t)v.s2 * b2))]));
      }
    }
    v.out[e][x] = acc;
  }
}

// out[k] = sum_t L[k][t] R[k][t], t = 0 .. len[k]-1 in order (the (link_a,
// link_b) contraction of batchevaluate, contraction.jl:325-329, a fastest).
__global__ void env_dot_kernel(const double* const* L, const double* const* R, const int32_t* len, int n,
                               double* out) {
  for (int64_t k = gtid(); k < n; k += gstride()) {
    const double* l = L[k];
    const double* r = R[k];
    double acc = 0.0;
    for (int t = 0; t < len[k]; ++t) acc = __dadd_rn(acc, __dmul_rn(l[t], r[t]));
    out[k] = acc;
  }
}

int grid_for(int64_t total) {
  int64_t g = (total + CT - 1) / CT;
  if (g < 1) g = 1;
  if (g > 152 * 32) g = 152 * 32;
  return (int)g;
}

}  // namespace

cudaError_t tci_naive_site_launch(const double* a, const double* b, double* out, int ra, int s1, int s2, int ra2,
                                  int rb, int s3, int rb2, cudaStream_t st) {
  const int64_t total = (int64_t)ra * rb * s1 * s3 * ra2 * rb2;
  naive_site_kernel<<<grid_for(total), CT, 0, st>>>(a, b, out, ra, s1, s2, ra2, rb, s3, rb2);
  return cudaGetLastError();
}

cudaError_t tci_zip_ra_launch(const double* R, const double* A, double* RA, int nab, int nan_, int nbn, int s,
                              int sp, int nan2, cudaStream_t st) {
  const int64_t total = (int64_t)nab * nbn * s * sp * nan2;
  zip_ra_kernel<<<grid_for(total), CT, 0, st>>>(R, A, RA, nab, nan_, nbn, s, sp, nan2);
  return cudaGetLastError();
}

cudaError_t tci_zip_c_launch(const double* RA, const double* B, double* C, int nab, int nbn, int s, int sp, int nan2,
                             int spp, int nbn2, cudaStream_t st) {
  const int64_t total = (int64_t)nab * s * spp * nan2 * nbn2;
  zip_c_kernel<<<grid_for(total), CT, 0, st>>>(RA, B, C, nab, nbn, s, sp, nan2, spp, nbn2);
  return cudaGetLastError();
}

cudaError_t tci_lu_left_right_launch(const double* F, const int32_t* rowperm, const int32_t* colperm, int m, int n,
                                     int K, int leftorth, double* left, double* right, cudaStream_t st) {
  const int64_t total = (left ? (int64_t)m * K : 0) + (right ? (int64_t)K * n : 0);
  if (total == 0) return cudaSuccess;
  lu_left_right_kernel<<<grid_for(total), CT, 0, st>>>(F, rowperm, colperm, m, n, K, leftorth, left, right);
  return cudaGetLastError();
}

cudaError_t tci_luci_left_right_launch(const double* F, const int32_t* rowperm, const int32_t* colperm, int m,
                                       int n, int K, int leftorth, double* left, double* right, cudaStream_t st) {
  const int64_t total = (int64_t)m + n;
  if (K == 0 || total == 0) return cudaSuccess;
  luci_left_right_kernel<<<grid_for(total), CT, 0, st>>>(F, rowperm, colperm, m, n, K, leftorth, left, right);
  return cudaGetLastError();
}

cudaError_t tci_gemm_launch(const double* A, int64_t lda, const double* B, int64_t ldb, double* C, int64_t ldc,
                            int M, int N, int K, cudaStream_t st) {
  const int64_t total = (int64_t)M * N;
  if (total == 0) return cudaSuccess;
  gemm_kernel<<<grid_for(total), CT, 0, st>>>(A, lda, B, ldb, C, ldc, M, N, K);
  return cudaGetLastError();
}

cudaError_t tci_env_level_launch(const double* A, const double* B, int ra, int s, int S, int ra2, int rb, int s2,
                                 int rb2, int right, int n, const double* const* parent, double* const* out,
                                 double* const* tmp, const int32_t* ii, const int32_t* jj, cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  EnvLevel v{A, B, ra, s, S, ra2, rb, s2, rb2, right, n, parent, out, tmp, ii, jj};
  const int64_t t1 = (right ? (int64_t)rb2 * S * ra : (int64_t)rb * S * ra2) * n;
  const int64_t t2 = (right ? (int64_t)ra * rb : (int64_t)ra2 * rb2) * n;
  env_tmp_kernel<<<grid_for(t1), CT, 0, st>>>(v);
  env_out_kernel<<<grid_for(t2), CT, 0, st>>>(v);
  return cudaGetLastError();
}

cudaError_t tci_env_dot_launch(const double* const* L, const double* const* R, const int32_t* len, int n, double* out,
                               cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  env_dot_kernel<<<grid_for(n), CT, 0, st>>>(L, R, len, n, out);
  return cudaGetLastError();
}
