// Split-precision (TF32 hi/lo) tensor-core GEMM on mapped FP64 operands.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

// Index map of one matrix index onto element offsets:
//   off(i) = (i % d0) * s0 + ((i / d0) % d1) * s1 + (i / (d0 * d1)) * s2.
// A plain stride s is {d0 = huge, d1 = 1, s0 = s, s1 = 0, s2 = 0}.
struct tci_map3 {
  int64_t d0, d1;
  int64_t s0, s1, s2;
};

inline tci_map3 tci_map_stride(int64_t s) { return tci_map3{INT64_MAX / 4, 1, s, 0, 0}; }
inline tci_map3 tci_map_2(int64_t d0, int64_t s0, int64_t s1) { return tci_map3{d0, 1, s0, 0, s1}; }
inline tci_map3 tci_map_3(int64_t d0, int64_t d1, int64_t s0, int64_t s1, int64_t s2) {
  return tci_map3{d0, d1, s0, s1, s2};
}

// Bytes of workspace tci_tc_gemm_split needs for an M x N x K product.
size_t tci_tc_gemm_workspace(int64_t M, int64_t N, int64_t K);

// C[c_row(m) + c_col(n)] = sum_k A[a_row(m) + a_k(k)] * B[b_row(n) + b_k(k)] for
// m < M, n < N, with TF32 hi/lo split products (hi*hi + hi*lo + lo*hi) on the
// tensor cores, FP32 accumulation, FP64 result.  a_kfast / b_kfast: the operand's
// unit stride runs along k (pack reads along k).  A wait that runs out writes a
// nonzero code to *err_dev.  Enqueued on `st`.
cudaError_t tci_tc_gemm_split(int64_t M, int64_t N, int64_t K, const double* A, tci_map3 a_row, tci_map3 a_k,
                              int a_kfast, const double* B, tci_map3 b_row, tci_map3 b_k, int b_kfast, double* C,
                              tci_map3 c_row, tci_map3 c_col, void* workspace, int* err_dev, cudaStream_t st);

// FP64 recomputation of `nsample` hashed entries of a product written by
// tci_tc_gemm_split: out2[0] = max |C - exact| and out2[1] = max |exact|, as
// double bit patterns merged by atomicMax (clear both words first).
cudaError_t tci_tc_gemm_sample_error(int64_t M, int64_t N, int64_t K, const double* A, tci_map3 a_row,
                                     tci_map3 a_k, const double* B, tci_map3 b_row, tci_map3 b_k, const double* C,
                                     tci_map3 c_row, tci_map3 c_col, int nsample, uint64_t seed,
                                     unsigned long long* out2, cudaStream_t st);

// Split-precision evaluation of a tensor train (abstracttensortrain.jl:124-132)
// at np points on the tensor cores.  dims[3b..3b+2] = (r0, d, r1) of core b;
// cores_dev[b] its FP64 values (column-major); pts_dev np x L 0-based local
// indices (uint8); out_dev np values.  The first nsample points are also
// evaluated in FP64 into sample_out_dev (for the error estimate).  Supported
// when tci_tc_eval_supported: bonds <= 128, outer bonds 1, and
// d * roundup(r_b, 16) <= 512 for every site after the first.
bool tci_tc_eval_supported(int L, const int64_t* dims);
size_t tci_tc_eval_workspace(int L, const int64_t* dims);
cudaError_t tci_tc_evaluate_split(int L, const int64_t* dims, const double* const* cores_dev, const uint8_t* pts_dev,
                                  int64_t np, double* out_dev, int nsample, double* sample_out_dev, void* workspace,
                                  int* err_dev, int nsm, cudaStream_t st);
