// Tensor trains with 4-leg cores (link, s_in, s_out, link') on the device and
// their contraction / recompression (contraction.jl, tensortrain.jl).
#pragma once
#include <cstdint>
#include <vector>

#include "engine.h"

namespace tci {

struct Tensor4 {
  double* p = nullptr;  // device, column-major d[0] x d[1] x d[2] x d[3]
  int64_t d[4] = {0, 0, 0, 0};
  size_t elems() const { return (size_t)(d[0] * d[1] * d[2] * d[3]); }
};

struct TT4 {
  std::vector<Tensor4> cores;
  void release(Engine& e);  // give every core back to the engine's pool
};

// Validation with the reference's messages: equal length (ArgumentError),
// consistent bonds, and for contract_naive the shared site index
// (contraction.jl:40-45).
int tt4_check_pair(const TT4& a, const TT4& b, bool sites_must_match);
int tt4_check(const TT4& t);

int tt4_contract_naive(Engine& e, const TT4& a, const TT4& b, TT4& out);

// Split-precision products (TF32 hi/lo on the tensor cores, tc_gemm.cu) for the
// site contractions, with the error of each product measured against FP64 at
// sampled entries; max_rel_err = max over products of max |C - exact| / max |exact|.
struct SplitRun {
  int samples = 64;
  double max_rel_err = 0.0;
  int64_t products = 0;
  double flops = 0.0;  // 2 M N K summed over the products
};

// ci selects _factorize(:CI) (MatrixLUCI's left/right) over _factorize(:LU);
// split != nullptr runs the two site contractions per site on the tensor cores.
int tt4_contract_zipup(Engine& e, const TT4& a, const TT4& b, double tolerance, int64_t maxbonddim, TT4& out,
                       bool ci = false, SplitRun* split = nullptr);

// C = A * B for column-major M x K and K x N device matrices (the matrix
// product of contraction.jl:92): the fixed-order FP64 kernel, or with split the
// tensor-core TF32 hi/lo product.
int device_matmul(Engine& e, const double* A, const double* B, double* C, int64_t M, int64_t N, int64_t K,
                  SplitRun* split);
int tt4_compress(Engine& e, TT4& tt, double tolerance, int64_t maxbonddim, bool normalizeerror, bool ci = false);
int device_rrlu_left_right(Engine& e, const double* A, int64_t m, int64_t n, int64_t maxrank, double reltol,
                           double abstol, bool leftorth, double** left, double** right, int64_t* npivot,
                           bool ci = false);

}  // namespace tci
