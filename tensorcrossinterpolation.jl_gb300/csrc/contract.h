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
// ci selects _factorize(:CI) (MatrixLUCI's left/right) over _factorize(:LU).
int tt4_contract_zipup(Engine& e, const TT4& a, const TT4& b, double tolerance, int64_t maxbonddim, TT4& out,
                       bool ci = false);
int tt4_compress(Engine& e, TT4& tt, double tolerance, int64_t maxbonddim, bool normalizeerror, bool ci = false);
int device_rrlu_left_right(Engine& e, const double* A, int64_t m, int64_t n, int64_t maxrank, double reltol,
                           double abstol, bool leftorth, double** left, double** right, int64_t* npivot,
                           bool ci = false);

}  // namespace tci
