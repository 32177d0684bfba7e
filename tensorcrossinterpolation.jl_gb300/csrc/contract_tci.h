// contract(A, B; algorithm = :TCI) on the device (contraction.jl:399-434).
#pragma once
#include <cstdint>
#include <vector>

#include "contract.h"

namespace tci {

// Interpolates the product of two trains of 4-leg cores with TCI2, the
// Contraction evaluator supplying f on the device; takes ownership of a and b.
// pivots: initial pivots over the fused local indices (0-based, A's index
// fastest); when empty, nmax starts of _findinitialpivots are used.  vf, if not
// null, maps every value of the product in place (contract's f).  The result
// keeps the two legs of each site split.
int tt4_contract_tci(Engine& e, TT4&& a, TT4&& b, const std::vector<std::vector<uint8_t>>& pivots, int nmax,
                     tci_value_fn vf, void* vuser, const tci_opts& o, TT4& out);

}  // namespace tci
