// Approximate minimum degree ordering (amd.cpp).
#pragma once

#include <cstdint>
#include <vector>

namespace sle_gb300 {

// Elimination record of one ordering: pivot k eliminates the supervariable at
// order positions [piv_end[k-1], piv_end[k]) (piv_end[-1] = 0), in that order,
// and lp[lp_ptr[k] .. lp_ptr[k+1]) lists the vertices of L's column structure
// below the supervariable (unsorted, each once).
struct AmdTrace {
    std::vector<int32_t> piv_end;
    std::vector<int64_t> lp_ptr;
    std::vector<int32_t> lp;
};

// Ordering of the symmetric graph (ptr, adj) (CSR, self loops ignored):
// order[k] = vertex eliminated k-th.  The trace, when given, is filled.
std::vector<int32_t> amd_order(int32_t n, const std::vector<int32_t>& ptr, const std::vector<int32_t>& adj,
                               AmdTrace* trace = nullptr);

}  // namespace sle_gb300
