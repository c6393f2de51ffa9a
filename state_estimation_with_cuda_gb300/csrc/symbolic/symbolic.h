// Symbolic analysis of one grid topology for the GPU WLS pipeline.
//
// Computed once per topology (bus/branch set, breaker statuses, measurement
// set) on the host, then uploaded; every Gauss-Newton iteration afterwards is
// numeric only.  Definitions (all deterministic functions of the input):
//
//  Ybus pattern      row i = [diagonal, then one entry per closed branch end at
//                    bus i, ordered by (column, branch index)].  Parallel
//                    branches stay separate entries.  This is the reference's
//                    pattern rule (sparse_matrix.cu:357-404: diagonal + one
//                    entry per closed branch end) with a canonical order in
//                    place of its atomic-arrival order (sparse_matrix.cu:476-481).
//  State vector      x = [theta_0..theta_{n-1} without slack, V_0..V_{n-1}]
//                    (sparse_matrix.cu:1677-1685, kernels.cu:732-745).
//  H pattern         row = measurement insertion index; columns = the exact
//                    set of states the row depends on, ascending, duplicates
//                    merged (the reference's intended pattern,
//                    sparse_matrix.cu:1458-1550, without the fixed 10-slot cap
//                    of sparse_matrix.cu:1574-1595).
//  Bus graph         buses i~j iff some active measurement row touches both.
//                    theta_i and V_i always have identical columns in
//                    G = H^T W H, so ordering and supernodes are found on this
//                    quotient graph and expanded to states (theta, then V).
//  Ordering          approximate minimum degree on the bus graph (default) or
//                    nested dissection with BFS level-set separators, then an
//                    elimination-tree postorder.  With minimum degree the
//                    elimination tree and the column structures come from the
//                    ordering's own elimination record (each pivot's element
//                    is its column structure); otherwise from Liu's algorithm
//                    and a merge up the tree.
//  Supernodes        fundamental supernodes of the bus-level etree, then
//                    relaxed amalgamation of each supernode into its parent
//                    when it immediately precedes it (bounded explicit zeros).
//  Fronts            multifrontal: front s has rows R_s = its columns followed by
//                    the sorted below-diagonal structure; its update matrix is
//                    extend-added into the parent through a relative-index map.
#pragma once

#include <cstdint>
#include <functional>
#include <memory>
#include <new>
#include <string>
#include <utility>
#include <vector>

namespace sle_gb300 {

// Allocator that leaves new elements of trivial types uninitialised.  The
// analysis writes every element of its largest arrays from several threads,
// so their pages are first touched by the writers instead of a serial fill.
template <typename T>
struct UninitAlloc : std::allocator<T> {
    template <typename U>
    struct rebind { using other = UninitAlloc<U>; };
    UninitAlloc() = default;
    template <typename U>
    UninitAlloc(const UninitAlloc<U>&) noexcept {}
    template <typename U>
    void construct(U* p) noexcept { ::new (static_cast<void*>(p)) U; }
    template <typename U, typename... A>
    void construct(U* p, A&&... a) { ::new (static_cast<void*>(p)) U(std::forward<A>(a)...); }
};
template <typename T>
using BigVec = std::vector<T, UninitAlloc<T>>;

struct Topology {
    int32_t n_bus = 0, n_branch = 0, n_meas = 0, slack = 0;
    const int32_t* br_from = nullptr;
    const int32_t* br_to = nullptr;
    const uint8_t* br_closed = nullptr;  // 1 closed, 0 open
    const int32_t* m_type = nullptr;
    const int32_t* m_loc = nullptr;
    const int32_t* m_end = nullptr;
    const uint8_t* m_active = nullptr;
};

struct SymbolicParams {
    int32_t ordering = 0;       // 0 approximate minimum degree, 1 natural order, 2 nested dissection
    int32_t leaf_size = 48;     // ND leaf size (buses)
    int32_t nrelax[3] = {2, 8, 24};        // relaxed amalgamation, in buses
    double zrelax[3] = {0.8, 0.1, 0.05};   // allowed explicit-zero fractions
};

// Measurement row kinds used by the evaluation kernel.
enum RowKind : int32_t { ROW_VMAG = 0, ROW_VANG = 1, ROW_INJ = 2, ROW_FLOW = 3, ROW_IMAG = 4, ROW_NONE = 5 };

struct Plan {
    int32_t n_bus = 0, n_state = 0, n_meas = 0, slack = 0;

    // Ybus pattern (CSR over buses). ysrc[e] = -1 for the diagonal, else
    // (branch << 1) | end, end 0 = this row is the branch's from bus.
    std::vector<int32_t> y_ptr, y_col, y_src;

    // H pattern (CSR over measurement rows), original state indices.
    std::vector<int32_t> h_ptr, h_col, h_row;
    // Per Ybus entry: position of theta_col / V_col inside the injection row
    // of the entry's row bus (relative to the row start), -1 when absent.
    std::vector<int32_t> y_hpos_t, y_hpos_v;
    // Per measurement row: kind and, for flow/current rows, packed positions
    // of (theta_from, V_from, theta_to, V_to), 8 bits each, 0xFF = absent.
    std::vector<int32_t> m_kind, m_fpos;

    // Ordering: bus position k -> bus; bus -> permuted state index of theta
    // (-1 for the slack) and of V.
    std::vector<int32_t> bus_perm, bus_ps_theta, bus_ps_v;
    // Permuted state index -> original state index.
    std::vector<int32_t> state_of_ps;

    // Supernodes / fronts (state level, permuted indices).
    int32_t n_super = 0;
    std::vector<int32_t> sn_c0;        // [n_super+1] first permuted column
    std::vector<int32_t> sn_f;         // front order
    std::vector<int32_t> sn_parent;    // -1 for roots
    std::vector<int64_t> sn_rows_off;  // [n_super+1] offsets into sn_rows
    std::vector<int32_t> sn_rows;      // row structures (permuted state indices)
    std::vector<int64_t> sn_lx_off;    // [n_super+1] L panel offsets (f x nc, column-major)
    std::vector<int64_t> sn_u_off;     // [n_super+1] update-matrix offsets ((f-nc)^2)
    std::vector<int64_t> sn_su_off;    // [n_super+1] solve-update offsets (f-nc)
    std::vector<int32_t> sn_child_ptr, sn_child;  // children lists
    std::vector<int32_t> sn_relmap;    // per supernode (f-nc) entries at sn_su_off: parent positions
    std::vector<int32_t> lvl_ptr, lvl_sn;  // bottom-up levels

    // Gain assembly: targets sorted by (front, local index); local index =
    // row + col * f within the front's L panel.  Pairs are H entry indices.
    std::vector<int32_t> sn_tgt_ptr;   // [n_super+1]
    BigVec<int32_t> tgt_local;         // [n_tgt]
    BigVec<int64_t> tgt_pair_ptr;      // [n_tgt+1]
    BigVec<int32_t> pair_a, pair_b;

    // RHS gather: per permuted state, the H entries in that column.
    std::vector<int32_t> rhs_ptr, rhs_h;
    // Permuted state index of each H entry (the entry's column).
    BigVec<int32_t> h_pcol;

    // Statistics.
    int64_t nnz_l = 0;        // stored entries of L (lower trapezoids of the panels)
    double flops = 0.0;       // multifrontal factorisation flops
    int32_t max_front = 0;
    int32_t n_levels = 0;
    int64_t lx_size = 0, u_size = 0, su_size = 0;
};

// Builds the plan; returns false and sets err on invalid input.  alongside,
// when given, runs once the fronts are complete (patterns, ordering, sn_*,
// children, relative maps, levels), on a thread of its own for all but small
// grids, and the analysis finishes after it; it may read those fields, not
// the RHS gather, h_pcol or the gain targets and pairs, which are built
// meanwhile.
bool build_plan(const Topology& t, const SymbolicParams& prm, Plan& plan, std::string& err,
                const std::function<void()>& alongside = nullptr);

// Block-diagonal union of independent grids' plans (a batch): every index
// array is shifted by the preceding grids' counts (buses, branches, rows,
// states, Ybus and H entries, supernodes, targets, pairs), so the batch is a
// plan of one grid whose elimination forest is the union of the grids'
// forests.  Level l of the batch is the union of the grids' levels l.
// Branch offsets come from br_count (branches per grid).
void merge_plans(const std::vector<const Plan*>& parts, const std::vector<int32_t>& br_count, Plan& out);

// Bus-level helpers exposed for tests / the oracle cross-check.
// Adjacency of the bus graph (CSR, sorted, no self loops).
void bus_graph(const Topology& t, const std::vector<int32_t>& y_ptr, const std::vector<int32_t>& y_col,
               std::vector<int32_t>& adj_ptr, std::vector<int32_t>& adj);

}  // namespace sle_gb300
