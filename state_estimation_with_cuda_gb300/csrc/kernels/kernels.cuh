// Device data views and kernel launchers of the GPU WLS pipeline.
#pragma once

#include <atomic>
#include <cstdint>
#include <cuda_runtime.h>

namespace sle_gb300 {

// Status bits written by kernels into DevStatus::flags.
enum StatusFlag : uint32_t {
    FLAG_SINGULAR = 1u,   // non-positive / non-finite pivot in the factorisation
    FLAG_NONFINITE = 2u,  // NaN/Inf in the state step
    FLAG_CONVERGED = 4u,  // max |dx| < tolerance
    FLAG_TIMEOUT = 8u,    // a dataflow wait gave up (bounded spin)
    FLAG_FROZEN = 16u,    // batch: this grid takes no further steps (inactive or finished)
    FLAG_INACTIVE = 32u,  // batch: this grid is not part of the current solve
    FLAG_FINAL = 64u,     // batch: the grid's final evaluation and objective are due
};

// Per-solve scalars kept on the device; read back once per iteration.
struct DevStatus {
    double max_mismatch;   // max |dx| of the last step
    double objective;      // sum w r^2 (base weights) at the last evaluation
    double huber_objective;
    double largest_residual;  // max |r| over active rows
    int32_t largest_idx;
    uint32_t flags;
    int32_t bad_count;     // rows with |r|/sigma > threshold (bad-data pass)
    int32_t pad;
};

// Static network data (device).
struct DevNet {
    int32_t n_bus, n_branch, n_meas, n_state, slack;
    // buses
    const int32_t* bus_type;
    const double* v_setpoint;
    // branches (inputs)
    const int32_t* br_from;
    const int32_t* br_to;
    const double* br_r;
    const double* br_x;
    const double* br_bch;   // total line charging
    const double* br_tap;
    const double* br_shift;
    const uint8_t* br_closed;
    // branch admittances (derived once per upload)
    double* br_g;
    double* br_b;
    double* br_bsf;
    double* br_bst;
    double* br_itap;  // 1 / max(tap, eps) and its square, for the flow rows (no FP64 division per row)
    double* br_itap2;
    // Ybus
    const int32_t* y_ptr;
    const int32_t* y_col;
    const int32_t* y_src;
    double* y_g;
    double* y_b;
    const int32_t* y_hpos_t;
    const int32_t* y_hpos_v;
    // measurements
    const int32_t* m_type;
    const int32_t* m_loc;
    const int32_t* m_end;
    const int32_t* m_kind;
    const int32_t* m_fpos;
    const uint8_t* m_active;
    const double* m_sigma;
    const double* m_w;       // base weights 1/max(sigma,eps)^2
    // H pattern
    const int32_t* h_ptr;
    const int32_t* h_row;
    const int32_t* h_pcol;   // column of each H entry in the permuted state order
    const int32_t* meas_grid;  // batch: grid of each measurement row (nullptr for one grid)
    const int32_t* bus_grid;   // batch: grid of each bus (nullptr for one grid)
    // Evaluation units: a row alone, or a P row with its Q twin (same bus,
    // or same branch end), (first row, twin or -1), in row order; per 32
    // units the row range [lo, hi) they cover when it is contiguous
    // (lo = -1 otherwise).
    const int2* ev_unit;
    const int2* ev_grp;
    int32_t n_units;
};

// Factorisation plan (device).
struct DevFactor {
    int32_t n_super, n_state;
    const int32_t* sn_c0;
    const int32_t* sn_f;
    const int32_t* sn_parent;
    const int64_t* sn_rows_off;
    const int32_t* sn_rows;
    const int64_t* sn_lx_off;
    const int64_t* sn_u_off;
    const int64_t* sn_su_off;
    const int32_t* sn_child_ptr;
    const int32_t* sn_child;
    const int32_t* sn_relmap;
    const int32_t* sn_tgt_ptr;
    const int32_t* tgt_local;
    const int64_t* tgt_pair_ptr;
    const int32_t* pair_a;
    const int32_t* pair_b;
    const int32_t* rhs_ptr;
    const int32_t* rhs_h;
    const int32_t* bus_ps_theta;
    const int32_t* bus_ps_v;
    // update-matrix leading dimension and location: small fronts keep a
    // compact (f-nc)^2 block in the update array; big fronts keep it in place
    // inside their f x f region of the factor array (sn_u_big = 1, ld = f)
    const int32_t* sn_u_ld;
    const uint8_t* sn_u_big;
    const int32_t* sn_grid;  // batch: grid of each front (nullptr for one grid)
    const int32_t* tgt_grid; // batch: grid of each gain target
    const int32_t* ps_grid;  // batch: grid of each permuted state
    // columns per panel of each front's factorisation (16 or 32); the
    // diagonal block of every panel is stored inverted (L11^-1) in L
    const int8_t* sn_pw;
};

// Mutable per-iteration state (device).
struct DevWork {
    double* v;        // [n_bus]
    double* th;       // [n_bus]
    double* z;        // [n_meas]
    double* h;        // [n_meas]
    double* r;        // [n_meas]
    double* w_eff;    // [n_meas] weights used for G and the RHS (Huber or base)
    double* wr;       // [n_meas] w_eff * r
    double* hval;     // [nnz_H]
    float* hval32;    // [nnz_H] FP32 copy (mixed-precision pipeline)
    double2* bus_cs;  // [n_bus] (cos theta, sin theta) of the state being evaluated
    double* hw;       // [nnz_H] FP64 pipeline: w_eff(row) * H entry, the gain sums' first factor
    float* hw32;      // [nnz_H] mixed pipeline: the same product rounded to FP32
    double* rhs;      // [n_state] permuted
    double* sol;      // [n_state] permuted (y after forward, x after backward)
    double* b0;       // [n_state] permuted gradient H^T W r of the iteration (mixed)
    double* dx;       // [n_state] permuted refined step (mixed)
    double* hdx;      // [n_meas] w * (H dx) (mixed refinement)
    double* lx;       // L panels (FP64 pipeline)
    double* u;        // update matrices (FP64 pipeline)
    float* lx32;      // L panels (mixed pipeline)
    float* u32;       // update matrices (mixed pipeline)
    double* su;       // solve update vectors
    void* gvals;      // [n_tgt] gain entries of the current factorisation (factor type)
    int* flow;        // dataflow flags and counters: [n_super + 8] factor, [2 n_super + 8] solves
    void* rdiag;      // [n_state] reciprocals of L's diagonal (factor type)
    float* rhs32;     // [n_state] FP32 right-hand side (mixed solves)
    float* sol32;     // [n_state] FP32 solution (mixed solves)
    float* su32;      // FP32 solve update vectors (mixed solves)
    double* p_inj;    // [n_bus]
    double* q_inj;
    double* pf;       // [n_branch] flows (filled by the result pass)
    double* qf;
    double* pt;
    double* qt;
    double* part;     // block partials: [2 * max_blocks]
    double* hpart;    // Huber-objective block partials of an evaluation
    double* opart;    // bad-data pass block partials: largest |r| per block
    int32_t* oidx;    //   its row
    int32_t* ocnt;    //   rows over the threshold per block
    DevStatus* status;
    uint32_t* grid_flags;  // batch: per-grid FLAG_* bits (nullptr for one grid)
    // Bounded dataflow waits: a wait gives up after spin_limit polls (about
    // 64 ns each), sets FLAG_TIMEOUT and lets the kernel finish, so the host
    // reports an error instead of the GPU hanging.
    long long spin_limit;
    // Test hook for that path: the backward sweeps never publish this front's
    // completion (-1: none), so its children's waits run out.
    int32_t hold_front;
};
constexpr long long kSpinLimitDefault = 1LL << 22;

// Batch of independent grids solved together (block-diagonal system).
struct DevBatch {
    int32_t n_grids;
    const int32_t* bus_off;   // [n_grids + 1]
    const int32_t* meas_off;  // [n_grids + 1]
    uint32_t* flags;          // [n_grids] FLAG_* (also DevWork::grid_flags)
    int32_t* iters;           // [n_grids] Gauss-Newton steps taken
    double* mismatch;         // [n_grids] max |dx| of the last step
    double* objective;        // [n_grids] sum w r^2 at the final state
    const uint8_t* active;    // [n_grids] 1 = solve this grid
    const uint8_t* flat;      // [n_grids] 1 = flat start first
    int32_t* running;         // [1] grids still iterating after this step
    // [4] Gauss-Newton loop run on the device by a graph's conditional while
    // node: [0] steps run, [1] step limit, [2] 1 = a dataflow wait timed out
    int32_t* loop;
    const uint8_t* retire;    // [n_grids] 1 = leave the running batch (stream mode)
    // Per-grid reductions spread over many CTAs: a grid's buses (rows) are cut
    // into items of kBatchChunk consecutive entries, items of a grid adjacent;
    // item k = (grid, first entry).  Each item writes a partial, and one thread
    // per grid combines its items' partials in item order (deterministic).
    const int2* bus_items;       // [n_bus_items]
    const int32_t* bus_item_ptr; // [n_grids + 1]
    int32_t n_bus_items;
    const int2* row_items;       // [n_row_items]
    const int32_t* row_item_ptr; // [n_grids + 1]
    int32_t n_row_items;
    double* part;                // [max(n_bus_items, n_row_items)] partial max |dx| or sum w r^2
    int32_t* part_bad;           // [n_bus_items] non-finite step seen
};
constexpr int kBatchChunk = 2048;

struct SolveParams {
    int32_t exact_jacobian;  // 1: analytic derivatives of h(x); 0: the reference's formulas
    int32_t mixed;           // 1: also store H in FP32 for the mixed-precision pipeline
    int32_t robust;          // Huber weights
    double huber_gamma;
    double tol;
    double vmin, vmax;
    uint32_t skip_flags;     // batch: grids whose flags intersect this mask are not evaluated
    uint32_t need_flags;     // batch: only grids whose flags hold every bit of this mask are evaluated
    int32_t huber_objective; // one grid: also sum the Huber objective of the evaluation into
                             // DevStatus::huber_objective (the robust solve's stall test)
    int32_t pad;
};

// Upload-time kernels.
cudaError_t launch_admittance_and_ybus(const DevNet& net, cudaStream_t st);

// One evaluation pass: h(x), r, H values, weights, objective partials.
cudaError_t launch_evaluate(const DevNet& net, const DevWork& w, const SolveParams& sp, cudaStream_t st);
// RHS b = H^T (w r), permuted.
cudaError_t launch_rhs(const DevNet& net, const DevFactor& f, const DevWork& w, cudaStream_t st);
// State update x += step (permuted step vector) + convergence / validity,
// then status finalisation.
cudaError_t launch_update(const DevNet& net, const DevFactor& f, const DevWork& w, const SolveParams& sp,
                          const double* step, cudaStream_t st);
// Mixed-precision refinement pieces (the solves run in FP32):
//   rhs32 = (float) rhs
cudaError_t launch_to_fp32(const DevFactor& f, const DevWork& w, cudaStream_t st);
//   b0 = rhs (kept), dx = sol32
cudaError_t launch_refine_begin(const DevFactor& f, const DevWork& w, cudaStream_t st);
//   rhs32 = b0 - H^T W H dx  (FP64 accumulation over the FP32 H)
cudaError_t launch_refine_residual(const DevNet& net, const DevFactor& f, const DevWork& w, cudaStream_t st);
//   dx += sol32
cudaError_t launch_refine_accumulate(const DevFactor& f, const DevWork& w, cudaStream_t st);
// Objective, largest residual and bad-data count after an evaluation pass.
cudaError_t launch_objective(const DevNet& net, const DevWork& w, double bad_threshold, cudaStream_t st);
// Flat start: V = setpoint for PV/slack, else 1; theta = 0.
cudaError_t launch_flat_start(const DevNet& net, const DevWork& w, cudaStream_t st);
// Injections and branch flows at the current state (result download).
cudaError_t launch_results(const DevNet& net, const DevWork& w, cudaStream_t st);

// A tiled front's assembly block (one CTA): tile column tj and row block rb
// (kAsmRows rows from the column's first row), the front's gain targets that
// land in the tile column, [tg_lo, tg_hi), and the children that add entries
// to the block, [ch_lo, ch_hi) of the AsmChild list, in child order.
struct AsmItem {
    int32_t s, tj, rb, tg_lo, tg_hi, ch_lo, ch_hi, pad;
};
// One child's part of an assembly block: its update-matrix columns [j0, j1)
// that land in the tile column and rows [ilo, ihi) that land in the row
// block (positions in the child's relative map).
struct AsmChild {
    int32_t c, j0, j1, ilo, ihi, pad0, pad1, pad2;
};

// One work item of the FP32 tiled fronts' dataflow factorisation (one
// persistent launch per synchronous level).  kind 0: the panel solve of
// chunk a (of b chunks) of step p, aux = the (front, step) pair of the
// step-0 tile-reader counter; kind 1: the trailing update of tile (a, b) at
// step p.  The item waits for the items dep[0, ndep) (level-local indices,
// all earlier in claim order) to publish their completion.  64 bytes: one
// load per item.
constexpr int kTileDeps = 8;
struct __align__(16) TileTask {
    int32_t kind, s, p, a, b, aux, ndep, pad;
    int32_t dep[kTileDeps];
};

// Level-scheduled multifrontal factorisation and solves.  Host-side copies
// of the schedule size the launches; device copies are read by kernels.
// Work-list entries are int4 (front, a, b, 0).
struct LevelSchedule {
    int32_t n_levels = 0;
    int32_t n_tgt = 0;                      // gain entries (targets)
    int32_t gain_acc32 = 0;                 // mixed pipeline: sum the gain entries in FP32 (else FP64)
    const int32_t* h_small_ptr = nullptr;   // [n_levels+1] offsets into d_small
    const int32_t* d_small = nullptr;       // single-CTA fronts, per level
    const int32_t* h_small_maxf = nullptr;  // [n_levels] largest single-CTA front
    const int32_t* h_asm_ptr = nullptr;     // [n_levels+1] offsets into d_asm
    const AsmItem* d_asm = nullptr;         // assembly blocks of the big fronts
    const AsmChild* d_asm_child = nullptr;  // their contributing children
    const int32_t* h_lvl_panels = nullptr;  // [n_levels] panel steps of the level
    const int32_t* h_step_ptr = nullptr;    // [n_levels+1] first step slot of a level
    const int32_t* h_pot_ptr = nullptr;     // [n_slots+1] offsets into d_pot
    const int4* d_pot = nullptr;            // FP64: (big front); FP32: (big front, chunk, chunks, step pair)
    int32_t* d_pot_cnt = nullptr;           // FP32: [n_pot_pairs] CTAs of a (front, step) done reading its tile
    int32_t n_pot_pairs = 0;
    const int32_t* h_pan_ptr = nullptr;     // [n_slots+1] offsets into d_pan (FP64 only)
    const int4* d_pan = nullptr;            // (big front, row tile below the panel)
    const int32_t* h_upd_ptr = nullptr;     // [n_slots+1] offsets into d_upd
    const int4* d_upd = nullptr;            // (big front, row tile, column tile)
    // FP32 tiled fronts as dataflow items, one persistent launch per level
    // (n_tt = 0: the per-step panel and update launches above)
    const int32_t* h_tt_ptr = nullptr;      // [n_levels+1] offsets into d_tt
    const TileTask* d_tt = nullptr;
    int32_t* d_tt_done = nullptr;           // [n_tt] completion flags, then [n_levels] claim counters
    int32_t n_tt = 0, tt_grid = 0;
    const int32_t* h_all_ptr = nullptr;     // [n_levels+1] offsets into d_all
    const int32_t* d_all = nullptr;         // every front, per level (solves)
    const int32_t* h_lvl_maxf = nullptr;    // [n_levels] largest front per level
    const int64_t* h_lvl_maxpanel = nullptr;  // [n_levels] largest f * nc per level
    // dataflow phases of the factorisation (fronts below every big front):
    // A = fronts whose whole subtree has f <= flow_small_f, B = the rest.  A
    // CTA claims an initially ready front of its phase (no children in the
    // phase) and, when it completes the last child of a parent in the same
    // phase, goes on with that parent; CTAs exit when nothing is left.
    const int32_t* d_flow_a = nullptr;  // initially ready fronts of phase A, claim order
    int32_t flow_a_n = 0, flow_a_maxf = 0, flow_a_grid = 0;
    const int32_t* d_flow_b = nullptr;  // initially ready fronts of phase B
    int32_t flow_b_n = 0, flow_b_maxf = 0, flow_b_grid = 0;
    const int8_t* d_phase = nullptr;         // [n_super] 1 = A, 2 = B, 0 = level-synchronous
    const int32_t* d_phase_nchild = nullptr; // [n_super] children in the same phase
    // dataflow solves over every front: forward by continuation from the
    // leaves (d_up, up_n), backward in top-down order (d_down) waiting on parents
    int32_t solve_flow = 0;
    const int32_t* d_up = nullptr;
    int32_t up_n = 0;
    const int32_t* d_nchild = nullptr;       // [n_super] children
    const int32_t* d_down = nullptr;
    int32_t solve_maxf = 0, solve_grid = 0, up_grid = 0;
    // warp phase: initially ready warp fronts (factor and forward sweep) and
    // every warp front top-down (backward sweep)
    const int32_t* d_flow_w = nullptr;
    int32_t flow_w_n = 0, flow_w_grid = 0;
    const int32_t* d_down_w = nullptr;
    int32_t down_w_n = 0, solve_w_grid = 0;
    // Lengths of the claim lists (A, B, up, down, warp, warp down) as the
    // kernels read them, on the device.  In a batch the lists above are
    // compacted copies: before every iteration launch_ready_compact keeps, in
    // order, the entries of src_lists whose grid takes the step, so that
    // fronts of frozen grids are never claimed and a pass costs what its
    // active grids cost.  Outside a batch the lists are the full ones and the
    // lengths fixed.
    int32_t* d_ready_n = nullptr;
    int32_t compact = 0;
    const int32_t* src_lists[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    int32_t* cmp_lists[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    int32_t src_n[6] = {0, 0, 0, 0, 0, 0};
    int32_t* d_chunk_cnt = nullptr;  // [ready_chunks(src_n)] scratch
};

// Claim lists and entries per CTA of their compaction.
constexpr int kReadyLists = 6;
constexpr int kCompactChunk = 2048;
inline int32_t ready_chunks(const int32_t* n) {
    int32_t c = 0;
    for (int l = 0; l < kReadyLists; ++l) c += (n[l] + kCompactChunk - 1) / kCompactChunk;
    return c;
}
// Batch: stable compaction of the claim lists to the fronts of grids that are
// not frozen (two launches).
cudaError_t launch_ready_compact(const DevFactor& f, const DevWork& w, const LevelSchedule& ls, cudaStream_t st);

// Batch control: begin (flags, flat starts), per-grid update + convergence,
// per-grid objective at the final state.
cudaError_t launch_batch_begin(const DevNet& net, const DevWork& w, const DevBatch& b, cudaStream_t st);
cudaError_t launch_batch_update(const DevNet& net, const DevFactor& f, const DevWork& w, const DevBatch& b,
                                const SolveParams& sp, const double* step, cudaStream_t st);
// Objective of every grid that is not inactive and whose flags hold `need`.
cudaError_t launch_batch_objective(const DevNet& net, const DevWork& w, const DevBatch& b, uint32_t need,
                                   cudaStream_t st);
// Stream mode: FLAG_FINAL on the grids with retire[g] = 1 (their final
// evaluation follows); launch_batch_retire then freezes them and clears it.
cudaError_t launch_batch_mark_final(const DevBatch& b, cudaStream_t st);
// Topological islands (connected components over closed branches) on the
// device: parent[n_bus] is scratch, out[0] = islands, out[1] = active rows.
// Hooking of component roots along every closed branch (the larger root
// points at the smaller) alternates with pointer jumping until no branch
// joins two components; bounded by `max_rounds` (out[2] = rounds used, -1
// when the bound was hit).
cudaError_t launch_islands(const DevNet& net, int32_t* parent, int32_t* out, int32_t max_rounds, cudaStream_t st);

// Stream mode (grids join and leave between iterations): activate the grids
// with active[g] = 1 (flags cleared, flat start if flat[g]), leaving the
// others as they are; retire the grids with retire[g] = 1 (frozen, inactive).
cudaError_t launch_batch_activate(const DevNet& net, const DevWork& w, const DevBatch& b, cudaStream_t st);
cudaError_t launch_batch_retire(const DevBatch& b, cudaStream_t st);
// Device Gauss-Newton loop of a batch solve: the host captures one step and
// launch_gn_loop_next into the body of a conditional while node; the node
// repeats the body while grids are running, no wait has timed out and fewer
// than `limit` steps have run (launch_gn_loop_init, before each launch).
cudaError_t launch_gn_loop_init(const DevBatch& b, int32_t limit, cudaStream_t st);
cudaError_t launch_gn_loop_next(cudaGraphConditionalHandle h, const DevBatch& b, const DevWork& w, cudaStream_t st);

// Largest front the high-occupancy dataflow phase may hold (its kernel keeps
// 16-column panels and a register budget for several CTAs per SM).
constexpr int32_t kFlowSmallFMax = 128;
// Panel width of the high-occupancy phase's fronts (all others use 32).
constexpr int32_t kPanelFlowA = 16;
// Fronts whose whole subtree is at most this wide are factorised and solved
// one front per warp (the warp phase, dataflow phase id 3).  By default a grid
// uses it as soon as it has kWarpPhaseMinFronts such fronts.  The phase adds
// a boundary to the factorisation and to each sweep, which a lone mid-size
// grid pays for (grid10k hot starts about 6 % slower), but a batch pays once
// for all its grids, and there the warp fronts' 8-fronts-a-CTA occupancy
// wins: on the 512-grid batch's loaded pass the factorisation falls from
// 3.78 to 1.62 ms and the solves from 1.97 to 0.69 ms.
constexpr int32_t kWarpFrontMax = 32;
constexpr int32_t kWarpPhaseMinFronts = 1;

// Resident-CTA grid sizes of the persistent dataflow kernels (0 = cannot run).
struct FlowGrids {
    int32_t a, b, solve, w, wsolve, tile;
};
FlowGrids flow_grids(bool mixed, int32_t maxf_a, int32_t maxf_b, int32_t solve_maxf);

// Allocation-free FP64 factor/solve (scratch in a static device array).
constexpr size_t kNoAllocScratchBytes = size_t(16) << 20;
struct NoAllocShape {
    int64_t u_elems;   // update-matrix entries of the small fronts (layout size)
    int64_t su_elems;  // solve update-vector entries
    int32_t n_state, n_super;
};
size_t noalloc_scratch_need(const NoAllocShape& sh);
// Looks the array up for the current device on first use.
cudaError_t noalloc_scratch_setup(void** out);
// rhs_host / x_host in state order; status flags land in W.status.
cudaError_t launch_factor_solve_noalloc(const DevNet& net, const DevFactor& F, const DevWork& W,
                                        const LevelSchedule& ls, const NoAllocShape& sh, const double* rhs_host,
                                        double* x_host, cudaStream_t st);

// Tile edge of the big-front kernels.
constexpr int kTile = 32;
// Rows per CTA of the FP32 panel solve of a tiled front.
constexpr int kPanelRows = 128;
// Rows per CTA of a tiled front's assembly (one CTA per tile column and row block).
constexpr int kAsmRows = 128;
// Edge of the trailing-update tiles of a tiled front (one CTA each; 64 left a
// single grid's step on too few SMs: grid200k FP64 179 -> 203 ms).
constexpr int kUpdTile = 32;

// Sets the kernel attributes (dynamic shared memory limits) on the current
// device; call before launching or capturing the factorisation.
cudaError_t prepare_factor_kernels();
cudaError_t launch_factor(const DevNet& net, const DevFactor& f, const DevWork& w, const LevelSchedule& ls,
                          cudaStream_t st);
cudaError_t launch_solve(const DevFactor& f, const DevWork& w, const LevelSchedule& ls, cudaStream_t st);
// FP32 gain / factor and mixed solves (FP32 L, FP64 vectors).
cudaError_t launch_factor32(const DevNet& net, const DevFactor& f, const DevWork& w, const LevelSchedule& ls,
                            cudaStream_t st);
cudaError_t launch_solve32(const DevFactor& f, const DevWork& w, const LevelSchedule& ls, cudaStream_t st);

// Kernels launched by this library since load (all engines of the process).
extern std::atomic<int64_t> g_kernel_launches;
// Launches issued by the calling thread (graph captures count their own
// launches without seeing other threads').
extern thread_local int64_t t_kernel_launches;
inline void count_launches(int64_t n) {
    g_kernel_launches += n;
    t_kernel_launches += n;
}

// Largest front (rows) handled by the single-CTA shared-memory kernel:
// 160 x 160 doubles or 224 x 224 floats (<= 200 KiB of shared memory).
constexpr int32_t kSmallFrontMax = 160;
constexpr int32_t kSmallFrontMax32 = 224;
template <typename T>
__host__ __device__ constexpr int32_t small_front_max() { return sizeof(T) == 4 ? kSmallFrontMax32 : kSmallFrontMax; }
// Leading dimension of a front held in shared memory: f rounded up to a
// multiple of 4 elements (16-byte aligned columns; 4-row tiles stay inside
// their column).
template <typename T>
__host__ __device__ constexpr int32_t front_ld(int32_t f) {
    return (f + 3) / 4 * 4;
}
template <typename T>
__host__ __device__ constexpr size_t front_smem(int32_t f) {
    return static_cast<size_t>(front_ld<T>(f)) * static_cast<size_t>(f) * sizeof(T);
}

}  // namespace sle_gb300
