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
};

// Factorisation plan (device).
struct DevFactor {
    int32_t n_super, n_state;
    const int32_t* sn_c0;
    const int32_t* sn_f;
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
    // big-front workspace offsets (-1 for fronts handled in shared memory)
    const int64_t* sn_big_off;
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
    double* rhs;      // [n_state] permuted
    double* sol;      // [n_state] permuted (y after forward, x after backward)
    double* lx;       // L panels
    double* u;        // update matrices
    double* su;       // solve update vectors
    double* big;      // big-front workspace
    double* p_inj;    // [n_bus]
    double* q_inj;
    double* pf;       // [n_branch] flows (filled by the result pass)
    double* qf;
    double* pt;
    double* qt;
    double* part;     // block partials: [2 * max_blocks]
    DevStatus* status;
};

struct SolveParams {
    int32_t exact_jacobian;  // 1: analytic derivatives of h(x); 0: the reference's formulas
    int32_t robust;          // Huber weights
    double huber_gamma;
    double tol;
    double vmin, vmax;
};

// Upload-time kernels.
cudaError_t launch_admittance_and_ybus(const DevNet& net, cudaStream_t st);

// One evaluation pass: h(x), r, H values, weights, objective partials.
cudaError_t launch_evaluate(const DevNet& net, const DevWork& w, const SolveParams& sp, cudaStream_t st);
// RHS b = H^T (w r), permuted.
cudaError_t launch_rhs(const DevNet& net, const DevFactor& f, const DevWork& w, cudaStream_t st);
// State update + convergence / validity, then status finalisation.
cudaError_t launch_update(const DevNet& net, const DevFactor& f, const DevWork& w, const SolveParams& sp,
                          cudaStream_t st);
// Objective, largest residual and bad-data count after an evaluation pass.
cudaError_t launch_objective(const DevNet& net, const DevWork& w, double bad_threshold, cudaStream_t st);
// Flat start: V = setpoint for PV/slack, else 1; theta = 0.
cudaError_t launch_flat_start(const DevNet& net, const DevWork& w, cudaStream_t st);
// Injections and branch flows at the current state (result download).
cudaError_t launch_results(const DevNet& net, const DevWork& w, cudaStream_t st);

// Level-scheduled multifrontal factorisation and solves.  Host-side copies
// of the plan arrays size the launches; device copies are read by kernels.
struct LevelSchedule {
    int32_t n_levels = 0;
    const int32_t* h_small_ptr = nullptr;  // [n_levels+1] offsets into d_small
    const int32_t* d_small = nullptr;      // fronts with f <= kSmallFrontMax, per level
    const int32_t* h_big_ptr = nullptr;    // [n_levels+1] offsets into h_big
    const int32_t* h_big = nullptr;        // fronts with f > kSmallFrontMax, per level
    const int32_t* h_all_ptr = nullptr;    // [n_levels+1] offsets into d_all
    const int32_t* d_all = nullptr;        // every front, per level (solves)
    const int32_t* h_lvl_maxf = nullptr;   // [n_levels] largest front per level
    const int32_t* h_sn_f = nullptr;
    const int32_t* h_sn_c0 = nullptr;
    const int64_t* h_big_off = nullptr;    // workspace offsets (host copy)
    const int32_t* h_tgt_ptr = nullptr;
    const int32_t* h_child_ptr = nullptr;
    const int32_t* h_child = nullptr;
    int32_t max_small_f = 0;
};

cudaError_t launch_factor(const DevNet& net, const DevFactor& f, const DevWork& w, const LevelSchedule& ls,
                          cudaStream_t st);
cudaError_t launch_solve(const DevFactor& f, const DevWork& w, const LevelSchedule& ls, cudaStream_t st);

// Kernels launched by this library since load (all engines of the process).
extern std::atomic<int64_t> g_kernel_launches;

// Largest front (rows) handled by the single-CTA shared-memory kernel.
constexpr int32_t kSmallFrontMax = 160;

}  // namespace sle_gb300
