// Engine: one network model resident on one GPU, solved by the level-scheduled
// multifrontal Gauss-Newton pipeline.  Mirrors the reference SLEEngine solve
// path (sle_engine.cu:450-682) and WLSSolver (wls_solver.cu:221-537).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>
#include <unordered_map>
#include <vector>

#include "../kernels/kernels.cuh"
#include "../model/model.h"
#include "../symbolic/symbolic.h"

namespace sle_gb300 {

// Reference EngineConfig defaults (sle_engine.h:84-122, sle_engine.config).
struct EngineConfig {
    int32_t device_id = 0;
    size_t max_buses = 200000, max_branches = 400000, max_measurements = 2000000, max_switching_devices = 100000;
    int32_t enable_robust = 0;
    double huber_gamma = 1.5;
    double convergence_tolerance = 1e-6;  // SLE_CONVERGENCE_TOL of the FP64 build (sle_types.cuh:63)
    int32_t max_realtime_iterations = 5;
    int32_t max_precision_iterations = 100;
    double realtime_time_limit_ms = 20.0;
    int32_t use_flat_start_default = 0;
    int32_t enable_profiling = 0;
    int32_t use_cuda_graphs = 1;
    int32_t block_size_standard = 256;
    int32_t block_size_reduction = 512;
    int32_t use_double_precision = 1;
    double voltage_min_pu = 0.5;
    double voltage_max_pu = 1.5;
    double bad_data_threshold = 3.0;
    int32_t auto_bad_data_rejection = 0;
    // Extensions (sle_ExSetOption).
    int32_t exact_jacobian = 1;  // 0: the reference's Jacobian formulas
    int32_t gain_policy = 0;     // 0: refactor every iteration; 1: reuse the factor until invalidated
    int32_t ordering = 0;        // symbolic ordering (see SymbolicParams)
    double big_front_flops = 2.0e5;  // FP64: fronts above this many factor flops use the tiled multi-CTA path
    int32_t refine_steps = 0;        // mixed precision: extra refinement steps per Gauss-Newton step
    int32_t dataflow = 1;            // persistent dataflow kernels below the big fronts and for the solves
    int32_t flow_small_f = 0;        // widest front of the high-occupancy dataflow phase (<= kFlowSmallFMax;
                                     // 0: 128 for the mixed pipeline, 64 for FP64)
    int32_t warp_fronts = -1;        // warp phase for fronts whose subtree is at most kWarpFrontMax wide:
                                     // 1 on, 0 off, -1 per grid with at least kWarpPhaseMinFronts of them
    int32_t stream_priority = 0;     // CUDA stream priority of the engine's stream (lower = more urgent)
    long long spin_limit = kSpinLimitDefault;  // polls before a dataflow wait gives up (FLAG_TIMEOUT)
    int32_t gain_acc32 = 1;          // mixed pipeline: gain entries summed in FP32 (1, default) or FP64 (0)
    double huber_stall = 0.0;        // robust solves: also stop when the Huber objective falls by no more
                                     // than this fraction in an iteration (0: the reference's test only)
    int32_t hold_front = -1;         // test hook: front whose backward-sweep completion is withheld
    int32_t eval_pair_rows = 1 << 18;  // evaluation: a P row and its Q twin share one thread from this many rows
    int32_t tile_flow = 0;           // FP32 tiled fronts: 1 = one dataflow launch per level; 0 = a panel and
                                     // an update launch per step (faster on the measured grids)
    int32_t device_loop = 1;         // batch solves: Gauss-Newton loop in a conditional graph node (needs
                                     // use_cuda_graphs and no profiling); 0: one host round trip per step
};

// Makes `dev` the calling thread's current device for the lifetime of the
// object and restores the caller's device afterwards.  Every engine call that
// touches device memory or the engine's stream opens one, so a handle created
// for device_id = k works while another device is current (the static
// scratch of the allocation-free entry point is looked up per current device).
struct DeviceScope {
    int prev = -1;
    explicit DeviceScope(int dev) {
        int cur = -1;
        if (cudaGetDevice(&cur) == cudaSuccess && cur != dev && cudaSetDevice(dev) == cudaSuccess) prev = cur;
    }
    ~DeviceScope() {
        if (prev >= 0) cudaSetDevice(prev);
    }
    DeviceScope(const DeviceScope&) = delete;
    DeviceScope& operator=(const DeviceScope&) = delete;
};

enum class Mode : int32_t { REALTIME = 0, PRECISION = 1 };

struct SolveRequest {
    Mode mode = Mode::REALTIME;
    int32_t max_iterations = 5;
    double tolerance = 1e-6;
    double huber_gamma = 1.5;
    int32_t robust = 0;
    int32_t flat_start = 0;
    double time_limit_ms = 0.0;
};

// ConvergenceStatus values (sle_types.cuh:142-149).
enum ConvStatus : int32_t { CONV_OK = 0, CONV_MAXIT = 1, CONV_DIVERGED = 2, CONV_SINGULAR = 3, CONV_NOTOBS = 4, CONV_RUNNING = 5 };

struct SolveResult {
    int32_t status = CONV_RUNNING;
    int32_t iterations = 0;
    double max_mismatch = 0.0;
    double objective = 0.0;
    double time_ms = 0.0;
    double largest_residual = 0.0;
    int32_t largest_idx = -1;
    int32_t bad_count = 0;
};

// Per-stage statistics (launch counts always; CUDA-event times when
// cfg.enable_profiling is set).
enum Stage : int32_t { ST_EVALUATE = 0, ST_FACTOR = 1, ST_RHS = 2, ST_SOLVE = 3, ST_UPDATE = 4, ST_OTHER = 5, ST_COUNT = 6 };
struct StageStats {
    int64_t launches[ST_COUNT] = {0, 0, 0, 0, 0, 0};
    double ms[ST_COUNT] = {0, 0, 0, 0, 0, 0};
    int64_t calls[ST_COUNT] = {0, 0, 0, 0, 0, 0};
    int64_t iterations = 0, solves = 0;
    int64_t analyses = 0, uploads = 0, branch_edits = 0;
    // Gauss-Newton steps after which the host waited for the device before
    // issuing the next (none inside a batch solve whose loop runs on the device)
    int64_t step_waits = 0;
    // host wall time: symbolic analyses, schedule builds, device arena builds
    // with their copies, CUDA graph captures with instantiation
    double analysis_ms = 0, schedule_ms = 0, upload_ms = 0, capture_ms = 0;
};

class Engine {
public:
    explicit Engine(const EngineConfig& c) : cfg(c) {}
    ~Engine();
    Engine(const Engine&) = delete;
    Engine& operator=(const Engine&) = delete;

    EngineConfig cfg;
    Model model;
    std::string config_path;
    std::string last_error;

    int32_t initialize();
    // Host-only symbolic analysis of the current model.  With `scheduled`
    // (one grid), the level schedule and evaluation units of the current
    // options are built alongside, and *scheduled says whether they were.
    int32_t analyze(bool* scheduled = nullptr);
    // Schedule summary (host-only before the first upload).
    struct ScheduleInfo {
        int32_t n_warp = 0, n_phase_a = 0, n_phase_b = 0, n_sync = 0;
        int32_t warp_ready = 0, a_ready = 0, b_ready = 0, up_ready = 0, down_n = 0, down_warp_n = 0;
        int32_t sync_levels = 0, panel_steps = 0, by_depth = 0, tile_tasks = 0;
        int64_t launches_by_height = 0, launches_by_depth = 0;
    };
    int32_t schedule_info(ScheduleInfo& out);
    int32_t upload();
    int32_t update_telemetry(const double* z, int32_t count);
    int32_t sync_measurements();
    int32_t solve(const SolveRequest& rq, SolveResult& out);
    int32_t flat_start();
    // Refresh the host model from the device; `what` is a mask of
    // DL_STATE (V, theta), DL_MEAS (h(x), residuals), DL_FLOWS (injections,
    // branch flows).  Only arrays changed since the last solve are copied.
    enum : int32_t { DL_STATE = 1, DL_MEAS = 2, DL_FLOWS = 4, DL_ALL = 7 };
    int32_t download_results(int32_t what = DL_ALL);

    // Stage-level access for parity tests.
    int32_t evaluate_at(const double* v, const double* th, int32_t exact);
    int32_t export_gain(std::vector<int32_t>& rows, std::vector<int32_t>& cols, std::vector<double>& vals);
    int32_t factor_and_solve(const double* rhs_orig, double* x_orig);
    // Same result as factor_and_solve, with every per-call scratch buffer in
    // a static device array (no host or device allocation); -11 when the
    // model needs more scratch than kNoAllocScratchBytes.
    int32_t factor_and_solve_noalloc(const double* rhs_orig, double* x_orig);
    int32_t export_ybus(std::vector<double>& g, std::vector<double>& b);
    // Topological islands of the uploaded network (closed branches) and the
    // active measurement rows, computed on the device.
    int32_t check_islands(int32_t* islands, int32_t* active_rows);
    int32_t export_eval(double* hval, double* hx, double* rhs_orig);

    // Measurement hooks.
    int32_t stage_telemetry(const double* z, int32_t count, int32_t slot);  // host -> device slot
    int32_t use_telemetry(int32_t slot);                                    // device slot -> z (on stream)
    int32_t flush_l2(size_t bytes);                                         // overwrite a scratch buffer
    // Copies cfg.spin_limit / cfg.hold_front into the device work view (the
    // next launches use them; captured iteration graphs are dropped).
    void apply_wait_options();
    // Device topology processor for one grid: breaker states and branch
    // parameters (r, x, charging, tap, phase shift) edited on the host model
    // reach the device as values -- the branch arrays are copied, admittances
    // and Ybus recomputed, the factor invalidated -- without a new symbolic
    // analysis, as long as every edited branch is in the uploaded pattern.
    int32_t apply_branch_edits();
    // True when branch k is in the pattern of the current plan (it is closed,
    // or a switching device can close it), so its edits are value edits.
    bool branch_in_pattern(int32_t k) const {
        return analyzed_ && k >= 0 && k < static_cast<int32_t>(br_in_pattern_.size()) && br_in_pattern_[k] != 0;
    }
    int32_t timer(int32_t op, double* ms);                                  // 0 start, 1 stop (+ elapsed)
    StageStats stats;

    bool initialized() const { return init_; }
    bool analyzed() const { return analyzed_; }
    bool uploaded() const { return uploaded_; }
    const Plan& plan() const { return plan_; }
    size_t device_bytes() const { return arena_bytes_; }
    double last_solve_ms() const { return last_.time_ms; }
    const SolveResult& last_result() const { return last_; }
    std::string device_info();

    // --- batch of independent grids (block-diagonal system) ---------------------
    // Grids are appended with batch_add_grid; the model is their union with
    // shifted indices, the symbolic plan the union of per-grid plans (built
    // with every branch in the pattern, so breaker edits only change values),
    // and batch_solve runs the Gauss-Newton loop for a subset of grids at once,
    // each grid stopping on its own convergence test.
    struct GridSpan {
        int32_t bus0, nbus, br0, nbr, m0, nm, slack;
    };
    struct GridResult {
        int32_t status, iterations;
        double max_mismatch, objective;
    };
    int32_t batch_add_grid(int32_t n_bus, const int32_t* bus_type, const double* vset, int32_t n_br,
                           const int32_t* from, const int32_t* to, const double* r, const double* x, const double* b,
                           const double* tap, const double* shift, const int32_t* status, int32_t n_meas,
                           const int32_t* mtype, const int32_t* mloc, const int32_t* mend, const double* sigma,
                           const double* z, int32_t* id);
    int32_t batch_solve(int32_t n, const int32_t* ids, const uint8_t* flat, const SolveRequest& rq, GridResult* out);
    int32_t batch_set_telemetry(int32_t grid, const double* z, int32_t count);
    int32_t batch_get_state(int32_t grid, double* v, double* th);
    int32_t batch_set_branch_status(int32_t grid, int32_t branch, int32_t closed);
    bool batch_mode() const { return !grids_.empty(); }
    // Stream mode of a batch (iteration-level continuous batching): after
    // stream_begin every grid is out of the batch; stream_activate adds grids
    // (their telemetry already set), stream_step runs one Gauss-Newton
    // iteration for the grids in the batch and returns those that finished
    // (converged, diverged, singular or at max_iterations), which leave it.
    int32_t stream_begin(const SolveRequest& rq);
    int32_t stream_activate(int32_t n, const int32_t* ids, const uint8_t* flat);
    int32_t stream_step(std::vector<int32_t>& done, std::vector<GridResult>& res);
    bool stream_in_flight(int32_t grid) const;
    // Admission: when non-zero, upload() refuses (-10, nothing allocated) a
    // model whose device arena would exceed this many bytes.
    size_t budget_bytes = 0;
    // Device arena size of the last upload attempt (set even when refused).
    size_t need_bytes = 0;
    // Frees the device arena after copying the state (V, theta) back to the
    // host model; the next upload() resumes from that state.
    int32_t evict();
    // Set by a caller that has just run analyze() on the unchanged model (e.g.
    // on a worker thread): the next upload() reuses that plan once.
    bool reuse_analysis_once = false;
    const std::vector<GridSpan>& grids() const { return grids_; }

    // Device copies of per-element results (downloaded lazily).
    std::vector<double> p_inj, q_inj, pf, qf, pt, qt;

private:
    bool init_ = false, analyzed_ = false, uploaded_ = false, factor_valid_ = false;
    std::vector<uint8_t> br_in_pattern_;  // per branch, of the current plan
    bool mixed_ = false;  // pipeline of the current upload: FP32 gain/factor + FP64 refinement
    int32_t stale_ = 0;  // DL_* mask of host copies older than the device
    cudaStream_t st_ = nullptr;
    cudaEvent_t ev0_ = nullptr, ev1_ = nullptr;
    void* arena_ = nullptr;
    size_t arena_bytes_ = 0;
    DevStatus* h_status_ = nullptr;
    double* h_stage_ = nullptr;  // pinned staging for telemetry
    size_t h_stage_n_ = 0;
    Plan plan_;
    DevNet net_{};
    DevFactor fac_{};
    DevWork work_{};
    LevelSchedule sched_{};
    // level schedule (host copies) and in-place storage layout
    std::vector<int32_t> sch_small_ptr_, sch_small_, sch_small_maxf_, sch_asm_ptr_, sch_panels_, sch_step_ptr_,
        sch_pot_ptr_, sch_pan_ptr_, sch_upd_ptr_, sch_all_ptr_, sch_all_, sch_maxf_;
    std::vector<int4> sch_pot_, sch_pan_, sch_upd_;
    std::vector<AsmItem> sch_asm_;
    std::vector<int2> ev_unit_, ev_grp_;  // evaluation units (DevNet::ev_unit / ev_grp)
    void build_eval_units();
    std::vector<AsmChild> sch_asm_child_;
    // FP32 tiled fronts as dataflow items (TileTask), per level
    std::vector<TileTask> sch_tt_;
    std::vector<int32_t> sch_tt_ptr_;
    std::vector<int64_t> sch_maxpanel_;
    std::vector<int32_t> sch_flow_a_, sch_flow_b_, sch_down_, sch_up_, sch_flow_w_, sch_down_w_, phase_nchild_, nchild_;
    std::vector<char> flow_phase_;
    int32_t sync_by_depth_ = 0;
    int64_t sync_cost_height_ = 0, sync_cost_depth_ = 0;
    int32_t flow_a_maxf_ = 0, flow_b_maxf_ = 0;
    int32_t* d_flow_a_ = nullptr;
    int32_t* d_flow_b_ = nullptr;
    int32_t* d_down_ = nullptr;
    int32_t* d_up_ = nullptr;
    int32_t* d_flow_w_ = nullptr;
    int32_t* d_down_w_ = nullptr;
    // the claim lists in LevelSchedule::src_lists order (A, B, up, down, warp, warp down)
    const std::vector<int32_t>& claim_list(int l) const {
        const std::vector<int32_t>* v[kReadyLists] = {&sch_flow_a_, &sch_flow_b_, &sch_up_, &sch_down_, &sch_flow_w_,
                                                      &sch_down_w_};
        return *v[l];
    }
    int32_t* claim_dev(int l) const {
        int32_t* v[kReadyLists] = {d_flow_a_, d_flow_b_, d_up_, d_down_, d_flow_w_, d_down_w_};
        return v[l];
    }
    int8_t* d_phase_ = nullptr;
    int32_t* d_phase_nchild_ = nullptr;
    int32_t* d_nchild_ = nullptr;
    int32_t* d_ready_n_ = nullptr;               // [4] claim-list lengths
    int32_t* d_pot_cnt_ = nullptr;               // FP32 tiled fronts: per (front, step) tile readers
    TileTask* d_tt_ = nullptr;
    int32_t* d_tt_done_ = nullptr;
    int32_t n_pot_pairs_ = 0;
    int32_t* d_cmp_[kReadyLists] = {};  // batch: compacted claim lists
    int32_t* d_chunk_cnt_ = nullptr;             // batch: compaction scratch
    std::vector<int2> bus_items_, row_items_;    // batch: per-grid reduction items
    std::vector<int32_t> bus_item_ptr_, row_item_ptr_;
    int32_t* isl_parent_ = nullptr;
    int32_t* isl_out_ = nullptr;
    int32_t max_solve_front() const;
    // batch state
    std::vector<GridSpan> grids_;
    std::vector<Plan> grid_plans_;
    DevBatch batch_{};
    uint8_t* h_batch_in_ = nullptr;   // pinned [2 * G]: active, flat
    void* h_batch_out_ = nullptr;     // pinned: flags, iters, mismatch, objective, running
    size_t h_batch_cap_ = 0;
    SolveRequest stream_rq_{};
    std::vector<uint8_t> in_flight_;
    std::vector<int32_t> stream_iters_;
    int32_t analyze_batch();
    std::vector<int64_t> lay_lx_off_, lay_u_off_;
    std::vector<int32_t> lay_u_ld_;
    std::vector<uint8_t> lay_u_big_;
    int64_t lay_lx_size_ = 0, lay_u_size_ = 0;
    int32_t* d_small_ = nullptr;
    int32_t* d_all_ = nullptr;
    AsmItem* d_asm_ = nullptr;
    AsmChild* d_asm_child_ = nullptr;
    int4* d_pot_ = nullptr;
    int4* d_pan_ = nullptr;
    int4* d_upd_ = nullptr;
    // targets_ready = false leaves the assembly items' target ranges to
    // fill_asm_targets(), for a schedule built before the gain targets exist.
    void build_schedule(bool targets_ready = true);
    void fill_asm_targets();
    void build_tile_tasks(const std::vector<int32_t>& bigs, const std::unordered_map<int64_t, int32_t>& pair_of);
    bool tile_tasks_bad_ = false;  // a dependency not earlier in claim order (never by construction)
    // CUDA graphs of one Gauss-Newton iteration, [0] without and [1] with
    // the refactorisation; re-captured when the solve parameters change.
    struct IterGraph {
        cudaGraphExec_t exec = nullptr;
        SolveParams sp{};
        int64_t launches[ST_COUNT] = {0, 0, 0, 0, 0, 0};
        int64_t total = 0;
    };
    IterGraph graphs_[2];
    // Batch solve's whole Gauss-Newton loop: a conditional while node whose
    // body is one step (with refactorisation) and the loop-control kernel.
    IterGraph loop_graph_;
    void drop_graphs();
    // host_copies: end the step with the status and running-count copies the
    // host loop reads (left out of the device loop's body).
    int32_t enqueue_iteration(const SolveParams& sp, bool refactor, int64_t* per_stage, bool host_copies = true);
    // Runs up to max_iter steps of a batch solve on the device; `steps` gets
    // the number run.  -1: the graph path is off (use the host loop).
    int32_t run_device_loop(const SolveParams& sp, int32_t max_iter, int32_t& steps);
    SolveResult last_{};
    double* d_slots_ = nullptr;
    int32_t n_slots_ = 0;
    void* d_scratch_ = nullptr;
    size_t scratch_bytes_ = 0;
    cudaEvent_t tm0_ = nullptr, tm1_ = nullptr;
    std::vector<cudaEvent_t> ev_pool_;
    std::vector<std::pair<int32_t, int32_t>> ev_marks_;  // (stage, pool index of the start event)
    size_t ev_used_ = 0;
    int32_t stage_begin(int32_t stage);
    void stage_end(int32_t stage, int32_t mark, int64_t launches_before);
    void collect_stage_times();

    void release_device();
    int32_t set_cuda_error(cudaError_t e, const char* where);
    SolveParams params(const SolveRequest& rq) const;
    int32_t run_iteration(const SolveParams& sp, bool refactor);
};

}  // namespace sle_gb300
