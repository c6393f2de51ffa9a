/*
 * sle_ex.h — additive entry points of the GB300-native WLS state estimator.
 *
 * None of these exist in the reference SLE Engine; existing sle_* symbols
 * keep their meaning.  They cover bulk model ingest, options the reference
 * does not expose, and stage-level access used by the parity tests.
 */
#ifndef SLE_EX_H
#define SLE_EX_H

#include "sle_api.h"

#ifdef __cplusplus
extern "C" {
#endif

/* sizeof(SLE_Real) the library was built with (8: the FP64 ABI). */
SLE_API int32_t SLE_CALL sle_ExRealSize(void);

/* Replace the model with plain SoA arrays (no string IDs; synthetic IDs
 * "BUS<i>", "BR<k>", "M<q>" are generated if an ID-based call needs one).
 * Index rules are those of sle_AddBus / sle_AddBranch / sle_AddMeasurement:
 * element index = array position; the last SLACK bus is the slack.  Branch
 * status may be NULL (all closed).  z are the initial telemetry values.
 * Replaces the per-element string calls for large grids (reference
 * network_model.cu:71-151 builds the same arrays one element at a time). */
SLE_API SLE_StatusCode SLE_CALL sle_ExLoadNetwork(SLE_Handle handle, int32_t n_bus, const int32_t* bus_type,
                                                  const SLE_Real* v_setpoint, int32_t n_branch, const int32_t* from,
                                                  const int32_t* to, const SLE_Real* r, const SLE_Real* x,
                                                  const SLE_Real* b, const SLE_Real* tap, const SLE_Real* shift,
                                                  const int32_t* status, int32_t n_meas, const int32_t* mtype,
                                                  const int32_t* mloc, const int32_t* mend, const SLE_Real* sigma,
                                                  const SLE_Real* z);

/* Options:
 *   "exact_jacobian"        1 (default): analytic derivatives of h(x);
 *                           0: the reference's Jacobian formulas
 *                              (sparse_matrix.cu:1627-2147, defects included)
 *   "gain_policy"           0 (default): refactorise G every iteration;
 *                           1: keep the factor until the model changes
 *                              (the reference's fixed-gain policy,
 *                              wls_solver.cu:416-419)
 *   "ordering"              0 approximate minimum degree, 1 natural,
 *                           2 nested dissection (takes effect at upload);
 *                           1 and 2 are for tests and comparisons: on a
 *                           20,000-bus synthetic grid their factors hold
 *                           530x and 33x the entries of the default's
 *   "use_double_precision"  as SLE_Config.use_double_precision (re-uploads)
 *   "refine_steps"          mixed precision: refinement steps per Gauss-Newton
 *                           step, each b - H^T W H dx in FP64 and an FP32 solve
 *                           (default 0: the Gauss-Newton loop itself re-forms
 *                           the FP64 residual and gradient every step)
 *   "big_front_flops"       FP64: fronts with more factor flops than this use
 *                           the tiled multi-CTA kernels (re-uploads)
 *   "dataflow"              1 (default): persistent dataflow kernels for the
 *                           fronts below the tiled ones and for the solves
 *   "flow_small_f"          widest front of the high-occupancy dataflow phase
 *                           (0 = default: 128 mixed, 64 FP64; at most 128;
 *                           re-uploads)
 *   "warp_fronts"           fronts whose whole subtree is at most 32 wide are
 *                           factorised and solved one per warp: 1 on, 0 off,
 *                           -1 (default) for each grid that has such fronts
 *                           (re-uploads)
 *   "spin_limit"            polls (about 64 ns each) after which a dataflow
 *                           wait of the solves gives up; the call then fails
 *                           with SLE_ERROR_CUDA_FAILURE and the message
 *                           "factorisation dataflow wait timed out" instead
 *                           of the GPU hanging (default 4194304)
 *   "gain_accumulate"       mixed pipeline: bits of the accumulator of each
 *                           gain entry's sum of FP32 products, 32 (default)
 *                           or 64 (re-uploads)
 *   "huber_stall"           robust (Huber) solves on one grid: also stop, as
 *                           converged, when an iteration lowers the Huber
 *                           objective by no more than this fraction of its
 *                           previous value (default 0: only the reference's
 *                           max |dx| < tolerance test).  The reference's
 *                           reweighting creeps when gross errors sit on
 *                           critical measurement pairs, whose Huber objective
 *                           is nearly flat along the states they alone fix
 *   "eval_pair_rows"        evaluation: from this many measurement rows on
 *                           (default 262144), a P injection or flow row and
 *                           its Q twin (same bus, or same branch end) are
 *                           evaluated by one thread, sharing their angle and
 *                           admittance terms; below it every row has its own
 *                           thread (re-uploads)
 *   "tile_flow"             mixed pipeline: 1 factorises the tiled fronts
 *                           of each synchronous level in one persistent
 *                           dataflow launch (panel chunks and update tiles
 *                           as items that wait, bounded, for their inputs);
 *                           0 (default): a panel launch and an update launch
 *                           per 32-column step.  Same arithmetic, same bits
 *                           (re-uploads)
 *   "device_loop"           batch solves: 1 (default) runs the Gauss-Newton
 *                           loop on the device, as a CUDA graph whose
 *                           conditional while node repeats one step while
 *                           grids are still iterating (one host wait per
 *                           solve); 0: the host decides after every step.
 *                           Needs use_cuda_graphs and enable_profiling = 0
 *   "hold_front"            failure-path test hook: the backward sweep never
 *                           publishes this front's completion, so the waits
 *                           of its children run out (-1, the default: none) */
SLE_API SLE_StatusCode SLE_CALL sle_ExSetOption(SLE_Handle handle, const char* key, double value);

typedef struct SLE_ExPlanInfo {
    int32_t n_bus, n_state, n_meas, nnz_ybus;
    int64_t nnz_h;
    int32_t n_super, n_levels, max_front, pad;
    int64_t nnz_l, lx_size, u_size, n_gain_targets, n_gain_pairs;
    double factor_flops;
    size_t device_bytes;
} SLE_ExPlanInfo;

/* Symbolic plan statistics (uploads the model if needed). */
SLE_API SLE_StatusCode SLE_CALL sle_ExGetPlanInfo(SLE_Handle handle, SLE_ExPlanInfo* info);

typedef struct SLE_ExScheduleInfo {
    int32_t n_warp, n_phase_a, n_phase_b, n_sync; /* fronts per factorisation phase (warp, dataflow A and B,
                                                      level-synchronous) */
    int32_t warp_ready, a_ready, b_ready;         /* initially ready fronts of the dataflow phases */
    int32_t up_ready, down_n, down_warp_n;        /* forward-sweep leaves; backward-sweep fronts (CTA, warp) */
    int32_t sync_levels, panel_steps;             /* non-empty synchronous levels; tiled-front panel steps */
    int32_t by_depth;                             /* 1: synchronous levels ordered by depth from the root */
    int32_t tile_tasks;                           /* FP32 tiled-front dataflow items (0: per-step launches) */
    int64_t launches_by_height, launches_by_depth; /* cost of the synchronous part under either order */
} SLE_ExScheduleInfo;

/* Kernel schedule of the current model and options (no counterpart in the
 * reference).  Host-only before the first upload (it runs the symbolic
 * analysis if needed); afterwards it reports the uploaded schedule. */
SLE_API SLE_StatusCode SLE_CALL sle_ExGetScheduleInfo(SLE_Handle handle, SLE_ExScheduleInfo* info);

/* Ybus in canonical CSR order: row_ptr[n_bus+1], col/g/b[nnz_ybus]. */
SLE_API SLE_StatusCode SLE_CALL sle_ExGetYbus(SLE_Handle handle, int32_t* row_ptr, int32_t* col, SLE_Real* g,
                                              SLE_Real* b);

/* Evaluate h(x), residuals, the Jacobian and b = H^T W r at the given state. */
SLE_API SLE_StatusCode SLE_CALL sle_ExEvaluateAt(SLE_Handle handle, const SLE_Real* v, const SLE_Real* theta,
                                                 int32_t exact_jacobian);

/* Last evaluation: H pattern row_ptr[n_meas+1], col[nnz_h] (state index),
 * values[nnz_h], h(x)[n_meas] and b[n_state] (state order).  Any may be NULL. */
SLE_API SLE_StatusCode SLE_CALL sle_ExGetJacobian(SLE_Handle handle, int32_t* row_ptr, int32_t* col, SLE_Real* val,
                                                  SLE_Real* hx, SLE_Real* rhs);

/* Lower triangle of G = H^T W H from the last evaluation as (row, col, value)
 * triplets in state indices, n_gain_targets entries. */
SLE_API SLE_StatusCode SLE_CALL sle_ExGetGain(SLE_Handle handle, int32_t* rows, int32_t* cols, SLE_Real* vals);

/* Factorise G from the last evaluation and solve G x = rhs (state order). */
SLE_API SLE_StatusCode SLE_CALL sle_ExFactorSolve(SLE_Handle handle, const SLE_Real* rhs, SLE_Real* x);

/* Allocation-free variant of sle_ExFactorSolve (no counterpart in the
 * reference SLE Engine): same inputs and result, but the call allocates no
 * host or device memory.  Its scratch (right-hand side and solution staging,
 * dataflow flags, solve update vectors, update matrices of the small fronts)
 * lives in one static device array of 16 MiB in the library.
 *   - The first call on a device looks the array up with that device current
 *     (one-time set-up); make that first call before any stream capture.
 *   - Every call on a device shares the array: calls that overlap in time
 *     (two threads, two handles) race and must be serialised by the caller.
 *   - Like sle_ExFactorSolve, the call also overwrites the handle's own
 *     factor, right-hand side and solution buffers in its device arena, so
 *     it must not overlap a solve or another stage call on the same handle.
 *   - The handle's device (SLE_Config.device_id) is made current for the
 *     call and the caller's current device is restored afterwards.
 *   - A model whose scratch exceeds 16 MiB is rejected with
 *     SLE_ERROR_INVALID_ARGUMENT and a message giving the bytes it needs.
 * FP64 pipeline only (use_double_precision = 1), after sle_ExEvaluateAt. */
SLE_API SLE_StatusCode SLE_CALL sle_ExFactorSolveNoAlloc(SLE_Handle handle, const SLE_Real* rhs, SLE_Real* x);

/* Symbolic analysis: bus_perm[n_bus] (position -> bus), state_of_ps[n_state]
 * (permuted -> state index), sn_c0[n_super+1], sn_parent[n_super],
 * sn_rows_off[n_super+1], sn_rows[sn_rows_off[n_super]].  Any may be NULL. */
SLE_API SLE_StatusCode SLE_CALL sle_ExGetSymbolic(SLE_Handle handle, int32_t* bus_perm, int32_t* state_of_ps,
                                                  int32_t* sn_c0, int32_t* sn_parent, int64_t* sn_rows_off,
                                                  int32_t* sn_rows);

/* Measurement hooks (device-resident inputs, L2 hygiene, stream timing). */
/* Copy a telemetry snapshot into device slot `slot` (host -> device, once). */
SLE_API SLE_StatusCode SLE_CALL sle_ExStageTelemetry(SLE_Handle handle, const SLE_Real* values, int32_t count,
                                                     int32_t slot);
/* Make slot `slot` the current telemetry (device -> device on the engine's
 * stream; the next solve reads it). */
SLE_API SLE_StatusCode SLE_CALL sle_ExUseTelemetry(SLE_Handle handle, int32_t slot);
/* Overwrite a scratch buffer of `bytes` bytes on the engine's stream and wait,
 * evicting the engine's working set from L2. */
SLE_API SLE_StatusCode SLE_CALL sle_ExFlushL2(SLE_Handle handle, size_t bytes);
/* op 0: record a start event on the engine's stream; op 1: record a stop
 * event, wait for it and return the elapsed milliseconds. */
SLE_API SLE_StatusCode SLE_CALL sle_ExTimer(SLE_Handle handle, int32_t op, double* elapsed_ms);

typedef struct SLE_ExStats {
    /* stages: 0 evaluate, 1 factorisation, 2 right-hand side, 3 solves,
     * 4 state update, 5 final evaluation / other */
    int64_t launches[6];
    double ms[6];          /* CUDA-event time per stage (enable_profiling = 1) */
    int64_t calls[6];
    int64_t iterations, solves;
    int64_t total_launches; /* kernels this library launched since load */
    int64_t analyses;       /* symbolic analyses of this handle */
    int64_t uploads;        /* device arenas built for this handle */
    int64_t branch_edits;   /* breaker / branch-parameter edits applied on the device */
    int64_t step_waits;     /* Gauss-Newton steps after which the host waited for the device before
                               issuing the next (none in a batch solve whose loop runs on the device) */
    /* host wall time in ms, summed since load or reset: symbolic analyses, schedule builds, device
     * arena builds with their host-to-device copies, CUDA graph captures with instantiation.  A single
     * grid's schedule is built beside the last passes of its analysis: that time overlaps analysis_ms. */
    double analysis_ms, schedule_ms, upload_ms, capture_ms;
} SLE_ExStats;

SLE_API SLE_StatusCode SLE_CALL sle_ExGetStats(SLE_Handle handle, SLE_ExStats* stats);
SLE_API SLE_StatusCode SLE_CALL sle_ExResetStats(SLE_Handle handle);

/* ---- Batch of independent grids (no counterpart in the reference) --------
 * One handle holds many grids, solved together: the union of the grids'
 * symbolic plans is factorised by the same kernels in one pass, and every
 * grid stops on its own convergence test, so each grid's result and
 * iteration count are those of solving it alone.  The pattern keeps every
 * branch, so sle_ExBatchSetBranchStatus changes values only (no new
 * symbolic analysis).  Grids are added before the first solve; adding a grid
 * later re-analyses the batch.  Per-grid retries from a flat start (single
 * grid: wls_solver.cu:326-332) are not performed: a grid that diverges or
 * meets a non-positive pivot reports that status. */
typedef struct SLE_ExGridResult {
    int32_t status;     /* SLE_ConvergenceStatus */
    int32_t iterations; /* Gauss-Newton steps taken */
    double max_mismatch;
    double objective;   /* sum w r^2 at the returned state */
} SLE_ExGridResult;

/* Append a grid (arrays and index rules of sle_ExLoadNetwork, indices local
 * to the grid); *grid_id receives its index in the batch. */
SLE_API SLE_StatusCode SLE_CALL sle_ExBatchAddGrid(SLE_Handle handle, int32_t n_bus, const int32_t* bus_type,
                                                   const SLE_Real* v_setpoint, int32_t n_branch, const int32_t* from,
                                                   const int32_t* to, const SLE_Real* r, const SLE_Real* x,
                                                   const SLE_Real* b, const SLE_Real* tap, const SLE_Real* shift,
                                                   const int32_t* status, int32_t n_meas, const int32_t* mtype,
                                                   const int32_t* mloc, const int32_t* mend, const SLE_Real* sigma,
                                                   const SLE_Real* z, int32_t* grid_id);
SLE_API int32_t SLE_CALL sle_ExBatchGridCount(SLE_Handle handle);
/* New telemetry of one grid (count = its measurement count). */
SLE_API SLE_StatusCode SLE_CALL sle_ExBatchUpdateTelemetry(SLE_Handle handle, int32_t grid, const SLE_Real* values,
                                                           int32_t count);
/* Solve grids[0..n) together (the others keep their state); flat_start may
 * be NULL (hot start from each grid's last state).  results may be NULL. */
SLE_API SLE_StatusCode SLE_CALL sle_ExBatchSolve(SLE_Handle handle, int32_t n, const int32_t* grids,
                                                 const uint8_t* flat_start, int32_t max_iterations, double tolerance,
                                                 int32_t robust, double huber_gamma, SLE_ExGridResult* results);
/* |V| and theta of one grid (its n_bus values each; either may be NULL). */
SLE_API SLE_StatusCode SLE_CALL sle_ExBatchGetState(SLE_Handle handle, int32_t grid, SLE_Real* v, SLE_Real* theta);
/* Breaker edit: open (0) or close (1) branch `branch` of grid `grid`. */
SLE_API SLE_StatusCode SLE_CALL sle_ExBatchSetBranchStatus(SLE_Handle handle, int32_t grid, int32_t branch,
                                                           int32_t closed);

/* ---- Serving runtime (no counterpart in the reference) --------------------
 * A resident fleet of grids answering measurement snapshots and breaker
 * edits as they arrive.  Grids share batch units by size (the sle_ExBatch
 * machinery); grids of at least own_unit_bus buses get a unit of their own.
 * Each unit has its own stream and worker thread and runs its batch one
 * Gauss-Newton iteration at a time: between iterations, grids with a pending
 * request join the batch (hot-started from their last state), and after each
 * iteration the grids that finished answer and leave (iteration-level
 * continuous batching).
 * Residency follows a device-memory budget: at start, units are made
 * resident in order (small units first) while their arenas fit; a unit left
 * out is made resident when a request for one of its grids arrives, after
 * evicting idle units (least recently used first; their states are kept on
 * the host and restored when they come back), so every request completes
 * and its result is the one the grid gives while resident.  Only a unit
 * whose arena alone exceeds the budget is never admitted: its requests
 * complete at once with admitted = 0.  Thread-safe: submit / wait may be
 * called from any thread. */
typedef struct SLE_ExServer SLE_ExServer;

typedef struct SLE_ExServerConfig {
    int32_t use_double_precision; /* 0: mixed form (default), 1: FP64 */
    int32_t max_iterations;       /* per request (default 20) */
    double tolerance;             /* max |dx| (default 1e-6) */
    int32_t robust;               /* Huber weights */
    double huber_gamma;
    int32_t bucket_bus[4];        /* upper bus bounds of the shared units, ascending, 0 = unused */
    int32_t own_unit_bus;         /* grids at least this large get their own unit */
    int32_t device_id;
    size_t memory_budget;         /* bytes; 0 = 90 % of the free device memory at start */
} SLE_ExServerConfig;

typedef struct SLE_ExServeResult {
    int32_t status;      /* SLE_ConvergenceStatus */
    int32_t iterations;
    double max_mismatch;
    double objective;
    int32_t admitted;    /* 0: the grid's unit is outside the memory budget */
    int32_t batch_size;  /* grids in the batch at the iteration that finished it */
    int64_t t_submit_ns, t_start_ns, t_done_ns; /* steady clock */
} SLE_ExServeResult;

typedef struct SLE_ExServerStats {
    int64_t submitted, completed, rejected, passes, grid_solves;
    int32_t units, admitted_units, grids, pad;
    size_t device_bytes, budget_bytes;  /* device_bytes: arenas resident now */
    int64_t admissions, evictions;      /* residency changes after start */
    int32_t resident_units, pad2;
} SLE_ExServerStats;

/* Defaults of SLE_ExServerConfig. */
SLE_API void SLE_CALL sle_ExServerDefaultConfig(SLE_ExServerConfig* config);
SLE_API SLE_StatusCode SLE_CALL sle_ExServerCreate(SLE_ExServer** server, const SLE_ExServerConfig* config);
SLE_API void SLE_CALL sle_ExServerDestroy(SLE_ExServer* server);
/* Arrays and index rules of sle_ExLoadNetwork; *grid_id is the fleet index. */
SLE_API SLE_StatusCode SLE_CALL sle_ExServerAddGrid(SLE_ExServer* server, int32_t n_bus, const int32_t* bus_type,
                                                    const SLE_Real* v_setpoint, int32_t n_branch, const int32_t* from,
                                                    const int32_t* to, const SLE_Real* r, const SLE_Real* x,
                                                    const SLE_Real* b, const SLE_Real* tap, const SLE_Real* shift,
                                                    const int32_t* status, int32_t n_meas, const int32_t* mtype,
                                                    const int32_t* mloc, const int32_t* mend, const SLE_Real* sigma,
                                                    const SLE_Real* z, int32_t* grid_id);
/* Partition, admit, upload, estimate every resident grid once from a flat
 * start, start the workers. */
SLE_API SLE_StatusCode SLE_CALL sle_ExServerStart(SLE_ExServer* server);
/* Queue a snapshot (count = the grid's measurement count, copied before
 * return); branch >= 0 opens (closed = 0) or closes that branch first. */
SLE_API SLE_StatusCode SLE_CALL sle_ExServerSubmit(SLE_ExServer* server, int32_t grid, const SLE_Real* values,
                                                   int32_t count, int32_t branch, int32_t closed, int64_t* ticket);
/* As sle_ExServerSubmit; when the request completes, the grid's |V| and
 * theta (its n_bus values each) are written to v_out / theta_out (either may
 * be NULL) before the ticket is ready.  The buffers belong to the caller and
 * must stay valid until sle_ExServerWait has returned the ticket. */
SLE_API SLE_StatusCode SLE_CALL sle_ExServerSubmitEx(SLE_ExServer* server, int32_t grid, const SLE_Real* values,
                                                     int32_t count, int32_t branch, int32_t closed, SLE_Real* v_out,
                                                     SLE_Real* theta_out, int64_t* ticket);
/* Wait for a ticket: returns 1 when done (result filled), 0 on timeout
 * (timeout_ms < 0 waits forever), negative on error.  A ticket is read once. */
SLE_API int32_t SLE_CALL sle_ExServerWait(SLE_ExServer* server, int64_t ticket, double timeout_ms,
                                          SLE_ExServeResult* result);
SLE_API SLE_StatusCode SLE_CALL sle_ExServerGetState(SLE_ExServer* server, int32_t grid, SLE_Real* v,
                                                     SLE_Real* theta);
SLE_API SLE_StatusCode SLE_CALL sle_ExServerGetStats(SLE_ExServer* server, SLE_ExServerStats* stats);
/* Last error of this server (valid until its next call). */
SLE_API const char* SLE_CALL sle_ExServerLastError(SLE_ExServer* server);

#ifdef __cplusplus
}
#endif
#endif /* SLE_EX_H */
