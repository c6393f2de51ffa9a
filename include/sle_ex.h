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
 *                           2 nested dissection (takes effect at upload)
 *   "use_double_precision"  as SLE_Config.use_double_precision (re-uploads)
 *   "refine_steps"          mixed precision: refinement steps per Gauss-Newton
 *                           step, each b - H^T W H dx in FP64 and an FP32 solve
 *                           (default 0: the Gauss-Newton loop itself re-forms
 *                           the FP64 residual and gradient every step)
 *   "big_front_flops"       FP64: fronts with more factor flops than this use
 *                           the tiled multi-CTA kernels (re-uploads) */
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
} SLE_ExStats;

SLE_API SLE_StatusCode SLE_CALL sle_ExGetStats(SLE_Handle handle, SLE_ExStats* stats);
SLE_API SLE_StatusCode SLE_CALL sle_ExResetStats(SLE_Handle handle);

#ifdef __cplusplus
}
#endif
#endif /* SLE_EX_H */
