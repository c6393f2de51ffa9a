/*
 * CPU FP64 oracle for the WLS Gauss-Newton state-estimation path.
 *
 * TEST INFRASTRUCTURE ONLY: the parity tests, the smoke check and the timed
 * CPU-baseline leg of the benchmark load this library to check or time the
 * GPU library; the product never links or calls it.
 *
 * It restates the SLE Engine's algorithm (reference alexdon256/
 * State_Estimation_with_CUDA) on the host, function by function:
 *   branch admittance      network_model.cu:595-612
 *   Ybus                   sparse_matrix.cu:410-492 (values), :357-404 (pattern)
 *   power injections       kernels.cu:129-230
 *   branch flows           kernels.cu:241-333, currents :335-375
 *   h(x) gather            kernels.cu:381-489
 *   residual / objective   kernels.cu:495-549
 *   Jacobian               sparse_matrix.cu:1627-2147 ("ref" mode keeps its
 *                          formulas; "exact" mode differentiates h(x))
 *   gain G = H^T W H       sparse_matrix.cu:979-1377
 *   Huber weights          kernels.cu:634-671
 *   state update / clamp   kernels.cu:721-750, max mismatch :752-782
 *   flat start             kernels.cu:799-817
 *   Gauss-Newton driver    wls_solver.cu:221-431 (retries, G reuse policy)
 *   bad-data flags         sle_engine.cu:959-977
 * The reference's own solve path (cuSOLVER csrlsvchol) is replaced by an
 * independent minimum-degree ordering and an up-looking simplicial Cholesky.
 *
 * Parity unpinned: the reference ships no tests, golden vectors or recorded
 * outputs, and its shipped solve path cannot run (Ybus is never assembled;
 * the FP64 build does not compile), so no output of the reference itself can
 * check this restatement.  The one fixture it ships, the IEEE 14-bus case
 * (data/ieee14bus.h), is loaded element for element by the tests; its
 * measurement set is unobservable (buses 10-14 carry only |V|), so every
 * correct WLS, this one included, reports a singular gain matrix on it.
 */
#ifndef SE_ORACLE_H
#define SE_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct OrParams {
    int32_t max_iterations;
    double tolerance;
    int32_t exact_jacobian;  /* 0: reference formulas, 1: analytic */
    int32_t gain_policy;     /* 0: refactor every iteration, 1: reuse until invalidated */
    int32_t robust;
    double huber_gamma;
    int32_t flat_start;
    int32_t realtime;        /* 1: no flat-start retries (REALTIME mode) */
    double vmin, vmax;
    double huber_stall;      /* robust: also converged when the Huber objective of an evaluation falls by no
                                more than this fraction of the previous one (0: off, the reference's test) */
} OrParams;

typedef struct OrResult {
    int32_t status;          /* 0 converged, 1 max iterations, 2 diverged, 3 singular */
    int32_t iterations;
    double max_mismatch;
    double objective;
    double largest_residual;
    int32_t largest_idx;
    int32_t pad;
} OrResult;

typedef struct OrGrid OrGrid;

OrGrid* or_create(int32_t n_bus, const int32_t* bus_type, const double* v_setpoint, int32_t n_branch,
                  const int32_t* from, const int32_t* to, const double* r, const double* x, const double* b,
                  const double* tap, const double* shift, const int32_t* status, int32_t n_meas,
                  const int32_t* mtype, const int32_t* mloc, const int32_t* mend, const double* sigma);
void or_destroy(OrGrid* g);

/* Ybus in canonical order; returns nnz.  Arrays may be NULL (size query). */
int32_t or_ybus(OrGrid* g, int32_t* row_ptr, int32_t* col, double* gv, double* bv);

/* H pattern size. */
int64_t or_nnz_h(OrGrid* g);

/* One evaluation at (v, th) with telemetry z: h(x), r, H (canonical CSR),
 * effective weights, b = H^T W r (state order) and J = sum w r^2. */
void or_evaluate(OrGrid* g, const double* v, const double* th, const double* z, int32_t exact, int32_t robust,
                 double gamma, double* hx, double* r, int32_t* h_ptr, int32_t* h_col, double* h_val, double* w_eff,
                 double* rhs, double* objective);

/* Lower triangle of G from the last evaluation as triplets (row >= col in
 * state indices, sorted by (col, row)); returns the count. */
int64_t or_gain(OrGrid* g, int32_t* rows, int32_t* cols, double* vals);

/* Factorise G from the last evaluation and solve G x = rhs; 0 or 3 (singular). */
int32_t or_solve_gain(OrGrid* g, const double* rhs, double* x);

/* Full Gauss-Newton WLS solve from the state in (v, th); writes the final
 * state back, plus residuals r[n_meas] if r != NULL. */
void or_wls(OrGrid* g, const double* z, double* v, double* th, const OrParams* p, OrResult* res, double* r);

/* Bad-data flags: active rows with sigma > 0 and |r|/sigma > threshold,
 * ascending; returns the count (writes at most max_count). */
int32_t or_bad_data(OrGrid* g, const double* r, double threshold, int32_t* idx, int32_t max_count);

/* Oracle minimum-degree bus ordering (position -> bus). */
void or_ordering(OrGrid* g, int32_t* bus_perm);

/* Bus-level elimination tree and column counts (incl. diagonal) of the bus
 * graph under the given ordering, by explicit symbolic elimination. */
void or_symbolic(OrGrid* g, const int32_t* bus_perm, int32_t* parent, int32_t* colcount);

/* Bus P/Q injections [n_bus] and branch flows P/Q at the from and to ends
 * [n_branch] at the state (v, th).  Any output may be NULL. */
void or_results(OrGrid* g, const double* v, const double* th, double* p_inj, double* q_inj, double* pf, double* qf,
                double* pt, double* qt);

/* Number of OpenMP threads the oracle uses. */
int32_t or_threads(void);

#ifdef __cplusplus
}
#endif
#endif
