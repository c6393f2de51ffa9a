/*
 * segen — deterministic synthetic power-grid + telemetry generator.
 *
 * Produces the seeded synthetic grids the WLS state-estimation benchmarks and
 * parity tests run on (meshed grid = random spanning tree + locality-biased
 * chords, pi-model branches with a tapped subset, a smooth "true" state, and
 * |V| / P,Q-injection / both-end P,Q-flow telemetry with Gaussian noise and
 * optional gross errors; where the random draw leaves the grid unobservable,
 * from-end P+Q flow pseudo-measurements restore a measured spanning tree).  Everything is a pure function of (parameters, seed):
 *   - PRNG: xoshiro256** seeded through splitmix64;
 *   - uniforms: 53-bit mantissa draws in [0,1);
 *   - normals: Box-Muller in double (cosine branch only).
 *
 * The measurement model used to synthesise z is the SLE Engine's h(x)
 * (injections from Ybus, pi-model flows with the from-end charging term
 * B/(2a^2) scaled again by V_i^2/a^2), restated here only to make inputs.
 *
 * Arrays returned by the accessors stay owned by the generator handle.
 */
#ifndef SEGEN_H
#define SEGEN_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct SEGenParams {
    int32_t n_bus;          /* number of buses (>= 2) */
    int32_t n_branch;       /* number of branches (>= n_bus - 1) */
    uint64_t seed;          /* master seed */
    double frac_vmag;       /* fraction of buses with |V| telemetry (0.30) */
    double frac_inj;        /* fraction of buses with P+Q injection (0.60) */
    double frac_flow;       /* fraction of branches with both-end P+Q flow (0.70) */
    int32_t n_vmag;         /* exact counts; < 0 means "use the fraction" */
    int32_t n_inj;
    int32_t n_flow;
    int32_t n_tap;          /* tapped branches; < 0 means 15 % of branches */
    double sigma_v;         /* 0.004 */
    double sigma_inj;       /* 0.010 */
    double sigma_flow;      /* 0.008 */
    double gross_frac;      /* fraction of measurements with +-(10..30) sigma errors */
    double sigma_pseudo;    /* sigma of the pseudo flow pairs added to restore
                               topological observability, 0.05 */
} SEGenParams;

typedef struct SEGrid SEGrid;

/* Fill p with the documented defaults for a grid of n_bus buses / n_branch branches. */
void segen_default_params(SEGenParams* p, int32_t n_bus, int32_t n_branch, uint64_t seed);

/* Build a grid; returns NULL on invalid parameters. */
SEGrid* segen_create(const SEGenParams* p);
void segen_destroy(SEGrid* g);

int32_t segen_n_bus(const SEGrid* g);
int32_t segen_n_branch(const SEGrid* g);
int32_t segen_n_meas(const SEGrid* g);
int32_t segen_slack(const SEGrid* g);

/* Bus arrays [n_bus]: type (0 PQ, 1 PV, 2 SLACK), setpoint, true |V|, true theta. */
const int32_t* segen_bus_type(const SEGrid* g);
const double* segen_v_setpoint(const SEGrid* g);
const double* segen_v_true(const SEGrid* g);
const double* segen_theta_true(const SEGrid* g);

/* Branch arrays [n_branch]. status: 1 closed, 0 open. */
const int32_t* segen_br_from(const SEGrid* g);
const int32_t* segen_br_to(const SEGrid* g);
const double* segen_br_r(const SEGrid* g);
const double* segen_br_x(const SEGrid* g);
const double* segen_br_b(const SEGrid* g);
const double* segen_br_tap(const SEGrid* g);
const double* segen_br_shift(const SEGrid* g);
const int32_t* segen_br_status(const SEGrid* g);

/* Measurement arrays [n_meas]: SLE measurement type codes, location index
 * (bus for bus types, branch for flow types), branch end (0 from, 1 to),
 * sigma, and the current telemetry values z. */
const int32_t* segen_meas_type(const SEGrid* g);
const int32_t* segen_meas_loc(const SEGrid* g);
const int32_t* segen_meas_end(const SEGrid* g);
const double* segen_meas_sigma(const SEGrid* g);
const double* segen_meas_z(const SEGrid* g);
/* 1 where the initial draw carries a gross error. */
const int32_t* segen_meas_gross(const SEGrid* g);
/* Noise-free h(x_true). */
const double* segen_meas_htrue(const SEGrid* g);

/* Hot-start telemetry update number `update`: re-draw the noise of a seeded
 * subset (round(frac * n_meas) rows) as z_i = h_i(x_true) + sigma_i N(0,1).
 * Writes the full updated z into out[n_meas] (and into the handle). Returns
 * the number of rows redrawn. */
int32_t segen_renoise(SEGrid* g, int32_t update, double frac, double* out);

/* Toggle the status of branch k (breaker edit) in the generator's copy. */
void segen_set_status(SEGrid* g, int32_t k, int32_t status);

/* Index of a seeded switchable branch, chosen by `draw`: closed, not a
 * bridge (removing it keeps the grid connected), without flow or current
 * rows, between buses of at least three branches; -1 if none is found. */
int32_t segen_pick_nonbridge(const SEGrid* g, uint64_t draw);

/* Fleet helpers: grid size draws used by the batched (log-uniform) and
 * serving (truncated Zipf) workloads. */
int32_t segen_draw_loguniform(uint64_t seed, int32_t index, int32_t lo, int32_t hi);
int32_t segen_draw_zipf(uint64_t seed, int32_t index, double s, int32_t lo, int32_t hi);

#ifdef __cplusplus
}
#endif
#endif
