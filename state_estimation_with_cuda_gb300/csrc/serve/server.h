// Serving runtime: a resident fleet of grids answering measurement snapshots
// (and breaker edits) as they arrive.
//
// Grids are partitioned by size into units.  Small grids share a unit: one
// batch Engine whose Gauss-Newton loop solves all grids with pending
// requests together.  A grid at or above `own_unit_bus` gets a unit of its
// own.  Every unit has its own CUDA stream and worker thread, so the units'
// work overlaps on the device.  A unit's worker runs its batch one
// Gauss-Newton iteration at a time; between iterations every grid with a
// pending request that is not already in the batch joins it (its oldest
// request), and after each iteration the grids that finished answer and
// leave (iteration-level continuous batching).  Each grid hot-starts from its
// last state and stops on its own convergence test, so its result does not
// depend on which other requests share the batch.
//
// Admission by device-memory budget: at start, units are made resident in
// order (small units first) while the sum of their device arenas stays
// within the budget.  A unit left out waits on the host; when a request for
// one of its grids arrives, its worker makes it resident, evicting idle
// resident units (least recently used first: their states are copied back
// to the host and their arenas freed) until it fits, or waiting until a
// unit goes idle.  An evicted unit resumes from its saved states, so every
// result is the one the grid gives when it stays resident.  Only a unit
// whose arena alone exceeds the budget is never admitted: its requests
// complete at once with `admitted = 0`.
#pragma once

#include <atomic>
#include <condition_variable>
#include <cstdint>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../engine/engine.h"

namespace sle_gb300 {

struct ServeConfig {
    int32_t use_double_precision = 0;
    int32_t max_iterations = 20;
    double tolerance = 1e-6;
    int32_t robust = 0;
    double huber_gamma = 1.5;
    // Upper bus-count bounds of the shared units (ascending; 0 = unused).  A
    // grid goes to the first unit whose bound is >= its size.
    int32_t bucket_bus[4] = {300, 2000, 20000, 0};
    int32_t own_unit_bus = 1 << 30;  // grids at least this large get a unit of their own
    size_t memory_budget = 0;      // bytes; 0 = 90 % of the free device memory at start
    int32_t device_id = 0;
};

struct ServeResult {
    int32_t status = CONV_RUNNING;
    int32_t iterations = 0;
    double max_mismatch = 0.0;
    double objective = 0.0;
    int32_t admitted = 1;
    int32_t batch_size = 0;  // grids in the batch at the iteration that finished this request
    int64_t t_submit_ns = 0, t_start_ns = 0, t_done_ns = 0;  // steady clock
};

struct ServeStats {
    int64_t submitted = 0, completed = 0, rejected = 0, passes = 0, grid_solves = 0;  // passes = iterations run
    int32_t units = 0, admitted_units = 0, grids = 0;
    size_t device_bytes = 0, budget_bytes = 0;  // device_bytes: arenas resident now
    int64_t admissions = 0, evictions = 0;      // residency changes after start
    int32_t resident_units = 0;
};

class Server {
public:
    explicit Server(const ServeConfig& c) : cfg_(c) {}
    ~Server();
    Server(const Server&) = delete;
    Server& operator=(const Server&) = delete;

    int32_t add_grid(int32_t n_bus, const int32_t* bus_type, const double* vset, int32_t n_br, const int32_t* from,
                     const int32_t* to, const double* r, const double* x, const double* b, const double* tap,
                     const double* shift, const int32_t* status, int32_t n_meas, const int32_t* mtype,
                     const int32_t* mloc, const int32_t* mend, const double* sigma, const double* z, int32_t* id);
    // Partition, admit, upload, solve every admitted grid once from a flat
    // start, and start the workers.
    int32_t start();
    // Queue a snapshot for `grid` (count = its measurement count); a breaker
    // edit (branch >= 0) is applied before the snapshot.  Returns a ticket.
    // v_out / th_out (either may be null) receive the grid's |V| and theta
    // when the request completes, before its ticket is ready; the caller
    // keeps them valid until then.
    int32_t submit(int32_t grid, const double* z, int32_t count, int32_t branch, int32_t closed, int64_t* ticket,
                   double* v_out = nullptr, double* th_out = nullptr);
    // Wait up to timeout_ms (< 0: forever) for a ticket; 1 = done, 0 = timed out.
    int32_t wait(int64_t ticket, double timeout_ms, ServeResult* out);
    int32_t get_state(int32_t grid, double* v, double* th);
    ServeStats stats();
    void stop();
    std::string last_error;

private:
    struct GridData {
        int32_t n_bus, n_br, n_meas;
        std::vector<int32_t> bus_type, from, to, status, mtype, mloc, mend;
        std::vector<double> vset, r, x, b, tap, shift, sigma, z;
    };
    struct Request {
        int64_t ticket;
        int32_t grid;
        std::vector<double> z;
        int32_t branch, closed;
        int64_t t_submit;
        double* v_out;
        double* th_out;
    };
    struct Unit {
        std::unique_ptr<Engine> eng;
        std::vector<int32_t> grids;                  // fleet grid ids, local order
        std::vector<std::deque<Request>> pending;    // per local grid
        int64_t n_pending = 0;
        bool admitted = false;  // its arena fits the budget (it can be made resident)
        std::thread worker;
        std::mutex mu;  // guards pending / n_pending
        std::condition_variable cv;
        std::mutex eng_mu;  // serialises engine use (worker, get_state, eviction); guards the fields below
        bool resident = false;    // arena allocated and the stream batch begun
        bool busy = false;        // the worker holds requests: not evictable
        bool solved_once = false; // the grids' first estimates (flat start) are done
        size_t need = 0;          // arena bytes when resident
        int64_t last_used_ns = 0;
    };
    ServeConfig cfg_;
    std::vector<GridData> fleet_;
    std::vector<int32_t> unit_of_, local_of_;
    std::vector<std::unique_ptr<Unit>> units_;
    bool started_ = false;
    std::atomic<bool> stopping_{false};
    std::mutex res_mu_;
    std::condition_variable res_cv_;
    std::unordered_map<int64_t, ServeResult> results_;
    int64_t next_ticket_ = 1;
    std::mutex st_mu_;
    ServeStats stats_;
    // residency: bytes of the resident arenas against the budget
    size_t budget_ = 0, used_ = 0;
    std::mutex mem_mu_;  // taken before any unit's eng_mu, never after
    std::condition_variable mem_cv_;
    SolveRequest request_params() const;
    int32_t first_estimates(Unit* u);  // caller holds u->eng_mu
    bool make_resident(Unit* u);       // worker thread, u->busy set
    bool evict_one(const Unit* except);  // caller holds mem_mu_
    void run_unit(Unit* u);
    void finish(int64_t ticket, const ServeResult& r);
};

}  // namespace sle_gb300
