#include "server.h"

#include <algorithm>
#include <chrono>
#include <numeric>

namespace sle_gb300 {

namespace {
int64_t now_ns() {
    return std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now().time_since_epoch())
        .count();
}
}  // namespace

Server::~Server() { stop(); }

int32_t Server::add_grid(int32_t nb, const int32_t* btype, const double* vset, int32_t nbr, const int32_t* from,
                         const int32_t* to, const double* r, const double* x, const double* b, const double* tap,
                         const double* shift, const int32_t* status, int32_t nm, const int32_t* mtype,
                         const int32_t* mloc, const int32_t* mend, const double* sigma, const double* z,
                         int32_t* id) {
    if (started_) {
        last_error = "grids are added before start";
        return -4;
    }
    if (nb <= 0 || nbr < 0 || nm < 0 || !btype || !vset || (nbr > 0 && (!from || !to || !r || !x || !b || !tap || !shift)) ||
        (nm > 0 && (!mtype || !mloc || !mend || !sigma || !z))) {
        last_error = "invalid grid arrays";
        return -4;
    }
    GridData g;
    g.n_bus = nb;
    g.n_br = nbr;
    g.n_meas = nm;
    g.bus_type.assign(btype, btype + nb);
    g.vset.assign(vset, vset + nb);
    g.from.assign(from, from + nbr);
    g.to.assign(to, to + nbr);
    g.r.assign(r, r + nbr);
    g.x.assign(x, x + nbr);
    g.b.assign(b, b + nbr);
    g.tap.assign(tap, tap + nbr);
    g.shift.assign(shift, shift + nbr);
    g.status.assign(nbr, 1);
    if (status) g.status.assign(status, status + nbr);
    g.mtype.assign(mtype, mtype + nm);
    g.mloc.assign(mloc, mloc + nm);
    g.mend.assign(mend, mend + nm);
    g.sigma.assign(sigma, sigma + nm);
    g.z.assign(z, z + nm);
    fleet_.push_back(std::move(g));
    if (id) *id = static_cast<int32_t>(fleet_.size()) - 1;
    return 0;
}

int32_t Server::start() {
    if (started_) return 0;
    const int32_t G = static_cast<int32_t>(fleet_.size());
    if (G == 0) {
        last_error = "no grids";
        return -4;
    }
    // partition: shared units by size bound, then one unit per large grid
    std::vector<int32_t> bounds;
    for (int32_t v : cfg_.bucket_bus)
        if (v > 0) bounds.push_back(v);
    std::sort(bounds.begin(), bounds.end());
    const int32_t nshared = static_cast<int32_t>(bounds.size()) + 1;  // the last shared unit takes the rest below own_unit_bus
    std::vector<std::vector<int32_t>> shared(nshared);
    std::vector<int32_t> own;
    for (int32_t g = 0; g < G; ++g) {
        const int32_t n = fleet_[g].n_bus;
        if (n >= cfg_.own_unit_bus) {
            own.push_back(g);
            continue;
        }
        int32_t k = 0;
        while (k < static_cast<int32_t>(bounds.size()) && n > bounds[k]) ++k;
        shared[k].push_back(g);
    }
    std::sort(own.begin(), own.end(), [&](int32_t a, int32_t b) { return fleet_[a].n_bus < fleet_[b].n_bus; });
    std::vector<std::vector<int32_t>> parts;
    for (auto& v : shared)
        if (!v.empty()) parts.push_back(v);
    for (int32_t g : own) parts.push_back({g});
    unit_of_.assign(G, -1);
    local_of_.assign(G, -1);
    // memory budget
    size_t budget = cfg_.memory_budget;
    if (budget == 0) {
        size_t fr = 0, tot = 0;
        cudaSetDevice(cfg_.device_id);
        if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) {
            last_error = "cudaMemGetInfo failed";
            return -3;
        }
        budget = static_cast<size_t>(0.9 * static_cast<double>(fr));
    }
    // stream priorities: units of smaller grids are more urgent (their
    // requests are short and plentiful), so their kernels are scheduled first
    int least = 0, greatest = 0;
    cudaSetDevice(cfg_.device_id);
    cudaDeviceGetStreamPriorityRange(&least, &greatest);
    const int32_t nparts = static_cast<int32_t>(parts.size());
    // build every unit's batch model, then analyse them in parallel (host only)
    for (auto& members : parts) {
        auto u = std::make_unique<Unit>();
        EngineConfig ec;
        ec.device_id = cfg_.device_id;
        ec.use_double_precision = cfg_.use_double_precision;
        {
            // parts are ordered small to large: spread them over the priority range
            const int32_t pi = static_cast<int32_t>(units_.size());
            const int span = least - greatest;  // >= 0; greatest is the most urgent
            ec.stream_priority = nparts > 1 ? greatest + static_cast<int>((static_cast<int64_t>(span) * pi) / (nparts - 1))
                                            : least;
        }
        u->eng = std::make_unique<Engine>(ec);
        u->grids = members;
        u->pending.resize(members.size());
        const int32_t ui = static_cast<int32_t>(units_.size());
        for (size_t li = 0; li < members.size(); ++li) {
            const GridData& d = fleet_[members[li]];
            int32_t lid = -1;
            const int32_t rc = u->eng->batch_add_grid(d.n_bus, d.bus_type.data(), d.vset.data(), d.n_br, d.from.data(),
                                                      d.to.data(), d.r.data(), d.x.data(), d.b.data(), d.tap.data(),
                                                      d.shift.data(), d.status.data(), d.n_meas, d.mtype.data(),
                                                      d.mloc.data(), d.mend.data(), d.sigma.data(), d.z.data(), &lid);
            if (rc) {
                last_error = u->eng->last_error;
                return rc;
            }
            unit_of_[members[li]] = ui;
            local_of_[members[li]] = lid;
        }
        units_.push_back(std::move(u));
    }
    const int32_t U = static_cast<int32_t>(units_.size());
    auto parallel = [&](auto&& fn) {
        std::atomic<int32_t> next{0};
        auto work = [&]() {
            for (int32_t i = next++; i < U; i = next++) fn(i);
        };
        const int32_t nt = std::max(1, std::min<int32_t>(U, static_cast<int32_t>(std::thread::hardware_concurrency())));
        std::vector<std::thread> pool;
        for (int32_t t = 1; t < nt; ++t) pool.emplace_back(work);
        work();
        for (auto& th : pool) th.join();
    };
    std::vector<int32_t> arc(U, 0);
    parallel([&](int32_t i) {
        arc[i] = units_[i]->eng->analyze();
        units_[i]->eng->reuse_analysis_once = (arc[i] == 0);
    });
    for (int32_t i = 0; i < U; ++i)
        if (arc[i]) {
            last_error = units_[i]->eng->last_error;
            return arc[i];
        }
    // admission in order (shared units first, then own units by size): the
    // units that fit are made resident now, the others when they are needed
    size_t used = 0;
    for (auto& u : units_) {
        u->eng->budget_bytes = budget > used ? budget - used : 1;
        const int32_t rc = u->eng->upload();
        u->need = u->eng->need_bytes;
        u->eng->budget_bytes = 0;
        if (rc == 0) {
            u->resident = true;
            used += u->eng->device_bytes();
        } else if (rc != -10) {
            last_error = u->eng->last_error;
            return rc;
        }
        u->admitted = u->need <= budget;
    }
    budget_ = budget;
    used_ = used;
    // first estimate of every resident grid from a flat start, units in parallel
    std::vector<int32_t> src(U, 0);
    parallel([&](int32_t i) {
        Unit* u = units_[i].get();
        if (!u->resident) return;
        std::lock_guard<std::mutex> lk(u->eng_mu);
        src[i] = first_estimates(u);
    });
    for (int32_t i = 0; i < U; ++i)
        if (src[i]) {
            last_error = units_[i]->eng->last_error;
            return src[i];
        }
    {
        std::lock_guard<std::mutex> lk(st_mu_);
        stats_.units = static_cast<int32_t>(units_.size());
        stats_.grids = G;
        stats_.budget_bytes = budget;
        stats_.device_bytes = used;
        for (auto& u : units_) {
            stats_.admitted_units += u->admitted ? 1 : 0;
            stats_.resident_units += u->resident ? 1 : 0;
        }
    }
    started_ = true;
    for (auto& u : units_)
        if (u->admitted) u->worker = std::thread(&Server::run_unit, this, u.get());
    return 0;
}

SolveRequest Server::request_params() const {
    SolveRequest rq;
    rq.mode = Mode::PRECISION;
    rq.max_iterations = cfg_.max_iterations;
    rq.tolerance = cfg_.tolerance;
    rq.robust = cfg_.robust;
    rq.huber_gamma = cfg_.huber_gamma;
    return rq;
}

// The grids' first estimates (flat start, the telemetry given at add_grid),
// then the stream batch is begun.
int32_t Server::first_estimates(Unit* u) {
    const SolveRequest rq = request_params();
    const int32_t n = static_cast<int32_t>(u->grids.size());
    std::vector<int32_t> ids(n);
    std::iota(ids.begin(), ids.end(), 0);
    std::vector<uint8_t> flat(n, 1);
    std::vector<Engine::GridResult> res(n);
    int32_t rc = u->eng->batch_solve(n, ids.data(), flat.data(), rq, res.data());
    if (rc == 0) u->solved_once = true;
    return rc;
}

// Picks the least recently used resident unit whose worker holds no requests
// (other than `except`), copies its states to the host and frees its arena.
bool Server::evict_one(const Unit* except) {
    Unit* best = nullptr;
    int64_t best_t = 0;
    for (auto& up : units_) {
        Unit* v = up.get();
        if (v == except) continue;
        std::unique_lock<std::mutex> el(v->eng_mu, std::try_to_lock);
        if (!el.owns_lock() || !v->resident || v->busy) continue;
        if (!best || v->last_used_ns < best_t) {
            best = v;
            best_t = v->last_used_ns;
        }
    }
    if (!best) return false;
    std::unique_lock<std::mutex> el(best->eng_mu, std::try_to_lock);
    if (!el.owns_lock() || !best->resident || best->busy) return false;  // its worker took work meanwhile
    if (best->eng->evict() != 0) return false;
    best->resident = false;
    used_ -= std::min(used_, best->need);
    std::lock_guard<std::mutex> lk(st_mu_);
    ++stats_.evictions;
    --stats_.resident_units;
    stats_.device_bytes = used_;
    return true;
}

// Runs on u's worker with u->busy set (so nothing evicts u meanwhile).
bool Server::make_resident(Unit* u) {
    {
        std::unique_lock<std::mutex> lk(mem_mu_);
        while (used_ + u->need > budget_) {
            if (stopping_) return false;
            if (!evict_one(u)) mem_cv_.wait_for(lk, std::chrono::milliseconds(20));
        }
        used_ += u->need;
    }
    int32_t rc;
    {
        std::lock_guard<std::mutex> el(u->eng_mu);
        u->eng->reuse_analysis_once = true;  // the plan does not depend on breaker states
        rc = u->eng->upload();
        if (rc == 0 && !u->solved_once) rc = first_estimates(u);
        if (rc == 0) rc = u->eng->stream_begin(request_params());
        if (rc == 0) {
            u->resident = true;
        } else {
            u->eng->evict();
        }
    }
    std::lock_guard<std::mutex> lk(mem_mu_);
    if (rc != 0) {
        used_ -= std::min(used_, u->need);
        mem_cv_.notify_all();
        return false;
    }
    std::lock_guard<std::mutex> sl(st_mu_);
    ++stats_.admissions;
    ++stats_.resident_units;
    stats_.device_bytes = used_;
    return true;
}

int32_t Server::submit(int32_t grid, const double* z, int32_t count, int32_t branch, int32_t closed, int64_t* ticket,
                       double* v_out, double* th_out) {
    if (!started_) {
        last_error = "server not started";
        return -4;
    }
    if (grid < 0 || grid >= static_cast<int32_t>(fleet_.size()) || !z || count != fleet_[grid].n_meas) {
        last_error = "invalid request";
        return -4;
    }
    if (branch >= fleet_[grid].n_br) {
        last_error = "branch index out of range";
        return -11;
    }
    int64_t t;
    {
        std::lock_guard<std::mutex> lk(res_mu_);
        t = next_ticket_++;
    }
    if (ticket) *ticket = t;
    {
        std::lock_guard<std::mutex> lk(st_mu_);
        ++stats_.submitted;
    }
    Unit* u = units_[unit_of_[grid]].get();
    if (!u->admitted) {
        ServeResult r;
        r.admitted = 0;
        r.status = CONV_NOTOBS;
        r.t_submit_ns = r.t_start_ns = r.t_done_ns = now_ns();
        {
            std::lock_guard<std::mutex> lk(st_mu_);
            ++stats_.rejected;
        }
        finish(t, r);
        return 0;
    }
    Request rq{t, grid, std::vector<double>(z, z + count), branch, closed, now_ns(), v_out, th_out};
    {
        std::lock_guard<std::mutex> lk(u->mu);
        u->pending[local_of_[grid]].push_back(std::move(rq));
        ++u->n_pending;
    }
    u->cv.notify_one();
    return 0;
}

void Server::finish(int64_t ticket, const ServeResult& r) {
    {
        std::lock_guard<std::mutex> lk(res_mu_);
        results_[ticket] = r;
    }
    res_cv_.notify_all();
}

// Iteration-level continuous batching: between two Gauss-Newton iterations
// of the unit's batch, every grid with a pending request that is not already
// in the batch joins it (its breaker edit and snapshot applied first); after
// the iteration, grids that finished answer their request and leave.  A unit
// that is not resident is made resident before it takes requests; an idle
// unit (no request in hand) may be evicted by another unit's worker.
void Server::run_unit(Unit* u) {
    const SolveRequest rq = request_params();
    {
        std::lock_guard<std::mutex> lk(u->eng_mu);
        if (u->resident && u->eng->stream_begin(rq) != 0) {
            // the next request brings the unit back (or fails its requests)
            u->eng->evict();
            u->resident = false;
            std::lock_guard<std::mutex> ml(mem_mu_);
            used_ -= std::min(used_, u->need);
            std::lock_guard<std::mutex> sl(st_mu_);
            --stats_.resident_units;
            stats_.device_bytes = used_;
        }
        u->last_used_ns = now_ns();
    }
    struct Running {
        Request req;
        int64_t t_start;
    };
    std::unordered_map<int32_t, Running> active;  // local grid -> its request
    std::vector<Request> starting;
    std::vector<int32_t> ids, done;
    std::vector<Engine::GridResult> res;
    auto fail_all = [&](std::vector<Request>& reqs, int32_t in_batch, int64_t t_start, int64_t t_done) {
        for (auto& r0 : reqs) {
            ServeResult r;
            r.status = CONV_DIVERGED;
            r.batch_size = in_batch;
            r.t_submit_ns = r0.t_submit;
            r.t_start_ns = t_start;
            r.t_done_ns = t_done;
            finish(r0.ticket, r);
        }
        std::lock_guard<std::mutex> lk(st_mu_);
        stats_.completed += static_cast<int64_t>(reqs.size());
    };
    for (;;) {
        starting.clear();
        {
            std::unique_lock<std::mutex> lk(u->mu);
            if (active.empty()) {
                if (u->n_pending == 0) {
                    {
                        std::lock_guard<std::mutex> el(u->eng_mu);
                        u->busy = false;  // evictable while it waits
                        u->last_used_ns = now_ns();
                    }
                    mem_cv_.notify_all();
                }
                u->cv.wait(lk, [&] { return stopping_.load() || u->n_pending > 0; });
            }
            if (stopping_ && u->n_pending == 0 && active.empty()) return;
            for (size_t lid = 0; lid < u->pending.size(); ++lid) {
                auto& q = u->pending[lid];
                if (q.empty() || active.count(static_cast<int32_t>(lid))) continue;
                starting.push_back(std::move(q.front()));
                q.pop_front();
                --u->n_pending;
            }
        }
        bool resident;
        {
            std::lock_guard<std::mutex> el(u->eng_mu);
            u->busy = true;
            resident = u->resident;
        }
        if (!resident && !make_resident(u)) {
            // stopping, or the unit could not be brought back: its requests fail
            const int64_t t = now_ns();
            fail_all(starting, 0, t, t);
            if (stopping_) {
                std::lock_guard<std::mutex> lk(u->mu);
                for (auto& q : u->pending) {
                    std::vector<Request> rest(std::make_move_iterator(q.begin()), std::make_move_iterator(q.end()));
                    q.clear();
                    fail_all(rest, 0, t, t);
                }
                u->n_pending = 0;
                return;
            }
            continue;
        }
        const int64_t t0 = now_ns();
        int32_t rc = 0;
        ids.clear();
        {
            std::lock_guard<std::mutex> lk(u->eng_mu);
            for (auto& r : starting) {
                const int32_t lid = local_of_[r.grid];
                if (rc == 0 && r.branch >= 0) rc = u->eng->batch_set_branch_status(lid, r.branch, r.closed);
                if (rc == 0) rc = u->eng->batch_set_telemetry(lid, r.z.data(), static_cast<int32_t>(r.z.size()));
                ids.push_back(lid);
            }
            if (rc == 0 && !ids.empty()) rc = u->eng->stream_activate(static_cast<int32_t>(ids.size()), ids.data(), nullptr);
            for (auto& r : starting) active[local_of_[r.grid]] = Running{std::move(r), t0};
            if (rc == 0) rc = u->eng->stream_step(done, res);
            // states of the finished grids into the callers' buffers, before their tickets complete
            for (size_t i = 0; rc == 0 && i < done.size(); ++i) {
                auto it = active.find(done[i]);
                if (it == active.end() || (!it->second.req.v_out && !it->second.req.th_out)) continue;
                rc = u->eng->batch_get_state(done[i], it->second.req.v_out, it->second.req.th_out);
            }
            u->last_used_ns = now_ns();
        }
        const int64_t t1 = now_ns();
        const int32_t in_batch = static_cast<int32_t>(active.size());
        int64_t completed = 0;
        if (rc != 0) {
            // an engine error ends every request in the batch
            for (auto& kv : active) {
                ServeResult r;
                r.status = CONV_DIVERGED;
                r.batch_size = in_batch;
                r.t_submit_ns = kv.second.req.t_submit;
                r.t_start_ns = kv.second.t_start;
                r.t_done_ns = t1;
                finish(kv.second.req.ticket, r);
                ++completed;
            }
            active.clear();
            std::lock_guard<std::mutex> lk(u->eng_mu);
            u->eng->stream_begin(rq);
        } else {
            for (size_t i = 0; i < done.size(); ++i) {
                auto it = active.find(done[i]);
                if (it == active.end()) continue;
                ServeResult r;
                r.status = res[i].status;
                r.iterations = res[i].iterations;
                r.max_mismatch = res[i].max_mismatch;
                r.objective = res[i].objective;
                r.batch_size = in_batch;
                r.t_submit_ns = it->second.req.t_submit;
                r.t_start_ns = it->second.t_start;
                r.t_done_ns = t1;
                finish(it->second.req.ticket, r);
                active.erase(it);
                ++completed;
            }
        }
        std::lock_guard<std::mutex> lk(st_mu_);
        stats_.completed += completed;
        stats_.grid_solves += completed;
        ++stats_.passes;
    }
}

int32_t Server::wait(int64_t ticket, double timeout_ms, ServeResult* out) {
    std::unique_lock<std::mutex> lk(res_mu_);
    auto ready = [&] { return results_.count(ticket) != 0; };
    if (timeout_ms < 0) {
        res_cv_.wait(lk, ready);
    } else if (!res_cv_.wait_for(lk, std::chrono::duration<double, std::milli>(timeout_ms), ready)) {
        return 0;
    }
    if (out) *out = results_[ticket];
    results_.erase(ticket);
    return 1;
}

int32_t Server::get_state(int32_t grid, double* v, double* th) {
    if (grid < 0 || grid >= static_cast<int32_t>(fleet_.size()) || !started_) {
        last_error = "invalid grid";
        return -4;
    }
    Unit* u = units_[unit_of_[grid]].get();
    if (!u->admitted) {
        last_error = "grid not admitted: its unit's arena exceeds the memory budget";
        return -10;
    }
    // a unit that is not resident answers from the states saved at eviction
    std::lock_guard<std::mutex> lk(u->eng_mu);
    const int32_t rc = u->eng->batch_get_state(local_of_[grid], v, th);
    if (rc) last_error = u->eng->last_error;
    return rc;
}

ServeStats Server::stats() {
    std::lock_guard<std::mutex> lk(st_mu_);
    return stats_;
}

void Server::stop() {
    if (!started_) return;
    stopping_ = true;
    for (auto& u : units_) {
        { std::lock_guard<std::mutex> lk(u->mu); }  // a worker between its predicate check and its wait sees the flag
        u->cv.notify_all();
    }
    {
        std::lock_guard<std::mutex> lk(mem_mu_);
        mem_cv_.notify_all();  // a worker waiting for memory gives up
    }
    for (auto& u : units_)
        if (u->worker.joinable()) u->worker.join();
    started_ = false;
}

}  // namespace sle_gb300
