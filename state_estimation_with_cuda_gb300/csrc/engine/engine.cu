#include "engine.h"

#include <atomic>
#include <thread>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <functional>

namespace sle_gb300 {

cudaError_t launch_gain_export(const DevNet& net, const DevFactor& f, const DevWork& w, int32_t n_tgt, double* out,
                               cudaStream_t st);

namespace {

// Sub-allocates one device arena with 256-byte alignment.
struct Carver {
    char* base;
    size_t off = 0;
    explicit Carver(void* b) : base(static_cast<char*>(b)) {}
    template <typename T>
    T* take(size_t n) {
        off = (off + 255) & ~static_cast<size_t>(255);
        T* p = reinterpret_cast<T*>(base + off);
        off += std::max<size_t>(n, 1) * sizeof(T);
        return p;
    }
};

template <typename T, typename A>
cudaError_t put(T* dst, const std::vector<T, A>& src, cudaStream_t st) {
    if (src.empty()) return cudaSuccess;
    return cudaMemcpyAsync(dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice, st);
}

inline int nblk(int n) { return (n + 255) / 256; }

// Adds the wall time of its scope to *acc, in milliseconds.
struct HostTimer {
    double* acc;
    std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
    explicit HostTimer(double* a) : acc(a) {}
    ~HostTimer() { *acc += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count(); }
};

}  // namespace

Engine::~Engine() {
    const DeviceScope dev_scope(cfg.device_id);
    release_device();
    if (st_) cudaStreamDestroy(st_);
    if (ev0_) cudaEventDestroy(ev0_);
    if (ev1_) cudaEventDestroy(ev1_);
    if (h_status_) cudaFreeHost(h_status_);
    if (h_stage_) cudaFreeHost(h_stage_);
    if (h_batch_in_) cudaFreeHost(h_batch_in_);
    if (h_batch_out_) cudaFreeHost(h_batch_out_);
    if (d_slots_) cudaFree(d_slots_);
    if (d_scratch_) cudaFree(d_scratch_);
    if (tm0_) cudaEventDestroy(tm0_);
    if (tm1_) cudaEventDestroy(tm1_);
    for (cudaEvent_t e : ev_pool_) cudaEventDestroy(e);
}

void Engine::release_device() {
    drop_graphs();
    if (d_slots_) cudaFree(d_slots_);
    d_slots_ = nullptr;
    n_slots_ = 0;
    if (arena_) cudaFree(arena_);
    arena_ = nullptr;
    arena_bytes_ = 0;
    uploaded_ = false;
    factor_valid_ = false;
}

int32_t Engine::set_cuda_error(cudaError_t e, const char* where) {
    last_error = std::string(where) + ": " + cudaGetErrorString(e);
    return -3;
}

std::string Engine::device_info() {
    cudaDeviceProp p{};
    if (cudaGetDeviceProperties(&p, cfg.device_id) != cudaSuccess) return "no CUDA device";
    char buf[256];
    snprintf(buf, sizeof(buf), "%s (sm_%d%d, %d SMs, %.1f GiB)", p.name, p.major, p.minor, p.multiProcessorCount,
             static_cast<double>(p.totalGlobalMem) / (1024.0 * 1024.0 * 1024.0));
    return buf;
}

int32_t Engine::initialize() {
    if (init_) return 0;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n == 0) {
        last_error = "no CUDA device available";
        return -3;
    }
    if (cfg.device_id < 0 || cfg.device_id >= n) {
        last_error = "device_id out of range";
        return -4;
    }
    if ((e = cudaSetDevice(cfg.device_id)) != cudaSuccess) return set_cuda_error(e, "cudaSetDevice");
    if ((e = cudaStreamCreateWithPriority(&st_, cudaStreamNonBlocking, cfg.stream_priority)) != cudaSuccess)
        return set_cuda_error(e, "stream");
    cudaEventCreate(&ev0_);
    cudaEventCreate(&ev1_);
    if ((e = cudaMallocHost(&h_status_, sizeof(DevStatus))) != cudaSuccess) return set_cuda_error(e, "cudaMallocHost");
    init_ = true;
    return 0;
}

int32_t Engine::analyze(bool* scheduled) {
    if (scheduled) *scheduled = false;
    if (batch_mode()) return analyze_batch();
    std::string err;
    if (!model.validate(err)) {
        last_error = err;
        return -5;
    }
    // The pattern holds the closed branches (the reference's rule,
    // sparse_matrix.cu:357-404) and every branch a switching device can
    // close, so breaker operations are value edits on the device; an open
    // switched branch contributes exact zeros.
    br_in_pattern_.assign(model.br_closed.begin(), model.br_closed.end());
    for (int32_t k : model.sd_branch)
        if (k >= 0 && k < model.n_branch()) br_in_pattern_[k] = 1;
    Topology t;
    t.n_bus = model.n_bus();
    t.n_branch = model.n_branch();
    t.n_meas = model.n_meas();
    t.slack = model.slack;
    t.br_from = model.br_from.data();
    t.br_to = model.br_to.data();
    t.br_closed = br_in_pattern_.data();
    t.m_type = model.m_type.data();
    t.m_loc = model.m_loc.data();
    t.m_end = model.m_end.data();
    t.m_active = model.m_active.data();
    SymbolicParams sp;
    sp.ordering = cfg.ordering;
    const HostTimer timer(&stats.analysis_ms);
    std::function<void()> alongside;
    if (scheduled)
        alongside = [this] {
            const HostTimer schedule_timer(&stats.schedule_ms);
            build_schedule(false);
            build_eval_units();
        };
    if (!build_plan(t, sp, plan_, err, alongside)) {
        last_error = "symbolic analysis: " + err;
        analyzed_ = false;
        return -5;
    }
    if (scheduled) {
        fill_asm_targets();
        *scheduled = true;
    }
    analyzed_ = true;
    ++stats.analyses;
    return 0;
}

// Splits every level into single-CTA fronts and big fronts (more factor
// flops than cfg.big_front_flops, or too large for shared memory), lays out
// the factor storage (big fronts in place in an f x f region) and builds the
// tile work lists of the big-front kernels.
// The FP32 tiled fronts of one synchronous level as dataflow items.  Items:
// P(p, k), the panel solve of chunk k of step p, and U(p, ti, tj), the step-p
// update of tile (ti, tj).  P(p, k) waits for U(p - 1) of its column-p tiles
// and of the diagonal tile (whose item also factors the block: look-ahead);
// U(p, ti, tj) waits for the panel chunks of step p that hold its rows and
// columns and for its own step p - 1 update.  Claim order: the panel items
// of step 0, then per step p the update tiles of the next step's panel
// column (its diagonal tile first), the panel items of step p + 1, and the
// rest of step p's update tiles (one step of look-ahead).  Every dependency
// comes earlier in the order, so a waiting CTA only waits for items that
// running CTAs hold, and a tile's successive updates are a step apart.
void Engine::build_tile_tasks(const std::vector<int32_t>& bigs,
                              const std::unordered_map<int64_t, int32_t>& pair_of) {
    const Plan& P = plan_;
    struct Front {
        int32_t s, f, nc, steps, ut;
        std::vector<int32_t> pid0;  // [steps] first panel item
        std::vector<int32_t> uid;   // [steps][ut][ut] update items
    };
    const int32_t base = static_cast<int32_t>(sch_tt_.size());  // item ids are level-local
    std::vector<Front> fr;
    for (int32_t s : bigs) {
        Front b;
        b.s = s;
        b.f = P.sn_f[s];
        b.nc = P.sn_c0[s + 1] - P.sn_c0[s];
        b.steps = (b.nc + kTile - 1) / kTile;
        b.ut = (b.f + kUpdTile - 1) / kUpdTile;
        b.pid0.assign(b.steps, -1);
        b.uid.assign(static_cast<size_t>(b.steps) * b.ut * b.ut, -1);
        fr.push_back(std::move(b));
    }
    auto q0_of = [](const Front& b, int32_t p) { return p * kTile + std::min(kTile, b.nc - p * kTile); };
    auto uid = [](Front& b, int32_t p, int32_t ti, int32_t tj) -> int32_t& {
        return b.uid[(static_cast<size_t>(p) * b.ut + ti) * b.ut + tj];
    };
    std::vector<int32_t> deps;
    auto add = [&](TileTask t) {
        const int32_t id = static_cast<int32_t>(sch_tt_.size()) - base;
        if (deps.size() > static_cast<size_t>(kTileDeps)) tile_tasks_bad_ = true;  // never for 32-row tiles
        t.ndep = static_cast<int32_t>(std::min<size_t>(deps.size(), kTileDeps));
        t.pad = 0;
        for (int32_t i = 0; i < kTileDeps; ++i) t.dep[i] = i < t.ndep ? deps[i] : 0;
        for (int32_t d : deps)
            if (d < 0 || d >= id) tile_tasks_bad_ = true;  // never by construction
        sch_tt_.push_back(t);
        return id;
    };
    auto push_dep = [&](int32_t d) {
        if (std::find(deps.begin(), deps.end(), d) == deps.end()) deps.push_back(d);
    };
    auto emit_panel = [&](Front& b, int32_t p) {
        const int32_t q0 = q0_of(b, p);
        const int32_t nch = std::max(1, (b.f - q0 + kPanelRows - 1) / kPanelRows);
        const auto it = pair_of.find((static_cast<int64_t>(b.s) << 20) | p);
        const int32_t pair = it == pair_of.end() ? 0 : it->second;
        for (int32_t k = 0; k < nch; ++k) {
            deps.clear();
            if (p > 0) {
                push_dep(uid(b, p - 1, p, p));
                const int32_t r0 = q0 + k * kPanelRows, r1 = std::min(r0 + kPanelRows, b.f);
                for (int32_t ti = r0 / kUpdTile; r0 < r1 && ti <= (r1 - 1) / kUpdTile; ++ti)
                    push_dep(uid(b, p - 1, ti, p));
            }
            TileTask t{};
            t.kind = 0, t.s = b.s, t.p = p, t.a = k, t.b = nch, t.aux = pair;
            const int32_t id = add(t);
            if (k == 0) b.pid0[p] = id;
        }
    };
    // U(p, ti, tj) for every ti >= tj in tile column tj
    auto emit_update_column = [&](Front& b, int32_t p, int32_t tj) {
        const int32_t q0 = q0_of(b, p);
        for (int32_t ti = tj; ti < b.ut; ++ti) {
            deps.clear();
            for (int32_t t : {ti, tj}) {
                const int32_t r0 = std::max(t * kUpdTile, q0), r1 = std::min(t * kUpdTile + kUpdTile, b.f);
                for (int32_t k = (r0 - q0) / kPanelRows; r0 < r1 && k <= (r1 - 1 - q0) / kPanelRows; ++k)
                    push_dep(b.pid0[p] + k);
            }
            if (p > 0) push_dep(uid(b, p - 1, ti, tj));
            TileTask t{};
            t.kind = 1, t.s = b.s, t.p = p, t.a = ti, t.b = tj;
            uid(b, p, ti, tj) = add(t);
        }
    };
    // step p updates tile columns q0(p) / 32 .. ut - 1; the first is the next
    // step's panel column (or, for a last step narrower than a tile, its own)
    auto emit_update = [&](Front& b, int32_t p, bool next_column) {
        const int32_t q0 = q0_of(b, p);
        if (q0 >= b.f) return;
        const int32_t tj0 = q0 / kUpdTile;
        if (next_column)
            emit_update_column(b, p, tj0);
        else
            for (int32_t tj = tj0 + 1; tj < b.ut; ++tj) emit_update_column(b, p, tj);
    };
    int32_t max_steps = 0;
    for (Front& b : fr) max_steps = std::max(max_steps, b.steps);
    for (Front& b : fr)
        if (b.steps > 0) emit_panel(b, 0);
    for (int32_t p = 0; p < max_steps; ++p) {
        for (Front& b : fr)
            if (p < b.steps) emit_update(b, p, true);
        for (Front& b : fr)
            if (p + 1 < b.steps) emit_panel(b, p + 1);
        for (Front& b : fr)
            if (p < b.steps) emit_update(b, p, false);
    }
}

// Evaluation units (one thread each in k_evaluate): a P injection row and
// the Q row of the same bus, or a P flow row and the Q row of the same branch
// end, share their angle differences and admittance products; every other
// row is a unit alone.  A row pairs with the first waiting twin of the other
// kind; units are in the order of their first rows.  Pairing halves the
// evaluation's threads, so it is used only where the units still fill the
// GPU (cfg.eval_pair_rows rows and more, 2^18 by default): a 54k-row grid evaluated in pairs ran
// with five warps per SM and took 75 % longer, the 2.6 M-row batch union 30 %
// less.
void Engine::build_eval_units() {
    const int32_t kEvalPairRows = std::max(0, cfg.eval_pair_rows);
    const Plan& P = plan_;
    const int32_t m = model.n_meas();
    std::vector<int32_t> twin(m, -1);
    if (m >= kEvalPairRows) {
        // A row waits in the slot of its (location, group, end), by P or Q,
        // until the opposite kind arrives there; a later row of the same kind
        // takes the slot over.  Slots: injections (groups 0, 1) per bus,
        // flows (group 2) per branch end.
        const int32_t nb = model.n_bus(), nbr = model.n_branch();
        std::vector<int32_t> wait(2 * (2 * static_cast<size_t>(nb) + 2 * static_cast<size_t>(nbr)), -1);
        for (int32_t q = 0; q < m; ++q) {
            if (P.m_kind[q] != ROW_INJ && P.m_kind[q] != ROW_FLOW) continue;
            const int32_t ty = model.m_type[q];
            const int32_t grp = (ty == 2 || ty == 3) ? 0 : (ty == 7 || ty == 8) ? 1 : (ty == 4 || ty == 5) ? 2 : -1;
            if (grp < 0) continue;
            const int32_t is_q = (ty == 3 || ty == 8 || ty == 5) ? 1 : 0;
            const int64_t loc = model.m_loc[q];
            const int64_t slot = grp < 2 ? loc * 2 + grp : 2 * static_cast<int64_t>(nb) + loc * 2 + (model.m_end[q] != 0 ? 1 : 0);
            int32_t& other = wait[slot * 2 + (is_q ^ 1)];
            if (other >= 0) {
                twin[other] = q;
                twin[q] = -2;
                other = -1;
            } else {
                wait[slot * 2 + is_q] = q;
            }
        }
    }
    ev_unit_.clear();
    for (int32_t q = 0; q < m; ++q)
        if (twin[q] != -2) ev_unit_.push_back(make_int2(q, twin[q] >= 0 ? twin[q] : -1));
    ev_grp_.clear();
    const int32_t nu = static_cast<int32_t>(ev_unit_.size());
    for (int32_t u0 = 0; u0 < nu; u0 += 32) {
        const int32_t u1 = std::min(u0 + 32, nu);
        int32_t lo = ev_unit_[u0].x, hi = lo, cnt = 0;
        for (int32_t u = u0; u < u1; ++u) {
            hi = std::max(hi, std::max(ev_unit_[u].x, ev_unit_[u].y));
            cnt += ev_unit_[u].y >= 0 ? 2 : 1;
        }
        ev_grp_.push_back(cnt == hi - lo + 1 ? make_int2(lo, hi + 1) : make_int2(-1, -1));
    }
}

// The gain targets of an assembly item: those of its front in its tile
// column, [tj * kTile, tj * kTile + kTile) (targets are sorted by local index
// row + col * f).
void Engine::fill_asm_targets() {
    const Plan& P = plan_;
    const int32_t* tl = P.tgt_local.data();
    for (AsmItem& it : sch_asm_) {
        const int32_t s = it.s, f = P.sn_f[s];
        const int32_t c0 = it.tj * kTile, c1 = std::min(c0 + kTile, f);
        it.tg_lo = static_cast<int32_t>(std::lower_bound(tl + P.sn_tgt_ptr[s], tl + P.sn_tgt_ptr[s + 1], c0 * f) - tl);
        it.tg_hi = static_cast<int32_t>(std::lower_bound(tl + it.tg_lo, tl + P.sn_tgt_ptr[s + 1], c1 * f) - tl);
    }
}

void Engine::build_schedule(bool targets_ready) {
    const Plan& P = plan_;
    const int32_t ns = P.n_super, nl = P.n_levels;
    sch_small_ptr_.assign(nl + 1, 0);
    sch_small_maxf_.assign(nl, 0);
    sch_asm_ptr_.assign(nl + 1, 0);
    sch_panels_.assign(nl, 0);
    sch_step_ptr_.assign(nl + 1, 0);
    sch_all_ptr_.assign(nl + 1, 0);
    sch_maxf_.assign(nl, 0);
    sch_maxpanel_.assign(nl, 0);
    sch_small_.clear();
    sch_all_.clear();
    sch_asm_.clear();
    sch_asm_child_.clear();
    sch_pot_.clear();
    n_pot_pairs_ = 0;
    sch_upd_.clear();
    sch_pot_ptr_.assign(1, 0);
    sch_pan_ptr_.assign(1, 0);
    sch_pan_.clear();
    sch_upd_ptr_.assign(1, 0);
    sch_tt_.clear();
    sch_tt_ptr_.assign(nl + 1, 0);
    tile_tasks_bad_ = false;
    sch_flow_a_.clear();
    sch_flow_w_.clear();
    sch_flow_b_.clear();
    sch_down_.clear();
    sch_up_.clear();
    flow_a_maxf_ = flow_b_maxf_ = 0;
    lay_lx_off_.assign(ns + 1, 0);
    lay_u_off_.assign(ns + 1, 0);
    lay_u_ld_.assign(ns, 0);
    lay_u_big_.assign(ns, 0);
    std::vector<char> big(ns, 0);
    for (int32_t s = 0; s < ns; ++s) {
        const int64_t f = P.sn_f[s], nc = P.sn_c0[s + 1] - P.sn_c0[s];
        double fl = 0.0;
        for (int64_t c = 0; c < nc; ++c) fl += static_cast<double>(f - c - 1) * (f - c);
        // FP64 work per front is costly on this GPU, so the FP64 pipeline moves
        // fronts with many flops to the tiled path; in FP32 only size decides
        const int64_t fmax = mixed_ ? kSmallFrontMax32 : kSmallFrontMax;
        big[s] = (f > fmax || (!mixed_ && fl > cfg.big_front_flops)) ? 1 : 0;
    }
    // Dataflow phases: a front whose subtree holds no big front is factorised
    // by the persistent kernels (phase A if no front of its subtree is wider
    // than cfg.flow_small_f, phase B otherwise); the rest stays level-synchronous.
    const int32_t want_f = cfg.flow_small_f > 0 ? cfg.flow_small_f : (mixed_ ? 128 : 64);
    const int32_t flow_small_f = std::max(8, std::min(want_f, kFlowSmallFMax));
    std::vector<char> sub_big(ns, 0);
    std::vector<int32_t> sub_maxf(ns, 0);
    for (int32_t l = 0; l < nl; ++l)
        for (int32_t x = P.lvl_ptr[l]; x < P.lvl_ptr[l + 1]; ++x) {
            const int32_t s = P.lvl_sn[x];
            sub_big[s] = static_cast<char>(sub_big[s] | big[s]);
            sub_maxf[s] = std::max(sub_maxf[s], P.sn_f[s]);
            const int32_t p = P.sn_parent[s];
            if (p >= 0) {
                sub_big[p] = static_cast<char>(sub_big[p] | sub_big[s]);
                sub_maxf[p] = std::max(sub_maxf[p], sub_maxf[s]);
            }
        }
    // The warp phase is decided per grid (by default: from kWarpPhaseMinFronts
    // candidate fronts of that grid on), so that a grid of a batch runs the
    // same kernels, and gets the same result, as when it is solved alone.
    std::vector<int32_t> front_grid(ns, 0);
    int32_t n_groups = 1;
    if (batch_mode()) {
        int64_t total = 0;
        for (const Plan& gp : grid_plans_) total += gp.n_super;
        if (total == ns) {
            int32_t x = 0;
            n_groups = static_cast<int32_t>(grid_plans_.size());
            for (int32_t g = 0; g < n_groups; ++g)
                for (int32_t k = 0; k < grid_plans_[g].n_super; ++k) front_grid[x++] = g;
        }
    }
    std::vector<int32_t> n_warp(n_groups, 0);
    for (int32_t s = 0; s < ns; ++s)
        if (cfg.dataflow && !sub_big[s] && sub_maxf[s] <= kWarpFrontMax) ++n_warp[front_grid[s]];
    std::vector<char> warp_phase(n_groups, 0);
    for (int32_t g = 0; g < n_groups; ++g)
        warp_phase[g] = cfg.warp_fronts > 0 || (cfg.warp_fronts < 0 && n_warp[g] >= kWarpPhaseMinFronts);
    flow_phase_.assign(ns, 0);
    for (int32_t s = 0; s < ns; ++s)
        if (cfg.dataflow && !sub_big[s])
            flow_phase_[s] = (warp_phase[front_grid[s]] && sub_maxf[s] <= kWarpFrontMax)
                                 ? 3
                                 : (sub_maxf[s] <= flow_small_f ? 1 : 2);
    int64_t lx = 0, uu = 0;
    for (int32_t s = 0; s < ns; ++s) {
        const int64_t f = P.sn_f[s], nc = P.sn_c0[s + 1] - P.sn_c0[s];
        lay_lx_off_[s] = lx;
        if (big[s]) {
            lay_u_off_[s] = lx + nc + nc * f;
            lay_u_ld_[s] = static_cast<int32_t>(f);
            lay_u_big_[s] = 1;
            lx += f * f;
        } else {
            lay_u_off_[s] = uu;
            lay_u_ld_[s] = static_cast<int32_t>(f - nc);
            lx += f * nc;
            uu += (f - nc) * (f - nc);
        }
    }
    lay_lx_off_[ns] = lx;
    lay_u_off_[ns] = uu;
    lay_lx_size_ = lx;
    lay_u_size_ = uu;
    // every front by level (solves without dataflow, backward order)
    std::vector<int32_t> lvl_of(ns, 0);
    for (int32_t l = 0; l < nl; ++l) {
        for (int32_t x = P.lvl_ptr[l]; x < P.lvl_ptr[l + 1]; ++x) {
            const int32_t s = P.lvl_sn[x];
            lvl_of[s] = l;
            sch_all_.push_back(s);
            sch_maxf_[l] = std::max(sch_maxf_[l], P.sn_f[s]);
            sch_maxpanel_[l] = std::max<int64_t>(sch_maxpanel_[l],
                                                 static_cast<int64_t>(P.sn_f[s]) * (P.sn_c0[s + 1] - P.sn_c0[s]));
            if (flow_phase_[s] == 1) flow_a_maxf_ = std::max(flow_a_maxf_, P.sn_f[s]);
            if (flow_phase_[s] == 2) flow_b_maxf_ = std::max(flow_b_maxf_, P.sn_f[s]);
        }
        sch_all_ptr_[l + 1] = static_cast<int32_t>(sch_all_.size());
    }
    // Level-synchronous fronts (not in a dataflow phase) are grouped either
    // by height (levels from the leaves, as above) or by depth (distance from
    // the root, deepest first).  Either order completes children first; the
    // one with fewer launches wins.  In a batch the wide fronts sit just below
    // each grid's root, so depth lines them up across grids where height does
    // not, and the union needs about as many panel steps as its largest grid.
    std::vector<int32_t> depth(ns, 0);
    int32_t dmax = 0;
    for (int32_t s = ns - 1; s >= 0; --s) {  // parents follow their children
        const int32_t p = P.sn_parent[s];
        depth[s] = p >= 0 ? depth[p] + 1 : 0;
        if (flow_phase_[s] == 0) dmax = std::max(dmax, depth[s]);
    }
    const int32_t per_panel = mixed_ ? 2 : 3;  // launches per panel step
    auto sync_cost = [&](bool by_depth) {
        std::vector<int32_t> pan(nl, 0);
        std::vector<char> has_small(nl, 0), has_big(nl, 0);
        for (int32_t s = 0; s < ns; ++s) {
            if (flow_phase_[s] != 0) continue;
            const int32_t l = by_depth ? dmax - depth[s] : lvl_of[s];
            if (big[s]) {
                has_big[l] = 1;
                pan[l] = std::max(pan[l], (P.sn_c0[s + 1] - P.sn_c0[s] + kTile - 1) / kTile);
            } else {
                has_small[l] = 1;
            }
        }
        int64_t c = 0;
        for (int32_t l = 0; l < nl; ++l) c += static_cast<int64_t>(pan[l]) * per_panel + has_small[l] + has_big[l];
        return c;
    };
    sync_cost_height_ = sync_cost(false);
    sync_cost_depth_ = dmax < nl ? sync_cost(true) : sync_cost_height_;
    const bool by_depth = dmax < nl && sync_cost_depth_ < sync_cost_height_;
    sync_by_depth_ = by_depth ? 1 : 0;
    std::vector<std::vector<int32_t>> sync_lvl(nl);
    for (int32_t l = 0; l < nl; ++l)
        for (int32_t x = P.lvl_ptr[l]; x < P.lvl_ptr[l + 1]; ++x) {
            const int32_t s = P.lvl_sn[x];
            if (flow_phase_[s] == 0) sync_lvl[by_depth ? dmax - depth[s] : l].push_back(s);
        }
    for (int32_t l = 0; l < nl; ++l) {
        std::vector<int32_t> bigs;
        for (int32_t s : sync_lvl[l]) {
            if (big[s]) {
                bigs.push_back(s);
            } else {
                sch_small_.push_back(s);
                sch_small_maxf_[l] = std::max(sch_small_maxf_[l], P.sn_f[s]);
            }
        }
        int32_t panels = 0;
        std::unordered_map<int64_t, int32_t> pair_of;  // (front, step) -> step-0 tile-reader counter
        for (int32_t s : bigs) {
            const int32_t f = P.sn_f[s], nc = P.sn_c0[s + 1] - P.sn_c0[s];
            const int32_t tiles = (f + kTile - 1) / kTile;
            for (int32_t tj = 0; tj < tiles; ++tj) {
                const int32_t rows = f - tj * kTile;  // the tile column's lower part
                const int32_t c0 = tj * kTile, c1 = std::min(c0 + kTile, f);
                for (int32_t rb = 0; rb * kAsmRows < rows; ++rb) {
                    const int32_t R0 = c0 + rb * kAsmRows, R1 = std::min(R0 + kAsmRows, f);
                    // target range [tg_lo, tg_hi) by fill_asm_targets()
                    AsmItem it{s, tj, rb, 0, 0, static_cast<int32_t>(sch_asm_child_.size()), 0, 0};
                    // the children that add entries to rows [R0, R1) of columns [c0, c1), in order
                    for (int32_t ci = P.sn_child_ptr[s]; ci < P.sn_child_ptr[s + 1]; ++ci) {
                        const int32_t c = P.sn_child[ci];
                        const int32_t m = P.sn_f[c] - (P.sn_c0[c + 1] - P.sn_c0[c]);
                        const int32_t* rel = P.sn_relmap.data() + P.sn_su_off[c];
                        const int32_t j0 = static_cast<int32_t>(std::lower_bound(rel, rel + m, c0) - rel);
                        const int32_t j1 = static_cast<int32_t>(std::lower_bound(rel + j0, rel + m, c1) - rel);
                        const int32_t ilo = static_cast<int32_t>(std::lower_bound(rel, rel + m, R0) - rel);
                        const int32_t ihi = static_cast<int32_t>(std::lower_bound(rel + ilo, rel + m, R1) - rel);
                        if (j0 < j1 && std::max(j0, ilo) < ihi)
                            sch_asm_child_.push_back(AsmChild{c, j0, j1, ilo, ihi, 0, 0, 0});
                    }
                    it.ch_hi = static_cast<int32_t>(sch_asm_child_.size());
                    sch_asm_.push_back(it);
                }
            }
            panels = std::max(panels, (nc + kTile - 1) / kTile);
        }
        sch_panels_[l] = panels;
        sch_step_ptr_[l + 1] = sch_step_ptr_[l] + panels;
        for (int32_t p = 0; p < panels; ++p) {
            for (int32_t s : bigs) {
                const int32_t f = P.sn_f[s], nc = P.sn_c0[s + 1] - P.sn_c0[s];
                if (nc <= p * kTile) continue;
                const int32_t tiles = (f + kTile - 1) / kTile;
                const int32_t pb = std::min(kTile, nc - p * kTile);
                const int32_t q0 = p * kTile + pb;
                if (mixed_) {
                    // one CTA per kPanelRows rows below the diagonal block
                    const int32_t nch = std::max(1, (f - q0 + kPanelRows - 1) / kPanelRows);
                    for (int32_t k = 0; k < nch; ++k) sch_pot_.push_back(make_int4(s, k, nch, n_pot_pairs_));
                    pair_of[(static_cast<int64_t>(s) << 20) | p] = n_pot_pairs_;
                    ++n_pot_pairs_;
                } else {
                    sch_pot_.push_back(make_int4(s, p, 0, 0));
                }
                if (!mixed_)  // FP64: the panel's row tiles below go to the multi-CTA solve
                    for (int32_t ti = p + 1; ti < tiles; ++ti) sch_pan_.push_back(make_int4(s, ti, 0, 0));
                if (q0 < f) {
                    const int32_t ut = (f + kUpdTile - 1) / kUpdTile;
                    for (int32_t tj = q0 / kUpdTile; tj < ut; ++tj)
                        for (int32_t ti = tj; ti < ut; ++ti) sch_upd_.push_back(make_int4(s, ti, tj, 0));
                }
            }
            sch_pot_ptr_.push_back(static_cast<int32_t>(sch_pot_.size()));
            sch_pan_ptr_.push_back(static_cast<int32_t>(sch_pan_.size()));
            sch_upd_ptr_.push_back(static_cast<int32_t>(sch_upd_.size()));
        }
        if (mixed_ && cfg.tile_flow && !bigs.empty()) build_tile_tasks(bigs, pair_of);
        sch_tt_ptr_[l + 1] = static_cast<int32_t>(sch_tt_.size());
        sch_small_ptr_[l + 1] = static_cast<int32_t>(sch_small_.size());
        sch_asm_ptr_[l + 1] = static_cast<int32_t>(sch_asm_.size());
    }
    // every front, top-down, for the backward dataflow sweep
    // every front top-down for the backward sweeps: warp fronts apart
    sch_down_.clear();
    sch_down_w_.clear();
    for (auto it = sch_all_.rbegin(); it != sch_all_.rend(); ++it)
        (flow_phase_[*it] == 3 ? sch_down_w_ : sch_down_).push_back(*it);
    // continuation sweeps: children counts and initially ready fronts, the
    // ones with the most factor work on their path to the root first
    phase_nchild_.assign(ns, 0);
    nchild_.assign(ns, 0);
    std::vector<double> up_cost(ns, 0.0);
    for (int32_t s = ns - 1; s >= 0; --s) {  // parents follow their children
        const int32_t p = P.sn_parent[s];
        const double f = P.sn_f[s], nc = P.sn_c0[s + 1] - P.sn_c0[s];
        up_cost[s] = f * f * nc + (p >= 0 ? up_cost[p] : 0.0);
        if (p >= 0) {
            if (flow_phase_[s] != 3) ++nchild_[p];  // the CTA forward sweep counts no warp fronts
            if (flow_phase_[p] != 0 && flow_phase_[p] == flow_phase_[s]) ++phase_nchild_[p];
        }
    }
    for (int32_t s = 0; s < ns; ++s) {
        if (flow_phase_[s] == 3 && phase_nchild_[s] == 0) sch_flow_w_.push_back(s);
        if (flow_phase_[s] == 1 && phase_nchild_[s] == 0) sch_flow_a_.push_back(s);
        if (flow_phase_[s] == 2 && phase_nchild_[s] == 0) sch_flow_b_.push_back(s);
        if (flow_phase_[s] != 3 && nchild_[s] == 0) sch_up_.push_back(s);
    }
    auto by_cost = [&](int32_t a, int32_t b) { return up_cost[a] > up_cost[b] || (up_cost[a] == up_cost[b] && a < b); };
    std::sort(sch_flow_w_.begin(), sch_flow_w_.end(), by_cost);
    std::sort(sch_flow_a_.begin(), sch_flow_a_.end(), by_cost);
    std::sort(sch_flow_b_.begin(), sch_flow_b_.end(), by_cost);
    std::sort(sch_up_.begin(), sch_up_.end(), by_cost);
    if (targets_ready) fill_asm_targets();
}

int32_t Engine::schedule_info(ScheduleInfo& out) {
    if (!uploaded_) {
        // Host-only: the schedule of the current options is built into the
        // engine's schedule members, which upload() rebuilds from scratch
        // (together with the pipeline precision) before it uses them; the
        // precision flag of the engine is left as it was.
        if (!(analyzed_ && !model.structure_dirty)) {
            const int32_t rc = analyze();
            if (rc) return rc;
        }
        const bool mixed_before = mixed_;
        mixed_ = cfg.use_double_precision == 0;
        build_schedule();
        mixed_ = mixed_before;
    }
    out = ScheduleInfo();
    for (char ph : flow_phase_) {
        out.n_warp += ph == 3;
        out.n_phase_a += ph == 1;
        out.n_phase_b += ph == 2;
        out.n_sync += ph == 0;
    }
    out.warp_ready = static_cast<int32_t>(sch_flow_w_.size());
    out.a_ready = static_cast<int32_t>(sch_flow_a_.size());
    out.b_ready = static_cast<int32_t>(sch_flow_b_.size());
    out.up_ready = static_cast<int32_t>(sch_up_.size());
    out.down_n = static_cast<int32_t>(sch_down_.size());
    out.down_warp_n = static_cast<int32_t>(sch_down_w_.size());
    for (size_t l = 0; l + 1 < sch_small_ptr_.size(); ++l)
        out.sync_levels += (sch_small_ptr_[l + 1] > sch_small_ptr_[l] || sch_asm_ptr_[l + 1] > sch_asm_ptr_[l]) ? 1 : 0;
    for (int32_t p : sch_panels_) out.panel_steps += p;
    out.tile_tasks = tile_tasks_bad_ ? -1 : static_cast<int32_t>(sch_tt_.size());
    out.by_depth = sync_by_depth_;
    out.launches_by_height = sync_cost_height_;
    out.launches_by_depth = sync_cost_depth_;
    return 0;
}

int32_t Engine::upload() {
    const DeviceScope dev_scope(cfg.device_id);
    int32_t rc = initialize();
    if (rc) return rc;
    // keep the hot-start state across re-uploads
    if (uploaded_) download_results();
    const bool mixed_before = mixed_;
    mixed_ = cfg.use_double_precision == 0;  // the schedule may be built during the analysis
    bool scheduled = false;
    if (!(reuse_analysis_once && analyzed_)) rc = analyze(&scheduled);
    reuse_analysis_once = false;
    if (rc) {
        mixed_ = mixed_before;
        return rc;
    }
    const int32_t n = model.n_bus(), nbr = model.n_branch(), m = model.n_meas();
    const Plan& P = plan_;
    if (!scheduled) {
        const HostTimer timer(&stats.schedule_ms);
        build_schedule();
        build_eval_units();
    }
    const HostTimer upload_timer(&stats.upload_ms);
    const int64_t nnz_h = static_cast<int64_t>(P.h_col.size());
    const int64_t nnz_y = static_cast<int64_t>(P.y_col.size());
    const int32_t ns = P.n_super;
    const int32_t nparts = std::max(nblk(std::max(m, 1)), nblk(n)) + 1;

    auto layout = [&](Carver& c) {
        // network
        net_.bus_type = c.take<int32_t>(n);
        net_.v_setpoint = c.take<double>(n);
        net_.br_from = c.take<int32_t>(nbr);
        net_.br_to = c.take<int32_t>(nbr);
        net_.br_r = c.take<double>(nbr);
        net_.br_x = c.take<double>(nbr);
        net_.br_bch = c.take<double>(nbr);
        net_.br_tap = c.take<double>(nbr);
        net_.br_shift = c.take<double>(nbr);
        net_.br_closed = c.take<uint8_t>(nbr);
        net_.br_g = c.take<double>(nbr);
        net_.br_b = c.take<double>(nbr);
        net_.br_bsf = c.take<double>(nbr);
        net_.br_bst = c.take<double>(nbr);
        net_.br_itap = c.take<double>(nbr);
        net_.br_itap2 = c.take<double>(nbr);
        net_.y_ptr = c.take<int32_t>(n + 1);
        net_.y_col = c.take<int32_t>(nnz_y);
        net_.y_src = c.take<int32_t>(nnz_y);
        net_.y_g = c.take<double>(nnz_y);
        net_.y_b = c.take<double>(nnz_y);
        net_.y_hpos_t = c.take<int32_t>(nnz_y);
        net_.y_hpos_v = c.take<int32_t>(nnz_y);
        net_.m_type = c.take<int32_t>(m);
        net_.m_loc = c.take<int32_t>(m);
        net_.m_end = c.take<int32_t>(m);
        net_.m_kind = c.take<int32_t>(m);
        net_.m_fpos = c.take<int32_t>(m);
        net_.m_active = c.take<uint8_t>(m);
        net_.m_sigma = c.take<double>(m);
        net_.m_w = c.take<double>(m);
        net_.h_ptr = c.take<int32_t>(m + 1);
        net_.h_row = c.take<int32_t>(nnz_h);
        net_.h_pcol = c.take<int32_t>(nnz_h);
        // factor plan
        fac_.sn_c0 = c.take<int32_t>(ns + 1);
        fac_.sn_f = c.take<int32_t>(ns);
        fac_.sn_parent = c.take<int32_t>(ns);
        fac_.sn_rows_off = c.take<int64_t>(ns + 1);
        fac_.sn_rows = c.take<int32_t>(P.sn_rows.size());
        fac_.sn_lx_off = c.take<int64_t>(ns + 1);
        fac_.sn_u_off = c.take<int64_t>(ns + 1);
        fac_.sn_su_off = c.take<int64_t>(ns + 1);
        fac_.sn_child_ptr = c.take<int32_t>(ns + 1);
        fac_.sn_child = c.take<int32_t>(P.sn_child.size());
        fac_.sn_relmap = c.take<int32_t>(P.sn_relmap.size());
        fac_.sn_tgt_ptr = c.take<int32_t>(ns + 1);
        fac_.tgt_local = c.take<int32_t>(P.tgt_local.size());
        fac_.tgt_pair_ptr = c.take<int64_t>(P.tgt_pair_ptr.size());
        fac_.pair_a = c.take<int32_t>(P.pair_a.size());
        fac_.pair_b = c.take<int32_t>(P.pair_b.size());
        fac_.rhs_ptr = c.take<int32_t>(P.rhs_ptr.size());
        fac_.rhs_h = c.take<int32_t>(P.rhs_h.size());
        fac_.bus_ps_theta = c.take<int32_t>(n);
        fac_.bus_ps_v = c.take<int32_t>(n);
        fac_.sn_u_ld = c.take<int32_t>(ns);
        fac_.sn_u_big = c.take<uint8_t>(ns);
        fac_.sn_pw = c.take<int8_t>(ns);
        fac_.sn_grid = batch_mode() ? c.take<int32_t>(ns) : nullptr;
        fac_.tgt_grid = batch_mode() ? c.take<int32_t>(P.tgt_local.size()) : nullptr;
        fac_.ps_grid = batch_mode() ? c.take<int32_t>(P.n_state) : nullptr;
        net_.meas_grid = batch_mode() ? c.take<int32_t>(m) : nullptr;
        net_.ev_unit = c.take<int2>(ev_unit_.size());
        net_.ev_grp = c.take<int2>(ev_grp_.size());
        net_.n_units = static_cast<int32_t>(ev_unit_.size());
        net_.bus_grid = batch_mode() ? c.take<int32_t>(n) : nullptr;
        if (batch_mode()) {
            const int32_t G = static_cast<int32_t>(grids_.size());
            batch_.n_grids = G;
            batch_.bus_off = c.take<int32_t>(G + 1);
            batch_.meas_off = c.take<int32_t>(G + 1);
            batch_.flags = c.take<uint32_t>(G);
            batch_.iters = c.take<int32_t>(G);
            batch_.mismatch = c.take<double>(G);
            batch_.objective = c.take<double>(G);
            uint8_t* af = c.take<uint8_t>(3 * static_cast<size_t>(G));  // active, flat, retire
            batch_.active = af;
            batch_.flat = af + G;
            batch_.retire = af + 2 * static_cast<size_t>(G);
            batch_.running = c.take<int32_t>(1);
            batch_.loop = c.take<int32_t>(4);
            // items of kBatchChunk buses / rows, a grid's items adjacent
            auto items = [&](bool rows, std::vector<int2>& it, std::vector<int32_t>& ptr) {
                it.clear();
                ptr.assign(1, 0);
                for (int32_t g = 0; g < G; ++g) {
                    const int32_t a = rows ? grids_[g].m0 : grids_[g].bus0;
                    const int32_t n = rows ? grids_[g].nm : grids_[g].nbus;
                    for (int32_t k = 0; k < n; k += kBatchChunk) it.push_back(make_int2(g, a + k));
                    ptr.push_back(static_cast<int32_t>(it.size()));
                }
            };
            items(false, bus_items_, bus_item_ptr_);
            items(true, row_items_, row_item_ptr_);
            batch_.n_bus_items = static_cast<int32_t>(bus_items_.size());
            batch_.n_row_items = static_cast<int32_t>(row_items_.size());
            batch_.bus_items = c.take<int2>(bus_items_.size());
            batch_.bus_item_ptr = c.take<int32_t>(G + 1);
            batch_.row_items = c.take<int2>(row_items_.size());
            batch_.row_item_ptr = c.take<int32_t>(G + 1);
            batch_.part = c.take<double>(std::max<size_t>(1, std::max(bus_items_.size(), row_items_.size())));
            batch_.part_bad = c.take<int32_t>(std::max<size_t>(1, bus_items_.size()));
        } else {
            batch_ = DevBatch{};
        }
        d_small_ = c.take<int32_t>(sch_small_.size());
        d_all_ = c.take<int32_t>(sch_all_.size());
        d_asm_ = c.take<AsmItem>(sch_asm_.size());
        d_asm_child_ = c.take<AsmChild>(sch_asm_child_.size());
        d_pot_ = c.take<int4>(sch_pot_.size());
        d_pot_cnt_ = c.take<int32_t>(std::max(1, n_pot_pairs_));
        d_pan_ = c.take<int4>(sch_pan_.size());
        d_upd_ = c.take<int4>(sch_upd_.size());
        d_tt_ = c.take<TileTask>(sch_tt_.size());
        d_tt_done_ = c.take<int32_t>(sch_tt_.size() + static_cast<size_t>(P.n_levels));
        d_flow_a_ = c.take<int32_t>(sch_flow_a_.size());
        d_flow_b_ = c.take<int32_t>(sch_flow_b_.size());
        d_down_ = c.take<int32_t>(sch_down_.size());
        d_up_ = c.take<int32_t>(sch_up_.size());
        d_flow_w_ = c.take<int32_t>(sch_flow_w_.size());
        d_down_w_ = c.take<int32_t>(sch_down_w_.size());
        d_phase_ = c.take<int8_t>(ns);
        d_phase_nchild_ = c.take<int32_t>(ns);
        d_nchild_ = c.take<int32_t>(ns);
        d_ready_n_ = c.take<int32_t>(kReadyLists);
        {
            int32_t src_n[kReadyLists];
            for (int l = 0; l < kReadyLists; ++l) src_n[l] = static_cast<int32_t>(claim_list(l).size());
            for (int l = 0; l < kReadyLists; ++l) d_cmp_[l] = batch_mode() ? c.take<int32_t>(src_n[l]) : nullptr;
            d_chunk_cnt_ = batch_mode() ? c.take<int32_t>(std::max(1, ready_chunks(src_n))) : nullptr;
        }
        // work
        work_.v = c.take<double>(n);
        work_.th = c.take<double>(n);
        work_.z = c.take<double>(m);
        work_.h = c.take<double>(m);
        work_.r = c.take<double>(m);
        work_.w_eff = c.take<double>(m);
        work_.wr = c.take<double>(m);
        work_.hval = c.take<double>(nnz_h);
        work_.rhs = c.take<double>(P.n_state);
        work_.sol = c.take<double>(P.n_state);
        work_.hval32 = mixed_ ? c.take<float>(nnz_h) : nullptr;
        work_.bus_cs = c.take<double2>(n);
        work_.hw = mixed_ ? nullptr : c.take<double>(nnz_h);
        work_.hw32 = mixed_ ? c.take<float>(nnz_h) : nullptr;
        work_.b0 = c.take<double>(P.n_state);
        work_.dx = c.take<double>(P.n_state);
        work_.hdx = c.take<double>(m);
        work_.lx = mixed_ ? nullptr : c.take<double>(lay_lx_size_);
        work_.u = mixed_ ? nullptr : c.take<double>(lay_u_size_);
        work_.lx32 = mixed_ ? c.take<float>(lay_lx_size_) : nullptr;
        work_.u32 = mixed_ ? c.take<float>(lay_u_size_) : nullptr;
        work_.su = c.take<double>(P.su_size);
        work_.gvals = c.take<double>(P.tgt_local.size());
        work_.flow = c.take<int32_t>(3 * static_cast<int64_t>(ns) + 16);
        work_.rdiag = c.take<double>(P.n_state);
        work_.rhs32 = mixed_ ? c.take<float>(P.n_state) : nullptr;
        work_.sol32 = mixed_ ? c.take<float>(P.n_state) : nullptr;
        work_.su32 = mixed_ ? c.take<float>(P.su_size) : nullptr;
        work_.p_inj = c.take<double>(n);
        work_.q_inj = c.take<double>(n);
        work_.pf = c.take<double>(nbr);
        work_.qf = c.take<double>(nbr);
        work_.pt = c.take<double>(nbr);
        work_.qt = c.take<double>(nbr);
        work_.part = c.take<double>(nparts);
        work_.hpart = c.take<double>(nparts);
        work_.opart = c.take<double>(nparts);
        work_.oidx = c.take<int32_t>(nparts);
        work_.ocnt = c.take<int32_t>(nparts);
        work_.status = c.take<DevStatus>(1);
        work_.grid_flags = batch_mode() ? batch_.flags : nullptr;
        work_.spin_limit = cfg.spin_limit;
        work_.hold_front = cfg.hold_front;
        isl_parent_ = c.take<int32_t>(n);
        isl_out_ = c.take<int32_t>(4);
    };
    Carver dry(nullptr);
    layout(dry);
    const size_t need = dry.off + 256;
    need_bytes = need;
    if (budget_bytes && need > budget_bytes) {
        last_error = "device arena of " + std::to_string(need) + " bytes exceeds the admission budget of " +
                     std::to_string(budget_bytes) + " bytes";
        return -10;
    }
    cudaError_t e = cudaStreamSynchronize(st_);
    if (e != cudaSuccess) return set_cuda_error(e, "stream sync");
    release_device();
    e = cudaMalloc(&arena_, need);
    if (e != cudaSuccess) {
        arena_ = nullptr;
        last_error = "device allocation of " + std::to_string(need) + " bytes failed";
        return -10;
    }
    arena_bytes_ = need;
    Carver real(arena_);
    layout(real);
    net_.n_bus = n;
    net_.n_branch = nbr;
    net_.n_meas = m;
    net_.n_state = P.n_state;
    net_.slack = model.slack;
    fac_.n_super = ns;
    fac_.n_state = P.n_state;

    std::vector<uint8_t> act(model.m_active);
    std::vector<int32_t> btype(model.bus_type);
    auto chk = [&](cudaError_t ee) { if (ee != cudaSuccess && e == cudaSuccess) e = ee; };
    chk(put(const_cast<int32_t*>(net_.bus_type), model.bus_type, st_));
    chk(put(const_cast<double*>(net_.v_setpoint), model.bus_vset, st_));
    chk(put(const_cast<int32_t*>(net_.br_from), model.br_from, st_));
    chk(put(const_cast<int32_t*>(net_.br_to), model.br_to, st_));
    chk(put(const_cast<double*>(net_.br_r), model.br_r, st_));
    chk(put(const_cast<double*>(net_.br_x), model.br_x, st_));
    chk(put(const_cast<double*>(net_.br_bch), model.br_b, st_));
    chk(put(const_cast<double*>(net_.br_tap), model.br_tap, st_));
    chk(put(const_cast<double*>(net_.br_shift), model.br_shift, st_));
    chk(put(const_cast<uint8_t*>(net_.br_closed), model.br_closed, st_));
    chk(put(const_cast<int32_t*>(net_.y_ptr), P.y_ptr, st_));
    chk(put(const_cast<int32_t*>(net_.y_col), P.y_col, st_));
    chk(put(const_cast<int32_t*>(net_.y_src), P.y_src, st_));
    chk(put(const_cast<int32_t*>(net_.y_hpos_t), P.y_hpos_t, st_));
    chk(put(const_cast<int32_t*>(net_.y_hpos_v), P.y_hpos_v, st_));
    chk(put(const_cast<int32_t*>(net_.m_type), model.m_type, st_));
    chk(put(const_cast<int32_t*>(net_.m_loc), model.m_loc, st_));
    chk(put(const_cast<int32_t*>(net_.m_end), model.m_end, st_));
    chk(put(const_cast<int32_t*>(net_.m_kind), P.m_kind, st_));
    chk(put(const_cast<int32_t*>(net_.m_fpos), P.m_fpos, st_));
    chk(put(const_cast<int2*>(net_.ev_unit), ev_unit_, st_));
    chk(put(const_cast<int2*>(net_.ev_grp), ev_grp_, st_));
    chk(put(const_cast<uint8_t*>(net_.m_active), model.m_active, st_));
    chk(put(const_cast<double*>(net_.m_sigma), model.m_sigma, st_));
    chk(put(const_cast<double*>(net_.m_w), model.m_w, st_));
    chk(put(const_cast<int32_t*>(net_.h_ptr), P.h_ptr, st_));
    chk(put(const_cast<int32_t*>(net_.h_row), P.h_row, st_));
    chk(put(const_cast<int32_t*>(net_.h_pcol), P.h_pcol, st_));
    chk(put(const_cast<int32_t*>(fac_.sn_c0), P.sn_c0, st_));
    chk(put(const_cast<int32_t*>(fac_.sn_f), P.sn_f, st_));
    chk(put(const_cast<int32_t*>(fac_.sn_parent), P.sn_parent, st_));
    chk(put(const_cast<int64_t*>(fac_.sn_rows_off), P.sn_rows_off, st_));
    chk(put(const_cast<int32_t*>(fac_.sn_rows), P.sn_rows, st_));
    chk(put(const_cast<int64_t*>(fac_.sn_lx_off), lay_lx_off_, st_));
    chk(put(const_cast<int64_t*>(fac_.sn_u_off), lay_u_off_, st_));
    chk(put(const_cast<int64_t*>(fac_.sn_su_off), P.sn_su_off, st_));
    chk(put(const_cast<int32_t*>(fac_.sn_child_ptr), P.sn_child_ptr, st_));
    chk(put(const_cast<int32_t*>(fac_.sn_child), P.sn_child, st_));
    chk(put(const_cast<int32_t*>(fac_.sn_relmap), P.sn_relmap, st_));
    chk(put(const_cast<int32_t*>(fac_.sn_tgt_ptr), P.sn_tgt_ptr, st_));
    chk(put(const_cast<int32_t*>(fac_.tgt_local), P.tgt_local, st_));
    chk(put(const_cast<int64_t*>(fac_.tgt_pair_ptr), P.tgt_pair_ptr, st_));
    chk(put(const_cast<int32_t*>(fac_.pair_a), P.pair_a, st_));
    chk(put(const_cast<int32_t*>(fac_.pair_b), P.pair_b, st_));
    chk(put(const_cast<int32_t*>(fac_.rhs_ptr), P.rhs_ptr, st_));
    chk(put(const_cast<int32_t*>(fac_.rhs_h), P.rhs_h, st_));
    chk(put(const_cast<int32_t*>(fac_.bus_ps_theta), P.bus_ps_theta, st_));
    chk(put(const_cast<int32_t*>(fac_.bus_ps_v), P.bus_ps_v, st_));
    chk(put(const_cast<int32_t*>(fac_.sn_u_ld), lay_u_ld_, st_));
    chk(put(const_cast<uint8_t*>(fac_.sn_u_big), lay_u_big_, st_));
    if (batch_mode()) {
        const int32_t G = static_cast<int32_t>(grids_.size());
        std::vector<int32_t> sg, boff(G + 1, 0), moff(G + 1, 0);
        sg.reserve(ns);
        for (int32_t g = 0; g < G; ++g) {
            sg.insert(sg.end(), grid_plans_[g].n_super, g);
            boff[g + 1] = grids_[g].bus0 + grids_[g].nbus;
            moff[g + 1] = grids_[g].m0 + grids_[g].nm;
        }
        chk(put(const_cast<int32_t*>(fac_.sn_grid), sg, st_));
        {
            std::vector<int32_t> tg(P.tgt_local.size()), pg(P.n_state), mg(m);
            for (int32_t sn = 0; sn < ns; ++sn)
                for (int32_t x = P.sn_tgt_ptr[sn]; x < P.sn_tgt_ptr[sn + 1]; ++x) tg[x] = sg[sn];
            for (int32_t sn = 0; sn < ns; ++sn)
                for (int32_t p = P.sn_c0[sn]; p < P.sn_c0[sn + 1]; ++p) pg[p] = sg[sn];
            for (int32_t g = 0; g < G; ++g)
                for (int32_t q = moff[g]; q < moff[g + 1]; ++q) mg[q] = g;
            chk(put(const_cast<int32_t*>(fac_.tgt_grid), tg, st_));
            chk(put(const_cast<int32_t*>(fac_.ps_grid), pg, st_));
            chk(put(const_cast<int32_t*>(net_.meas_grid), mg, st_));
            std::vector<int32_t> bg(n);
            for (int32_t g = 0; g < G; ++g)
                for (int32_t i = boff[g]; i < boff[g + 1]; ++i) bg[i] = g;
            chk(put(const_cast<int32_t*>(net_.bus_grid), bg, st_));
        }
        chk(put(const_cast<int32_t*>(batch_.bus_off), boff, st_));
        chk(put(const_cast<int32_t*>(batch_.meas_off), moff, st_));
        chk(put(const_cast<int2*>(batch_.bus_items), bus_items_, st_));
        chk(put(const_cast<int32_t*>(batch_.bus_item_ptr), bus_item_ptr_, st_));
        chk(put(const_cast<int2*>(batch_.row_items), row_items_, st_));
        chk(put(const_cast<int32_t*>(batch_.row_item_ptr), row_item_ptr_, st_));
        // flags, iterations, mismatch, objective per grid; running count (+4
        // spare); the device loop's four words
        const size_t out_bytes = static_cast<size_t>(G) * (4 + 4 + 8 + 8) + 8 + 16;
        if (h_batch_cap_ < static_cast<size_t>(G)) {
            if (h_batch_in_) cudaFreeHost(h_batch_in_);
            if (h_batch_out_) cudaFreeHost(h_batch_out_);
            h_batch_in_ = nullptr;
            h_batch_out_ = nullptr;
            h_batch_cap_ = 0;
            chk(cudaMallocHost(reinterpret_cast<void**>(&h_batch_in_), 3 * static_cast<size_t>(G)));
            chk(cudaMallocHost(&h_batch_out_, out_bytes));
            if (e == cudaSuccess) h_batch_cap_ = G;
        }
    }
    chk(put(d_small_, sch_small_, st_));
    chk(put(d_all_, sch_all_, st_));
    chk(put(d_asm_, sch_asm_, st_));
    chk(put(d_asm_child_, sch_asm_child_, st_));
    chk(put(d_pot_, sch_pot_, st_));
    chk(put(d_pan_, sch_pan_, st_));
    chk(put(d_upd_, sch_upd_, st_));
    chk(put(d_tt_, sch_tt_, st_));
    chk(put(d_flow_a_, sch_flow_a_, st_));
    chk(put(d_flow_b_, sch_flow_b_, st_));
    chk(put(d_down_, sch_down_, st_));
    chk(put(d_up_, sch_up_, st_));
    chk(put(d_flow_w_, sch_flow_w_, st_));
    chk(put(d_down_w_, sch_down_w_, st_));
    {
        std::vector<int8_t> ph(flow_phase_.begin(), flow_phase_.end());
        chk(put(d_phase_, ph, st_));
    }
    chk(put(d_phase_nchild_, phase_nchild_, st_));
    {
        // phase-A fronts are factorised with kPanelFlowA-column panels, all
        // others (warp fronts: one block of at most kWarpFrontMax) kTile
        std::vector<int8_t> pw(ns);
        for (int32_t x = 0; x < ns; ++x) pw[x] = static_cast<int8_t>(flow_phase_[x] == 1 ? kPanelFlowA : kTile);
        chk(put(const_cast<int8_t*>(fac_.sn_pw), pw, st_));
    }
    chk(put(d_nchild_, nchild_, st_));
    {
        std::vector<int32_t> nl(kReadyLists);
        for (int l = 0; l < kReadyLists; ++l) nl[l] = static_cast<int32_t>(claim_list(l).size());
        chk(put(d_ready_n_, nl, st_));
        // until the first compaction the batch lists are the full ones (every
        // factor or solve launch then finds valid lists)
        for (int l = 0; l < kReadyLists; ++l)
            if (d_cmp_[l] && nl[l] > 0)
                chk(cudaMemcpyAsync(d_cmp_[l], claim_dev(l), sizeof(int32_t) * nl[l], cudaMemcpyDeviceToDevice, st_));
    }
    chk(put(work_.v, model.bus_v, st_));
    chk(put(work_.th, model.bus_th, st_));
    chk(put(work_.z, model.m_value, st_));
    chk(cudaMemsetAsync(work_.status, 0, sizeof(DevStatus), st_));
    chk(launch_admittance_and_ybus(net_, st_));
    chk(prepare_factor_kernels());
    chk(cudaStreamSynchronize(st_));
    if (e != cudaSuccess) return set_cuda_error(e, "upload");

    sched_.n_levels = P.n_levels;
    sched_.n_tgt = static_cast<int32_t>(P.tgt_local.size());
    sched_.gain_acc32 = mixed_ && cfg.gain_acc32 ? 1 : 0;
    sched_.h_small_ptr = sch_small_ptr_.data();
    sched_.d_small = d_small_;
    sched_.h_small_maxf = sch_small_maxf_.data();
    sched_.h_asm_ptr = sch_asm_ptr_.data();
    sched_.d_asm = d_asm_;
    sched_.d_asm_child = d_asm_child_;
    sched_.h_lvl_panels = sch_panels_.data();
    sched_.h_step_ptr = sch_step_ptr_.data();
    sched_.h_pot_ptr = sch_pot_ptr_.data();
    sched_.d_pot = d_pot_;
    sched_.d_pot_cnt = d_pot_cnt_;
    sched_.n_pot_pairs = n_pot_pairs_;
    sched_.h_pan_ptr = sch_pan_ptr_.data();
    sched_.d_pan = d_pan_;
    sched_.h_upd_ptr = sch_upd_ptr_.data();
    sched_.d_upd = d_upd_;
    sched_.h_all_ptr = sch_all_ptr_.data();
    sched_.d_all = d_all_;
    sched_.h_lvl_maxf = sch_maxf_.data();
    sched_.h_lvl_maxpanel = sch_maxpanel_.data();
    {
        const int32_t ms = max_solve_front();
        FlowGrids g = flow_grids(mixed_, flow_a_maxf_, flow_b_maxf_, ms);
        const bool tt = mixed_ && !sch_tt_.empty() && !tile_tasks_bad_ && g.tile > 0;
        sched_.h_tt_ptr = sch_tt_ptr_.data();
        sched_.d_tt = d_tt_;
        sched_.d_tt_done = d_tt_done_;
        sched_.n_tt = tt ? static_cast<int32_t>(sch_tt_.size()) : 0;
        sched_.tt_grid = g.tile;
        sched_.d_flow_w = d_flow_w_;
        sched_.flow_w_n = static_cast<int32_t>(sch_flow_w_.size());
        sched_.flow_w_grid = std::max(1, std::min(g.w, sched_.flow_w_n));
        sched_.d_down_w = d_down_w_;
        sched_.down_w_n = static_cast<int32_t>(sch_down_w_.size());
        sched_.solve_w_grid = std::max(1, std::min(g.wsolve, std::max(sched_.flow_w_n, sched_.down_w_n)));
        sched_.d_flow_a = d_flow_a_;
        sched_.flow_a_n = static_cast<int32_t>(sch_flow_a_.size());
        sched_.flow_a_maxf = flow_a_maxf_;
        sched_.flow_a_grid = std::max(1, std::min(g.a, sched_.flow_a_n));
        sched_.d_flow_b = d_flow_b_;
        sched_.flow_b_n = static_cast<int32_t>(sch_flow_b_.size());
        sched_.flow_b_maxf = flow_b_maxf_;
        sched_.flow_b_grid = std::max(1, std::min(g.b, sched_.flow_b_n));
        sched_.d_phase = d_phase_;
        sched_.d_phase_nchild = d_phase_nchild_;
        sched_.solve_flow = (cfg.dataflow && g.solve > 0) ? 1 : 0;
        sched_.d_up = d_up_;
        sched_.up_n = static_cast<int32_t>(sch_up_.size());
        sched_.d_nchild = d_nchild_;
        sched_.d_down = d_down_;
        sched_.solve_maxf = ms;
        sched_.solve_grid = std::max(1, std::min(g.solve, ns));
        sched_.up_grid = std::max(1, std::min(g.solve, sched_.up_n));
        // claim-list lengths on the device; a batch claims from compacted copies
        sched_.d_ready_n = d_ready_n_;
        sched_.compact = batch_mode() ? 1 : 0;
        sched_.d_chunk_cnt = d_chunk_cnt_;
        for (int l = 0; l < kReadyLists; ++l) {
            sched_.src_lists[l] = claim_dev(l);
            sched_.src_n[l] = static_cast<int32_t>(claim_list(l).size());
            sched_.cmp_lists[l] = d_cmp_[l];
        }
        if (sched_.compact) {
            sched_.d_flow_a = d_cmp_[0];
            sched_.d_flow_b = d_cmp_[1];
            sched_.d_up = d_cmp_[2];
            sched_.d_down = d_cmp_[3];
            sched_.d_flow_w = d_cmp_[4];
            sched_.d_down_w = d_cmp_[5];
        }
    }

    if (h_stage_n_ < static_cast<size_t>(m)) {
        if (h_stage_) cudaFreeHost(h_stage_);
        h_stage_ = nullptr;
        h_stage_n_ = 0;
        if (cudaMallocHost(&h_stage_, std::max<size_t>(m, 1) * sizeof(double)) == cudaSuccess) h_stage_n_ = m;
    }
    p_inj.assign(n, 0.0);
    q_inj.assign(n, 0.0);
    pf.assign(nbr, 0.0);
    qf.assign(nbr, 0.0);
    pt.assign(nbr, 0.0);
    qt.assign(nbr, 0.0);
    uploaded_ = true;
    factor_valid_ = false;
    stale_ = 0;
    model.structure_dirty = false;
    model.branch_values_dirty = false;  // the upload took the current branch values
    ++stats.uploads;
    model.values_dirty = false;
    return 0;
}

int32_t Engine::update_telemetry(const double* z, int32_t count) {
    const DeviceScope dev_scope(cfg.device_id);
    if (count != model.n_meas()) {
        last_error = "telemetry count does not match the measurement count";
        return -4;
    }
    std::memcpy(model.m_value.data(), z, sizeof(double) * count);
    if (!uploaded_ || model.structure_dirty) {
        model.values_dirty = true;
        return 0;
    }
    cudaError_t e;
    if (h_stage_ && h_stage_n_ >= static_cast<size_t>(count)) {
        // wait for the previous staged copy before overwriting the staging buffer
        e = cudaStreamSynchronize(st_);
        if (e != cudaSuccess) return set_cuda_error(e, "telemetry");
        std::memcpy(h_stage_, z, sizeof(double) * count);
        e = cudaMemcpyAsync(work_.z, h_stage_, sizeof(double) * count, cudaMemcpyHostToDevice, st_);
    } else {
        e = cudaMemcpyAsync(work_.z, z, sizeof(double) * count, cudaMemcpyHostToDevice, st_);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st_);
    }
    if (e != cudaSuccess) return set_cuda_error(e, "telemetry");
    model.values_dirty = false;
    return 0;
}

int32_t Engine::sync_measurements() {
    if (!uploaded_) return 0;
    return update_telemetry(model.m_value.data(), model.n_meas());
}

int32_t Engine::flat_start() {
    const DeviceScope dev_scope(cfg.device_id);
    for (int32_t i = 0; i < model.n_bus(); ++i) {
        const int32_t t = model.bus_type[i];
        model.bus_v[i] = (t == 1 || t == 2) ? model.bus_vset[i] : 1.0;
        model.bus_th[i] = 0.0;
    }
    if (!uploaded_) return 0;
    cudaError_t e = launch_flat_start(net_, work_, st_);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st_);
    if (e != cudaSuccess) return set_cuda_error(e, "flat start");
    return 0;
}

SolveParams Engine::params(const SolveRequest& rq) const {
    SolveParams sp{};
    sp.exact_jacobian = cfg.exact_jacobian;
    sp.mixed = mixed_ ? 1 : 0;
    sp.robust = rq.robust;
    sp.huber_gamma = rq.huber_gamma;
    sp.tol = rq.tolerance;
    sp.vmin = cfg.voltage_min_pu;
    sp.vmax = cfg.voltage_max_pu;
    sp.skip_flags = FLAG_FROZEN;
    sp.huber_objective = (rq.robust && cfg.huber_stall > 0.0 && !batch_mode()) ? 1 : 0;
    return sp;
}

int32_t Engine::stage_begin(int32_t stage) {
    if (!cfg.enable_profiling) return -1;
    while (ev_pool_.size() < ev_used_ + 2) {
        cudaEvent_t e;
        cudaEventCreate(&e);
        ev_pool_.push_back(e);
    }
    const int32_t mark = static_cast<int32_t>(ev_used_);
    ev_used_ += 2;
    cudaEventRecord(ev_pool_[mark], st_);
    ev_marks_.push_back({stage, mark});
    return mark;
}

void Engine::stage_end(int32_t stage, int32_t mark, int64_t launches_before) {
    stats.launches[stage] += t_kernel_launches - launches_before;
    stats.calls[stage] += 1;
    if (mark >= 0) cudaEventRecord(ev_pool_[mark + 1], st_);
}

void Engine::collect_stage_times() {
    for (auto& m : ev_marks_) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, ev_pool_[m.second], ev_pool_[m.second + 1]) == cudaSuccess)
            stats.ms[m.first] += ms;
    }
    ev_marks_.clear();
    ev_used_ = 0;
}

int32_t Engine::enqueue_iteration(const SolveParams& sp, bool refactor, int64_t* per_stage, bool host_copies) {
    cudaError_t e = cudaMemsetAsync(&work_.status->flags, 0, sizeof(uint32_t), st_);
    if (e == cudaSuccess && batch_mode()) e = cudaMemsetAsync(batch_.running, 0, sizeof(int32_t), st_);
    auto update = [&](const double* step) {
        return batch_mode() ? launch_batch_update(net_, fac_, work_, batch_, sp, step, st_)
                            : launch_update(net_, fac_, work_, sp, step, st_);
    };
    auto stage = [&](int32_t st, auto&& fn) {
        if (e != cudaSuccess) return;
        const int64_t l0 = t_kernel_launches;
        const int32_t mk = stage_begin(st);
        e = fn();
        if (per_stage) per_stage[st] += t_kernel_launches - l0;
        if (mk >= 0) cudaEventRecord(ev_pool_[mk + 1], st_);
    };
    if (sched_.compact) stage(ST_OTHER, [&] { return launch_ready_compact(fac_, work_, sched_, st_); });
    stage(ST_EVALUATE, [&] { return launch_evaluate(net_, work_, sp, st_); });
    if (!mixed_) {
        if (refactor) stage(ST_FACTOR, [&] { return launch_factor(net_, fac_, work_, sched_, st_); });
        stage(ST_RHS, [&] { return launch_rhs(net_, fac_, work_, st_); });
        stage(ST_SOLVE, [&] { return launch_solve(fac_, work_, sched_, st_); });
        stage(ST_UPDATE, [&] { return update(work_.sol); });
    } else {
        if (refactor) stage(ST_FACTOR, [&] { return launch_factor32(net_, fac_, work_, sched_, st_); });
        stage(ST_RHS, [&] { return launch_rhs(net_, fac_, work_, st_); });
        stage(ST_SOLVE, [&] {
            cudaError_t ee = launch_to_fp32(fac_, work_, st_);
            if (ee == cudaSuccess) ee = launch_solve32(fac_, work_, sched_, st_);
            if (ee == cudaSuccess) ee = launch_refine_begin(fac_, work_, st_);
            for (int32_t k = 0; k < cfg.refine_steps && ee == cudaSuccess; ++k) {
                ee = launch_refine_residual(net_, fac_, work_, st_);
                if (ee == cudaSuccess) ee = launch_solve32(fac_, work_, sched_, st_);
                if (ee == cudaSuccess) ee = launch_refine_accumulate(fac_, work_, st_);
            }
            return ee;
        });
        stage(ST_UPDATE, [&] { return update(work_.dx); });
    }
    if (e == cudaSuccess && host_copies)
        e = cudaMemcpyAsync(h_status_, work_.status, sizeof(DevStatus), cudaMemcpyDeviceToHost, st_);
    if (e == cudaSuccess && host_copies && batch_mode()) {
        const int32_t G = batch_.n_grids;
        int32_t* h_running = reinterpret_cast<int32_t*>(static_cast<char*>(h_batch_out_) + static_cast<size_t>(G) * 24);
        e = cudaMemcpyAsync(h_running, batch_.running, sizeof(int32_t), cudaMemcpyDeviceToHost, st_);
    }
    if (e != cudaSuccess) {
        set_cuda_error(e, "iteration");
        return -3;
    }
    return 0;
}

void Engine::apply_wait_options() {
    work_.spin_limit = cfg.spin_limit;
    work_.hold_front = cfg.hold_front;
    drop_graphs();  // the captured launches hold the previous values
}

void Engine::drop_graphs() {
    for (auto& g : graphs_) {
        if (g.exec) cudaGraphExecDestroy(g.exec);
        g = IterGraph();
    }
    if (loop_graph_.exec) cudaGraphExecDestroy(loop_graph_.exec);
    loop_graph_ = IterGraph();
}

int32_t Engine::run_device_loop(const SolveParams& sp, int32_t max_iter, int32_t& steps) {
    steps = 0;
    if (!cfg.device_loop || !cfg.use_cuda_graphs || cfg.enable_profiling) return -1;
    IterGraph& g = loop_graph_;
    if (!g.exec || std::memcmp(&g.sp, &sp, sizeof(sp)) != 0) {
        const HostTimer timer(&stats.capture_ms);
        if (g.exec) cudaGraphExecDestroy(g.exec);
        g = IterGraph();
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaGraphCreate(&graph, 0);
        if (e != cudaSuccess) return set_cuda_error(e, "loop graph");
        cudaGraphConditionalHandle h{};
        // the node's condition starts at 1 on every launch: the first step
        // always runs (max_iter >= 1)
        e = cudaGraphConditionalHandleCreate(&h, graph, 1u, cudaGraphCondAssignDefault);
        cudaGraphNodeParams np{};
        np.type = cudaGraphNodeTypeConditional;
        np.conditional.handle = h;
        np.conditional.type = cudaGraphCondTypeWhile;
        np.conditional.size = 1;
        cudaGraphNode_t node = nullptr;
        if (e == cudaSuccess) e = cudaGraphAddNode(&node, graph, nullptr, nullptr, 0, &np);
        int32_t rc = 0;
        const int64_t before = t_kernel_launches;
        if (e == cudaSuccess) {
            cudaGraph_t body = np.conditional.phGraph_out[0];
            e = cudaStreamBeginCaptureToGraph(st_, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
            if (e == cudaSuccess) {
                rc = enqueue_iteration(sp, true, g.launches, false);
                cudaError_t ek = rc == 0 ? launch_gn_loop_next(h, batch_, work_, st_) : cudaSuccess;
                g.launches[ST_OTHER] += 1;
                e = cudaStreamEndCapture(st_, &body);
                if (e == cudaSuccess) e = ek;
            }
        }
        g.total = t_kernel_launches - before;
        g_kernel_launches -= g.total;  // counted per step run
        t_kernel_launches -= g.total;
        if (e == cudaSuccess && rc == 0) e = cudaGraphInstantiate(&g.exec, graph, 0);
        cudaGraphDestroy(graph);
        if (rc) {
            g = IterGraph();
            return rc;
        }
        if (e != cudaSuccess) {
            g = IterGraph();
            return set_cuda_error(e, "loop graph");
        }
        g.sp = sp;
    }
    cudaError_t e = launch_gn_loop_init(batch_, max_iter, st_);
    if (e == cudaSuccess) e = cudaGraphLaunch(g.exec, st_);
    int32_t* h_loop = reinterpret_cast<int32_t*>(static_cast<char*>(h_batch_out_) + static_cast<size_t>(batch_.n_grids) * 24 + 8);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h_loop, batch_.loop, 4 * sizeof(int32_t), cudaMemcpyDeviceToHost, st_);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st_);
    if (e != cudaSuccess) return set_cuda_error(e, "device loop");
    steps = h_loop[0];
    g_kernel_launches += g.total * steps;
    t_kernel_launches += g.total * steps;
    for (int i = 0; i < ST_COUNT; ++i) {
        stats.launches[i] += g.launches[i] * steps;
        if (i != ST_OTHER) stats.calls[i] += steps;
    }
    stats.iterations += steps;
    if (h_loop[2]) {
        last_error = "factorisation dataflow wait timed out";
        return -3;
    }
    return 0;
}

int32_t Engine::run_iteration(const SolveParams& sp, bool refactor) {
    int64_t per_stage[ST_COUNT] = {0, 0, 0, 0, 0, 0};
    const bool use_graph = cfg.use_cuda_graphs && !cfg.enable_profiling;
    if (!use_graph) {
        const int32_t rc = enqueue_iteration(sp, refactor, per_stage);
        if (rc) return rc;
    } else {
        IterGraph& g = graphs_[refactor ? 1 : 0];
        if (!g.exec || std::memcmp(&g.sp, &sp, sizeof(sp)) != 0) {
            const HostTimer timer(&stats.capture_ms);
            if (g.exec) cudaGraphExecDestroy(g.exec);
            g = IterGraph();
            cudaGraph_t graph = nullptr;
            cudaError_t e = cudaStreamBeginCapture(st_, cudaStreamCaptureModeThreadLocal);
            if (e != cudaSuccess) return set_cuda_error(e, "graph capture");
            const int64_t before = t_kernel_launches;
            const int32_t rc = enqueue_iteration(sp, refactor, g.launches);
            e = cudaStreamEndCapture(st_, &graph);
            g.total = t_kernel_launches - before;
            g_kernel_launches -= g.total;  // counted when the graph runs
            t_kernel_launches -= g.total;
            if (rc) {
                if (graph) cudaGraphDestroy(graph);
                return rc;
            }
            if (e == cudaSuccess) e = cudaGraphInstantiate(&g.exec, graph, 0);
            if (graph) cudaGraphDestroy(graph);
            if (e != cudaSuccess) {
                g.exec = nullptr;
                return set_cuda_error(e, "graph instantiate");
            }
            g.sp = sp;
        }
        cudaError_t e = cudaGraphLaunch(g.exec, st_);
        if (e != cudaSuccess) return set_cuda_error(e, "graph launch");
        g_kernel_launches += g.total;
        for (int i = 0; i < ST_COUNT; ++i) per_stage[i] = g.launches[i];
    }
    for (int i = 0; i < ST_COUNT; ++i) {
        if (i == ST_FACTOR && !refactor) continue;
        if (i == ST_OTHER) continue;
        stats.launches[i] += per_stage[i];
        stats.calls[i] += 1;
    }
    cudaError_t e = cudaStreamSynchronize(st_);
    ++stats.iterations;
    ++stats.step_waits;
    if (e != cudaSuccess) {
        set_cuda_error(e, "iteration");
        return -3;
    }
    return 0;
}

int32_t Engine::solve(const SolveRequest& rq, SolveResult& out) {
    const DeviceScope dev_scope(cfg.device_id);
    out = SolveResult();
    if (batch_mode()) {
        last_error = "a batch handle is solved with batch_solve";
        out.status = CONV_NOTOBS;
        return -4;
    }
    if (!init_ || !uploaded_ || model.structure_dirty) {
        const int32_t rc = upload();
        if (rc) {
            out.status = CONV_NOTOBS;
            last_ = out;
            return rc;
        }
    }
    if (model.branch_values_dirty) {
        const int32_t rc = apply_branch_edits();
        if (rc) {
            out.status = CONV_SINGULAR;
            last_ = out;
            return rc;
        }
        if (model.structure_dirty) {  // an edit needs a new pattern
            const int32_t rc2 = upload();
            if (rc2) {
                out.status = CONV_NOTOBS;
                last_ = out;
                return rc2;
            }
        }
    }
    if (model.values_dirty) {
        const int32_t rc = sync_measurements();
        if (rc) return rc;
    }
    const SolveParams sp = params(rq);
    cudaEventRecord(ev0_, st_);
    if (rq.flat_start) launch_flat_start(net_, work_, st_);
    const int32_t max_iter = rq.max_iterations;
    bool converged = false, diverged = false, retry = false;
    int32_t retries = 0;
    double jh_prev = -1.0;  // Huber objective of the previous evaluation (stall test)
    out.status = CONV_RUNNING;
    do {
        if (retry) {
            launch_flat_start(net_, work_, st_);
            converged = diverged = retry = false;
            factor_valid_ = false;
            jh_prev = -1.0;
        }
        for (int32_t it = 0; it < max_iter && !converged && !diverged; ++it) {
            const bool refactor = !factor_valid_ || rq.robust || cfg.gain_policy == 0;
            if (run_iteration(sp, refactor) != 0) {
                out.status = CONV_SINGULAR;  // wls_solver.cu:296-300
                diverged = true;
                break;
            }
            const uint32_t fl = h_status_->flags;
            if (fl & FLAG_TIMEOUT) {
                // a failure inside an iteration ends the solve as SINGULAR_MATRIX
                // (wls_solver.cu:296-300); the message names the cause
                last_error = "factorisation dataflow wait timed out";
                out.status = CONV_SINGULAR;
                factor_valid_ = false;
                last_ = out;
                return -3;
            }
            if (fl & FLAG_SINGULAR) {
                out.status = CONV_SINGULAR;
                factor_valid_ = false;
                diverged = true;
                break;
            }
            if (refactor) factor_valid_ = true;
            out.max_mismatch = h_status_->max_mismatch;
            converged = (fl & FLAG_CONVERGED) != 0;
            diverged = (fl & FLAG_NONFINITE) != 0;
            if (sp.huber_objective && !diverged) {
                // robust stall test (option huber_stall): the Huber objective of
                // this iteration's evaluation fell by no more than
                // huber_stall x its previous value -> the estimate stands
                const double jh = h_status_->huber_objective;
                if (jh_prev > 0.0 && jh_prev - jh <= cfg.huber_stall * jh_prev) converged = true;
                jh_prev = jh;
            }
            out.iterations = it + 1;
            if (rq.mode == Mode::REALTIME && rq.time_limit_ms > 0.0) {
                cudaEventRecord(ev1_, st_);
                cudaEventSynchronize(ev1_);
                float ms = 0.f;
                cudaEventElapsedTime(&ms, ev0_, ev1_);
                if (ms > rq.time_limit_ms && !converged && !diverged) {
                    out.status = CONV_MAXIT;
                    break;
                }
            }
        }
        if (diverged && retries < 2 && rq.mode != Mode::REALTIME) {  // wls_solver.cu:326-332
            retry = true;
            ++retries;
            out.iterations = 0;
            if (out.status == CONV_RUNNING) {
                // retry from a flat start
            }
        }
    } while (retry);
    if (out.status == CONV_RUNNING) out.status = converged ? CONV_OK : (diverged ? CONV_DIVERGED : CONV_MAXIT);
    if (diverged) factor_valid_ = false;
    // final evaluation at the returned state: objective, residuals, bad data
    {
        const int64_t l0 = t_kernel_launches;
        const int32_t mk = stage_begin(ST_OTHER);
        launch_evaluate(net_, work_, sp, st_);
        launch_objective(net_, work_, cfg.bad_data_threshold, st_);
        stage_end(ST_OTHER, mk, l0);
    }
    cudaEventRecord(ev1_, st_);
    cudaMemcpyAsync(h_status_, work_.status, sizeof(DevStatus), cudaMemcpyDeviceToHost, st_);
    cudaError_t e = cudaStreamSynchronize(st_);
    if (e != cudaSuccess) {
        set_cuda_error(e, "solve");
        out.status = CONV_SINGULAR;
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ev0_, ev1_);
    out.time_ms = ms;
    out.objective = h_status_->objective;
    out.largest_residual = h_status_->largest_residual;
    out.largest_idx = h_status_->largest_idx;
    out.bad_count = h_status_->bad_count;
    stale_ = DL_ALL;
    last_ = out;
    ++stats.solves;
    collect_stage_times();
    return 0;
}

int32_t Engine::apply_branch_edits() {
    if (!model.branch_values_dirty) return 0;
    if (!uploaded_ || model.structure_dirty) return 0;  // the next upload takes the host values
    const DeviceScope dev_scope(cfg.device_id);
    for (int32_t k = 0; k < model.n_branch(); ++k)
        if (model.br_closed[k] && !branch_in_pattern(k)) {
            model.structure_dirty = true;  // a branch outside the pattern closed: analyse again
            return 0;
        }
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t x) {
        if (e == cudaSuccess) e = x;
    };
    chk(put(const_cast<double*>(net_.br_r), model.br_r, st_));
    chk(put(const_cast<double*>(net_.br_x), model.br_x, st_));
    chk(put(const_cast<double*>(net_.br_bch), model.br_b, st_));
    chk(put(const_cast<double*>(net_.br_tap), model.br_tap, st_));
    chk(put(const_cast<double*>(net_.br_shift), model.br_shift, st_));
    chk(put(const_cast<uint8_t*>(net_.br_closed), model.br_closed, st_));
    chk(launch_admittance_and_ybus(net_, st_));
    chk(cudaStreamSynchronize(st_));
    if (e != cudaSuccess) return set_cuda_error(e, "branch edits");
    model.branch_values_dirty = false;
    factor_valid_ = false;
    stale_ = DL_ALL;
    ++stats.branch_edits;
    return 0;
}

int32_t Engine::evict() {
    const DeviceScope dev_scope(cfg.device_id);
    if (!uploaded_) return 0;
    stale_ |= DL_STATE;  // the device state is the one to keep
    const int32_t rc = download_results(DL_STATE);
    if (rc) return rc;
    const cudaError_t e = cudaStreamSynchronize(st_);
    if (e != cudaSuccess) return set_cuda_error(e, "evict");
    release_device();
    return 0;
}

int32_t Engine::download_results(int32_t what) {
    const DeviceScope dev_scope(cfg.device_id);
    what &= stale_;
    if (!uploaded_ || !what) return 0;
    const int32_t n = model.n_bus(), m = model.n_meas(), nbr = model.n_branch();
    cudaError_t e = cudaSuccess;
    auto get = [&](double* dst, const double* src, int32_t cnt) {
        if (cnt > 0 && e == cudaSuccess) e = cudaMemcpyAsync(dst, src, sizeof(double) * cnt, cudaMemcpyDeviceToHost, st_);
    };
    if (what & DL_STATE) {
        get(model.bus_v.data(), work_.v, n);
        get(model.bus_th.data(), work_.th, n);
    }
    if (what & DL_MEAS) {
        get(model.m_est.data(), work_.h, m);
        get(model.m_res.data(), work_.r, m);
    }
    if (what & DL_FLOWS) {
        e = launch_results(net_, work_, st_);
        get(p_inj.data(), work_.p_inj, n);
        get(q_inj.data(), work_.q_inj, n);
        get(pf.data(), work_.pf, nbr);
        get(qf.data(), work_.qf, nbr);
        get(pt.data(), work_.pt, nbr);
        get(qt.data(), work_.qt, nbr);
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(st_);
    if (e != cudaSuccess) return set_cuda_error(e, "download");
    stale_ &= ~what;
    return 0;
}

int32_t Engine::evaluate_at(const double* v, const double* th, int32_t exact) {
    const DeviceScope dev_scope(cfg.device_id);
    if (!uploaded_ || model.structure_dirty) {
        const int32_t rc = upload();
        if (rc) return rc;
    }
    if (model.branch_values_dirty) {
        int32_t rc = apply_branch_edits();
        if (rc == 0 && model.structure_dirty) rc = upload();
        if (rc) return rc;
    }
    if (model.values_dirty) sync_measurements();
    const int32_t n = model.n_bus();
    cudaError_t e = cudaMemcpyAsync(work_.v, v, sizeof(double) * n, cudaMemcpyHostToDevice, st_);
    if (e == cudaSuccess) e = cudaMemcpyAsync(work_.th, th, sizeof(double) * n, cudaMemcpyHostToDevice, st_);
    SolveParams sp{};
    sp.exact_jacobian = exact;
    sp.mixed = mixed_ ? 1 : 0;
    sp.robust = 0;
    sp.huber_gamma = cfg.huber_gamma;
    sp.tol = cfg.convergence_tolerance;
    sp.vmin = cfg.voltage_min_pu;
    sp.vmax = cfg.voltage_max_pu;
    if (e == cudaSuccess) e = launch_evaluate(net_, work_, sp, st_);
    if (e == cudaSuccess) e = launch_objective(net_, work_, cfg.bad_data_threshold, st_);
    if (e == cudaSuccess) e = launch_rhs(net_, fac_, work_, st_);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st_);
    if (e != cudaSuccess) return set_cuda_error(e, "evaluate");
    stale_ = DL_ALL;
    factor_valid_ = false;
    return 0;
}

int32_t Engine::export_gain(std::vector<int32_t>& rows, std::vector<int32_t>& cols, std::vector<double>& vals) {
    const DeviceScope dev_scope(cfg.device_id);
    const Plan& P = plan_;
    if (mixed_) {
        last_error = "stage access needs the FP64 pipeline (use_double_precision = 1)";
        return -4;
    }
    const int32_t nt = static_cast<int32_t>(P.tgt_local.size());
    double* d = nullptr;
    cudaError_t e = cudaMalloc(&d, sizeof(double) * std::max(nt, 1));
    if (e != cudaSuccess) return set_cuda_error(e, "export gain");
    e = launch_gain_export(net_, fac_, work_, nt, d, st_);
    vals.assign(nt, 0.0);
    if (e == cudaSuccess && nt > 0) e = cudaMemcpyAsync(vals.data(), d, sizeof(double) * nt, cudaMemcpyDeviceToHost, st_);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st_);
    cudaFree(d);
    if (e != cudaSuccess) return set_cuda_error(e, "export gain");
    rows.resize(nt);
    cols.resize(nt);
    for (int32_t s = 0; s < P.n_super; ++s) {
        const int32_t f = P.sn_f[s];
        for (int32_t tg = P.sn_tgt_ptr[s]; tg < P.sn_tgt_ptr[s + 1]; ++tg) {
            const int32_t lr = P.tgt_local[tg] % f, lc = P.tgt_local[tg] / f;
            rows[tg] = P.state_of_ps[P.sn_rows[P.sn_rows_off[s] + lr]];
            cols[tg] = P.state_of_ps[P.sn_c0[s] + lc];
        }
    }
    return 0;
}

int32_t Engine::factor_and_solve(const double* rhs_orig, double* x_orig) {
    const DeviceScope dev_scope(cfg.device_id);
    const Plan& P = plan_;
    if (mixed_) {
        last_error = "stage access needs the FP64 pipeline (use_double_precision = 1)";
        return -4;
    }
    std::vector<double> b(P.n_state);
    for (int32_t p = 0; p < P.n_state; ++p) b[p] = rhs_orig[P.state_of_ps[p]];
    cudaError_t e = cudaMemsetAsync(&work_.status->flags, 0, sizeof(uint32_t), st_);
    if (e == cudaSuccess) e = launch_factor(net_, fac_, work_, sched_, st_);
    if (e == cudaSuccess) e = cudaMemcpyAsync(work_.rhs, b.data(), sizeof(double) * P.n_state, cudaMemcpyHostToDevice, st_);
    if (e == cudaSuccess) e = launch_solve(fac_, work_, sched_, st_);
    std::vector<double> x(P.n_state);
    if (e == cudaSuccess) e = cudaMemcpyAsync(x.data(), work_.sol, sizeof(double) * P.n_state, cudaMemcpyDeviceToHost, st_);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h_status_, work_.status, sizeof(DevStatus), cudaMemcpyDeviceToHost, st_);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st_);
    if (e != cudaSuccess) return set_cuda_error(e, "factor/solve");
    for (int32_t p = 0; p < P.n_state; ++p) x_orig[P.state_of_ps[p]] = x[p];
    factor_valid_ = false;
    if (h_status_->flags & FLAG_TIMEOUT) {
        last_error = "factorisation dataflow wait timed out";
        return -3;
    }
    return (h_status_->flags & FLAG_SINGULAR) ? -7 : 0;
}

int32_t Engine::factor_and_solve_noalloc(const double* rhs_orig, double* x_orig) {
    const DeviceScope dev_scope(cfg.device_id);
    if (batch_mode()) {
        last_error = "not available on a batch handle";
        return -4;
    }
    if (!uploaded_) {
        last_error = "no model on the device (upload and evaluate first)";
        return -4;
    }
    if (mixed_) {
        last_error = "stage access needs the FP64 pipeline (use_double_precision = 1)";
        return -4;
    }
    const NoAllocShape sh{lay_u_size_, plan_.su_size, plan_.n_state, plan_.n_super};
    const size_t need = noalloc_scratch_need(sh);
    if (need > kNoAllocScratchBytes) {
        last_error = "allocation-free factor/solve needs " + std::to_string(need) + " bytes of scratch; the static limit is " +
                     std::to_string(kNoAllocScratchBytes) + " bytes";
        return -11;
    }
    cudaError_t e = cudaMemsetAsync(&work_.status->flags, 0, sizeof(uint32_t), st_);
    if (e == cudaSuccess) e = launch_factor_solve_noalloc(net_, fac_, work_, sched_, sh, rhs_orig, x_orig, st_);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h_status_, work_.status, sizeof(DevStatus), cudaMemcpyDeviceToHost, st_);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st_);
    if (e != cudaSuccess) return set_cuda_error(e, "allocation-free factor/solve");
    factor_valid_ = false;
    if (h_status_->flags & FLAG_TIMEOUT) {
        last_error = "factorisation dataflow wait timed out";
        return -3;
    }
    return (h_status_->flags & FLAG_SINGULAR) ? -7 : 0;
}

int32_t Engine::check_islands(int32_t* islands, int32_t* active_rows) {
    const DeviceScope dev_scope(cfg.device_id);
    if (!uploaded_) {
        last_error = "no model on the device";
        return -4;
    }
    cudaError_t e = launch_islands(net_, isl_parent_, isl_out_, 1000, st_);
    int32_t out[4] = {0, 0, 0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, isl_out_, sizeof(out), cudaMemcpyDeviceToHost, st_);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st_);
    if (e != cudaSuccess) return set_cuda_error(e, "islands");
    if (out[2] < 0) {
        last_error = "island labelling did not settle";
        return -3;
    }
    if (islands) *islands = out[0];
    if (active_rows) *active_rows = out[1];
    return 0;
}

int32_t Engine::max_solve_front() const {
    int32_t m = 0;
    for (int32_t f : plan_.sn_f) m = std::max(m, f);
    return m;
}

int32_t Engine::export_ybus(std::vector<double>& g, std::vector<double>& b) {
    const DeviceScope dev_scope(cfg.device_id);
    const size_t nnz = plan_.y_col.size();
    g.assign(nnz, 0.0);
    b.assign(nnz, 0.0);
    cudaError_t e = cudaMemcpyAsync(g.data(), net_.y_g, sizeof(double) * nnz, cudaMemcpyDeviceToHost, st_);
    if (e == cudaSuccess) e = cudaMemcpyAsync(b.data(), net_.y_b, sizeof(double) * nnz, cudaMemcpyDeviceToHost, st_);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st_);
    if (e != cudaSuccess) return set_cuda_error(e, "export ybus");
    return 0;
}

int32_t Engine::export_eval(double* hval, double* hx, double* rhs_orig) {
    const DeviceScope dev_scope(cfg.device_id);
    const Plan& P = plan_;
    std::vector<double> b(P.n_state);
    cudaError_t e = cudaSuccess;
    if (hval && !P.h_col.empty())
        e = cudaMemcpyAsync(hval, work_.hval, sizeof(double) * P.h_col.size(), cudaMemcpyDeviceToHost, st_);
    if (e == cudaSuccess && hx && P.n_meas > 0)
        e = cudaMemcpyAsync(hx, work_.h, sizeof(double) * P.n_meas, cudaMemcpyDeviceToHost, st_);
    if (e == cudaSuccess && rhs_orig)
        e = cudaMemcpyAsync(b.data(), work_.rhs, sizeof(double) * P.n_state, cudaMemcpyDeviceToHost, st_);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st_);
    if (e != cudaSuccess) return set_cuda_error(e, "export eval");
    if (rhs_orig)
        for (int32_t p = 0; p < P.n_state; ++p) rhs_orig[P.state_of_ps[p]] = b[p];
    return 0;
}

int32_t Engine::stage_telemetry(const double* z, int32_t count, int32_t slot) {
    const DeviceScope dev_scope(cfg.device_id);
    if (!uploaded_ || model.structure_dirty) {
        const int32_t rc = upload();
        if (rc) return rc;
    }
    const int32_t m = model.n_meas();
    if (count != m || slot < 0 || slot >= 4096) {
        last_error = "telemetry count or slot out of range";
        return -4;
    }
    if (slot >= n_slots_) {
        const int32_t ns = std::max(slot + 1, std::max(2 * n_slots_, 8));
        double* d = nullptr;
        cudaError_t e = cudaMalloc(&d, sizeof(double) * static_cast<size_t>(ns) * std::max(m, 1));
        if (e != cudaSuccess) return set_cuda_error(e, "telemetry slots");
        if (d_slots_) {
            cudaMemcpyAsync(d, d_slots_, sizeof(double) * static_cast<size_t>(n_slots_) * m, cudaMemcpyDeviceToDevice, st_);
            cudaStreamSynchronize(st_);
            cudaFree(d_slots_);
        }
        d_slots_ = d;
        n_slots_ = ns;
    }
    cudaError_t e = cudaMemcpyAsync(d_slots_ + static_cast<size_t>(slot) * m, z, sizeof(double) * m,
                                    cudaMemcpyHostToDevice, st_);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st_);
    if (e != cudaSuccess) return set_cuda_error(e, "stage telemetry");
    return 0;
}

int32_t Engine::use_telemetry(int32_t slot) {
    const DeviceScope dev_scope(cfg.device_id);
    if (slot < 0 || slot >= n_slots_ || !uploaded_) {
        last_error = "telemetry slot not staged";
        return -4;
    }
    const int32_t m = model.n_meas();
    cudaError_t e = cudaMemcpyAsync(work_.z, d_slots_ + static_cast<size_t>(slot) * m, sizeof(double) * m,
                                    cudaMemcpyDeviceToDevice, st_);
    if (e != cudaSuccess) return set_cuda_error(e, "use telemetry");
    model.values_dirty = false;
    return 0;
}

int32_t Engine::flush_l2(size_t bytes) {
    const DeviceScope dev_scope(cfg.device_id);
    int32_t rc = initialize();
    if (rc) return rc;
    if (bytes > scratch_bytes_) {
        if (d_scratch_) cudaFree(d_scratch_);
        d_scratch_ = nullptr;
        scratch_bytes_ = 0;
        cudaError_t e = cudaMalloc(&d_scratch_, bytes);
        if (e != cudaSuccess) return set_cuda_error(e, "l2 flush buffer");
        scratch_bytes_ = bytes;
    }
    static int salt = 0;
    cudaError_t e = cudaMemsetAsync(d_scratch_, (++salt) & 0xFF, bytes, st_);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st_);
    if (e != cudaSuccess) return set_cuda_error(e, "l2 flush");
    return 0;
}

int32_t Engine::timer(int32_t op, double* ms) {
    const DeviceScope dev_scope(cfg.device_id);
    int32_t rc = initialize();
    if (rc) return rc;
    if (!tm0_) {
        cudaEventCreate(&tm0_);
        cudaEventCreate(&tm1_);
    }
    if (op == 0) {
        cudaEventRecord(tm0_, st_);
        return 0;
    }
    cudaEventRecord(tm1_, st_);
    cudaError_t e = cudaEventSynchronize(tm1_);
    float f = 0.f;
    if (e == cudaSuccess) e = cudaEventElapsedTime(&f, tm0_, tm1_);
    if (e != cudaSuccess) return set_cuda_error(e, "timer");
    if (ms) *ms = f;
    return 0;
}


// ---------------------------------------------------------------------------
// Batch of independent grids
// ---------------------------------------------------------------------------
int32_t Engine::batch_add_grid(int32_t nb, const int32_t* btype, const double* vset, int32_t nbr, const int32_t* from,
                               const int32_t* to, const double* r, const double* x, const double* b,
                               const double* tap, const double* shift, const int32_t* status, int32_t nm,
                               const int32_t* mtype, const int32_t* mloc, const int32_t* mend, const double* sigma,
                               const double* z, int32_t* id) {
    if (nb <= 0 || nbr < 0 || nm < 0 || !btype || !vset || (nbr > 0 && (!from || !to || !r || !x || !b || !tap || !shift)) ||
        (nm > 0 && (!mtype || !mloc || !mend || !sigma || !z))) {
        last_error = "invalid grid arrays";
        return -4;
    }
    if (!batch_mode() && model.n_bus() > 0) {
        last_error = "the handle already holds a single-grid model";
        return -4;
    }
    int32_t slack = -1;
    for (int32_t i = 0; i < nb; ++i)
        if (btype[i] == 2) slack = i;  // the last SLACK, as for one grid
    if (slack < 0) {
        last_error = "grid has no slack bus";
        return -4;
    }
    for (int32_t k = 0; k < nbr; ++k)
        if (from[k] < 0 || from[k] >= nb || to[k] < 0 || to[k] >= nb) {
            last_error = "branch references an unknown bus";
            return -11;
        }
    for (int32_t q = 0; q < nm; ++q) {
        const int32_t ty = mtype[q];
        const bool on_branch = (ty == 4 || ty == 5 || ty == 6);
        if (ty < 0 || ty > 8 || mloc[q] < 0 || mloc[q] >= (on_branch ? nbr : nb)) {
            last_error = "measurement references an unknown element";
            return -11;
        }
    }
    GridSpan sp{model.n_bus(), nb, model.n_branch(), nbr, model.n_meas(), nm, model.n_bus() + slack};
    model.append_soa(nb, btype, vset, nbr, from, to, r, x, b, tap, shift, status, nm, mtype, mloc, mend, sigma, z);
    grids_.push_back(sp);
    analyzed_ = false;
    if (id) *id = static_cast<int32_t>(grids_.size()) - 1;
    return 0;
}

int32_t Engine::analyze_batch() {
    const HostTimer timer(&stats.analysis_ms);
    const int32_t G = static_cast<int32_t>(grids_.size());
    grid_plans_.assign(G, Plan());
    std::vector<std::string> errs(G);
    std::atomic<int32_t> next{0};
    auto work = [&]() {
        for (int32_t g = next++; g < G; g = next++) {
            const GridSpan& S = grids_[g];
            std::vector<int32_t> from(S.nbr), to(S.nbr), loc(S.nm);
            for (int32_t k = 0; k < S.nbr; ++k) {
                from[k] = model.br_from[S.br0 + k] - S.bus0;
                to[k] = model.br_to[S.br0 + k] - S.bus0;
            }
            for (int32_t q = 0; q < S.nm; ++q) {
                const int32_t ty = model.m_type[S.m0 + q];
                const bool on_branch = (ty == 4 || ty == 5 || ty == 6);
                loc[q] = model.m_loc[S.m0 + q] - (on_branch ? S.br0 : S.bus0);
            }
            // every branch is in the pattern: opening a breaker changes values only
            std::vector<uint8_t> all_closed(S.nbr, 1);
            Topology t;
            t.n_bus = S.nbus;
            t.n_branch = S.nbr;
            t.n_meas = S.nm;
            t.slack = S.slack - S.bus0;
            t.br_from = from.data();
            t.br_to = to.data();
            t.br_closed = all_closed.data();
            t.m_type = model.m_type.data() + S.m0;
            t.m_loc = loc.data();
            t.m_end = model.m_end.data() + S.m0;
            t.m_active = model.m_active.data() + S.m0;
            SymbolicParams prm;
            prm.ordering = cfg.ordering;
            if (!build_plan(t, prm, grid_plans_[g], errs[g])) errs[g] = "grid " + std::to_string(g) + ": " + errs[g];
        }
    };
    const int32_t nt = std::max(1, std::min<int32_t>(G, static_cast<int32_t>(std::thread::hardware_concurrency())));
    std::vector<std::thread> pool;
    for (int32_t i = 1; i < nt; ++i) pool.emplace_back(work);
    work();
    for (auto& th : pool) th.join();
    for (int32_t g = 0; g < G; ++g)
        if (!errs[g].empty()) {
            last_error = "symbolic analysis: " + errs[g];
            analyzed_ = false;
            return -5;
        }
    std::vector<const Plan*> parts(G);
    std::vector<int32_t> brc(G);
    for (int32_t g = 0; g < G; ++g) {
        parts[g] = &grid_plans_[g];
        brc[g] = grids_[g].nbr;
    }
    merge_plans(parts, brc, plan_);
    analyzed_ = true;
    return 0;
}

int32_t Engine::batch_solve(int32_t n, const int32_t* ids, const uint8_t* flat, const SolveRequest& rq,
                            GridResult* out) {
    const DeviceScope dev_scope(cfg.device_id);
    if (!batch_mode()) {
        last_error = "no batch grids";
        return -4;
    }
    const int32_t G = static_cast<int32_t>(grids_.size());
    for (int32_t i = 0; i < n; ++i)
        if (!ids || ids[i] < 0 || ids[i] >= G) {
            last_error = "grid index out of range";
            return -4;
        }
    if (!init_ || !uploaded_ || model.structure_dirty) {
        const int32_t rc = upload();
        if (rc) return rc;
    }
    if (model.values_dirty) {
        const int32_t rc = sync_measurements();
        if (rc) return rc;
    }
    const SolveParams sp = params(rq);
    std::memset(h_batch_in_, 0, 2 * static_cast<size_t>(G));
    for (int32_t i = 0; i < n; ++i) {
        h_batch_in_[ids[i]] = 1;
        h_batch_in_[G + ids[i]] = (flat && flat[i]) ? 1 : 0;
    }
    cudaError_t e = cudaMemcpyAsync(const_cast<uint8_t*>(batch_.active), h_batch_in_, 2 * static_cast<size_t>(G),
                                    cudaMemcpyHostToDevice, st_);  // active and flat are adjacent in the arena
    if (e != cudaSuccess) return set_cuda_error(e, "batch inputs");
    cudaEventRecord(ev0_, st_);
    e = launch_batch_begin(net_, work_, batch_, st_);
    if (e != cudaSuccess) return set_cuda_error(e, "batch begin");
    char* ob = static_cast<char*>(h_batch_out_);
    uint32_t* h_flags = reinterpret_cast<uint32_t*>(ob);
    int32_t* h_iters = reinterpret_cast<int32_t*>(ob + 4 * static_cast<size_t>(G));
    double* h_mis = reinterpret_cast<double*>(ob + 8 * static_cast<size_t>(G));
    double* h_obj = reinterpret_cast<double*>(ob + 16 * static_cast<size_t>(G));
    int32_t* h_running = reinterpret_cast<int32_t*>(ob + 24 * static_cast<size_t>(G));
    int32_t steps = 0;
    const int32_t lrc = rq.max_iterations > 0 ? run_device_loop(sp, rq.max_iterations, steps) : 0;
    if (lrc != 0 && lrc != -1) return -3;
    for (int32_t it = 0; lrc == -1 && it < rq.max_iterations; ++it) {
        if (run_iteration(sp, true) != 0) return -3;
        if (h_status_->flags & FLAG_TIMEOUT) {
            last_error = "factorisation dataflow wait timed out";
            return -3;
        }
        if (*h_running == 0) break;
    }
    SolveParams spf = sp;
    spf.skip_flags = FLAG_INACTIVE;  // converged grids need their final residuals
    e = launch_evaluate(net_, work_, spf, st_);
    if (e == cudaSuccess) e = launch_batch_objective(net_, work_, batch_, 0u, st_);
    cudaEventRecord(ev1_, st_);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h_flags, batch_.flags, 4 * static_cast<size_t>(G), cudaMemcpyDeviceToHost, st_);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h_iters, batch_.iters, 4 * static_cast<size_t>(G), cudaMemcpyDeviceToHost, st_);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h_mis, batch_.mismatch, 8 * static_cast<size_t>(G), cudaMemcpyDeviceToHost, st_);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h_obj, batch_.objective, 8 * static_cast<size_t>(G), cudaMemcpyDeviceToHost, st_);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st_);
    if (e != cudaSuccess) return set_cuda_error(e, "batch solve");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ev0_, ev1_);
    last_.time_ms = ms;
    collect_stage_times();
    for (int32_t i = 0; i < n; ++i) {
        const int32_t g = ids[i];
        const uint32_t fl = h_flags[g];
        GridResult r;
        r.status = (fl & FLAG_SINGULAR) ? CONV_SINGULAR
                   : (fl & FLAG_NONFINITE) ? CONV_DIVERGED
                   : (fl & FLAG_CONVERGED) ? CONV_OK
                                           : CONV_MAXIT;
        r.iterations = h_iters[g];
        r.max_mismatch = h_mis[g];
        r.objective = h_obj[g];
        if (out) out[i] = r;
    }
    stale_ = DL_ALL;
    ++stats.solves;
    return 0;
}

int32_t Engine::batch_set_telemetry(int32_t grid, const double* z, int32_t count) {
    const DeviceScope dev_scope(cfg.device_id);
    if (grid < 0 || grid >= static_cast<int32_t>(grids_.size()) || !z) {
        last_error = "grid index out of range";
        return -4;
    }
    const GridSpan& S = grids_[grid];
    if (count != S.nm) {
        last_error = "telemetry count does not match the grid's measurement count";
        return -4;
    }
    std::memcpy(model.m_value.data() + S.m0, z, sizeof(double) * count);
    if (!uploaded_ || model.structure_dirty || count == 0) {
        model.values_dirty = true;
        return 0;
    }
    cudaError_t e;
    if (h_stage_ && h_stage_n_ >= static_cast<size_t>(S.m0 + count)) {
        // this grid's slice of the pinned staging buffer; the copy is ordered
        // before the next solve on the engine stream
        e = cudaStreamSynchronize(st_);
        if (e == cudaSuccess) {
            std::memcpy(h_stage_ + S.m0, z, sizeof(double) * count);
            e = cudaMemcpyAsync(work_.z + S.m0, h_stage_ + S.m0, sizeof(double) * count, cudaMemcpyHostToDevice, st_);
        }
    } else {
        e = cudaMemcpy(work_.z + S.m0, z, sizeof(double) * count, cudaMemcpyHostToDevice);
    }
    if (e != cudaSuccess) return set_cuda_error(e, "telemetry");
    return 0;
}

int32_t Engine::batch_get_state(int32_t grid, double* v, double* th) {
    const DeviceScope dev_scope(cfg.device_id);
    if (grid < 0 || grid >= static_cast<int32_t>(grids_.size())) {
        last_error = "grid index out of range";
        return -4;
    }
    const GridSpan& S = grids_[grid];
    if (!uploaded_) {
        if (v) std::memcpy(v, model.bus_v.data() + S.bus0, sizeof(double) * S.nbus);
        if (th) std::memcpy(th, model.bus_th.data() + S.bus0, sizeof(double) * S.nbus);
        return 0;
    }
    cudaError_t e = cudaSuccess;
    if (v) e = cudaMemcpyAsync(v, work_.v + S.bus0, sizeof(double) * S.nbus, cudaMemcpyDeviceToHost, st_);
    if (th && e == cudaSuccess) e = cudaMemcpyAsync(th, work_.th + S.bus0, sizeof(double) * S.nbus, cudaMemcpyDeviceToHost, st_);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st_);
    if (e != cudaSuccess) return set_cuda_error(e, "batch state");
    return 0;
}

int32_t Engine::batch_set_branch_status(int32_t grid, int32_t branch, int32_t closed) {
    const DeviceScope dev_scope(cfg.device_id);
    if (grid < 0 || grid >= static_cast<int32_t>(grids_.size())) {
        last_error = "grid index out of range";
        return -4;
    }
    const GridSpan& S = grids_[grid];
    if (branch < 0 || branch >= S.nbr) {
        last_error = "branch index out of range";
        return -11;
    }
    const int32_t k = S.br0 + branch;
    model.br_closed[k] = closed ? 1 : 0;
    if (!uploaded_ || model.structure_dirty) return 0;
    // value-only topology change: every branch is in the batch pattern
    cudaError_t e = cudaMemcpyAsync(const_cast<uint8_t*>(net_.br_closed) + k, &model.br_closed[k], 1,
                                    cudaMemcpyHostToDevice, st_);
    if (e == cudaSuccess) e = launch_admittance_and_ybus(net_, st_);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st_);
    if (e != cudaSuccess) return set_cuda_error(e, "breaker edit");
    return 0;
}


// ---------------------------------------------------------------------------
// Stream mode: grids join and leave the running batch between iterations.
// ---------------------------------------------------------------------------
int32_t Engine::stream_begin(const SolveRequest& rq) {
    const DeviceScope dev_scope(cfg.device_id);
    if (!batch_mode()) {
        last_error = "no batch grids";
        return -4;
    }
    if (!init_ || !uploaded_ || model.structure_dirty) {
        const int32_t rc = upload();
        if (rc) return rc;
    }
    if (model.values_dirty) {
        const int32_t rc = sync_measurements();
        if (rc) return rc;
    }
    stream_rq_ = rq;
    const int32_t G = static_cast<int32_t>(grids_.size());
    in_flight_.assign(G, 0);
    stream_iters_.assign(G, 0);
    std::memset(h_batch_in_, 0, 3 * static_cast<size_t>(G));
    // every grid starts out of the batch
    cudaError_t e = cudaMemcpyAsync(const_cast<uint8_t*>(batch_.active), h_batch_in_, 3 * static_cast<size_t>(G),
                                    cudaMemcpyHostToDevice, st_);
    if (e == cudaSuccess) e = launch_batch_begin(net_, work_, batch_, st_);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st_);
    if (e != cudaSuccess) return set_cuda_error(e, "stream begin");
    return 0;
}

int32_t Engine::stream_activate(int32_t n, const int32_t* ids, const uint8_t* flat) {
    const DeviceScope dev_scope(cfg.device_id);
    const int32_t G = static_cast<int32_t>(grids_.size());
    if (n <= 0) return 0;
    std::memset(h_batch_in_, 0, 3 * static_cast<size_t>(G));
    for (int32_t i = 0; i < n; ++i) {
        const int32_t g = ids[i];
        if (g < 0 || g >= G || in_flight_[g]) {
            last_error = "grid index out of range or already in the batch";
            return -4;
        }
        h_batch_in_[g] = 1;
        h_batch_in_[G + g] = (flat && flat[i]) ? 1 : 0;
        in_flight_[g] = 1;
        stream_iters_[g] = 0;
    }
    cudaError_t e = cudaMemcpyAsync(const_cast<uint8_t*>(batch_.active), h_batch_in_, 2 * static_cast<size_t>(G),
                                    cudaMemcpyHostToDevice, st_);
    if (e == cudaSuccess) e = launch_batch_activate(net_, work_, batch_, st_);
    if (e != cudaSuccess) return set_cuda_error(e, "stream activate");
    return 0;
}

int32_t Engine::stream_step(std::vector<int32_t>& done, std::vector<GridResult>& res) {
    const DeviceScope dev_scope(cfg.device_id);
    done.clear();
    res.clear();
    const int32_t G = static_cast<int32_t>(grids_.size());
    bool any = false;
    for (int32_t g = 0; g < G && !any; ++g) any = in_flight_[g] != 0;
    if (!any) return 0;
    const SolveParams sp = params(stream_rq_);
    if (run_iteration(sp, true) != 0) return -3;
    if (h_status_->flags & FLAG_TIMEOUT) {
        last_error = "factorisation dataflow wait timed out";
        return -3;
    }
    char* ob = static_cast<char*>(h_batch_out_);
    uint32_t* h_flags = reinterpret_cast<uint32_t*>(ob);
    int32_t* h_iters = reinterpret_cast<int32_t*>(ob + 4 * static_cast<size_t>(G));
    double* h_mis = reinterpret_cast<double*>(ob + 8 * static_cast<size_t>(G));
    double* h_obj = reinterpret_cast<double*>(ob + 16 * static_cast<size_t>(G));
    cudaError_t e = cudaMemcpyAsync(h_flags, batch_.flags, 4 * static_cast<size_t>(G), cudaMemcpyDeviceToHost, st_);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h_iters, batch_.iters, 4 * static_cast<size_t>(G), cudaMemcpyDeviceToHost, st_);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h_mis, batch_.mismatch, 8 * static_cast<size_t>(G), cudaMemcpyDeviceToHost, st_);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st_);
    if (e != cudaSuccess) return set_cuda_error(e, "stream step");
    collect_stage_times();
    for (int32_t g = 0; g < G; ++g) {
        if (!in_flight_[g]) continue;
        ++stream_iters_[g];
        if ((h_flags[g] & FLAG_FROZEN) || stream_iters_[g] >= stream_rq_.max_iterations) done.push_back(g);
    }
    if (done.empty()) return 0;
    // final evaluation and objective of the finished grids only (marked
    // FLAG_FINAL); then they leave the batch
    std::memset(h_batch_in_ + 2 * static_cast<size_t>(G), 0, G);
    for (int32_t g : done) h_batch_in_[2 * static_cast<size_t>(G) + g] = 1;
    SolveParams spf = sp;
    spf.skip_flags = FLAG_INACTIVE;
    spf.need_flags = FLAG_FINAL;
    e = cudaMemcpyAsync(const_cast<uint8_t*>(batch_.retire), h_batch_in_ + 2 * static_cast<size_t>(G), G,
                        cudaMemcpyHostToDevice, st_);
    if (e == cudaSuccess) e = launch_batch_mark_final(batch_, st_);
    if (e == cudaSuccess) e = launch_evaluate(net_, work_, spf, st_);
    if (e == cudaSuccess) e = launch_batch_objective(net_, work_, batch_, FLAG_FINAL, st_);
    if (e == cudaSuccess) e = launch_batch_retire(batch_, st_);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h_obj, batch_.objective, 8 * static_cast<size_t>(G), cudaMemcpyDeviceToHost, st_);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st_);
    if (e != cudaSuccess) return set_cuda_error(e, "stream retire");
    for (int32_t g : done) {
        const uint32_t fl = h_flags[g];
        GridResult r;
        r.status = (fl & FLAG_SINGULAR) ? CONV_SINGULAR
                   : (fl & FLAG_NONFINITE) ? CONV_DIVERGED
                   : (fl & FLAG_CONVERGED) ? CONV_OK
                                           : CONV_MAXIT;
        r.iterations = h_iters[g];
        r.max_mismatch = h_mis[g];
        r.objective = h_obj[g];
        res.push_back(r);
        in_flight_[g] = 0;
    }
    stale_ = DL_ALL;
    return 0;
}

bool Engine::stream_in_flight(int32_t grid) const {
    return grid >= 0 && grid < static_cast<int32_t>(in_flight_.size()) && in_flight_[grid] != 0;
}

}  // namespace sle_gb300
