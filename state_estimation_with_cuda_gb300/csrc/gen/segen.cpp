// Deterministic synthetic power-grid generator (see segen.h for the contract).
#include "segen.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <queue>
#include <unordered_set>
#include <vector>

namespace {

constexpr double kPi = 3.14159265358979323846;
constexpr double kEps = 1e-12;

uint64_t splitmix64(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

struct Rng {
    uint64_t s[4];
    explicit Rng(uint64_t seed) {
        uint64_t x = seed;
        for (auto& v : s) v = splitmix64(x);
    }
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t next() {
        const uint64_t result = rotl(s[1] * 5, 7) * 9;
        const uint64_t t = s[1] << 17;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return result;
    }
    double uniform() { return static_cast<double>(next() >> 11) * 0x1.0p-53; }
    double uniform(double lo, double hi) { return lo + (hi - lo) * uniform(); }
    // Unbiased integer in [0, n) by rejection on the top bits.
    uint64_t below(uint64_t n) {
        if (n <= 1) return 0;
        const uint64_t lim = UINT64_MAX - (UINT64_MAX % n);
        uint64_t v;
        do { v = next(); } while (v >= lim);
        return v % n;
    }
    double normal() {
        const double u1 = 1.0 - uniform();  // (0, 1]
        const double u2 = uniform();
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(2.0 * kPi * u2);
    }
};

uint64_t mix_seed(uint64_t a, uint64_t b) {
    uint64_t s = a ^ (b * 0x9E3779B97F4A7C15ULL);
    return splitmix64(s);
}

// Uniform grid spatial index over [0,1]^2 for k-nearest-neighbour queries.
struct SpatialGrid {
    int cells;
    std::vector<std::vector<int32_t>> bucket;
    const std::vector<double>* px;
    const std::vector<double>* py;
    SpatialGrid(int n, const std::vector<double>& x, const std::vector<double>& y)
        : px(&x), py(&y) {
        cells = std::max(1, static_cast<int>(std::sqrt(static_cast<double>(n) / 2.0)));
        bucket.assign(static_cast<size_t>(cells) * cells, {});
    }
    int cell_of(double v) const {
        int c = static_cast<int>(v * cells);
        return std::min(std::max(c, 0), cells - 1);
    }
    void insert(int32_t i) {
        bucket[static_cast<size_t>(cell_of((*py)[i])) * cells + cell_of((*px)[i])].push_back(i);
    }
    // k nearest inserted points to point q (excluding q), sorted by (distance, index).
    std::vector<int32_t> knn(int32_t q, int k) const {
        const double qx = (*px)[q], qy = (*py)[q];
        const int cx = cell_of(qx), cy = cell_of(qy);
        std::vector<std::pair<double, int32_t>> cand;
        for (int ring = 0; ring <= cells; ++ring) {
            for (int dy = -ring; dy <= ring; ++dy) {
                for (int dx = -ring; dx <= ring; ++dx) {
                    if (std::max(std::abs(dx), std::abs(dy)) != ring) continue;
                    const int X = cx + dx, Y = cy + dy;
                    if (X < 0 || Y < 0 || X >= cells || Y >= cells) continue;
                    for (int32_t j : bucket[static_cast<size_t>(Y) * cells + X]) {
                        if (j == q) continue;
                        const double ddx = (*px)[j] - qx, ddy = (*py)[j] - qy;
                        cand.emplace_back(ddx * ddx + ddy * ddy, j);
                    }
                }
            }
            if (static_cast<int>(cand.size()) >= k) {
                // Every point outside the scanned square is at least ring/cells away.
                std::sort(cand.begin(), cand.end());
                const double reach = static_cast<double>(ring) / cells;
                if (cand[k - 1].first <= reach * reach) break;
            }
        }
        std::sort(cand.begin(), cand.end());
        std::vector<int32_t> out;
        for (int t = 0; t < static_cast<int>(cand.size()) && t < k; ++t) out.push_back(cand[t].second);
        return out;
    }
};

}  // namespace

struct SEGrid {
    SEGenParams p{};
    int32_t n = 0, nbr = 0, m = 0, slack = 0;
    std::vector<int32_t> bus_type;
    std::vector<double> v_set, v_true, th_true;
    std::vector<int32_t> from, to, status;
    std::vector<double> r, x, b, tap, shift;
    std::vector<int32_t> mtype, mloc, mend, gross;
    std::vector<double> sigma, z, htrue;
};

namespace {

// h(x) of the SLE measurement model at (V, theta), FP64.
void eval_h(const SEGrid& g, const std::vector<double>& V, const std::vector<double>& th,
            std::vector<double>& h) {
    const int32_t n = g.n;
    std::vector<double> P(n, 0.0), Q(n, 0.0);
    std::vector<double> pf(g.nbr), qf(g.nbr), pt(g.nbr), qt(g.nbr);
    // Injections through Ybus, accumulated branch by branch.
    std::vector<double> Gii(n, 0.0), Bii(n, 0.0);
    for (int32_t k = 0; k < g.nbr; ++k) {
        if (!g.status[k]) continue;
        const int32_t i = g.from[k], j = g.to[k];
        double den = g.r[k] * g.r[k] + g.x[k] * g.x[k];
        if (den < kEps) den = kEps;
        const double gs = g.r[k] / den, bs = -g.x[k] / den;
        const double bsf = g.b[k] / (2.0 * g.tap[k] * g.tap[k]);
        const double bst = g.b[k] / 2.0;
        const double a = std::max(g.tap[k], kEps);
        const double cph = std::cos(g.shift[k]), sph = std::sin(g.shift[k]);
        const double yij_g = -(gs * cph + bs * sph) / a, yij_b = -(-gs * sph + bs * cph) / a;
        const double yji_g = -(gs * cph - bs * sph) / a, yji_b = -(gs * sph + bs * cph) / a;
        Gii[i] += gs / (a * a);
        Bii[i] += bs / (a * a) + bsf;
        Gii[j] += gs;
        Bii[j] += bs + bst;
        {
            const double t = th[i] - th[j];
            const double c = std::cos(t), s = std::sin(t);
            P[i] += V[i] * V[j] * (yij_g * c + yij_b * s);
            Q[i] += V[i] * V[j] * (yij_g * s - yij_b * c);
        }
        {
            const double t = th[j] - th[i];
            const double c = std::cos(t), s = std::sin(t);
            P[j] += V[j] * V[i] * (yji_g * c + yji_b * s);
            Q[j] += V[j] * V[i] * (yji_g * s - yji_b * c);
        }
    }
    for (int32_t i = 0; i < n; ++i) {
        P[i] += V[i] * V[i] * Gii[i];
        Q[i] -= V[i] * V[i] * Bii[i];
    }
    for (int32_t k = 0; k < g.nbr; ++k) {
        const int32_t i = g.from[k], j = g.to[k];
        double den = g.r[k] * g.r[k] + g.x[k] * g.x[k];
        if (den < kEps) den = kEps;
        const double gs = g.r[k] / den, bs = -g.x[k] / den;
        const double bsf = g.b[k] / (2.0 * g.tap[k] * g.tap[k]);
        const double bst = g.b[k] / 2.0;
        const double a = std::max(g.tap[k], kEps);
        const double t = th[i] - th[j] - g.shift[k];
        const double c = std::cos(t), s = std::sin(t);
        const double vv = V[i] * V[j] / a;
        const double on = g.status[k] ? 1.0 : 0.0;
        pf[k] = on * (V[i] * V[i] / (a * a) * gs - vv * (gs * c + bs * s));
        qf[k] = on * (-(V[i] * V[i] / (a * a)) * (bs + bsf) - vv * (gs * s - bs * c));
        pt[k] = on * (V[j] * V[j] * gs - vv * (gs * c - bs * s));
        qt[k] = on * (-(V[j] * V[j]) * (bs + bst) + vv * (gs * s + bs * c));
    }
    h.assign(g.m, 0.0);
    for (int32_t q = 0; q < g.m; ++q) {
        const int32_t loc = g.mloc[q];
        const bool to_end = g.mend[q] != 0;
        switch (g.mtype[q]) {
            case 0: h[q] = V[loc]; break;
            case 1: h[q] = th[loc]; break;
            case 2: case 7: h[q] = P[loc]; break;
            case 3: case 8: h[q] = Q[loc]; break;
            case 4: h[q] = to_end ? pt[loc] : pf[loc]; break;
            case 5: h[q] = to_end ? qt[loc] : qf[loc]; break;
            case 6: {
                const double pp = to_end ? pt[loc] : pf[loc];
                const double qq = to_end ? qt[loc] : qf[loc];
                const double vv = std::max(V[to_end ? g.to[loc] : g.from[loc]], kEps);
                h[q] = std::sqrt(pp * pp + qq * qq) / vv * (g.status[loc] ? 1.0 : 0.0);
                break;
            }
            default: h[q] = 0.0;
        }
    }
}

std::vector<int32_t> sample_sorted(Rng& rng, int32_t pool, int32_t k) {
    k = std::max(0, std::min(k, pool));
    std::vector<int32_t> idx(pool);
    for (int32_t i = 0; i < pool; ++i) idx[i] = i;
    for (int32_t i = 0; i < k; ++i) {
        const int32_t j = i + static_cast<int32_t>(rng.below(static_cast<uint64_t>(pool - i)));
        std::swap(idx[i], idx[j]);
    }
    idx.resize(k);
    std::sort(idx.begin(), idx.end());
    return idx;
}

bool connected_without(const SEGrid& g, int32_t skip) {
    std::vector<std::vector<int32_t>> adj(g.n);
    for (int32_t k = 0; k < g.nbr; ++k) {
        if (k == skip || !g.status[k]) continue;
        adj[g.from[k]].push_back(g.to[k]);
        adj[g.to[k]].push_back(g.from[k]);
    }
    std::vector<char> seen(g.n, 0);
    std::vector<int32_t> stack{0};
    seen[0] = 1;
    int32_t cnt = 1;
    while (!stack.empty()) {
        const int32_t u = stack.back();
        stack.pop_back();
        for (int32_t v : adj[u]) {
            if (!seen[v]) { seen[v] = 1; ++cnt; stack.push_back(v); }
        }
    }
    return cnt == g.n;
}

}  // namespace

extern "C" {

void segen_default_params(SEGenParams* p, int32_t n_bus, int32_t n_branch, uint64_t seed) {
    std::memset(p, 0, sizeof(*p));
    p->n_bus = n_bus;
    p->n_branch = n_branch;
    p->seed = seed;
    p->frac_vmag = 0.30;
    p->frac_inj = 0.60;
    p->frac_flow = 0.70;
    p->n_vmag = p->n_inj = p->n_flow = -1;
    p->n_tap = -1;
    p->sigma_v = 0.004;
    p->sigma_inj = 0.010;
    p->sigma_flow = 0.008;
    p->gross_frac = 0.0;
    p->sigma_pseudo = 0.05;
}

SEGrid* segen_create(const SEGenParams* p) {
    if (!p || p->n_bus < 2 || p->n_branch < p->n_bus - 1) return nullptr;
    auto* g = new SEGrid();
    g->p = *p;
    const int32_t n = p->n_bus, nbr = p->n_branch;
    g->n = n;
    g->nbr = nbr;
    g->slack = 0;

    // --- topology -----------------------------------------------------------
    Rng rng_topo(mix_seed(p->seed, 1));
    std::vector<double> px(n), py(n);
    for (int32_t i = 0; i < n; ++i) {
        px[i] = rng_topo.uniform();
        py[i] = rng_topo.uniform();
    }
    SpatialGrid grid(n, px, py);
    std::unordered_set<uint64_t> edges;
    auto key = [](int32_t a, int32_t b) {
        const uint32_t lo = static_cast<uint32_t>(std::min(a, b));
        const uint32_t hi = static_cast<uint32_t>(std::max(a, b));
        return (static_cast<uint64_t>(lo) << 32) | hi;
    };
    grid.insert(0);
    for (int32_t k = 1; k < n; ++k) {
        std::vector<int32_t> nb = grid.knn(k, 8);  // only earlier buses are inserted
        const int32_t par = nb[rng_topo.below(nb.size())];
        g->from.push_back(par);
        g->to.push_back(k);
        edges.insert(key(par, k));
        grid.insert(k);
    }
    // Chords between k-NN pairs (k = 8) over all buses.
    std::vector<std::vector<int32_t>> knn_all(n);
    for (int32_t i = 0; i < n; ++i) knn_all[i] = grid.knn(i, 8);
    int64_t attempts = 0;
    while (static_cast<int32_t>(g->from.size()) < nbr) {
        int32_t u, v;
        if (attempts < 64LL * nbr + 1024) {
            u = static_cast<int32_t>(rng_topo.below(n));
            const auto& nb = knn_all[u];
            v = nb[rng_topo.below(nb.size())];
        } else {  // k-NN pairs exhausted (tiny grids): any pair
            u = static_cast<int32_t>(rng_topo.below(n));
            v = static_cast<int32_t>(rng_topo.below(n));
        }
        ++attempts;
        if (u == v || edges.count(key(u, v))) {
            if (attempts > 1024LL * nbr + 100000) break;
            continue;
        }
        edges.insert(key(u, v));
        g->from.push_back(u);
        g->to.push_back(v);
    }
    g->nbr = static_cast<int32_t>(g->from.size());

    // --- branch parameters --------------------------------------------------
    Rng rng_par(mix_seed(p->seed, 2));
    g->r.resize(g->nbr);
    g->x.resize(g->nbr);
    g->b.resize(g->nbr);
    g->tap.assign(g->nbr, 1.0);
    g->shift.assign(g->nbr, 0.0);
    g->status.assign(g->nbr, 1);
    for (int32_t k = 0; k < g->nbr; ++k) {
        g->r[k] = rng_par.uniform(0.01, 0.08);
        g->x[k] = g->r[k] * rng_par.uniform(3.0, 8.0);
        g->b[k] = rng_par.uniform(0.0, 0.06);
    }
    const int32_t ntap = p->n_tap >= 0 ? p->n_tap : (3 * g->nbr) / 20;
    for (int32_t k : sample_sorted(rng_par, g->nbr, ntap)) g->tap[k] = rng_par.uniform(0.95, 1.05);

    // --- buses and true state -----------------------------------------------
    g->bus_type.assign(n, 0);
    g->bus_type[0] = 2;
    g->v_set.assign(n, 1.0);
    Rng rng_state(mix_seed(p->seed, 3));
    g->v_true.resize(n);
    for (int32_t i = 0; i < n; ++i) g->v_true[i] = rng_state.uniform(0.97, 1.06);
    g->th_true.assign(n, 0.0);
    {
        std::vector<std::vector<int32_t>> adj(n);
        for (int32_t k = 0; k < g->nbr; ++k) {
            adj[g->from[k]].push_back(g->to[k]);
            adj[g->to[k]].push_back(g->from[k]);
        }
        std::vector<char> seen(n, 0);
        std::queue<int32_t> q;
        q.push(0);
        seen[0] = 1;
        const double rho = 0.9, innov = std::sqrt(1.0 - rho * rho) * 0.08;
        while (!q.empty()) {
            const int32_t u = q.front();
            q.pop();
            for (int32_t v : adj[u]) {
                if (seen[v]) continue;
                seen[v] = 1;
                g->th_true[v] = rho * g->th_true[u] + innov * rng_state.normal();
                q.push(v);
            }
        }
    }

    // --- measurements ---------------------------------------------------------
    Rng rng_meas(mix_seed(p->seed, 4));
    const int32_t nv = p->n_vmag >= 0 ? p->n_vmag : static_cast<int32_t>(std::lround(p->frac_vmag * n));
    const int32_t ni = p->n_inj >= 0 ? p->n_inj : static_cast<int32_t>(std::lround(p->frac_inj * n));
    const int32_t nf = p->n_flow >= 0 ? p->n_flow : static_cast<int32_t>(std::lround(p->frac_flow * g->nbr));
    auto add = [&](int32_t type, int32_t loc, int32_t end, double sig) {
        g->mtype.push_back(type);
        g->mloc.push_back(loc);
        g->mend.push_back(end);
        g->sigma.push_back(sig);
    };
    for (int32_t i : sample_sorted(rng_meas, n, nv)) add(0, i, 0, p->sigma_v);
    for (int32_t i : sample_sorted(rng_meas, n, ni)) {
        add(2, i, 0, p->sigma_inj);
        add(3, i, 0, p->sigma_inj);
    }
    for (int32_t k : sample_sorted(rng_meas, g->nbr, nf)) {
        add(4, k, 0, p->sigma_flow);
        add(5, k, 0, p->sigma_flow);
        add(4, k, 1, p->sigma_flow);
        add(5, k, 1, p->sigma_flow);
    }
    const int32_t m_tele = static_cast<int32_t>(g->mtype.size());  // telemetry rows (before pseudo rows)
    // Observability restoration (topological observability: a spanning tree
    // whose branches each carry a distinct measurement).  Flow-measured
    // branches join their ends; each injection-measured bus then joins one
    // incident branch still crossing components (lowest branch index); every
    // branch that still crosses components gets a from-end P+Q flow pair with
    // the pseudo-measurement sigma.  These rows are appended after the mix.
    {
        std::vector<int32_t> uf(n);
        for (int32_t i = 0; i < n; ++i) uf[i] = i;
        auto find = [&](int32_t x) {
            while (uf[x] != x) x = uf[x] = uf[uf[x]];
            return x;
        };
        std::vector<std::vector<int32_t>> inc(n);
        for (int32_t k = 0; k < g->nbr; ++k) {
            inc[g->from[k]].push_back(k);
            inc[g->to[k]].push_back(k);
        }
        std::vector<char> has_inj(n, 0);
        for (size_t q = 0; q < g->mtype.size(); ++q) {
            const int32_t ty = g->mtype[q], loc = g->mloc[q];
            if (ty == 4) {
                const int32_t a = find(g->from[loc]), b = find(g->to[loc]);
                if (a != b) uf[a] = b;
            } else if (ty == 2) {
                has_inj[loc] = 1;
            }
        }
        for (int32_t i = 0; i < n; ++i) {
            if (!has_inj[i]) continue;
            for (int32_t k : inc[i]) {
                const int32_t a = find(g->from[k]), b = find(g->to[k]);
                if (a != b) {
                    uf[a] = b;
                    break;
                }
            }
        }
        for (int32_t k = 0; k < g->nbr; ++k) {
            const int32_t a = find(g->from[k]), b = find(g->to[k]);
            if (a == b) continue;
            uf[a] = b;
            add(4, k, 0, p->sigma_pseudo);
            add(5, k, 0, p->sigma_pseudo);
        }
    }
    g->m = static_cast<int32_t>(g->mtype.size());
    eval_h(*g, g->v_true, g->th_true, g->htrue);
    Rng rng_noise(mix_seed(p->seed, 5));
    g->z.resize(g->m);
    for (int32_t q = 0; q < g->m; ++q) g->z[q] = g->htrue[q] + g->sigma[q] * rng_noise.normal();
    g->gross.assign(g->m, 0);
    // Gross errors model telemetry failures: they hit a seeded fraction of the
    // telemetry rows only, never the pseudo-measurements that restore
    // observability (a +-30 sigma error on a pseudo flow, sigma 0.05, is a
    // 1.5 pu error on the only row covering a leaf and drives |V| into the
    // clamp, so the iteration cannot converge).
    if (p->gross_frac > 0.0) {
        Rng rng_gross(mix_seed(p->seed, 6));
        const int32_t ng = static_cast<int32_t>(std::lround(p->gross_frac * m_tele));
        for (int32_t q : sample_sorted(rng_gross, m_tele, ng)) {
            const double mag = 10.0 + 20.0 * rng_gross.uniform();
            const double sgn = (rng_gross.next() >> 63) ? -1.0 : 1.0;
            g->z[q] += sgn * mag * g->sigma[q];
            g->gross[q] = 1;
        }
    }
    return g;
}

void segen_destroy(SEGrid* g) { delete g; }

int32_t segen_n_bus(const SEGrid* g) { return g->n; }
int32_t segen_n_branch(const SEGrid* g) { return g->nbr; }
int32_t segen_n_meas(const SEGrid* g) { return g->m; }
int32_t segen_slack(const SEGrid* g) { return g->slack; }
const int32_t* segen_bus_type(const SEGrid* g) { return g->bus_type.data(); }
const double* segen_v_setpoint(const SEGrid* g) { return g->v_set.data(); }
const double* segen_v_true(const SEGrid* g) { return g->v_true.data(); }
const double* segen_theta_true(const SEGrid* g) { return g->th_true.data(); }
const int32_t* segen_br_from(const SEGrid* g) { return g->from.data(); }
const int32_t* segen_br_to(const SEGrid* g) { return g->to.data(); }
const double* segen_br_r(const SEGrid* g) { return g->r.data(); }
const double* segen_br_x(const SEGrid* g) { return g->x.data(); }
const double* segen_br_b(const SEGrid* g) { return g->b.data(); }
const double* segen_br_tap(const SEGrid* g) { return g->tap.data(); }
const double* segen_br_shift(const SEGrid* g) { return g->shift.data(); }
const int32_t* segen_br_status(const SEGrid* g) { return g->status.data(); }
const int32_t* segen_meas_type(const SEGrid* g) { return g->mtype.data(); }
const int32_t* segen_meas_loc(const SEGrid* g) { return g->mloc.data(); }
const int32_t* segen_meas_end(const SEGrid* g) { return g->mend.data(); }
const double* segen_meas_sigma(const SEGrid* g) { return g->sigma.data(); }
const double* segen_meas_z(const SEGrid* g) { return g->z.data(); }
const int32_t* segen_meas_gross(const SEGrid* g) { return g->gross.data(); }
const double* segen_meas_htrue(const SEGrid* g) { return g->htrue.data(); }

int32_t segen_renoise(SEGrid* g, int32_t update, double frac, double* out) {
    Rng rng(mix_seed(g->p.seed ^ 0xA5A5A5A5ULL, static_cast<uint64_t>(update) + 1));
    const int32_t k = static_cast<int32_t>(std::lround(frac * g->m));
    const std::vector<int32_t> rows = sample_sorted(rng, g->m, k);
    for (int32_t q : rows) g->z[q] = g->htrue[q] + g->sigma[q] * rng.normal();
    if (out) std::memcpy(out, g->z.data(), sizeof(double) * g->m);
    return static_cast<int32_t>(rows.size());
}

void segen_set_status(SEGrid* g, int32_t k, int32_t status) {
    if (k >= 0 && k < g->nbr) g->status[k] = status ? 1 : 0;
    eval_h(*g, g->v_true, g->th_true, g->htrue);
}

int32_t segen_pick_nonbridge(const SEGrid* g, uint64_t draw) {
    // A switchable branch: closed, not a bridge, carrying no flow or current
    // rows, between buses of at least three branches each.  Opening a branch
    // can still leave a grid unobservable (its injection rows lose their
    // coupling); the rules make that rare: about 7 % of openings of any
    // non-bridge branch, under 1 % with them (seeded 1,500-bus grids).
    std::vector<uint8_t> metered(g->nbr, 0);
    for (int32_t q = 0; q < g->m; ++q)
        if (g->mtype[q] == 4 || g->mtype[q] == 5 || g->mtype[q] == 6) metered[g->mloc[q]] = 1;
    std::vector<int32_t> deg(g->n, 0);
    for (int32_t k = 0; k < g->nbr; ++k)
        if (g->status[k]) {
            ++deg[g->from[k]];
            ++deg[g->to[k]];
        }
    Rng rng(mix_seed(g->p.seed ^ 0x5EEDULL, draw));
    for (int t = 0; t < 256; ++t) {
        const int32_t k = static_cast<int32_t>(rng.below(g->nbr));
        if (g->status[k] && !metered[k] && deg[g->from[k]] >= 3 && deg[g->to[k]] >= 3 && connected_without(*g, k))
            return k;
    }
    return -1;
}

int32_t segen_draw_loguniform(uint64_t seed, int32_t index, int32_t lo, int32_t hi) {
    Rng rng(mix_seed(seed, static_cast<uint64_t>(index) + 0x100));
    const double u = rng.uniform();
    return static_cast<int32_t>(std::lround(lo * std::pow(static_cast<double>(hi) / lo, u)));
}

int32_t segen_draw_zipf(uint64_t seed, int32_t index, double s, int32_t lo, int32_t hi) {
    // Continuous inverse-CDF draw of density ~ n^-s on [lo, hi + 1), floored.
    Rng rng(mix_seed(seed, static_cast<uint64_t>(index) + 0x200));
    const double u = rng.uniform();
    const double e = 1.0 - s;
    const double a = std::pow(static_cast<double>(lo), e), b = std::pow(static_cast<double>(hi) + 1.0, e);
    const int32_t v = static_cast<int32_t>(std::floor(std::pow(a + u * (b - a), 1.0 / e)));
    return std::min(std::max(v, lo), hi);
}

}  // extern "C"
