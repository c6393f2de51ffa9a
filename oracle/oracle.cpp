// CPU FP64 oracle (test infrastructure; see oracle.h for the reference map).
#include "oracle.h"

#include <algorithm>
#include <limits>
#include <cmath>
#include <cstring>
#include <set>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr double kEps = 1e-12;  // SLE_REAL_EPSILON, FP64 build (sle_types.cuh:62)

inline bool bus_type_meas(int t) { return t == 0 || t == 1 || t == 2 || t == 3 || t == 7 || t == 8; }
inline bool inj_type(int t) { return t == 2 || t == 3 || t == 7 || t == 8; }

}  // namespace

struct OrGrid {
    int n = 0, nbr = 0, m = 0, slack = -1;
    std::vector<int> btype, from, to, status, mtype, mloc, mend;
    std::vector<double> vset, r, x, b, tap, shift, sigma, w;
    // derived admittances
    std::vector<double> gs, bs, bsf, bst;
    // canonical Ybus
    std::vector<int> yptr, ycol;
    std::vector<double> yg, yb;
    // canonical H pattern
    std::vector<int> hptr, hcol;
    // last evaluation
    std::vector<double> hval, weff, res, hx;
    // factorisation
    bool have_symbolic = false, factor_valid = false;
    std::vector<int> sperm, sinv;  // state permutation (new -> old), inverse
    std::vector<int> Cp, Ci;       // upper triangle of permuted G, CSC
    std::vector<double> Cx;
    std::vector<int> pair_slot;    // per H row pair (row-major enumeration) -> Cx slot
    std::vector<int> parent, Lp, Li;
    std::vector<double> Lx;
};

namespace {

int col_theta(const OrGrid& g, int i) { return i == g.slack ? -1 : (i < g.slack ? i : i - 1); }
int col_v(const OrGrid& g, int i) { return g.n - 1 + i; }

void build_static(OrGrid& g) {
    // a1: admittances (network_model.cu:595-612)
    g.gs.resize(g.nbr);
    g.bs.resize(g.nbr);
    g.bsf.resize(g.nbr);
    g.bst.resize(g.nbr);
    for (int k = 0; k < g.nbr; ++k) {
        double den = g.r[k] * g.r[k] + g.x[k] * g.x[k];
        if (den < kEps) den = kEps;
        g.gs[k] = g.r[k] / den;
        g.bs[k] = -g.x[k] / den;
        g.bsf[k] = g.b[k] / (2.0 * g.tap[k] * g.tap[k]);
        g.bst[k] = g.b[k] / 2.0;
    }
    // a2: Ybus, diagonal first, then (column, branch, end) order
    struct Ent { int col, k, end; };
    std::vector<std::vector<Ent>> rows(g.n);
    for (int k = 0; k < g.nbr; ++k) {
        if (!g.status[k]) continue;
        rows[g.from[k]].push_back({g.to[k], k, 0});
        rows[g.to[k]].push_back({g.from[k], k, 1});
    }
    g.yptr.assign(g.n + 1, 0);
    g.ycol.clear();
    g.yg.clear();
    g.yb.clear();
    for (int i = 0; i < g.n; ++i) {
        auto& rw = rows[i];
        std::sort(rw.begin(), rw.end(), [](const Ent& a, const Ent& c) {
            if (a.col != c.col) return a.col < c.col;
            if (a.k != c.k) return a.k < c.k;
            return a.end < c.end;
        });
        const size_t diag = g.ycol.size();
        g.ycol.push_back(i);
        g.yg.push_back(0.0);
        g.yb.push_back(0.0);
        double dg = 0.0, db = 0.0;
        for (const Ent& e : rw) {
            const int k = e.k;
            const double a = std::max(g.tap[k], kEps);
            const double cph = std::cos(g.shift[k]), sph = std::sin(g.shift[k]);
            const double gg = g.gs[k], bb = g.bs[k];
            double yv_g, yv_b;
            if (e.end == 0) {
                yv_g = -(gg * cph + bb * sph) / a;
                yv_b = -(-gg * sph + bb * cph) / a;
                dg += gg / (a * a);
                db += bb / (a * a) + g.bsf[k];
            } else {
                yv_g = -(gg * cph - bb * sph) / a;
                yv_b = -(gg * sph + bb * cph) / a;
                dg += gg;
                db += bb + g.bst[k];
            }
            g.ycol.push_back(e.col);
            g.yg.push_back(yv_g);
            g.yb.push_back(yv_b);
        }
        g.yg[diag] = dg;
        g.yb[diag] = db;
        g.yptr[i + 1] = static_cast<int>(g.ycol.size());
    }
    // H pattern: exact state set of every active row, ascending
    g.hptr.assign(g.m + 1, 0);
    g.hcol.clear();
    std::vector<int> cols;
    for (int q = 0; q < g.m; ++q) {
        cols.clear();
        const int t = g.mtype[q], loc = g.mloc[q];
        std::vector<int> buses;
        if (t == 0) {
            cols.push_back(col_v(g, loc));
        } else if (t == 1) {
            if (col_theta(g, loc) >= 0) cols.push_back(col_theta(g, loc));
        } else if (inj_type(t)) {
            buses.push_back(loc);
            for (int e = g.yptr[loc]; e < g.yptr[loc + 1]; ++e) buses.push_back(g.ycol[e]);
        } else {
            buses.push_back(g.from[loc]);
            buses.push_back(g.to[loc]);
        }
        for (int bb : buses) {
            if (col_theta(g, bb) >= 0) cols.push_back(col_theta(g, bb));
            cols.push_back(col_v(g, bb));
        }
        std::sort(cols.begin(), cols.end());
        cols.erase(std::unique(cols.begin(), cols.end()), cols.end());
        g.hcol.insert(g.hcol.end(), cols.begin(), cols.end());
        g.hptr[q + 1] = static_cast<int>(g.hcol.size());
    }
}

// P and Q at one branch end with the four derivatives (theta_i, V_i, theta_j, V_j).
void flow(const OrGrid& g, const double* V, const double* th, int k, bool q_flow, bool to_end, bool exact,
          double& val, double d[4]) {
    const int i = g.from[k], j = g.to[k];
    const double Vi = V[i], Vj = V[j];
    const double t = th[i] - th[j] - g.shift[k];
    const double c = std::cos(t), s = std::sin(t);
    const double gg = g.gs[k], bb = g.bs[k];
    const double a = std::max(g.tap[k], kEps);
    const double on = g.status[k] ? 1.0 : 0.0;
    const double k1 = Vi * Vj / a;
    if (!q_flow && !to_end) {
        // P_ij = Vi^2 g / a^2 - (Vi Vj / a)(g cos + b sin)
        val = Vi * Vi / (a * a) * gg - k1 * (gg * c + bb * s);
        d[0] = k1 * (gg * s - bb * c);
        d[2] = -k1 * (gg * s - bb * c);
        d[1] = 2.0 * Vi * gg / (a * a) - Vj / a * (gg * c + bb * s);
        d[3] = -Vi / a * (gg * c + bb * s);
    } else if (q_flow && !to_end) {
        // Q_ij = -(Vi^2/a^2)(b + bsh_from) - (Vi Vj / a)(g sin - b cos)
        val = -(Vi * Vi / (a * a)) * (bb + g.bsf[k]) - k1 * (gg * s - bb * c);
        d[0] = -k1 * (gg * c + bb * s);
        d[2] = k1 * (gg * c + bb * s);
        d[1] = (exact ? -2.0 * Vi * (bb + g.bsf[k]) / (a * a) : -2.0 * Vi * bb / (a * a)) - Vj / a * (gg * s - bb * c);
        d[3] = -Vi / a * (gg * s - bb * c);
    } else if (!q_flow && to_end) {
        // P_ji = Vj^2 g - (Vi Vj / a)(g cos - b sin)
        val = Vj * Vj * gg - k1 * (gg * c - bb * s);
        const double dti = exact ? k1 * (gg * s + bb * c) : k1 * (-gg * s - bb * c);
        d[0] = dti;
        d[2] = -dti;
        d[1] = -Vj / a * (gg * c - bb * s);
        d[3] = 2.0 * Vj * gg - Vi / a * (gg * c - bb * s);
    } else {
        // Q_ji = -Vj^2 (b + bsh_to) + (Vi Vj / a)(g sin + b cos)
        val = -Vj * Vj * (bb + g.bst[k]) + k1 * (gg * s + bb * c);
        d[0] = k1 * (gg * c - bb * s);
        d[2] = -k1 * (gg * c - bb * s);
        d[1] = Vj / a * (gg * s + bb * c);
        d[3] = (exact ? -2.0 * Vj * (bb + g.bst[k]) : -2.0 * Vj * bb) + Vi / a * (gg * s + bb * c);
    }
    val *= on;
    if (exact)
        for (int x = 0; x < 4; ++x) d[x] *= on;
}

// Evaluates row q: value and derivative map (state col -> value) into a
// small dense buffer aligned with the row's canonical columns.
double eval_row(const OrGrid& g, const double* V, const double* th, int q, bool exact, double* hrow) {
    const int t = g.mtype[q], loc = g.mloc[q];
    const int h0 = g.hptr[q], nh = g.hptr[q + 1] - h0;
    const int* cols = g.hcol.data() + h0;
    for (int x = 0; x < nh; ++x) hrow[x] = 0.0;
    auto add = [&](int col, double v) {
        if (col < 0) return;
        const int* it = std::lower_bound(cols, cols + nh, col);
        hrow[it - cols] += v;
    };
    if (t == 0) {
        add(col_v(g, loc), 1.0);
        return V[loc];
    }
    if (t == 1) {
        add(col_theta(g, loc), 1.0);
        return th[loc];
    }
    if (inj_type(t)) {
        const bool is_q = (t == 3 || t == 8);
        const double Vi = V[loc];
        double val = 0.0, dvi = 0.0, dti = 0.0;
        for (int e = g.yptr[loc]; e < g.yptr[loc + 1]; ++e) {
            const int j = g.ycol[e];
            const double G = g.yg[e], B = g.yb[e];
            if (j == loc) {
                // self term V_i^2 (G cos0 + B sin0) / V_i^2 (G sin0 - B cos0)
                if (!is_q) {
                    val += Vi * Vi * G;
                    dvi += 2.0 * Vi * G;
                    if (!exact) dti += Vi * Vi * B;  // reference A1 term
                } else {
                    val += -Vi * Vi * B;
                    dvi += -2.0 * Vi * B;
                    if (!exact) dti += Vi * Vi * G;
                }
                continue;
            }
            const double Vj = V[j];
            const double ang = th[loc] - th[j];
            const double c = std::cos(ang), s = std::sin(ang);
            if (!is_q) {
                val += Vi * Vj * (G * c + B * s);
                dvi += Vj * (G * c + B * s);
                dti += -Vi * Vj * (G * s - B * c);
                add(col_theta(g, j), Vi * Vj * (G * s - B * c));
                add(col_v(g, j), Vi * (G * c + B * s));
            } else {
                val += Vi * Vj * (G * s - B * c);
                dvi += Vj * (G * s - B * c);
                dti += Vi * Vj * (G * c + B * s);
                add(col_theta(g, j), -Vi * Vj * (G * c + B * s));
                add(col_v(g, j), Vi * (G * s - B * c));
            }
        }
        add(col_theta(g, loc), dti);
        add(col_v(g, loc), dvi);
        return val;
    }
    const int k = loc;
    const bool to_end = g.mend[q] != 0;
    const int i = g.from[k], j = g.to[k];
    double d[4], val;
    if (t == 4 || t == 5) {
        flow(g, V, th, k, t == 5, to_end, exact, val, d);
    } else {  // I_MAG
        double pv, qv, dp[4], dq[4];
        flow(g, V, th, k, false, to_end, exact, pv, dp);
        flow(g, V, th, k, true, to_end, exact, qv, dq);
        const int eb = to_end ? j : i;
        const double ve = V[eb], vs = std::max(ve, kEps);
        const double on = g.status[k] ? 1.0 : 0.0;
        const double S = std::sqrt(pv * pv + qv * qv);
        val = S / vs * on;
        if (!exact) {
            for (int x = 0; x < 4; ++x) d[x] = dp[x];  // reference A4: P-flow derivatives
        } else {
            for (int x = 0; x < 4; ++x) d[x] = S > 0.0 ? (pv * dp[x] + qv * dq[x]) / (S * vs) * on : 0.0;
            if (ve > kEps) d[to_end ? 3 : 1] -= S / (vs * vs) * on;
        }
    }
    add(col_theta(g, i), d[0]);
    add(col_v(g, i), d[1]);
    add(col_theta(g, j), d[2]);
    add(col_v(g, j), d[3]);
    return val;
}

double evaluate(OrGrid& g, const double* V, const double* th, const double* z, bool exact, bool robust,
                double gamma) {
    g.hval.assign(g.hcol.size(), 0.0);
    g.weff.assign(g.m, 0.0);
    g.res.assign(g.m, 0.0);
    g.hx.assign(g.m, 0.0);
    double J = 0.0;
#pragma omp parallel for schedule(static) reduction(+ : J)
    for (int q = 0; q < g.m; ++q) {
        const double h = eval_row(g, V, th, q, exact, g.hval.data() + g.hptr[q]);
        const double rr = z[q] - h;
        double we = g.w[q];
        if (robust) {
            const double rn = std::fabs(rr / g.sigma[q]);
            if (!(rn <= gamma)) we = gamma / (g.sigma[q] * std::fabs(rr) + kEps);
        }
        g.hx[q] = h;
        g.res[q] = rr;
        g.weff[q] = we;
        J += g.w[q] * rr * rr;
    }
    return J;
}

// ---------------------------------------------------------------------------
// Oracle ordering: exact minimum degree on the bus graph (ties: lowest bus).
// ---------------------------------------------------------------------------
std::vector<std::vector<int>> bus_adjacency(const OrGrid& g) {
    std::vector<std::vector<int>> adj(g.n);
    std::vector<int> buses;
    for (int q = 0; q < g.m; ++q) {
        if (g.hptr[q + 1] == g.hptr[q]) continue;
        buses.clear();
        const int t = g.mtype[q], loc = g.mloc[q];
        if (inj_type(t)) {
            buses.push_back(loc);
            for (int e = g.yptr[loc]; e < g.yptr[loc + 1]; ++e) buses.push_back(g.ycol[e]);
        } else if (t == 4 || t == 5 || t == 6) {
            buses.push_back(g.from[loc]);
            buses.push_back(g.to[loc]);
        }
        for (int a : buses)
            for (int c : buses)
                if (a != c) adj[a].push_back(c);
    }
    for (auto& v : adj) {
        std::sort(v.begin(), v.end());
        v.erase(std::unique(v.begin(), v.end()), v.end());
    }
    return adj;
}

std::vector<int> min_degree(const OrGrid& g) {
    auto adj = bus_adjacency(g);
    const int n = g.n;
    std::vector<char> gone(n, 0);
    std::set<std::pair<int, int>> pq;
    for (int i = 0; i < n; ++i) pq.insert({static_cast<int>(adj[i].size()), i});
    std::vector<int> order, tmp;
    order.reserve(n);
    while (!pq.empty()) {
        const int p = pq.begin()->second;
        pq.erase(pq.begin());
        gone[p] = 1;
        order.push_back(p);
        std::vector<int> nb;
        for (int u : adj[p])
            if (!gone[u]) nb.push_back(u);
        for (int u : nb) {
            pq.erase({static_cast<int>(adj[u].size()), u});
            tmp.clear();
            std::set_union(adj[u].begin(), adj[u].end(), nb.begin(), nb.end(), std::back_inserter(tmp));
            adj[u].clear();
            for (int v : tmp)
                if (v != u && !gone[v]) adj[u].push_back(v);
            pq.insert({static_cast<int>(adj[u].size()), u});
        }
        std::vector<int>().swap(adj[p]);
    }
    return order;
}

// ---------------------------------------------------------------------------
// Up-looking simplicial Cholesky of the permuted gain matrix.
// ---------------------------------------------------------------------------
void symbolic(OrGrid& g) {
    const int ns = 2 * g.n - 1;
    const std::vector<int> bus_order = min_degree(g);
    g.sperm.clear();
    for (int b : bus_order) {
        if (col_theta(g, b) >= 0) g.sperm.push_back(col_theta(g, b));
        g.sperm.push_back(col_v(g, b));
    }
    g.sinv.assign(ns, 0);
    for (int k = 0; k < ns; ++k) g.sinv[g.sperm[k]] = k;
    // Upper-triangle pattern of the permuted gain: (min, max) per H row pair.
    std::vector<std::pair<int, int>> ent;  // (col, row)
    for (int q = 0; q < g.m; ++q)
        for (int a = g.hptr[q]; a < g.hptr[q + 1]; ++a)
            for (int c = a; c < g.hptr[q + 1]; ++c) {
                const int pa = g.sinv[g.hcol[a]], pc = g.sinv[g.hcol[c]];
                ent.push_back({std::max(pa, pc), std::min(pa, pc)});
            }
    std::vector<std::pair<int, int>> uniq = ent;
    std::sort(uniq.begin(), uniq.end());
    uniq.erase(std::unique(uniq.begin(), uniq.end()), uniq.end());
    g.Cp.assign(ns + 1, 0);
    g.Ci.resize(uniq.size());
    for (auto& e : uniq) ++g.Cp[e.first + 1];
    for (int k = 0; k < ns; ++k) g.Cp[k + 1] += g.Cp[k];
    for (size_t t = 0; t < uniq.size(); ++t) g.Ci[t] = uniq[t].second;
    g.Cx.assign(uniq.size(), 0.0);
    g.pair_slot.resize(ent.size());
    for (size_t t = 0; t < ent.size(); ++t) {
        const int col = ent[t].first;
        const int* it = std::lower_bound(g.Ci.data() + g.Cp[col], g.Ci.data() + g.Cp[col + 1], ent[t].second);
        g.pair_slot[t] = static_cast<int>(it - g.Ci.data());
    }
    // etree (Liu, path compression)
    g.parent.assign(ns, -1);
    std::vector<int> anc(ns, -1);
    for (int k = 0; k < ns; ++k)
        for (int p = g.Cp[k]; p < g.Cp[k + 1]; ++p) {
            int i = g.Ci[p];
            while (i != -1 && i < k) {
                const int nx = anc[i];
                anc[i] = k;
                if (nx == -1) g.parent[i] = k;
                i = nx;
            }
        }
    // column counts through row patterns (ereach)
    std::vector<int> cnt(ns, 1), flag(ns, -1);
    for (int k = 0; k < ns; ++k) {
        flag[k] = k;
        for (int p = g.Cp[k]; p < g.Cp[k + 1]; ++p)
            for (int i = g.Ci[p]; i < k && flag[i] != k; i = g.parent[i]) {
                ++cnt[i];
                flag[i] = k;
            }
    }
    g.Lp.assign(ns + 1, 0);
    for (int k = 0; k < ns; ++k) g.Lp[k + 1] = g.Lp[k] + cnt[k];
    g.Li.assign(g.Lp[ns], 0);
    g.Lx.assign(g.Lp[ns], 0.0);
    g.have_symbolic = true;
}

bool numeric(OrGrid& g) {
    const int ns = 2 * g.n - 1;
    std::fill(g.Cx.begin(), g.Cx.end(), 0.0);
    size_t t = 0;
    for (int q = 0; q < g.m; ++q)
        for (int a = g.hptr[q]; a < g.hptr[q + 1]; ++a)
            for (int c = a; c < g.hptr[q + 1]; ++c) g.Cx[g.pair_slot[t++]] += g.weff[q] * g.hval[a] * g.hval[c];
    std::vector<double> xw(ns, 0.0);
    std::vector<int> next(g.Lp.begin(), g.Lp.end() - 1), flag(ns, -1), stack(ns);
    bool ok = true;
    for (int k = 0; k < ns; ++k) {
        int top = ns;
        flag[k] = k;
        for (int p = g.Cp[k]; p < g.Cp[k + 1]; ++p) {
            int i = g.Ci[p];
            xw[i] = g.Cx[p];
            int len = 0;
            for (; i < k && flag[i] != k; i = g.parent[i]) {
                stack[len++] = i;
                flag[i] = k;
            }
            while (len > 0) stack[--top] = stack[--len];
        }
        double d = xw[k];
        xw[k] = 0.0;
        for (; top < ns; ++top) {
            const int i = stack[top];
            const double lki = xw[i] / g.Lx[g.Lp[i]];
            xw[i] = 0.0;
            for (int p = g.Lp[i] + 1; p < next[i]; ++p) xw[g.Li[p]] -= g.Lx[p] * lki;
            d -= lki * lki;
            const int p = next[i]++;
            g.Li[p] = k;
            g.Lx[p] = lki;
        }
        if (!(d > 0.0) || !std::isfinite(d)) {
            ok = false;
            d = 1.0;
        }
        const int p = next[k]++;
        g.Li[p] = k;
        g.Lx[p] = std::sqrt(d);
    }
    return ok;
}

void solve_factor(const OrGrid& g, const double* rhs, double* x) {
    const int ns = 2 * g.n - 1;
    std::vector<double> y(ns);
    for (int k = 0; k < ns; ++k) y[k] = rhs[g.sperm[k]];
    for (int j = 0; j < ns; ++j) {
        y[j] /= g.Lx[g.Lp[j]];
        for (int p = g.Lp[j] + 1; p < g.Lp[j + 1]; ++p) y[g.Li[p]] -= g.Lx[p] * y[j];
    }
    for (int j = ns - 1; j >= 0; --j) {
        for (int p = g.Lp[j] + 1; p < g.Lp[j + 1]; ++p) y[j] -= g.Lx[p] * y[g.Li[p]];
        y[j] /= g.Lx[g.Lp[j]];
    }
    for (int k = 0; k < ns; ++k) x[g.sperm[k]] = y[k];
}

void rhs_of(const OrGrid& g, double* b) {
    const int ns = 2 * g.n - 1;
    std::fill(b, b + ns, 0.0);
    for (int q = 0; q < g.m; ++q)
        for (int a = g.hptr[q]; a < g.hptr[q + 1]; ++a) b[g.hcol[a]] += g.hval[a] * g.weff[q] * g.res[q];
}

}  // namespace

extern "C" {

OrGrid* or_create(int32_t n_bus, const int32_t* bus_type, const double* v_setpoint, int32_t n_branch,
                  const int32_t* from, const int32_t* to, const double* r, const double* x, const double* b,
                  const double* tap, const double* shift, const int32_t* status, int32_t n_meas,
                  const int32_t* mtype, const int32_t* mloc, const int32_t* mend, const double* sigma) {
    auto* g = new OrGrid();
    g->n = n_bus;
    g->nbr = n_branch;
    g->m = n_meas;
    g->btype.assign(bus_type, bus_type + n_bus);
    g->vset.assign(v_setpoint, v_setpoint + n_bus);
    for (int i = 0; i < n_bus; ++i)
        if (bus_type[i] == 2) g->slack = i;  // last SLACK wins (network_model.cu:86-88)
    g->from.assign(from, from + n_branch);
    g->to.assign(to, to + n_branch);
    g->r.assign(r, r + n_branch);
    g->x.assign(x, x + n_branch);
    g->b.assign(b, b + n_branch);
    g->tap.assign(tap, tap + n_branch);
    g->shift.assign(shift, shift + n_branch);
    g->status.resize(n_branch);
    for (int k = 0; k < n_branch; ++k) g->status[k] = status ? (status[k] ? 1 : 0) : 1;
    g->mtype.assign(mtype, mtype + n_meas);
    g->mloc.assign(mloc, mloc + n_meas);
    g->mend.assign(mend, mend + n_meas);
    g->sigma.assign(sigma, sigma + n_meas);
    g->w.resize(n_meas);
    for (int q = 0; q < n_meas; ++q) {
        const double s = std::max(sigma[q], kEps);  // network_model.cu:142-143
        g->w[q] = 1.0 / (s * s);
    }
    build_static(*g);
    return g;
}

void or_destroy(OrGrid* g) { delete g; }

int32_t or_ybus(OrGrid* g, int32_t* row_ptr, int32_t* col, double* gv, double* bv) {
    if (row_ptr) std::copy(g->yptr.begin(), g->yptr.end(), row_ptr);
    if (col) std::copy(g->ycol.begin(), g->ycol.end(), col);
    if (gv) std::copy(g->yg.begin(), g->yg.end(), gv);
    if (bv) std::copy(g->yb.begin(), g->yb.end(), bv);
    return static_cast<int32_t>(g->ycol.size());
}

int64_t or_nnz_h(OrGrid* g) { return static_cast<int64_t>(g->hcol.size()); }

void or_evaluate(OrGrid* g, const double* v, const double* th, const double* z, int32_t exact, int32_t robust,
                 double gamma, double* hx, double* r, int32_t* h_ptr, int32_t* h_col, double* h_val, double* w_eff,
                 double* rhs, double* objective) {
    const double J = evaluate(*g, v, th, z, exact != 0, robust != 0, gamma);
    if (hx) std::copy(g->hx.begin(), g->hx.end(), hx);
    if (r) std::copy(g->res.begin(), g->res.end(), r);
    if (h_ptr) std::copy(g->hptr.begin(), g->hptr.end(), h_ptr);
    if (h_col) std::copy(g->hcol.begin(), g->hcol.end(), h_col);
    if (h_val) std::copy(g->hval.begin(), g->hval.end(), h_val);
    if (w_eff) std::copy(g->weff.begin(), g->weff.end(), w_eff);
    if (rhs) rhs_of(*g, rhs);
    if (objective) *objective = J;
    g->factor_valid = false;
}

int64_t or_gain(OrGrid* g, int32_t* rows, int32_t* cols, double* vals) {
    std::vector<std::pair<std::pair<int, int>, double>> ent;  // ((col, row), value) in state indices
    for (int q = 0; q < g->m; ++q)
        for (int a = g->hptr[q]; a < g->hptr[q + 1]; ++a)
            for (int c = a; c < g->hptr[q + 1]; ++c)
                ent.push_back({{g->hcol[a], g->hcol[c]}, g->weff[q] * g->hval[a] * g->hval[c]});
    std::stable_sort(ent.begin(), ent.end(), [](const auto& u, const auto& w) { return u.first < w.first; });
    int64_t cnt = 0;
    for (size_t t = 0; t < ent.size();) {
        size_t e = t;
        double s = 0.0;
        while (e < ent.size() && ent[e].first == ent[t].first) s += ent[e++].second;
        if (rows) rows[cnt] = ent[t].first.second;
        if (cols) cols[cnt] = ent[t].first.first;
        if (vals) vals[cnt] = s;
        ++cnt;
        t = e;
    }
    return cnt;
}

int32_t or_solve_gain(OrGrid* g, const double* rhs, double* x) {
    if (!g->have_symbolic) symbolic(*g);
    const bool ok = numeric(*g);
    g->factor_valid = ok;
    if (!ok) return 3;
    solve_factor(*g, rhs, x);
    return 0;
}

void or_wls(OrGrid* g, const double* z, double* v, double* th, const OrParams* p, OrResult* res, double* r) {
    const int n = g->n, ns = 2 * n - 1;
    std::vector<double> dx(ns), b(ns);
    auto flat = [&]() {  // kernels.cu:799-817
        for (int i = 0; i < n; ++i) {
            v[i] = (g->btype[i] == 1 || g->btype[i] == 2) ? g->vset[i] : 1.0;
            th[i] = 0.0;
        }
    };
    if (!g->have_symbolic) symbolic(*g);
    if (p->flat_start) flat();
    std::memset(res, 0, sizeof(*res));
    res->status = 5;
    bool converged = false, diverged = false, retry = false;
    int retries = 0;
    const bool stall_test = p->robust && p->huber_stall > 0.0;
    double jh_prev = -1.0, jh = 0.0;
    do {
        if (retry) {
            flat();
            g->factor_valid = false;
            converged = diverged = retry = false;
            jh_prev = -1.0;
        }
        for (int it = 0; it < p->max_iterations && !converged && !diverged; ++it) {
            evaluate(*g, v, th, z, p->exact_jacobian != 0, p->robust != 0, p->huber_gamma);
            if (stall_test) {  // Huber objective of this evaluation
                jh = 0.0;
                for (int q = 0; q < g->m; ++q) {  // every row is active in the oracle
                    const double u = std::fabs(g->res[q]) / std::max(g->sigma[q], kEps);
                    jh += u <= p->huber_gamma ? 0.5 * u * u : p->huber_gamma * u - 0.5 * p->huber_gamma * p->huber_gamma;
                }
            }
            const bool refactor = !g->factor_valid || p->robust || p->gain_policy == 0;
            if (refactor) {
                if (!numeric(*g)) {
                    res->status = 3;
                    g->factor_valid = false;
                    diverged = true;
                    break;
                }
                g->factor_valid = true;
            }
            rhs_of(*g, b.data());
            solve_factor(*g, b.data(), dx.data());
            double mx = 0.0;
            bool bad = false;
            for (int i = 0; i < n; ++i) {  // kernels.cu:721-750
                const int ct = col_theta(*g, i);
                const double dt = ct >= 0 ? dx[ct] : 0.0, dv = dx[col_v(*g, i)];
                if (ct >= 0) th[i] += dt;
                double vn = v[i] + dv;
                vn = std::max(vn, p->vmin);
                vn = std::min(vn, p->vmax);
                v[i] = vn;
                if (!std::isfinite(dt) || !std::isfinite(dv)) bad = true;
                double a = std::max(std::fabs(dt), std::fabs(dv));
                if (a != a) a = 0.0;
                mx = std::max(mx, a);
            }
            // a non-finite step: the reference's max reduction yields NaN
            // (kernels.cu:557-574,752-782), "NaN < tol" fails, and the
            // validity flag makes the step diverged (wls_solver.cu:493-517)
            res->max_mismatch = bad ? std::numeric_limits<double>::quiet_NaN() : mx;
            converged = !bad && mx < p->tolerance;
            diverged = bad;
            if (stall_test && !diverged) {
                if (jh_prev > 0.0 && jh_prev - jh <= p->huber_stall * jh_prev) converged = true;
                jh_prev = jh;
            }
            res->iterations = it + 1;
        }
        if (diverged && retries < 2 && !p->realtime) {
            retry = true;
            ++retries;
            res->iterations = 0;
        }
    } while (retry);
    if (res->status == 5) res->status = converged ? 0 : (diverged ? 2 : 1);
    if (diverged) g->factor_valid = false;
    res->objective = evaluate(*g, v, th, z, p->exact_jacobian != 0, p->robust != 0, p->huber_gamma);
    double best = -1.0;
    int bi = -1;
    for (int q = 0; q < g->m; ++q) {
        if (g->hptr[q + 1] == g->hptr[q] && g->mtype[q] != 1) continue;
        const double a = std::fabs(g->res[q]);
        if (a > best) { best = a; bi = q; }
    }
    res->largest_residual = best < 0 ? 0.0 : best;
    res->largest_idx = bi;
    if (r) std::copy(g->res.begin(), g->res.end(), r);
}

int32_t or_bad_data(OrGrid* g, const double* r, double threshold, int32_t* idx, int32_t max_count) {
    int32_t c = 0;
    for (int q = 0; q < g->m; ++q) {
        if (g->sigma[q] > 0 && std::fabs(r[q]) / g->sigma[q] > threshold) {
            if (idx && c < max_count) idx[c] = q;
            ++c;
        }
    }
    return c;
}

void or_ordering(OrGrid* g, int32_t* bus_perm) {
    const std::vector<int> o = min_degree(*g);
    std::copy(o.begin(), o.end(), bus_perm);
}

void or_symbolic(OrGrid* g, const int32_t* bus_perm, int32_t* parent, int32_t* colcount) {
    // Explicit elimination on the bus graph in the given order: the filled
    // graph's higher neighbours of position j are column j's structure.
    const int n = g->n;
    auto adj = bus_adjacency(*g);
    std::vector<int> pos(n);
    for (int k = 0; k < n; ++k) pos[bus_perm[k]] = k;
    std::vector<std::set<int>> higher(n);
    for (int b = 0; b < n; ++b)
        for (int c : adj[b])
            if (pos[c] > pos[b]) higher[pos[b]].insert(pos[c]);
    for (int j = 0; j < n; ++j) {
        const auto& s = higher[j];
        parent[j] = s.empty() ? -1 : *s.begin();
        colcount[j] = static_cast<int32_t>(s.size()) + 1;
        if (!s.empty()) {
            const int p = *s.begin();
            for (int x : s)
                if (x != p) higher[p].insert(x);
        }
    }
}

void or_results(OrGrid* g, const double* v, const double* th, double* p_inj, double* q_inj, double* pf, double* qf,
                double* pt, double* qt) {
    // bus injections from Ybus at (v, th) (kernels.cu:129-230) and both-end
    // branch flows (kernels.cu:241-333), the arrays the reference's result
    // accessors read after a solve (sle_engine.cu:841-977)
    for (int i = 0; i < g->n; ++i) {
        double P = 0.0, Q = 0.0;
        for (int e = g->yptr[i]; e < g->yptr[i + 1]; ++e) {
            const int j = g->ycol[e];
            const double ang = th[i] - th[j];
            const double c = std::cos(ang), s = std::sin(ang);
            P += v[i] * v[j] * (g->yg[e] * c + g->yb[e] * s);
            Q += v[i] * v[j] * (g->yg[e] * s - g->yb[e] * c);
        }
        if (p_inj) p_inj[i] = P;
        if (q_inj) q_inj[i] = Q;
    }
    double d[4];
    for (int k = 0; k < g->nbr; ++k) {
        double val;
        flow(*g, v, th, k, false, false, true, val, d);
        if (pf) pf[k] = val;
        flow(*g, v, th, k, true, false, true, val, d);
        if (qf) qf[k] = val;
        flow(*g, v, th, k, false, true, true, val, d);
        if (pt) pt[k] = val;
        flow(*g, v, th, k, true, true, true, val, d);
        if (qt) qt[k] = val;
    }
}

int32_t or_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

}  // extern "C"
