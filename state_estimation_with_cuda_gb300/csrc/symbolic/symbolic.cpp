// Symbolic analysis for the GPU WLS pipeline (definitions in symbolic.h).
#include "symbolic.h"

#include "amd.h"

#include <algorithm>
#include <atomic>
#include <cstring>
#include <memory>
#include <numeric>
#include <functional>
#include <thread>

namespace sle_gb300 {

namespace {

inline bool is_bus_type(int32_t t) { return t == 0 || t == 1 || t == 2 || t == 3 || t == 7 || t == 8; }
inline bool is_inj_type(int32_t t) { return t == 2 || t == 3 || t == 7 || t == 8; }

// Buses + measurement rows from which a side task of the analysis (the H
// pattern, the caller's work beside the last passes) gets a thread of its own.
constexpr int64_t kOwnThreadItems = 1 << 15;

// Host threads for the analysis: at most the hardware's less `reserved`
// (cores left to other work), and few enough that each gets at least `grain`
// items.  Ranges are split statically, so a pass is as slow as its slowest
// thread: the threads must not outnumber the free cores.
int32_t host_threads(int64_t items, int64_t grain, int32_t reserved = 0) {
    const int64_t hw = std::max<int64_t>(1, static_cast<int64_t>(std::thread::hardware_concurrency()) - reserved);
    return static_cast<int32_t>(std::max<int64_t>(1, std::min<int64_t>(hw, items / std::max<int64_t>(1, grain))));
}

// fn(t, begin, end) on `parts` contiguous ranges of [0, n), one thread each;
// range t is the same for any machine, so results merged in t order are too.
template <typename Fn>
void parallel_ranges(int64_t n, int32_t parts, Fn&& fn) {
    auto range = [&](int32_t t) {
        return std::make_pair(n * t / parts, n * (t + 1) / parts);
    };
    std::vector<std::thread> pool;
    for (int32_t t = 1; t < parts; ++t)
        pool.emplace_back([&, t] {
            const auto r = range(t);
            fn(t, r.first, r.second);
        });
    const auto r0 = range(0);
    fn(0, r0.first, r0.second);
    for (auto& th : pool) th.join();
}

// Per-range output lists of a parallel pass, concatenated in range order
// into a CSR structure (ptr[i + 1] - ptr[i] = length of item i's list).
struct RangeLists {
    std::vector<std::vector<int32_t>> data, len;
    explicit RangeLists(int32_t parts) : data(parts), len(parts) {}
    void gather(int64_t n, std::vector<int32_t>& ptr, std::vector<int32_t>& out) const {
        const int32_t parts = static_cast<int32_t>(data.size());
        ptr.assign(static_cast<size_t>(n) + 1, 0);
        std::vector<size_t> o(parts + 1, 0);
        std::vector<int64_t> i0(parts + 1, 0);
        for (int32_t t = 0; t < parts; ++t) {
            o[t + 1] = o[t] + data[t].size();
            i0[t + 1] = i0[t] + static_cast<int64_t>(len[t].size());
        }
        out.resize(o[parts]);
        parallel_ranges(parts, parts, [&](int32_t t, int64_t, int64_t) {
            std::copy(data[t].begin(), data[t].end(), out.begin() + o[t]);
            int32_t run = static_cast<int32_t>(o[t]);
            for (size_t x = 0; x < len[t].size(); ++x) {
                run += len[t][x];
                ptr[i0[t] + static_cast<int64_t>(x) + 1] = run;
            }
        });
    }
};

// ---------------------------------------------------------------------------
// Nested dissection on the bus graph.
// ---------------------------------------------------------------------------
class NestedDissection {
public:
    NestedDissection(int32_t n, const std::vector<int32_t>& ptr, const std::vector<int32_t>& adj, int32_t leaf)
        : n_(n), ptr_(ptr), adj_(adj), leaf_(std::max(leaf, 4)), stamp_(n, -1), level_(n, -1) {}

    std::vector<int32_t> run() {
        order_.clear();
        order_.reserve(n_);
        std::vector<int32_t> all(n_);
        std::iota(all.begin(), all.end(), 0);
        dissect(all, 0);
        return order_;
    }

private:
    int32_t n_;
    const std::vector<int32_t>& ptr_;
    const std::vector<int32_t>& adj_;
    int32_t leaf_;
    std::vector<int32_t> stamp_, level_;
    int32_t next_stamp_ = 0;
    std::vector<int32_t> order_;

    int32_t new_stamp(const std::vector<int32_t>& nodes) {
        const int32_t s = next_stamp_++;
        for (int32_t v : nodes) stamp_[v] = s;
        return s;
    }

    // BFS inside the stamped subset; returns visit order, fills level_.
    std::vector<int32_t> bfs(int32_t root, int32_t s) {
        std::vector<int32_t> q{root};
        level_[root] = 0;
        std::vector<int32_t> seen{root};
        const int32_t mark = -2 - s;  // temporary visited marker in level_ is not used; use a local set
        (void)mark;
        std::vector<int32_t> visited_flag;
        size_t head = 0;
        while (head < q.size()) {
            const int32_t u = q[head++];
            for (int32_t e = ptr_[u]; e < ptr_[u + 1]; ++e) {
                const int32_t v = adj_[e];
                if (stamp_[v] != s || level_[v] >= 0) continue;
                level_[v] = level_[u] + 1;
                q.push_back(v);
            }
        }
        return q;
    }

    void clear_levels(const std::vector<int32_t>& nodes) {
        for (int32_t v : nodes) level_[v] = -1;
    }

    int32_t degree_in(int32_t v, int32_t s) const {
        int32_t d = 0;
        for (int32_t e = ptr_[v]; e < ptr_[v + 1]; ++e) d += (stamp_[adj_[e]] == s);
        return d;
    }

    void leaf_order(const std::vector<int32_t>& nodes) {
        // Minimum degree on the induced subgraph (exact degrees, ties -> lowest bus).
        const int32_t k = static_cast<int32_t>(nodes.size());
        if (k == 0) return;
        std::vector<int32_t> sorted = nodes;
        std::sort(sorted.begin(), sorted.end());
        std::vector<int32_t> local(k);
        // map bus -> local through a temporary use of level_
        for (int32_t i = 0; i < k; ++i) level_[sorted[i]] = i;
        std::vector<std::vector<char>> a(k, std::vector<char>(k, 0));
        for (int32_t i = 0; i < k; ++i) {
            const int32_t u = sorted[i];
            for (int32_t e = ptr_[u]; e < ptr_[u + 1]; ++e) {
                const int32_t v = adj_[e];
                if (level_[v] >= 0 && level_[v] < k && v != u && sorted[level_[v]] == v) a[i][level_[v]] = 1;
            }
        }
        for (int32_t i = 0; i < k; ++i) level_[sorted[i]] = -1;
        std::vector<char> alive(k, 1);
        std::vector<int32_t> deg(k, 0);
        for (int32_t i = 0; i < k; ++i)
            for (int32_t j = 0; j < k; ++j) deg[i] += a[i][j];
        for (int32_t step = 0; step < k; ++step) {
            int32_t best = -1;
            for (int32_t i = 0; i < k; ++i)
                if (alive[i] && (best < 0 || deg[i] < deg[best])) best = i;
            order_.push_back(sorted[best]);
            alive[best] = 0;
            std::vector<int32_t> nb;
            for (int32_t j = 0; j < k; ++j)
                if (alive[j] && a[best][j]) nb.push_back(j);
            for (int32_t j : nb) {
                a[j][best] = 0;
                --deg[j];
            }
            for (size_t x = 0; x < nb.size(); ++x)
                for (size_t y = x + 1; y < nb.size(); ++y) {
                    const int32_t p = nb[x], q = nb[y];
                    if (!a[p][q]) {
                        a[p][q] = a[q][p] = 1;
                        ++deg[p];
                        ++deg[q];
                    }
                }
        }
    }

    void dissect(std::vector<int32_t> nodes, int depth) {
        if (static_cast<int32_t>(nodes.size()) <= leaf_ || depth > 200) {
            leaf_order(nodes);
            return;
        }
        const int32_t s = new_stamp(nodes);
        // Connected components inside the subset.
        std::vector<int32_t> sorted = nodes;
        std::sort(sorted.begin(), sorted.end());
        std::vector<std::vector<int32_t>> comps;
        for (int32_t v : sorted) {
            if (level_[v] >= 0) continue;
            comps.push_back(bfs(v, s));
        }
        clear_levels(nodes);
        if (comps.size() > 1) {
            for (auto& c : comps) dissect(c, depth + 1);
            return;
        }
        // Pseudo-peripheral root: start at the min-degree vertex.
        int32_t root = sorted[0];
        int32_t best_deg = degree_in(root, s);
        for (int32_t v : sorted) {
            const int32_t d = degree_in(v, s);
            if (d < best_deg) { best_deg = d; root = v; }
        }
        std::vector<int32_t> q;
        int32_t ecc = -1;
        for (int it = 0; it < 6; ++it) {
            q = bfs(root, s);
            const int32_t e = level_[q.back()];
            if (e <= ecc) { break; }
            ecc = e;
            // min-degree vertex in the last level
            int32_t cand = q.back();
            int32_t cd = degree_in(cand, s);
            for (auto itq = q.rbegin(); itq != q.rend() && level_[*itq] == e; ++itq) {
                const int32_t d = degree_in(*itq, s);
                if (d < cd || (d == cd && *itq < cand)) { cd = d; cand = *itq; }
            }
            clear_levels(q);
            root = cand;
        }
        clear_levels(q);
        q = bfs(root, s);
        const int32_t depth_levels = level_[q.back()];
        if (depth_levels < 2) {
            clear_levels(q);
            leaf_order(nodes);
            return;
        }
        std::vector<int32_t> cnt(depth_levels + 1, 0);
        for (int32_t v : q) ++cnt[level_[v]];
        const int32_t total = static_cast<int32_t>(q.size());
        // Choose the smallest level among those keeping 40..60 % balance;
        // fall back to the median level.
        int32_t cum = 0, median = 1;
        std::vector<int32_t> below(depth_levels + 1, 0);
        for (int32_t l = 0; l <= depth_levels; ++l) {
            below[l] = cum;
            cum += cnt[l];
        }
        for (int32_t l = 1; l < depth_levels; ++l) {
            if (below[l] + cnt[l] >= total / 2) { median = l; break; }
            median = l;
        }
        int32_t sep = median;
        for (int32_t l = 1; l < depth_levels; ++l) {
            const double lo = static_cast<double>(below[l]) / total;
            const double hi = static_cast<double>(total - below[l] - cnt[l]) / total;
            if (lo >= 0.35 && hi >= 0.35 && cnt[l] < cnt[sep]) sep = l;
        }
        // Parts: 0 = A (levels < sep), 1 = separator, 2 = B.
        std::vector<int32_t> A, S, B;
        for (int32_t v : q) {
            const int32_t l = level_[v];
            if (l < sep) A.push_back(v);
            else if (l == sep) S.push_back(v);
            else B.push_back(v);
        }
        // Thin the separator: a separator vertex with no neighbour in B joins A,
        // then one with no neighbour in A joins B.
        auto part_of = [&](int32_t v) { return level_[v] < sep ? 0 : (level_[v] == sep ? 1 : 2); };
        std::vector<int32_t> S2;
        for (int32_t v : S) {
            bool touches_b = false;
            for (int32_t e = ptr_[v]; e < ptr_[v + 1] && !touches_b; ++e) {
                const int32_t u = adj_[e];
                if (stamp_[u] == s && part_of(u) == 2) touches_b = true;
            }
            if (!touches_b) {
                A.push_back(v);
                level_[v] = sep - 1;  // now part of A
            } else {
                S2.push_back(v);
            }
        }
        std::vector<int32_t> S3;
        for (int32_t v : S2) {
            bool touches_a = false;
            for (int32_t e = ptr_[v]; e < ptr_[v + 1] && !touches_a; ++e) {
                const int32_t u = adj_[e];
                if (stamp_[u] == s && part_of(u) == 0) touches_a = true;
            }
            if (!touches_a) {
                B.push_back(v);
                level_[v] = sep + 1;
            } else {
                S3.push_back(v);
            }
        }
        clear_levels(q);
        if (A.empty() || B.empty()) {
            leaf_order(nodes);
            return;
        }
        dissect(std::move(A), depth + 1);
        dissect(std::move(B), depth + 1);
        // Separator last, ordered by minimum degree among itself.
        leaf_order_small_or_natural(S3);
    }

    void leaf_order_small_or_natural(std::vector<int32_t>& S) {
        if (static_cast<int32_t>(S.size()) <= 4 * leaf_) {
            leaf_order(S);
        } else {
            std::sort(S.begin(), S.end());
            for (int32_t v : S) order_.push_back(v);
        }
    }
};

int64_t trapezoid(int64_t nc, int64_t f) { return nc * f - nc * (nc - 1) / 2; }

}  // namespace

void bus_graph(const Topology& t, const std::vector<int32_t>& y_ptr, const std::vector<int32_t>& y_col,
               std::vector<int32_t>& adj_ptr, std::vector<int32_t>& adj) {
    // Buses a and b are adjacent when an active row couples them: an
    // injection row at c couples every pair of {c} and c's Ybus neighbours,
    // a flow or current row couples the branch's two ends.  Bus a's list is
    // therefore the Ybus rows of the injection-measured buses of a's own Ybus
    // row, plus the far ends of a's flow-measured branches; each list is
    // built on its own (sorted, unique), buses in parallel ranges.
    const int32_t n = t.n_bus, nbr = t.n_branch;
    // marks: injection-measured buses, flow-measured branches (rows in
    // parallel ranges; a mark is only ever set to 1)
    std::unique_ptr<std::atomic<uint8_t>[]> has_inj(new std::atomic<uint8_t>[n]);
    std::unique_ptr<std::atomic<uint8_t>[]> has_flow(new std::atomic<uint8_t>[std::max(nbr, 1)]);
    parallel_ranges(n, host_threads(n, 1 << 16), [&](int32_t, int64_t i0, int64_t i1) {
        for (int64_t i = i0; i < i1; ++i) has_inj[i].store(0, std::memory_order_relaxed);
    });
    parallel_ranges(nbr, host_threads(nbr, 1 << 16), [&](int32_t, int64_t k0, int64_t k1) {
        for (int64_t k = k0; k < k1; ++k) has_flow[k].store(0, std::memory_order_relaxed);
    });
    parallel_ranges(t.n_meas, host_threads(t.n_meas, 1 << 16), [&](int32_t, int64_t q0, int64_t q1) {
        for (int64_t q = q0; q < q1; ++q) {
            if (t.m_active && !t.m_active[q]) continue;
            const int32_t ty = t.m_type[q], loc = t.m_loc[q];
            if (is_inj_type(ty)) has_inj[loc].store(1, std::memory_order_relaxed);
            if ((ty == 4 || ty == 5 || ty == 6) && t.br_from[loc] != t.br_to[loc])
                has_flow[loc].store(1, std::memory_order_relaxed);
        }
    });
    // flow-measured branches by end bus (CSR)
    std::vector<int32_t> fptr(static_cast<size_t>(n) + 1, 0), fpart;
    for (int32_t k = 0; k < nbr; ++k)
        if (has_flow[k].load(std::memory_order_relaxed)) {
            ++fptr[t.br_from[k] + 1];
            ++fptr[t.br_to[k] + 1];
        }
    for (int32_t i = 0; i < n; ++i) fptr[i + 1] += fptr[i];
    fpart.resize(fptr[n]);
    {
        std::vector<int32_t> fill(fptr.begin(), fptr.end() - 1);
        for (int32_t k = 0; k < nbr; ++k)
            if (has_flow[k].load(std::memory_order_relaxed)) {
                const int32_t i = t.br_from[k], j = t.br_to[k];
                fpart[fill[i]++] = j;
                fpart[fill[j]++] = i;
            }
    }
    const int32_t parts = host_threads(n, 4096);
    RangeLists out(parts);
    parallel_ranges(n, parts, [&](int32_t th, int64_t b0, int64_t b1) {
        std::vector<int32_t> mark(n, -1), list;
        auto& d = out.data[th];
        auto& len = out.len[th];
        for (int64_t a64 = b0; a64 < b1; ++a64) {
            const int32_t a = static_cast<int32_t>(a64);
            list.clear();
            mark[a] = a;
            for (int32_t e = y_ptr[a]; e < y_ptr[a + 1]; ++e) {
                const int32_t c = y_col[e];
                if (!has_inj[c].load(std::memory_order_relaxed)) continue;
                for (int32_t f = y_ptr[c]; f < y_ptr[c + 1]; ++f) {
                    const int32_t b = y_col[f];
                    if (mark[b] != a) {
                        mark[b] = a;
                        list.push_back(b);
                    }
                }
            }
            for (int32_t f = fptr[a]; f < fptr[a + 1]; ++f) {
                const int32_t b = fpart[f];
                if (mark[b] != a) {
                    mark[b] = a;
                    list.push_back(b);
                }
            }
            std::sort(list.begin(), list.end());
            d.insert(d.end(), list.begin(), list.end());
            len.push_back(static_cast<int32_t>(list.size()));
        }
    });
    out.gather(n, adj_ptr, adj);
}

bool build_plan(const Topology& t, const SymbolicParams& prm, Plan& P, std::string& err,
                const std::function<void()>& alongside) {
    const int32_t n = t.n_bus, nbr = t.n_branch, m = t.n_meas, s = t.slack;
    if (n < 1 || s < 0 || s >= n) { err = "invalid bus count or slack index"; return false; }
    P = Plan();
    P.n_bus = n;
    P.n_state = 2 * n - 1;
    P.n_meas = m;
    P.slack = s;
    for (int32_t k = 0; k < nbr; ++k) {
        if (t.br_from[k] < 0 || t.br_from[k] >= n || t.br_to[k] < 0 || t.br_to[k] >= n) {
            err = "branch references an unknown bus";
            return false;
        }
    }
    for (int32_t q = 0; q < m; ++q) {
        const int32_t ty = t.m_type[q], loc = t.m_loc[q];
        if (ty < 0 || ty > 8) { err = "unknown measurement type"; return false; }
        const int32_t lim = is_bus_type(ty) ? n : nbr;
        if (loc < 0 || loc >= lim) { err = "measurement location out of range"; return false; }
    }
    auto col_t = [&](int32_t i) { return i == s ? -1 : (i < s ? i : i - 1); };
    auto col_v = [&](int32_t i) { return n - 1 + i; };

    // --- Ybus pattern -----------------------------------------------------------
    // Row i: the diagonal, then (column, 2k + end) of each closed branch k at
    // bus i, sorted.
    {
        std::vector<int32_t> cnt(static_cast<size_t>(n) + 1, 0);
        for (int32_t k = 0; k < nbr; ++k) {
            if (!t.br_closed[k]) continue;
            ++cnt[t.br_from[k] + 1];
            ++cnt[t.br_to[k] + 1];
        }
        P.y_ptr.assign(static_cast<size_t>(n) + 1, 0);
        for (int32_t i = 0; i < n; ++i) {
            P.y_ptr[i + 1] = P.y_ptr[i] + 1 + cnt[i + 1];
            cnt[i + 1] += cnt[i];
        }
        std::vector<std::pair<int32_t, int32_t>> ent(static_cast<size_t>(cnt[n]));
        {
            std::vector<int32_t> fill(cnt.begin(), cnt.end() - 1);
            for (int32_t k = 0; k < nbr; ++k) {
                if (!t.br_closed[k]) continue;
                ent[fill[t.br_from[k]]++] = {t.br_to[k], (k << 1) | 0};
                ent[fill[t.br_to[k]]++] = {t.br_from[k], (k << 1) | 1};
            }
        }
        P.y_col.resize(P.y_ptr[n]);
        P.y_src.resize(P.y_ptr[n]);
        parallel_ranges(n, host_threads(n, 8192), [&](int32_t, int64_t i0, int64_t i1) {
            for (int64_t i = i0; i < i1; ++i) {
                auto* r0 = ent.data() + cnt[i];
                auto* r1 = ent.data() + cnt[i + 1];
                std::sort(r0, r1);
                int32_t o = P.y_ptr[i];
                P.y_col[o] = static_cast<int32_t>(i);
                P.y_src[o] = -1;
                for (auto* e = r0; e < r1; ++e) {
                    ++o;
                    P.y_col[o] = e->first;
                    P.y_src[o] = e->second;
                }
            }
        });
    }

    // --- bus graph -------------------------------------------------------------------
    std::vector<int32_t> gptr, gadj;
    bus_graph(t, P.y_ptr, P.y_col, gptr, gadj);

    // --- H pattern ------------------------------------------------------------------
    // Built on a thread of its own while the bus graph is ordered (the ordering
    // does not read it), joined before anything else returns or reads it; a
    // small grid builds it in place (a thread costs more than it hides).
    auto h_pattern_build = [&] {
        // Injection-row column lists per bus (computed once per bus, in
        // parallel ranges): the angle and magnitude columns of the bus's Ybus
        // row, sorted and unique, with each Ybus entry's positions in it.
        std::vector<int32_t> inj_cols_ptr, inj_cols;
        P.y_hpos_t.assign(P.y_col.size(), -1);
        P.y_hpos_v.assign(P.y_col.size(), -1);
        {
            const int32_t parts = host_threads(n, 8192);
            RangeLists out(parts);
            parallel_ranges(n, parts, [&](int32_t th, int64_t i0, int64_t i1) {
                std::vector<int32_t> cols;
                for (int64_t i = i0; i < i1; ++i) {
                    cols.clear();
                    for (int32_t e = P.y_ptr[i]; e < P.y_ptr[i + 1]; ++e) {
                        const int32_t j = P.y_col[e];
                        if (col_t(j) >= 0) cols.push_back(col_t(j));
                        cols.push_back(col_v(j));
                    }
                    std::sort(cols.begin(), cols.end());
                    cols.erase(std::unique(cols.begin(), cols.end()), cols.end());
                    for (int32_t e = P.y_ptr[i]; e < P.y_ptr[i + 1]; ++e) {
                        const int32_t j = P.y_col[e];
                        if (col_t(j) >= 0)
                            P.y_hpos_t[e] =
                                static_cast<int32_t>(std::lower_bound(cols.begin(), cols.end(), col_t(j)) - cols.begin());
                        P.y_hpos_v[e] =
                            static_cast<int32_t>(std::lower_bound(cols.begin(), cols.end(), col_v(j)) - cols.begin());
                    }
                    out.data[th].insert(out.data[th].end(), cols.begin(), cols.end());
                    out.len[th].push_back(static_cast<int32_t>(cols.size()));
                }
            });
            out.gather(n, inj_cols_ptr, inj_cols);
        }
        // Rows: the columns of each active row (a pass of lengths, then each
        // row written at its offset, rows in parallel ranges).
        P.m_kind.assign(m, ROW_NONE);
        P.m_fpos.assign(m, -1);
        auto row_cols = [&](int32_t q, int32_t* dst, int32_t& kind, int32_t& fpos) {
            const int32_t ty = t.m_type[q], loc = t.m_loc[q];
            if (t.m_active && !t.m_active[q]) return 0;
            if (ty == 0) {
                kind = ROW_VMAG;
                if (dst) dst[0] = col_v(loc);
                return 1;
            }
            if (ty == 1) {
                kind = ROW_VANG;
                if (col_t(loc) < 0) return 0;
                if (dst) dst[0] = col_t(loc);
                return 1;
            }
            if (is_inj_type(ty)) {
                kind = ROW_INJ;
                const int32_t c0 = inj_cols_ptr[loc], c1 = inj_cols_ptr[loc + 1];
                if (dst) std::copy(inj_cols.begin() + c0, inj_cols.begin() + c1, dst);
                return c1 - c0;
            }
            kind = (ty == 6) ? ROW_IMAG : ROW_FLOW;
            const int32_t i = t.br_from[loc], j = t.br_to[loc];
            const int32_t c4[4] = {col_t(i), col_v(i), col_t(j), col_v(j)};
            int32_t cols[4], nc = 0;
            for (int32_t c : c4)
                if (c >= 0) cols[nc++] = c;
            std::sort(cols, cols + nc);
            nc = static_cast<int32_t>(std::unique(cols, cols + nc) - cols);
            uint32_t packed = 0;
            for (int x = 0; x < 4; ++x) {
                uint32_t pos = 0xFF;
                if (c4[x] >= 0) pos = static_cast<uint32_t>(std::lower_bound(cols, cols + nc, c4[x]) - cols);
                packed |= pos << (8 * x);
            }
            fpos = static_cast<int32_t>(packed);
            if (dst) std::copy(cols, cols + nc, dst);
            return nc;
        };
        P.h_ptr.assign(static_cast<size_t>(m) + 1, 0);
        const int32_t parts = host_threads(m, 16384);
        parallel_ranges(m, parts, [&](int32_t, int64_t q0, int64_t q1) {
            for (int64_t q = q0; q < q1; ++q) {
                int32_t kind = ROW_NONE, fpos = -1;
                P.h_ptr[q + 1] = row_cols(static_cast<int32_t>(q), nullptr, kind, fpos);
                P.m_kind[q] = kind;
                P.m_fpos[q] = fpos;
            }
        });
        for (int32_t q = 0; q < m; ++q) P.h_ptr[q + 1] += P.h_ptr[q];
        P.h_col.resize(P.h_ptr[m]);
        P.h_row.resize(P.h_ptr[m]);
        parallel_ranges(m, parts, [&](int32_t, int64_t q0, int64_t q1) {
            for (int64_t q = q0; q < q1; ++q) {
                int32_t kind = ROW_NONE, fpos = -1;
                row_cols(static_cast<int32_t>(q), P.h_col.data() + P.h_ptr[q], kind, fpos);
                for (int32_t h = P.h_ptr[q]; h < P.h_ptr[q + 1]; ++h) P.h_row[h] = static_cast<int32_t>(q);
            }
        });
    };
    std::thread h_pattern;
    if (static_cast<int64_t>(n) + m >= kOwnThreadItems) h_pattern = std::thread(h_pattern_build);
    else h_pattern_build();

    // --- ordering on the bus graph -----------------------------------------------------
    std::vector<int32_t> order;
    AmdTrace trace;
    const bool traced = prm.ordering != 1 && prm.ordering != 2;
    if (prm.ordering == 1) {
        order.resize(n);
        std::iota(order.begin(), order.end(), 0);
    } else if (prm.ordering == 2) {
        NestedDissection nd(n, gptr, gadj, prm.leaf_size);
        order = nd.run();
    } else {
        order = amd_order(n, gptr, gadj, &trace);
    }
    if (h_pattern.joinable()) h_pattern.join();
    if (static_cast<int32_t>(order.size()) != n) { err = "ordering failed"; return false; }
    std::vector<int32_t> pos(n, -1);
    for (int32_t k = 0; k < n; ++k) pos[order[k]] = k;
    const int32_t n_piv = static_cast<int32_t>(trace.piv_end.size());
    const int32_t piv_parts = host_threads(n_piv, 4096);

    // --- elimination tree and postorder -----------------------------------------------------
    // From the ordering's trace: a supervariable's members form a chain, and
    // the last one's parent is the first vertex of its column structure.
    // Otherwise Liu's algorithm on the bus graph.
    std::vector<int32_t> parent(n, -1);
    if (traced) {
        parallel_ranges(n_piv, piv_parts, [&](int32_t, int64_t k0, int64_t k1) {
            for (int64_t k = k0; k < k1; ++k) {
                const int32_t b0 = k ? trace.piv_end[k - 1] : 0, b1 = trace.piv_end[k];
                for (int32_t q = b0; q + 1 < b1; ++q) parent[q] = q + 1;
                int32_t first = n;
                for (int64_t y = trace.lp_ptr[k]; y < trace.lp_ptr[k + 1]; ++y) first = std::min(first, pos[trace.lp[y]]);
                parent[b1 - 1] = first < n ? first : -1;
            }
        });
    } else {
        std::vector<int32_t> anc(n, -1);
        for (int32_t j = 0; j < n; ++j) {
            const int32_t b = order[j];
            for (int32_t e = gptr[b]; e < gptr[b + 1]; ++e) {
                int32_t i = pos[gadj[e]];
                if (i >= j) continue;
                while (anc[i] != -1 && anc[i] != j) {
                    const int32_t nx = anc[i];
                    anc[i] = j;
                    i = nx;
                }
                if (anc[i] == -1) {
                    anc[i] = j;
                    parent[i] = j;
                }
            }
        }
    }
    std::vector<int32_t> post, new_of(n);  // new position -> old, old -> new
    post.reserve(n);
    {
        std::vector<int32_t> head(n, -1), next(n, -1);
        for (int32_t j = n - 1; j >= 0; --j) {
            if (parent[j] >= 0) {
                next[j] = head[parent[j]];
                head[parent[j]] = j;
            }
        }
        std::vector<int32_t> stack;
        for (int32_t r = 0; r < n; ++r) {
            if (parent[r] != -1) continue;
            stack.push_back(r);
            while (!stack.empty()) {
                const int32_t v = stack.back();
                if (head[v] != -1) {
                    const int32_t c = head[v];
                    head[v] = next[c];
                    stack.push_back(c);
                } else {
                    stack.pop_back();
                    post.push_back(v);
                }
            }
        }
        // renumbering (positions in parallel ranges); a postorder is an
        // equivalent ordering: its elimination tree is the same tree, renumbered
        const int32_t parts = host_threads(n, 1 << 15);
        std::vector<int32_t> order2(n), parent2(n);
        parallel_ranges(n, parts, [&](int32_t, int64_t k0, int64_t k1) {
            for (int64_t k = k0; k < k1; ++k) {
                order2[k] = order[post[k]];
                pos[order2[k]] = static_cast<int32_t>(k);
                new_of[post[k]] = static_cast<int32_t>(k);
            }
        });
        parallel_ranges(n, parts, [&](int32_t, int64_t k0, int64_t k1) {
            for (int64_t k = k0; k < k1; ++k) {
                const int32_t pa = parent[post[k]];
                parent2[k] = pa < 0 ? -1 : new_of[pa];
            }
        });
        order.swap(order2);
        parent.swap(parent2);
    }

    // --- column structures (bus level, strictly below the diagonal) ----------------------
    // csize[j] = |struct(L(:, j))|; col_struct(j, out) writes the sorted
    // structure.  A postorder keeps the structures as vertex sets, so from
    // the trace column j is the later members of its supervariable plus the
    // supervariable's element, renumbered.  Otherwise the structures are
    // merged up the tree from the bus graph.
    std::vector<int32_t> csize(n);
    std::vector<std::vector<int32_t>> cstruct;
    std::vector<int32_t> piv_of_old;
    if (traced) {
        piv_of_old.resize(n);
        parallel_ranges(n_piv, piv_parts, [&](int32_t, int64_t k0, int64_t k1) {
            for (int64_t k = k0; k < k1; ++k)
                for (int32_t q = k ? trace.piv_end[k - 1] : 0; q < trace.piv_end[k]; ++q)
                    piv_of_old[q] = static_cast<int32_t>(k);
        });
        for (int32_t j = 0; j < n; ++j) {
            const int32_t q = post[j], k = piv_of_old[q];
            csize[j] = trace.piv_end[k] - 1 - q + static_cast<int32_t>(trace.lp_ptr[k + 1] - trace.lp_ptr[k]);
        }
    } else {
        cstruct.resize(n);
        std::vector<std::vector<int32_t>> kids(n);
        for (int32_t j = 0; j < n; ++j)
            if (parent[j] >= 0) kids[parent[j]].push_back(j);
        std::vector<int32_t> tmp, merged;
        for (int32_t j = 0; j < n; ++j) {
            tmp.clear();
            const int32_t b = order[j];
            for (int32_t e = gptr[b]; e < gptr[b + 1]; ++e) {
                const int32_t i = pos[gadj[e]];
                if (i > j) tmp.push_back(i);
            }
            std::sort(tmp.begin(), tmp.end());
            for (int32_t c : kids[j]) {
                merged.clear();
                const auto& cs = cstruct[c];
                auto it = std::upper_bound(cs.begin(), cs.end(), j);
                std::set_union(tmp.begin(), tmp.end(), it, cs.end(), std::back_inserter(merged));
                tmp.swap(merged);
            }
            cstruct[j] = tmp;
            csize[j] = static_cast<int32_t>(tmp.size());
        }
    }
    auto col_struct = [&](int32_t j, int32_t* out) {
        if (!traced) {
            std::copy(cstruct[j].begin(), cstruct[j].end(), out);
            return;
        }
        const int32_t q = post[j], k = piv_of_old[q];
        int32_t o = 0;
        for (int32_t q2 = q + 1; q2 < trace.piv_end[k]; ++q2) out[o++] = new_of[q2];
        for (int64_t y = trace.lp_ptr[k]; y < trace.lp_ptr[k + 1]; ++y) out[o++] = pos[trace.lp[y]];
        std::sort(out, out + o);
    };

    // --- fundamental supernodes + relaxed amalgamation (bus level) ------------------------
    std::vector<int32_t> nkids(n, 0);
    for (int32_t j = 0; j < n; ++j)
        if (parent[j] >= 0) ++nkids[parent[j]];
    std::vector<int32_t> fs_start;  // fundamental supernode starts
    for (int32_t j = 0; j < n; ++j) {
        const bool joins_prev = j > 0 && parent[j - 1] == j && nkids[j] == 1 &&
                                csize[j - 1] == csize[j] + 1;
        if (!joins_prev) fs_start.push_back(j);
    }
    const int32_t nfs = static_cast<int32_t>(fs_start.size());
    fs_start.push_back(n);
    std::vector<int32_t> fs_of(n);
    for (int32_t f = 0; f < nfs; ++f)
        for (int32_t j = fs_start[f]; j < fs_start[f + 1]; ++j) fs_of[j] = f;
    std::vector<int32_t> g_start(nfs), g_nc(nfs), g_f(nfs);
    std::vector<int64_t> g_true(nfs);
    std::vector<char> merged_up(nfs, 0);
    for (int32_t f = 0; f < nfs; ++f) {
        const int32_t last = fs_start[f + 1] - 1;
        g_start[f] = fs_start[f];
        g_nc[f] = fs_start[f + 1] - fs_start[f];
        g_f[f] = g_nc[f] + csize[last];
        g_true[f] = trapezoid(g_nc[f], g_f[f]);
    }
    for (int32_t f = 0; f < nfs; ++f) {
        const int32_t last = fs_start[f + 1] - 1;
        const int32_t pj = parent[last];
        if (pj < 0) continue;
        const int32_t p = fs_of[pj];
        if (fs_start[f + 1] != g_start[p]) continue;  // not immediately before the parent
        const int64_t nc = g_nc[f] + g_nc[p];
        const int64_t ff = g_nc[f] + g_f[p];
        const int64_t ent = trapezoid(nc, ff);
        const double z = static_cast<double>(ent - g_true[f] - g_true[p]) / static_cast<double>(ent);
        bool merge = false;
        if (nc <= prm.nrelax[0]) merge = true;
        else if (nc <= prm.nrelax[1]) merge = z < prm.zrelax[0];
        else if (nc <= prm.nrelax[2]) merge = z < prm.zrelax[1];
        else merge = z < prm.zrelax[2];
        if (!merge) continue;
        merged_up[f] = 1;
        g_start[p] = g_start[f];
        g_nc[p] = static_cast<int32_t>(nc);
        g_f[p] = static_cast<int32_t>(ff);
        g_true[p] += g_true[f];
    }
    // Final supernodes: surviving groups, ordered by start column (= index order).
    std::vector<int32_t> sn_b0, sn_b1, sn_top;  // bus position ranges, top fundamental
    for (int32_t f = 0; f < nfs; ++f) {
        if (merged_up[f]) continue;
        sn_b0.push_back(g_start[f]);
        sn_b1.push_back(fs_start[f + 1]);
        sn_top.push_back(f);
    }
    const int32_t ns = static_cast<int32_t>(sn_b0.size());
    std::vector<int32_t> sn_of_pos(n);
    for (int32_t k = 0; k < ns; ++k)
        for (int32_t j = sn_b0[k]; j < sn_b1[k]; ++j) sn_of_pos[j] = k;

    // --- expansion to states --------------------------------------------------------------
    // ps0[k] = first permuted state of bus position k: two states a bus, one
    // for the slack (theta, then V); buses in parallel ranges
    std::vector<int32_t> ps0(n + 1);
    const int32_t pos_s = pos[s];
    const int32_t bus_parts = host_threads(n, 1 << 15);
    P.bus_perm = order;
    P.bus_ps_theta.assign(n, -1);
    P.bus_ps_v.assign(n, -1);
    P.state_of_ps.assign(P.n_state, -1);
    parallel_ranges(n + 1, bus_parts, [&](int32_t, int64_t k0, int64_t k1) {
        for (int64_t k = k0; k < k1; ++k) ps0[k] = static_cast<int32_t>(2 * k - (k > pos_s ? 1 : 0));
    });
    parallel_ranges(n, bus_parts, [&](int32_t, int64_t k0, int64_t k1) {
        for (int64_t k = k0; k < k1; ++k) {
            const int32_t b = order[k];
            if (b == s) {
                P.bus_ps_v[b] = ps0[k];
            } else {
                P.bus_ps_theta[b] = ps0[k];
                P.bus_ps_v[b] = ps0[k] + 1;
                P.state_of_ps[ps0[k]] = col_t(b);
            }
            P.state_of_ps[P.bus_ps_v[b]] = col_v(b);
        }
    });
    std::vector<int32_t> ps_of_state(P.n_state);
    parallel_ranges(P.n_state, bus_parts, [&](int32_t, int64_t p0, int64_t p1) {
        for (int64_t p = p0; p < p1; ++p) ps_of_state[P.state_of_ps[p]] = static_cast<int32_t>(p);
    });

    P.n_super = ns;
    P.sn_c0.assign(ns + 1, 0);
    P.sn_f.assign(ns, 0);
    P.sn_parent.assign(ns, -1);
    P.sn_rows_off.assign(ns + 1, 0);
    P.sn_lx_off.assign(ns + 1, 0);
    P.sn_u_off.assign(ns + 1, 0);
    P.sn_su_off.assign(ns + 1, 0);
    std::vector<int32_t> sn_of_ps(P.n_state);
    // Rows of front k: its own columns, then the structure of its last column,
    // each bus expanded to its states.
    std::vector<int64_t> sb_off(ns + 1, 0);
    for (int32_t k = 0; k < ns; ++k) sb_off[k + 1] = sb_off[k] + csize[sn_b1[k] - 1];
    std::vector<int32_t> sb(static_cast<size_t>(sb_off[ns]));
    const int32_t sn_parts = host_threads(ns, 2048);
    parallel_ranges(ns, sn_parts, [&](int32_t, int64_t k0, int64_t k1) {
        for (int64_t k = k0; k < k1; ++k) {
            col_struct(sn_b1[k] - 1, sb.data() + sb_off[k]);
            int32_t f = ps0[sn_b1[k]] - ps0[sn_b0[k]];
            for (int64_t y = sb_off[k]; y < sb_off[k + 1]; ++y) f += ps0[sb[y] + 1] - ps0[sb[y]];
            P.sn_f[k] = f;
        }
    });
    for (int32_t k = 0; k < ns; ++k) P.sn_rows_off[k + 1] = P.sn_rows_off[k] + P.sn_f[k];
    P.sn_rows.resize(static_cast<size_t>(P.sn_rows_off[ns]));
    parallel_ranges(ns, sn_parts, [&](int32_t, int64_t k0, int64_t k1) {
        for (int64_t k = k0; k < k1; ++k) {
            P.sn_c0[k] = ps0[sn_b0[k]];
            int32_t* row = P.sn_rows.data() + P.sn_rows_off[k];
            for (int32_t x = ps0[sn_b0[k]]; x < ps0[sn_b1[k]]; ++x) {
                *row++ = x;
                sn_of_ps[x] = static_cast<int32_t>(k);
            }
            for (int64_t y = sb_off[k]; y < sb_off[k + 1]; ++y)
                for (int32_t x = ps0[sb[y]]; x < ps0[sb[y] + 1]; ++x) *row++ = x;
            const int32_t pj = parent[sn_b1[k] - 1];
            P.sn_parent[k] = pj >= 0 ? sn_of_pos[pj] : -1;
        }
    });
    P.sn_c0[ns] = P.n_state;
    int64_t lx = 0, uu = 0, su = 0;
    P.nnz_l = 0;
    P.flops = 0.0;
    P.max_front = 0;
    for (int32_t k = 0; k < ns; ++k) {
        const int64_t nc = P.sn_c0[k + 1] - P.sn_c0[k];
        const int64_t f = P.sn_f[k];
        P.sn_lx_off[k] = lx;
        P.sn_u_off[k] = uu;
        P.sn_su_off[k] = su;
        lx += f * nc;
        uu += (f - nc) * (f - nc);
        su += f - nc;
        P.nnz_l += trapezoid(nc, f);
        for (int64_t c = 0; c < nc; ++c) {
            const double below = static_cast<double>(f - c - 1);
            P.flops += below * (below + 1.0) + below + 1.0;
        }
        P.max_front = std::max<int32_t>(P.max_front, static_cast<int32_t>(f));
    }
    P.sn_lx_off[ns] = lx;
    P.sn_u_off[ns] = uu;
    P.sn_su_off[ns] = su;
    P.lx_size = lx;
    P.u_size = uu;
    P.su_size = su;

    // children, relative maps, levels
    P.sn_child_ptr.assign(ns + 1, 0);
    for (int32_t k = 0; k < ns; ++k)
        if (P.sn_parent[k] >= 0) ++P.sn_child_ptr[P.sn_parent[k] + 1];
    for (int32_t k = 0; k < ns; ++k) P.sn_child_ptr[k + 1] += P.sn_child_ptr[k];
    P.sn_child.assign(P.sn_child_ptr[ns], 0);
    {
        std::vector<int32_t> fill(P.sn_child_ptr.begin(), P.sn_child_ptr.end() - 1);
        for (int32_t k = 0; k < ns; ++k)
            if (P.sn_parent[k] >= 0) P.sn_child[fill[P.sn_parent[k]]++] = k;
    }
    P.sn_relmap.assign(su, 0);
    {
        // 1: a front with below rows has no parent; 2: a row missing from the parent
        std::vector<uint8_t> bad(sn_parts, 0);
        parallel_ranges(ns, sn_parts, [&](int32_t t, int64_t k0, int64_t k1) {
            for (int64_t k = k0; k < k1 && !bad[t]; ++k) {
                const int32_t p = P.sn_parent[k];
                const int64_t nc = P.sn_c0[k + 1] - P.sn_c0[k];
                const int64_t f = P.sn_f[k];
                if (f > nc && p < 0) bad[t] = 1;
                if (p < 0) continue;
                const int32_t* pr = P.sn_rows.data() + P.sn_rows_off[p];
                const int32_t pf = P.sn_f[p];
                for (int64_t r = nc; r < f; ++r) {
                    const int32_t row = P.sn_rows[P.sn_rows_off[k] + r];
                    const int32_t* it = std::lower_bound(pr, pr + pf, row);
                    if (it == pr + pf || *it != row) {
                        bad[t] = 2;
                        break;
                    }
                    P.sn_relmap[P.sn_su_off[k] + (r - nc)] = static_cast<int32_t>(it - pr);
                }
            }
        });
        for (uint8_t b : bad) {  // the first failing range names the error
            if (b == 1) { err = "front has below rows but no parent"; return false; }
            if (b == 2) { err = "child row missing from parent front"; return false; }
        }
    }
    {
        std::vector<int32_t> lvl(ns, 0);
        int32_t maxl = 0;
        for (int32_t k = 0; k < ns; ++k) {  // children precede parents
            for (int32_t c = P.sn_child_ptr[k]; c < P.sn_child_ptr[k + 1]; ++c)
                lvl[k] = std::max(lvl[k], lvl[P.sn_child[c]] + 1);
            maxl = std::max(maxl, lvl[k]);
        }
        P.n_levels = ns ? maxl + 1 : 0;
        P.lvl_ptr.assign(P.n_levels + 1, 0);
        for (int32_t k = 0; k < ns; ++k) ++P.lvl_ptr[lvl[k] + 1];
        for (int32_t l = 0; l < P.n_levels; ++l) P.lvl_ptr[l + 1] += P.lvl_ptr[l];
        P.lvl_sn.assign(ns, 0);
        std::vector<int32_t> fill(P.lvl_ptr.begin(), P.lvl_ptr.end() - 1);
        for (int32_t k = 0; k < ns; ++k) P.lvl_sn[fill[lvl[k]]++] = k;
    }
    // the caller's work that needs only the fronts runs from here on, joined
    // on every way out
    struct Joiner {
        std::thread th;
        ~Joiner() {
            if (th.joinable()) th.join();
        }
    } beside;
    if (alongside && static_cast<int64_t>(n) + m >= kOwnThreadItems) beside.th = std::thread(alongside);
    else if (alongside) alongside();
    const int32_t busy = beside.th.joinable() ? 1 : 0;  // cores taken from the passes below

    // --- RHS gather ------------------------------------------------------------------------
    // Each H entry's permuted column, then the entries by permuted state (a
    // CSR transpose): ranges of entries count per thread, the offsets run
    // state-major then range-minor, so each state's entries stay in
    // ascending order.
    {
        const int64_t nnz = static_cast<int64_t>(P.h_col.size());
        const int32_t ns_ = P.n_state;
        const int32_t parts = host_threads(nnz, 1 << 18, busy);
        P.h_pcol.resize(static_cast<size_t>(nnz));
        std::vector<std::vector<int32_t>> cnt(parts);
        parallel_ranges(nnz, parts, [&](int32_t t, int64_t h0, int64_t h1) {
            auto& c = cnt[t];
            c.assign(static_cast<size_t>(ns_), 0);
            for (int64_t h = h0; h < h1; ++h) {
                const int32_t pc = ps_of_state[P.h_col[h]];
                P.h_pcol[h] = pc;
                ++c[pc];
            }
        });
        // per state: the ranges' first slots relative to the state's start
        P.rhs_ptr.assign(static_cast<size_t>(ns_) + 1, 0);
        parallel_ranges(ns_, host_threads(ns_, 1 << 15, busy), [&](int32_t, int64_t p0, int64_t p1) {
            for (int64_t p = p0; p < p1; ++p) {
                int32_t run = 0;
                for (int32_t t = 0; t < parts; ++t) {
                    const int32_t c = cnt[t][p];
                    cnt[t][p] = run;
                    run += c;
                }
                P.rhs_ptr[p + 1] = run;
            }
        });
        for (int32_t p = 0; p < ns_; ++p) P.rhs_ptr[p + 1] += P.rhs_ptr[p];
        P.rhs_h.resize(nnz);
        parallel_ranges(nnz, parts, [&](int32_t t, int64_t h0, int64_t h1) {
            auto& o = cnt[t];
            for (int64_t h = h0; h < h1; ++h) {
                const int32_t pc = P.h_pcol[h];
                P.rhs_h[P.rhs_ptr[pc] + o[pc]++] = static_cast<int32_t>(h);
            }
        });
    }
    // --- gain assembly targets --------------------------------------------------------
    // Every pair (x, y), x <= y, of H entries of one row contributes to the G
    // entry (lo, hi), lo <= hi their permuted columns, of the front owning
    // column lo.  A front's pairs are generated column by column from the
    // column lists of H (the RHS gather): for each entry of column lo, in
    // ascending row order, the entries of its row at columns >= lo.  They are
    // stably sorted by the entry's local index (row + col * f in the front's
    // panel), and each run of equal indices becomes one target with its pair
    // list; a target gets at most one pair per row, so its pairs are in row
    // order.  Fronts are cut into ranges of about equal pair counts, one host
    // thread each; every front is written at its own offsets, so the plan
    // does not depend on the thread count.
    {
        struct PairRec { int32_t local; int32_t a; int32_t b; };
        const int64_t nnz = static_cast<int64_t>(P.h_col.size());
        int64_t run = 0;
        for (int32_t q = 0; q < m; ++q) {
            const int64_t L = P.h_ptr[q + 1] - P.h_ptr[q];
            run += L * (L + 1) / 2;
        }
        P.pair_a.resize(static_cast<size_t>(run));  // written (first touched) by the workers below
        P.pair_b.resize(static_cast<size_t>(run));
        // ge[h] = entries of h's row at permuted columns >= h's, h included;
        // hrow[h] = h's row range
        const BigVec<int32_t>& hps = P.h_pcol;
        BigVec<int32_t> ge(static_cast<size_t>(nnz));
        struct RowRange { int32_t beg, end; };
        BigVec<RowRange> hrow(static_cast<size_t>(nnz));
        parallel_ranges(m, host_threads(m, 4096, busy), [&](int32_t, int64_t q0, int64_t q1) {
            for (int64_t q = q0; q < q1; ++q) {
                const int32_t h0 = P.h_ptr[q], h1 = P.h_ptr[q + 1];
                for (int32_t x = h0; x < h1; ++x) {
                    int32_t c = 0;
                    for (int32_t y = h0; y < h1; ++y) c += hps[y] >= hps[x];
                    ge[x] = c;
                    hrow[x] = RowRange{h0, h1};
                }
            }
        });
        std::vector<int64_t> fr_off(ns + 1, 0);
        parallel_ranges(ns, host_threads(ns, 2048, busy), [&](int32_t, int64_t k0, int64_t k1) {
            for (int64_t k = k0; k < k1; ++k) {
                int64_t c = 0;
                for (int32_t i = P.rhs_ptr[P.sn_c0[k]]; i < P.rhs_ptr[P.sn_c0[k + 1]]; ++i) c += ge[P.rhs_h[i]];
                fr_off[k + 1] = c;
            }
        });
        for (int32_t k = 0; k < ns; ++k) fr_off[k + 1] += fr_off[k];
        const int32_t nthr = host_threads(run, 1 << 16, busy);
        std::vector<int32_t> fr_cut(nthr + 1, ns);
        fr_cut[0] = 0;
        for (int32_t t = 1, k = 0; t < nthr; ++t) {
            const int64_t goal = run * t / nthr;
            while (k < ns && fr_off[k] < goal) ++k;
            fr_cut[t] = k;
        }
        std::vector<int32_t> ntg(ns, 0);
        std::vector<std::vector<int32_t>> t_local(nthr);
        std::vector<std::vector<int64_t>> t_start(nthr);
        std::vector<uint8_t> bad(nthr, 0);
        parallel_ranges(nthr, nthr, [&](int32_t t, int64_t, int64_t) {
            std::vector<PairRec> rec;
            std::vector<int32_t> hist;
            std::vector<int32_t> where(static_cast<size_t>(P.n_state), -1);  // state -> row in the front
            for (int32_t k = fr_cut[t]; k < fr_cut[t + 1]; ++k) {
                const int32_t f = P.sn_f[k], c0 = P.sn_c0[k], nc = P.sn_c0[k + 1] - c0;
                const int32_t* rows = P.sn_rows.data() + P.sn_rows_off[k];
                for (int32_t r = 0; r < f; ++r) where[rows[r]] = r;
                rec.resize(static_cast<size_t>(fr_off[k + 1] - fr_off[k]));
                size_t nr = 0;
                for (int32_t lo = c0; lo < c0 + nc; ++lo)
                    for (int32_t i = P.rhs_ptr[lo]; i < P.rhs_ptr[lo + 1]; ++i) {
                        const int32_t h = P.rhs_h[i];
                        for (int32_t h2 = hrow[h].beg; h2 < hrow[h].end; ++h2) {
                            const int32_t hi = hps[h2];
                            if (hi < lo) continue;
                            const int32_t r = where[hi];
                            if (r < 0) {  // outside the front's structure
                                bad[t] = 1;
                                return;
                            }
                            rec[nr++] = {r + (lo - c0) * f, std::min(h, h2), std::max(h, h2)};
                        }
                    }
                for (int32_t r = 0; r < f; ++r) where[rows[r]] = -1;
                // stable counting sort by local index (local < f * nc), the
                // targets found in the prefix pass, the pairs scattered into
                // place
                const int32_t range = f * nc;
                const int64_t o = fr_off[k];
                hist.assign(static_cast<size_t>(range) + 1, 0);
                for (const PairRec& x : rec) ++hist[x.local + 1];
                int32_t c = 0;
                for (int32_t v = 0; v < range; ++v) {
                    if (hist[v + 1] > 0) {
                        t_local[t].push_back(v);
                        t_start[t].push_back(o + hist[v]);
                        ++c;
                    }
                    hist[v + 1] += hist[v];
                }
                for (const PairRec& x : rec) {
                    const int64_t at = o + hist[x.local]++;
                    P.pair_a[at] = x.a;
                    P.pair_b[at] = x.b;
                }
                ntg[k] = c;
            }
        });
        for (uint8_t b : bad)
            if (b) {
                err = "gain entry outside the front structure";
                return false;
            }
        P.sn_tgt_ptr.assign(ns + 1, 0);
        for (int32_t k = 0; k < ns; ++k) P.sn_tgt_ptr[k + 1] = P.sn_tgt_ptr[k] + ntg[k];
        const int32_t n_tgt = P.sn_tgt_ptr[ns];
        P.tgt_local.resize(n_tgt);
        P.tgt_pair_ptr.resize(static_cast<size_t>(n_tgt) + 1);
        P.tgt_pair_ptr[n_tgt] = run;
        parallel_ranges(nthr, nthr, [&](int32_t t, int64_t, int64_t) {
            const int32_t g0 = P.sn_tgt_ptr[fr_cut[t]];
            std::copy(t_local[t].begin(), t_local[t].end(), P.tgt_local.begin() + g0);
            std::copy(t_start[t].begin(), t_start[t].end(), P.tgt_pair_ptr.begin() + g0);
        });
    }
    return true;
}


namespace {
template <typename T, typename A, typename B>
void append_shift(std::vector<T, A>& dst, const std::vector<T, B>& src, T shift, bool keep_negative = false) {
    for (T v : src) dst.push_back((keep_negative && v < 0) ? v : static_cast<T>(v + shift));
}
// CSR row pointers: drop the leading 0 of every part after the first.
template <typename T, typename A, typename B>
void append_ptr(std::vector<T, A>& dst, const std::vector<T, B>& src, T shift) {
    if (dst.empty()) dst.push_back(0);
    for (size_t i = 1; i < src.size(); ++i) dst.push_back(static_cast<T>(src[i] + shift));
}
}  // namespace

void merge_plans(const std::vector<const Plan*>& parts, const std::vector<int32_t>& br_count, Plan& M) {
    M = Plan();
    int32_t bus0 = 0, br0 = 0, m0 = 0, st0 = 0, ns0 = 0;
    int32_t y0 = 0, h0 = 0, tg0 = 0;
    int64_t rows0 = 0, su0 = 0, pair0 = 0, lx0 = 0, u0 = 0;
    int32_t maxl = 0;
    for (const Plan* P : parts) maxl = std::max(maxl, P->n_levels);
    for (size_t g = 0; g < parts.size(); ++g) {
        const Plan& P = *parts[g];
        if (g == 0) M.slack = P.slack;
        append_ptr(M.y_ptr, P.y_ptr, y0);
        append_shift(M.y_col, P.y_col, bus0);
        for (int32_t v : P.y_src) M.y_src.push_back(v < 0 ? v : (((v >> 1) + br0) << 1) | (v & 1));
        M.y_hpos_t.insert(M.y_hpos_t.end(), P.y_hpos_t.begin(), P.y_hpos_t.end());
        M.y_hpos_v.insert(M.y_hpos_v.end(), P.y_hpos_v.begin(), P.y_hpos_v.end());
        append_ptr(M.h_ptr, P.h_ptr, h0);
        append_shift(M.h_col, P.h_col, st0);
        append_shift(M.h_row, P.h_row, m0);
        M.m_kind.insert(M.m_kind.end(), P.m_kind.begin(), P.m_kind.end());
        M.m_fpos.insert(M.m_fpos.end(), P.m_fpos.begin(), P.m_fpos.end());
        append_shift(M.bus_perm, P.bus_perm, bus0);
        append_shift(M.bus_ps_theta, P.bus_ps_theta, st0, true);
        append_shift(M.bus_ps_v, P.bus_ps_v, st0, true);
        append_shift(M.state_of_ps, P.state_of_ps, st0);
        append_ptr(M.sn_c0, P.sn_c0, st0);
        M.sn_f.insert(M.sn_f.end(), P.sn_f.begin(), P.sn_f.end());
        append_shift(M.sn_parent, P.sn_parent, ns0, true);
        append_ptr(M.sn_rows_off, P.sn_rows_off, rows0);
        append_shift(M.sn_rows, P.sn_rows, st0);
        append_ptr(M.sn_lx_off, P.sn_lx_off, lx0);
        append_ptr(M.sn_u_off, P.sn_u_off, u0);
        append_ptr(M.sn_su_off, P.sn_su_off, su0);
        append_ptr(M.sn_child_ptr, P.sn_child_ptr, static_cast<int32_t>(M.sn_child.size()));
        append_shift(M.sn_child, P.sn_child, ns0);
        M.sn_relmap.insert(M.sn_relmap.end(), P.sn_relmap.begin(), P.sn_relmap.end());
        append_ptr(M.sn_tgt_ptr, P.sn_tgt_ptr, tg0);
        M.tgt_local.insert(M.tgt_local.end(), P.tgt_local.begin(), P.tgt_local.end());
        append_ptr(M.tgt_pair_ptr, P.tgt_pair_ptr, pair0);
        append_shift(M.pair_a, P.pair_a, h0);
        append_shift(M.pair_b, P.pair_b, h0);
        append_ptr(M.rhs_ptr, P.rhs_ptr, static_cast<int32_t>(M.rhs_h.size()));
        append_shift(M.rhs_h, P.rhs_h, h0);
        append_shift(M.h_pcol, P.h_pcol, st0);
        M.nnz_l += P.nnz_l;
        M.flops += P.flops;
        M.max_front = std::max(M.max_front, P.max_front);
        M.lx_size += P.lx_size;
        M.u_size += P.u_size;
        M.su_size += P.su_size;
        bus0 += P.n_bus;
        br0 += br_count[g];
        m0 += P.n_meas;
        st0 += P.n_state;
        ns0 += P.n_super;
        y0 += static_cast<int32_t>(P.y_col.size());
        h0 += static_cast<int32_t>(P.h_col.size());
        tg0 += static_cast<int32_t>(P.tgt_local.size());
        rows0 += static_cast<int64_t>(P.sn_rows.size());
        su0 += P.su_size;
        pair0 += static_cast<int64_t>(P.pair_a.size());
        lx0 += P.lx_size;
        u0 += P.u_size;
    }
    if (M.y_ptr.empty()) M.y_ptr.push_back(0);
    if (M.h_ptr.empty()) M.h_ptr.push_back(0);
    if (M.sn_c0.empty()) M.sn_c0.push_back(0);
    if (M.sn_rows_off.empty()) M.sn_rows_off.push_back(0);
    if (M.sn_lx_off.empty()) M.sn_lx_off.push_back(0);
    if (M.sn_u_off.empty()) M.sn_u_off.push_back(0);
    if (M.sn_su_off.empty()) M.sn_su_off.push_back(0);
    if (M.sn_child_ptr.empty()) M.sn_child_ptr.push_back(0);
    if (M.sn_tgt_ptr.empty()) M.sn_tgt_ptr.push_back(0);
    if (M.tgt_pair_ptr.empty()) M.tgt_pair_ptr.push_back(0);
    if (M.rhs_ptr.empty()) M.rhs_ptr.push_back(0);
    M.n_bus = bus0;
    M.n_meas = m0;
    M.n_state = st0;
    M.n_super = ns0;
    M.n_levels = maxl;
    M.lvl_ptr.assign(maxl + 1, 0);
    for (int32_t l = 0; l < maxl; ++l) {
        int32_t off = 0;
        for (const Plan* P : parts) {
            if (l < P->n_levels)
                for (int32_t x = P->lvl_ptr[l]; x < P->lvl_ptr[l + 1]; ++x) M.lvl_sn.push_back(P->lvl_sn[x] + off);
            off += P->n_super;
        }
        M.lvl_ptr[l + 1] = static_cast<int32_t>(M.lvl_sn.size());
    }
}

}  // namespace sle_gb300
