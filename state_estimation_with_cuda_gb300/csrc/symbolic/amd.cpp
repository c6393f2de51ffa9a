// Approximate minimum degree ordering on a quotient graph.
//
// Follows the published AMD method (Amestoy, Davis & Duff, "An approximate
// minimum degree ordering algorithm", SIAM J. Matrix Anal. Appl. 17(4), 1996):
// eliminated variables become elements, a variable's degree is bounded by
//   min(n - k, d_old + |Lp \ i|, |A_i \ i| + |Lp \ i| + sum_e |Le \ Lp|),
// indistinguishable variables are merged into supervariables (mass
// elimination) and elements whose variables are all in the new element are
// absorbed.  Ties are broken by bucket order, so the result is deterministic.
//
// Storage is flat: a variable's remaining neighbours are a shrinking range of
// one copy of the adjacency; element lists (Le) are ranges of a bump pool,
// compacted in place; a variable's element list (Ei) is a range of a second
// pool that moves to the pool's end when it outgrows its capacity; the
// members of a supervariable are a linked chain.  Every list keeps the order
// the list-per-node form had, so the ordering is the same.
#include <algorithm>
#include <cstdint>
#include <vector>

namespace sle_gb300 {

std::vector<int32_t> amd_order(int32_t n, const std::vector<int32_t>& ptr, const std::vector<int32_t>& adj) {
    enum : uint8_t { VAR = 0, ELEM = 1, DEAD = 2 };
    std::vector<uint8_t> status(n, VAR);
    std::vector<int32_t> nv(n, 1), deg(n, 0);
    // A: [a_beg, a_beg + a_len) of a_pool (self loops dropped)
    std::vector<int32_t> a_pool;
    a_pool.reserve(adj.size());
    std::vector<int64_t> a_beg(n);
    std::vector<int32_t> a_len(n);
    for (int32_t i = 0; i < n; ++i) {
        a_beg[i] = static_cast<int64_t>(a_pool.size());
        for (int32_t e = ptr[i]; e < ptr[i + 1]; ++e)
            if (adj[e] != i) a_pool.push_back(adj[e]);
        a_len[i] = static_cast<int32_t>(a_pool.size() - a_beg[i]);
        deg[i] = a_len[i];
    }
    // L (elements): [l_beg, l_beg + l_len) of l_pool
    std::vector<int32_t> l_pool;
    l_pool.reserve(adj.size() + static_cast<size_t>(n));
    std::vector<int64_t> l_beg(n, 0);
    std::vector<int32_t> l_len(n, 0);
    // E (variables' elements): [e_beg, e_beg + e_len) of e_pool, capacity e_cap
    std::vector<int32_t> e_pool;
    e_pool.reserve(4 * static_cast<size_t>(n));
    std::vector<int64_t> e_beg(n, 0);
    std::vector<int32_t> e_len(n, 0), e_cap(n, 0);
    auto e_push = [&](int32_t i, int32_t v) {
        if (e_len[i] == e_cap[i]) {
            const int32_t cap = std::max(4, 2 * e_cap[i]);
            const int64_t nb = static_cast<int64_t>(e_pool.size());
            e_pool.resize(e_pool.size() + cap);
            std::copy(e_pool.begin() + e_beg[i], e_pool.begin() + e_beg[i] + e_len[i], e_pool.begin() + nb);
            e_beg[i] = nb;
            e_cap[i] = cap;
        }
        e_pool[e_beg[i] + e_len[i]++] = v;
    };
    // members of supervariable i: chain from m_head[i] to m_tail[i] through m_next
    std::vector<int32_t> m_head(n), m_tail(n), m_next(n, -1);
    for (int32_t i = 0; i < n; ++i) m_head[i] = m_tail[i] = i;

    // Degree buckets (doubly linked lists).
    std::vector<int32_t> head(n + 1, -1), nxt(n, -1), prv(n, -1);
    auto bucket_insert = [&](int32_t i) {
        const int32_t d = std::min(deg[i], n);
        nxt[i] = head[d];
        prv[i] = -1;
        if (head[d] >= 0) prv[head[d]] = i;
        head[d] = i;
    };
    auto bucket_remove = [&](int32_t i) {
        const int32_t d = std::min(deg[i], n);
        if (prv[i] >= 0) nxt[prv[i]] = nxt[i];
        else head[d] = nxt[i];
        if (nxt[i] >= 0) prv[nxt[i]] = prv[i];
        nxt[i] = prv[i] = -1;
    };
    for (int32_t i = n - 1; i >= 0; --i) bucket_insert(i);

    std::vector<int32_t> flag(n, -1), wtag(n, -1), w(n, 0);
    std::vector<int32_t> order;
    order.reserve(n);
    int32_t tag = 0, mindeg = 0, eliminated = 0;
    std::vector<int32_t> Lp;
    std::vector<std::pair<uint64_t, int32_t>> hashes;
    std::vector<int32_t> si, sj, ai, aj, ai2, aj2;

    while (eliminated < n) {
        while (mindeg <= n && head[mindeg] < 0) ++mindeg;
        if (mindeg > n) break;
        const int32_t p = head[mindeg];
        bucket_remove(p);
        ++tag;
        // --- new element Lp -------------------------------------------------------
        Lp.clear();
        flag[p] = tag;
        for (int32_t x = 0; x < e_len[p]; ++x) {
            const int32_t e = e_pool[e_beg[p] + x];
            if (status[e] != ELEM) continue;
            for (int32_t y = 0; y < l_len[e]; ++y) {
                const int32_t i = l_pool[l_beg[e] + y];
                if (status[i] == VAR && flag[i] != tag) {
                    flag[i] = tag;
                    Lp.push_back(i);
                }
            }
            status[e] = DEAD;  // absorbed into p
            l_len[e] = 0;
        }
        for (int32_t x = 0; x < a_len[p]; ++x) {
            const int32_t i = a_pool[a_beg[p] + x];
            if (status[i] == VAR && flag[i] != tag) {
                flag[i] = tag;
                Lp.push_back(i);
            }
        }
        a_len[p] = 0;
        e_len[p] = 0;
        status[p] = ELEM;
        for (int32_t mb = m_head[p]; mb >= 0; mb = m_next[mb]) order.push_back(mb);
        eliminated += nv[p];
        int32_t lp_w = 0;
        for (int32_t i : Lp) {
            bucket_remove(i);
            lp_w += nv[i];
        }
        // --- |Le \ Lp| for elements adjacent to Lp -------------------------------
        ++tag;  // second tag for w
        const int32_t wt = tag;
        for (int32_t i : Lp) {
            for (int32_t x = 0; x < e_len[i]; ++x) {
                const int32_t e = e_pool[e_beg[i] + x];
                if (status[e] != ELEM) continue;
                if (wtag[e] != wt) {
                    // weighted size of L[e], compacting dead entries
                    int32_t sz = 0, k2 = 0;
                    int32_t* le = l_pool.data() + l_beg[e];
                    for (int32_t y = 0; y < l_len[e]; ++y) {
                        const int32_t v = le[y];
                        if (status[v] == VAR) {
                            le[k2++] = v;
                            sz += nv[v];
                        }
                    }
                    l_len[e] = k2;
                    w[e] = sz;
                    wtag[e] = wt;
                }
                w[e] -= nv[i];
            }
        }
        // --- update variables in Lp ---------------------------------------------------
        // flag[] == tag - 1 marks membership in Lp.
        const int32_t lp_tag = tag - 1;
        for (int32_t i : Lp) {
            int32_t* ei = e_pool.data() + e_beg[i];
            int32_t k2 = 0, ext = 0;
            for (int32_t x = 0; x < e_len[i]; ++x) {
                const int32_t e = ei[x];
                if (status[e] != ELEM || e == p) continue;
                if (wtag[e] == wt && w[e] <= 0) {  // Le subset of Lp: absorb into p
                    status[e] = DEAD;
                    l_len[e] = 0;
                    continue;
                }
                ei[k2++] = e;
                ext += (wtag[e] == wt) ? w[e] : 0;
            }
            e_len[i] = k2;
            e_push(i, p);
            int32_t* ap = a_pool.data() + a_beg[i];
            int32_t aw = 0;
            k2 = 0;
            for (int32_t x = 0; x < a_len[i]; ++x) {
                const int32_t v = ap[x];
                if (status[v] != VAR || v == p || flag[v] == lp_tag) continue;
                ap[k2++] = v;
                aw += nv[v];
            }
            a_len[i] = k2;
            const int32_t remaining = n - eliminated;
            const int32_t d1 = deg[i] + lp_w - nv[i];
            const int32_t d2 = aw + (lp_w - nv[i]) + ext;
            deg[i] = std::max(0, std::min(std::min(d1, d2), remaining - nv[i]));
        }
        // --- supervariable detection among Lp ------------------------------------------
        hashes.clear();
        for (int32_t i : Lp) {
            if (status[i] != VAR) continue;
            uint64_t h = 0;
            for (int32_t x = 0; x < e_len[i]; ++x)
                h += static_cast<uint64_t>(e_pool[e_beg[i] + x]) * 0x9E3779B97F4A7C15ULL + 1;
            for (int32_t x = 0; x < a_len[i]; ++x)
                h += static_cast<uint64_t>(a_pool[a_beg[i] + x]) * 0xC2B2AE3D27D4EB4FULL + 7;
            hashes.emplace_back(h, i);
        }
        std::sort(hashes.begin(), hashes.end());
        for (size_t a = 0; a < hashes.size();) {
            size_t b = a;
            while (b < hashes.size() && hashes[b].first == hashes[a].first) ++b;
            for (size_t x = a; x + 1 < b; ++x) {  // a variable alone in its hash group has no twin
                const int32_t i = hashes[x].second;
                if (status[i] != VAR) continue;
                si.assign(e_pool.begin() + e_beg[i], e_pool.begin() + e_beg[i] + e_len[i]);
                std::sort(si.begin(), si.end());
                ai.assign(a_pool.begin() + a_beg[i], a_pool.begin() + a_beg[i] + a_len[i]);
                std::sort(ai.begin(), ai.end());
                for (size_t y = x + 1; y < b; ++y) {
                    const int32_t j = hashes[y].second;
                    if (status[j] != VAR) continue;
                    if (e_len[j] != e_len[i]) continue;
                    sj.assign(e_pool.begin() + e_beg[j], e_pool.begin() + e_beg[j] + e_len[j]);
                    std::sort(sj.begin(), sj.end());
                    if (si != sj) continue;
                    aj.assign(a_pool.begin() + a_beg[j], a_pool.begin() + a_beg[j] + a_len[j]);
                    std::sort(aj.begin(), aj.end());
                    ai2.clear();
                    aj2.clear();
                    for (int32_t v : ai) if (v != j) ai2.push_back(v);
                    for (int32_t v : aj) if (v != i) aj2.push_back(v);
                    if (ai2 != aj2) continue;
                    // merge j into i
                    nv[i] += nv[j];
                    deg[i] = std::max(0, deg[i] - nv[j]);
                    nv[j] = 0;
                    status[j] = DEAD;
                    m_next[m_tail[i]] = m_head[j];
                    m_tail[i] = m_tail[j];
                    a_len[j] = 0;
                    e_len[j] = 0;
                    ai.erase(std::remove(ai.begin(), ai.end(), j), ai.end());
                    int32_t* ap = a_pool.data() + a_beg[i];
                    a_len[i] = static_cast<int32_t>(std::remove(ap, ap + a_len[i], j) - ap);
                }
            }
            a = b;
        }
        // --- finalise element p and reinsert variables ------------------------------------
        l_beg[p] = static_cast<int64_t>(l_pool.size());
        for (int32_t i : Lp) {
            if (status[i] != VAR) continue;
            l_pool.push_back(i);
            bucket_insert(i);
            mindeg = std::min(mindeg, std::min(deg[i], n));
        }
        l_len[p] = static_cast<int32_t>(l_pool.size() - l_beg[p]);
    }
    return order;
}

}  // namespace sle_gb300
