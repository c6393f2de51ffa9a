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
// one copy of the adjacency; element lists (Le) are ranges of a bump pool;
// a variable's element list (Ei) is a range of a second
// pool that moves to the pool's end when it outgrows its capacity; the
// members of a supervariable are a linked chain.  Every list keeps the order
// the list-per-node form had, so the ordering is the same.
//
// The new element Lp of a pivot is the exact set of variables adjacent to it
// in the elimination graph, so, expanded to the members of its
// supervariables, it is the below-diagonal structure of the L column of the
// pivot's last member (and, with the later members, of every member).  The
// optional trace keeps it, which gives the elimination tree and the column
// counts without a second symbolic pass.
#include "amd.h"

#include <algorithm>

namespace sle_gb300 {

std::vector<int32_t> amd_order(int32_t n, const std::vector<int32_t>& ptr, const std::vector<int32_t>& adj,
                               AmdTrace* trace) {
    if (trace) {
        trace->piv_end.clear();
        trace->lp_ptr.assign(1, 0);
        trace->lp.clear();
        trace->lp.reserve(adj.size());
    }
    enum : uint8_t { VAR = 0, ELEM = 1, DEAD = 2 };
    std::vector<uint8_t> status(n, VAR);
    // The per-variable (and per-element) fields the elimination loop reads
    // together share one cache line: bus numbers carry no locality, so every
    // list entry visited is a random access.
    struct Node {
        int64_t a_beg, e_beg, l_beg;     // list starts in a_pool, e_pool, l_pool
        int32_t a_len, e_len, e_cap, l_len;
        int32_t nv, deg, flag, wtag;
        int32_t w, l_w;
    };
    static_assert(sizeof(Node) == 64, "one cache line per node");
    std::vector<Node> nd(n, Node{0, 0, 0, 0, 0, 0, 0, 1, 0, -1, -1, 0, 0});
    // A: [a_beg, a_beg + a_len) of a_pool (self loops dropped)
    std::vector<int32_t> a_pool;
    a_pool.reserve(adj.size());
    for (int32_t i = 0; i < n; ++i) {
        nd[i].a_beg = static_cast<int64_t>(a_pool.size());
        for (int32_t e = ptr[i]; e < ptr[i + 1]; ++e)
            if (adj[e] != i) a_pool.push_back(adj[e]);
        nd[i].a_len = static_cast<int32_t>(a_pool.size() - nd[i].a_beg);
        nd[i].deg = nd[i].a_len;
    }
    // L (elements): [l_beg, l_beg + l_len) of l_pool
    std::vector<int32_t> l_pool;
    l_pool.reserve(adj.size() + static_cast<size_t>(n));
    // l_w of element e = sum of nv over its live variables.  It holds while e lives: a
    // variable leaves Le only by elimination, which absorbs e, or by merging
    // into a twin that is in Le too.  Dead entries stay in Le until e dies.
    // E (variables' elements): [e_beg, e_beg + e_len) of e_pool, capacity e_cap
    std::vector<int32_t> e_pool;
    e_pool.reserve(4 * static_cast<size_t>(n));
    auto e_push = [&](int32_t i, int32_t v) {
        if (nd[i].e_len == nd[i].e_cap) {
            const int32_t cap = std::max(4, 2 * nd[i].e_cap);
            const int64_t nb = static_cast<int64_t>(e_pool.size());
            e_pool.resize(e_pool.size() + cap);
            std::copy(e_pool.begin() + nd[i].e_beg, e_pool.begin() + nd[i].e_beg + nd[i].e_len, e_pool.begin() + nb);
            nd[i].e_beg = nb;
            nd[i].e_cap = cap;
        }
        e_pool[nd[i].e_beg + nd[i].e_len++] = v;
    };
    // members of supervariable i: chain from mc[i].head to mc[i].tail through .next
    struct Chain { int32_t head, tail, next; };
    std::vector<Chain> mc(n);
    for (int32_t i = 0; i < n; ++i) mc[i] = Chain{i, i, -1};

    // Degree buckets (doubly linked lists).
    struct Link { int32_t nxt, prv; };  // one line per node for both neighbours
    std::vector<int32_t> head(n + 1, -1);
    std::vector<Link> lk(n, Link{-1, -1});
    auto bucket_insert = [&](int32_t i) {
        const int32_t d = std::min(nd[i].deg, n);
        lk[i].nxt = head[d];
        lk[i].prv = -1;
        if (head[d] >= 0) lk[head[d]].prv = i;
        head[d] = i;
    };
    auto bucket_remove = [&](int32_t i) {
        const int32_t d = std::min(nd[i].deg, n);
        const Link l = lk[i];
        if (l.prv >= 0) lk[l.prv].nxt = l.nxt;
        else head[d] = l.nxt;
        if (l.nxt >= 0) lk[l.nxt].prv = l.prv;
        lk[i] = Link{-1, -1};
    };
    for (int32_t i = n - 1; i >= 0; --i) bucket_insert(i);

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
        nd[p].flag = tag;
        // (list lengths and starts are read once: the loops store only into
        // other nodes)
        const int32_t* ep = e_pool.data() + nd[p].e_beg;
        for (int32_t x = 0, ne = nd[p].e_len; x < ne; ++x) {
            const int32_t e = ep[x];
            if (status[e] != ELEM) continue;
            const int32_t* le = l_pool.data() + nd[e].l_beg;
            for (int32_t y = 0, nl = nd[e].l_len; y < nl; ++y) {
                const int32_t i = le[y];
                if (status[i] == VAR && nd[i].flag != tag) {
                    nd[i].flag = tag;
                    Lp.push_back(i);
                }
            }
            status[e] = DEAD;  // absorbed into p
            nd[e].l_len = 0;
        }
        const int32_t* pa = a_pool.data() + nd[p].a_beg;
        for (int32_t x = 0, na = nd[p].a_len; x < na; ++x) {
            const int32_t i = pa[x];
            if (status[i] == VAR && nd[i].flag != tag) {
                nd[i].flag = tag;
                Lp.push_back(i);
            }
        }
        nd[p].a_len = 0;
        nd[p].e_len = 0;
        status[p] = ELEM;
        for (int32_t mb = mc[p].head; mb >= 0; mb = mc[mb].next) order.push_back(mb);
        eliminated += nd[p].nv;
        int32_t lp_w = 0;
        for (int32_t i : Lp) {
            bucket_remove(i);
            lp_w += nd[i].nv;
            __builtin_prefetch(&e_pool[nd[i].e_beg]);
            __builtin_prefetch(&a_pool[nd[i].a_beg]);
        }
        // --- |Le \ Lp| for elements adjacent to Lp -------------------------------
        ++tag;  // second tag for w
        const int32_t wt = tag;
        for (int32_t i : Lp) {
            const Node ni = nd[i];
            const int32_t* ei = e_pool.data() + ni.e_beg;
            for (int32_t x = 0; x < ni.e_len; ++x) {
                const int32_t e = ei[x];
                if (status[e] != ELEM) continue;
                if (nd[e].wtag != wt) {
                    nd[e].w = nd[e].l_w;
                    nd[e].wtag = wt;
                }
                nd[e].w -= ni.nv;
            }
            // the next pass reads the nodes of i's remaining neighbours
            const int32_t* ap = a_pool.data() + ni.a_beg;
            for (int32_t x = 0; x < ni.a_len; ++x) __builtin_prefetch(&nd[ap[x]]);
        }
        // --- update variables in Lp ---------------------------------------------------
        // flag == tag - 1 marks membership in Lp.
        const int32_t lp_tag = tag - 1;
        for (int32_t i : Lp) {
            int32_t* ei = e_pool.data() + nd[i].e_beg;
            int32_t k2 = 0, ext = 0;
            for (int32_t x = 0, ne = nd[i].e_len; x < ne; ++x) {
                const int32_t e = ei[x];
                if (status[e] != ELEM || e == p) continue;
                if (nd[e].wtag == wt && nd[e].w <= 0) {  // Le subset of Lp: absorb into p
                    status[e] = DEAD;
                    nd[e].l_len = 0;
                    continue;
                }
                ei[k2++] = e;
                ext += (nd[e].wtag == wt) ? nd[e].w : 0;
            }
            nd[i].e_len = k2;
            e_push(i, p);
            int32_t* ap = a_pool.data() + nd[i].a_beg;
            int32_t aw = 0;
            k2 = 0;
            for (int32_t x = 0, na = nd[i].a_len; x < na; ++x) {
                const int32_t v = ap[x];
                if (status[v] != VAR || v == p || nd[v].flag == lp_tag) continue;
                ap[k2++] = v;
                aw += nd[v].nv;
            }
            nd[i].a_len = k2;
            const int32_t remaining = n - eliminated;
            const int32_t d1 = nd[i].deg + lp_w - nd[i].nv;
            const int32_t d2 = aw + (lp_w - nd[i].nv) + ext;
            nd[i].deg = std::max(0, std::min(std::min(d1, d2), remaining - nd[i].nv));
        }
        // --- supervariable detection among Lp ------------------------------------------
        hashes.clear();
        for (int32_t i : Lp) {
            if (status[i] != VAR) continue;
            uint64_t h = 0;
            for (int32_t x = 0; x < nd[i].e_len; ++x)
                h += static_cast<uint64_t>(e_pool[nd[i].e_beg + x]) * 0x9E3779B97F4A7C15ULL + 1;
            for (int32_t x = 0; x < nd[i].a_len; ++x)
                h += static_cast<uint64_t>(a_pool[nd[i].a_beg + x]) * 0xC2B2AE3D27D4EB4FULL + 7;
            hashes.emplace_back(h, i);
        }
        std::sort(hashes.begin(), hashes.end());
        for (size_t a = 0; a < hashes.size();) {
            size_t b = a;
            while (b < hashes.size() && hashes[b].first == hashes[a].first) ++b;
            for (size_t x = a; x + 1 < b; ++x) {  // a variable alone in its hash group has no twin
                const int32_t i = hashes[x].second;
                if (status[i] != VAR) continue;
                si.assign(e_pool.begin() + nd[i].e_beg, e_pool.begin() + nd[i].e_beg + nd[i].e_len);
                std::sort(si.begin(), si.end());
                ai.assign(a_pool.begin() + nd[i].a_beg, a_pool.begin() + nd[i].a_beg + nd[i].a_len);
                std::sort(ai.begin(), ai.end());
                for (size_t y = x + 1; y < b; ++y) {
                    const int32_t j = hashes[y].second;
                    if (status[j] != VAR) continue;
                    if (nd[j].e_len != nd[i].e_len) continue;
                    sj.assign(e_pool.begin() + nd[j].e_beg, e_pool.begin() + nd[j].e_beg + nd[j].e_len);
                    std::sort(sj.begin(), sj.end());
                    if (si != sj) continue;
                    aj.assign(a_pool.begin() + nd[j].a_beg, a_pool.begin() + nd[j].a_beg + nd[j].a_len);
                    std::sort(aj.begin(), aj.end());
                    ai2.clear();
                    aj2.clear();
                    for (int32_t v : ai) if (v != j) ai2.push_back(v);
                    for (int32_t v : aj) if (v != i) aj2.push_back(v);
                    if (ai2 != aj2) continue;
                    // merge j into i
                    nd[i].nv += nd[j].nv;
                    nd[i].deg = std::max(0, nd[i].deg - nd[j].nv);
                    nd[j].nv = 0;
                    status[j] = DEAD;
                    mc[mc[i].tail].next = mc[j].head;
                    mc[i].tail = mc[j].tail;
                    nd[j].a_len = 0;
                    nd[j].e_len = 0;
                    ai.erase(std::remove(ai.begin(), ai.end(), j), ai.end());
                    int32_t* ap = a_pool.data() + nd[i].a_beg;
                    nd[i].a_len = static_cast<int32_t>(std::remove(ap, ap + nd[i].a_len, j) - ap);
                }
            }
            a = b;
        }
        // --- finalise element p and reinsert variables ------------------------------------
        nd[p].l_beg = static_cast<int64_t>(l_pool.size());
        for (int32_t i : Lp) {
            if (status[i] != VAR) continue;
            l_pool.push_back(i);
            nd[p].l_w += nd[i].nv;
            bucket_insert(i);
            mindeg = std::min(mindeg, std::min(nd[i].deg, n));
        }
        nd[p].l_len = static_cast<int32_t>(l_pool.size() - nd[p].l_beg);
        if (trace) {
            trace->piv_end.push_back(eliminated);
            for (int64_t y = nd[p].l_beg; y < nd[p].l_beg + nd[p].l_len; ++y)
                for (int32_t mb = mc[l_pool[y]].head; mb >= 0; mb = mc[mb].next) trace->lp.push_back(mb);
            trace->lp_ptr.push_back(static_cast<int64_t>(trace->lp.size()));
        }
    }
    return order;
}

}  // namespace sle_gb300
