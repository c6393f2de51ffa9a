// Approximate minimum degree ordering on a quotient graph.
//
// Follows the published AMD method (Amestoy, Davis & Duff, "An approximate
// minimum degree ordering algorithm", SIAM J. Matrix Anal. Appl. 17(4), 1996):
// eliminated variables become elements, a variable's degree is bounded by
//   min(n - k, d_old + |Lp \ i|, |A_i \ i| + |Lp \ i| + sum_e |Le \ Lp|),
// indistinguishable variables are merged into supervariables (mass
// elimination) and elements whose variables are all in the new element are
// absorbed.  Written with explicit per-node lists rather than AMD's in-place
// workspace; ties are broken by bucket order, so the result is deterministic.
#include <algorithm>
#include <cstdint>
#include <vector>

namespace sle_gb300 {

std::vector<int32_t> amd_order(int32_t n, const std::vector<int32_t>& ptr, const std::vector<int32_t>& adj) {
    enum : uint8_t { VAR = 0, ELEM = 1, DEAD = 2 };
    std::vector<uint8_t> status(n, VAR);
    std::vector<int32_t> nv(n, 1), deg(n, 0);
    std::vector<std::vector<int32_t>> A(n), E(n), L(n), members(n);
    for (int32_t i = 0; i < n; ++i) {
        A[i].assign(adj.begin() + ptr[i], adj.begin() + ptr[i + 1]);
        A[i].erase(std::remove(A[i].begin(), A[i].end(), i), A[i].end());
        deg[i] = static_cast<int32_t>(A[i].size());
        members[i].push_back(i);
    }
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

    while (eliminated < n) {
        while (mindeg <= n && head[mindeg] < 0) ++mindeg;
        if (mindeg > n) break;
        const int32_t p = head[mindeg];
        bucket_remove(p);
        ++tag;
        // --- new element Lp -------------------------------------------------------
        Lp.clear();
        flag[p] = tag;
        for (int32_t e : E[p]) {
            if (status[e] != ELEM) continue;
            for (int32_t i : L[e]) {
                if (status[i] == VAR && flag[i] != tag) {
                    flag[i] = tag;
                    Lp.push_back(i);
                }
            }
            status[e] = DEAD;  // absorbed into p
            std::vector<int32_t>().swap(L[e]);
        }
        for (int32_t i : A[p]) {
            if (status[i] == VAR && flag[i] != tag) {
                flag[i] = tag;
                Lp.push_back(i);
            }
        }
        std::vector<int32_t>().swap(A[p]);
        std::vector<int32_t>().swap(E[p]);
        status[p] = ELEM;
        for (int32_t m : members[p]) order.push_back(m);
        eliminated += nv[p];
        std::vector<int32_t>().swap(members[p]);
        int32_t lp_w = 0;
        for (int32_t i : Lp) {
            bucket_remove(i);
            lp_w += nv[i];
        }
        // --- |Le \ Lp| for elements adjacent to Lp -------------------------------
        ++tag;  // second tag for w
        const int32_t wt = tag;
        for (int32_t i : Lp) {
            for (int32_t e : E[i]) {
                if (status[e] != ELEM) continue;
                if (wtag[e] != wt) {
                    // weighted size of L[e], compacting dead entries
                    int32_t sz = 0;
                    auto& le = L[e];
                    size_t k2 = 0;
                    for (int32_t v : le)
                        if (status[v] == VAR) {
                            le[k2++] = v;
                            sz += nv[v];
                        }
                    le.resize(k2);
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
            auto& ei = E[i];
            size_t k2 = 0;
            int32_t ext = 0;
            for (int32_t e : ei) {
                if (status[e] != ELEM || e == p) continue;
                if (wtag[e] == wt && w[e] <= 0) {  // Le subset of Lp: absorb into p
                    status[e] = DEAD;
                    std::vector<int32_t>().swap(L[e]);
                    continue;
                }
                ei[k2++] = e;
                ext += (wtag[e] == wt) ? w[e] : 0;
            }
            ei.resize(k2);
            ei.push_back(p);
            auto& ai = A[i];
            k2 = 0;
            int32_t aw = 0;
            for (int32_t v : ai) {
                if (status[v] != VAR || v == p || flag[v] == lp_tag) continue;
                ai[k2++] = v;
                aw += nv[v];
            }
            ai.resize(k2);
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
            for (int32_t e : E[i]) h += static_cast<uint64_t>(e) * 0x9E3779B97F4A7C15ULL + 1;
            for (int32_t v : A[i]) h += static_cast<uint64_t>(v) * 0xC2B2AE3D27D4EB4FULL + 7;
            hashes.emplace_back(h, i);
        }
        std::sort(hashes.begin(), hashes.end());
        std::vector<int32_t> si, sj;
        for (size_t a = 0; a < hashes.size();) {
            size_t b = a;
            while (b < hashes.size() && hashes[b].first == hashes[a].first) ++b;
            for (size_t x = a; x + 1 < b; ++x) {  // a variable alone in its hash group has no twin
                const int32_t i = hashes[x].second;
                if (status[i] != VAR) continue;
                si.assign(E[i].begin(), E[i].end());
                std::sort(si.begin(), si.end());
                std::vector<int32_t> ai(A[i].begin(), A[i].end());
                std::sort(ai.begin(), ai.end());
                for (size_t y = x + 1; y < b; ++y) {
                    const int32_t j = hashes[y].second;
                    if (status[j] != VAR) continue;
                    if (E[j].size() != E[i].size()) continue;
                    sj.assign(E[j].begin(), E[j].end());
                    std::sort(sj.begin(), sj.end());
                    if (si != sj) continue;
                    std::vector<int32_t> aj(A[j].begin(), A[j].end());
                    std::sort(aj.begin(), aj.end());
                    std::vector<int32_t> ai2, aj2;
                    for (int32_t v : ai) if (v != j) ai2.push_back(v);
                    for (int32_t v : aj) if (v != i) aj2.push_back(v);
                    if (ai2 != aj2) continue;
                    // merge j into i
                    nv[i] += nv[j];
                    deg[i] = std::max(0, deg[i] - nv[j]);
                    nv[j] = 0;
                    status[j] = DEAD;
                    members[i].insert(members[i].end(), members[j].begin(), members[j].end());
                    std::vector<int32_t>().swap(members[j]);
                    std::vector<int32_t>().swap(A[j]);
                    std::vector<int32_t>().swap(E[j]);
                    ai.erase(std::remove(ai.begin(), ai.end(), j), ai.end());
                    A[i].erase(std::remove(A[i].begin(), A[i].end(), j), A[i].end());
                }
            }
            a = b;
        }
        // --- finalise element p and reinsert variables ------------------------------------
        auto& lpe = L[p];
        lpe.clear();
        for (int32_t i : Lp) {
            if (status[i] != VAR) continue;
            lpe.push_back(i);
            bucket_insert(i);
            mindeg = std::min(mindeg, std::min(deg[i], n));
        }
    }
    return order;
}

}  // namespace sle_gb300
