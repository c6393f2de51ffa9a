// Network-side kernels: branch admittances, Ybus assembly, the fused
// measurement evaluation (h(x), residual, weights, Jacobian values), the
// gain right-hand side, state update / convergence and the result pass.
#include "kernels.cuh"

#include <cfloat>

namespace sle_gb300 {
namespace {

constexpr double kEps = 1e-12;   // SLE_REAL_EPSILON of the FP64 build (sle_types.cuh:62)
constexpr int kBlock = 256;

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__device__ __forceinline__ double warp_max(double v) {
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_down_sync(0xffffffffu, v, o));
    return v;
}

// Deterministic block sum (fixed tree), result valid in thread 0.
__device__ double block_sum(double v, double* sh) {
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    v = (threadIdx.x < (blockDim.x >> 5)) ? sh[lane] : 0.0;
    if (wid == 0) v = warp_sum(v);
    __syncthreads();
    return v;
}
__device__ double block_max(double v, double* sh) {
    v = warp_max(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) sh[wid] = v;
    __syncthreads();
    v = (threadIdx.x < (blockDim.x >> 5)) ? sh[lane] : 0.0;
    if (wid == 0) v = warp_max(v);
    __syncthreads();
    return v;
}

// a1: per-branch series admittance and charging split
// (network_model.cu:595-612 / sparse_matrix.cu:321-355).
__global__ void k_admittance(DevNet net) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= net.n_branch) return;
    const double r = net.br_r[k], x = net.br_x[k], bt = net.br_bch[k], a = net.br_tap[k];
    double den = r * r + x * x;
    if (den < kEps) den = kEps;
    net.br_g[k] = r / den;
    net.br_b[k] = -x / den;
    net.br_bsf[k] = bt / (2.0 * a * a);
    net.br_bst[k] = bt / 2.0;
    const double A = fmax(a, kEps), ia = 1.0 / A;
    net.br_itap[k] = ia;
    net.br_itap2[k] = 1.0 / (A * A);
}

// a2: Ybus values on the canonical pattern, one thread per bus row; the
// diagonal accumulates the row's branch contributions in entry order
// (sparse_matrix.cu:410-492 without floating-point atomics).
__global__ void k_ybus(DevNet net) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= net.n_bus) return;
    const int e0 = net.y_ptr[i], e1 = net.y_ptr[i + 1];
    double dg = 0.0, db = 0.0;
    for (int e = e0 + 1; e < e1; ++e) {
        const int src = net.y_src[e];
        const int k = src >> 1, end = src & 1;
        // an open branch in the pattern (batch patterns keep every branch)
        // contributes nothing
        const double on = net.br_closed[k] ? 1.0 : 0.0;
        const double g = net.br_g[k] * on, b = net.br_b[k] * on;
        const double a = fmax(net.br_tap[k], kEps);
        const double phi = net.br_shift[k];
        double sph, cph;
        sincos(phi, &sph, &cph);
        const double inv_a = 1.0 / a;
        if (end == 0) {  // row = from bus: Y_ij = -(g+jb) e^{-j phi} / a
            net.y_g[e] = -(g * cph + b * sph) * inv_a;
            net.y_b[e] = -(-g * sph + b * cph) * inv_a;
            dg += g / (a * a);
            db += b / (a * a) + net.br_bsf[k] * on;
        } else {         // row = to bus: Y_ji = -(g+jb) e^{+j phi} / a
            net.y_g[e] = -(g * cph - b * sph) * inv_a;
            net.y_b[e] = -(g * sph + b * cph) * inv_a;
            dg += g;
            db += b + net.br_bst[k] * on;
        }
    }
    net.y_g[e0] = dg;
    net.y_b[e0] = db;
}

struct FlowTerms {
    double val;
    double d[4];  // theta_i, V_i, theta_j, V_j
};

// a4 + a8 flow rows: value of P/Q at one end and its derivatives, given
// s, c = sin, cos of theta_i - theta_j - shift.
__device__ FlowTerms flow_terms_sc(const DevNet& net, const double* v, int k, bool is_q, bool to_end, bool exact,
                                   double s, double c) {
    const int i = net.br_from[k], j = net.br_to[k];
    const double Vi = v[i], Vj = v[j];
    const double g = net.br_g[k], b = net.br_b[k];
    // 1 / a and 1 / a^2 of the tap a (clamped as the reference clamps it),
    // computed once per branch: the rows multiply instead of dividing
    const double inv = net.br_itap[k], ia2 = net.br_itap2[k];
    const double on = net.br_closed[k] ? 1.0 : 0.0;
    const double vv = Vi * Vj * inv;
    FlowTerms f;
    if (!is_q && !to_end) {
        f.val = Vi * Vi * ia2 * g - vv * (g * c + b * s);
        f.d[0] = vv * (g * s - b * c);
        f.d[1] = 2.0 * Vi * ia2 * g - Vj * inv * (g * c + b * s);
        f.d[2] = -f.d[0];
        f.d[3] = -Vi * inv * (g * c + b * s);
    } else if (is_q && !to_end) {
        const double bsf = net.br_bsf[k];
        f.val = -(Vi * Vi * ia2) * (b + bsf) - vv * (g * s - b * c);
        f.d[0] = -vv * (g * c + b * s);
        f.d[1] = (exact ? -2.0 * Vi * (b + bsf) * ia2 : -2.0 * Vi * b * ia2) - Vj * inv * (g * s - b * c);
        f.d[2] = -f.d[0];
        f.d[3] = -Vi * inv * (g * s - b * c);
    } else if (!is_q && to_end) {
        f.val = Vj * Vj * g - vv * (g * c - b * s);
        // exact: dP_t/dtheta_i = (ViVj/a)(g s + b c); the reference flips the sign.
        f.d[0] = exact ? vv * (g * s + b * c) : vv * (-g * s - b * c);
        f.d[1] = -Vj * inv * (g * c - b * s);
        f.d[2] = -f.d[0];
        f.d[3] = 2.0 * Vj * g - Vi * inv * (g * c - b * s);
    } else {
        const double bst = net.br_bst[k];
        f.val = -Vj * Vj * (b + bst) + vv * (g * s + b * c);
        f.d[0] = vv * (g * c - b * s);
        f.d[1] = Vj * inv * (g * s + b * c);
        f.d[2] = -f.d[0];
        f.d[3] = (exact ? -2.0 * Vj * (b + bst) : -2.0 * Vj * b) + Vi * inv * (g * s + b * c);
    }
    f.val *= on;
    if (exact) {
        for (int x = 0; x < 4; ++x) f.d[x] *= on;
    }
    return f;
}

__device__ FlowTerms flow_terms(const DevNet& net, const double* v, const double* th, int k, bool is_q,
                                bool to_end, bool exact) {
    double s, c;
    sincos(th[net.br_from[k]] - th[net.br_to[k]] - net.br_shift[k], &s, &c);
    return flow_terms_sc(net, v, k, is_q, to_end, exact, s, c);
}

// sin and cos of theta_i - theta_j from the buses' (cos, sin): four FMAs in
// place of an FP64 sincos per use (the evaluation meets each angle difference
// in up to eight rows); absolute error a few ulps of 1.
__device__ __forceinline__ void angle_diff(const double2 a, const double2 b, double* s, double* c) {
    *c = a.x * b.x + a.y * b.y;
    *s = a.y * b.x - a.x * b.y;
}

// sin and cos of theta_i - theta_j - shift of branch k.
__device__ __forceinline__ void branch_angle(const DevNet& net, const double2* cs, int k, double* s, double* c) {
    angle_diff(cs[net.br_from[k]], cs[net.br_to[k]], s, c);
    const double phi = net.br_shift[k];
    if (phi != 0.0) {
        double sp, cp;
        sincos(phi, &sp, &cp);
        const double c2 = *c * cp + *s * sp;
        *s = *s * cp - *c * sp;
        *c = c2;
    }
}

__device__ __forceinline__ FlowTerms flow_terms_cs(const DevNet& net, const double* v, const double2* cs, int k,
                                                   bool is_q, bool to_end, bool exact) {
    double s, c;
    branch_angle(net, cs, k, &s, &c);
    return flow_terms_sc(net, v, k, is_q, to_end, exact, s, c);
}

// cos and sin of every bus angle of the grids being evaluated.
__global__ void k_bus_trig(DevNet net, DevWork w, SolveParams sp) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= net.n_bus) return;
    if (net.bus_grid) {
        const uint32_t gf = w.grid_flags[net.bus_grid[i]];
        if ((gf & sp.skip_flags) || (gf & sp.need_flags) != sp.need_flags) return;
    }
    double s, c;
    sincos(w.th[i], &s, &c);
    w.bus_cs[i] = make_double2(c, s);
}

__device__ __forceinline__ void put_flow(double* hrow, int fpos, const double d[4]) {
    for (int x = 0; x < 4; ++x) {
        const int p = (fpos >> (8 * x)) & 0xFF;
        if (p != 0xFF) hrow[p] += d[x];
    }
}

// a3/a6/a7/a8/a9 fused: one thread per measurement row.
// P and Q flow at one end of branch k from the same angle difference: the
// two rows' values and derivatives with the expressions of flow_terms_sc.
__device__ __forceinline__ void flow_terms_pq(const DevNet& net, const double* v, int k, bool to_end, bool exact,
                                              double s, double c, FlowTerms& P, FlowTerms& Q) {
    const int i = net.br_from[k], j = net.br_to[k];
    const double Vi = v[i], Vj = v[j];
    const double g = net.br_g[k], b = net.br_b[k];
    const double inv = net.br_itap[k], ia2 = net.br_itap2[k];
    const double on = net.br_closed[k] ? 1.0 : 0.0;
    const double vv = Vi * Vj * inv;
    if (!to_end) {
        P.val = Vi * Vi * ia2 * g - vv * (g * c + b * s);
        P.d[0] = vv * (g * s - b * c);
        P.d[1] = 2.0 * Vi * ia2 * g - Vj * inv * (g * c + b * s);
        P.d[2] = -P.d[0];
        P.d[3] = -Vi * inv * (g * c + b * s);
        const double bsf = net.br_bsf[k];
        Q.val = -(Vi * Vi * ia2) * (b + bsf) - vv * (g * s - b * c);
        Q.d[0] = -vv * (g * c + b * s);
        Q.d[1] = (exact ? -2.0 * Vi * (b + bsf) * ia2 : -2.0 * Vi * b * ia2) - Vj * inv * (g * s - b * c);
        Q.d[2] = -Q.d[0];
        Q.d[3] = -Vi * inv * (g * s - b * c);
    } else {
        P.val = Vj * Vj * g - vv * (g * c - b * s);
        P.d[0] = exact ? vv * (g * s + b * c) : vv * (-g * s - b * c);
        P.d[1] = -Vj * inv * (g * c - b * s);
        P.d[2] = -P.d[0];
        P.d[3] = 2.0 * Vj * g - Vi * inv * (g * c - b * s);
        const double bst = net.br_bst[k];
        Q.val = -Vj * Vj * (b + bst) + vv * (g * s + b * c);
        Q.d[0] = vv * (g * c - b * s);
        Q.d[1] = Vj * inv * (g * s + b * c);
        Q.d[2] = -Q.d[0];
        Q.d[3] = (exact ? -2.0 * Vj * (b + bst) : -2.0 * Vj * b) + Vi * inv * (g * s + b * c);
    }
    P.val *= on;
    Q.val *= on;
    if (exact) {
        for (int x = 0; x < 4; ++x) {
            P.d[x] *= on;
            Q.d[x] *= on;
        }
    }
}

// H entries of a warp's rows (a contiguous range of the CSR values) staged
// in shared memory by k_evaluate.
constexpr int kEvalSpan = 512;

// a3/a6/a7/a8/a9 fused, one thread per evaluation unit (one row, or a P row
// and its Q twin): h(x), the H row values, the residual, the (Huber) weight,
// the FP32 and weighted copies of the H row, and per-block partials of the
// objective.  A warp's 32 units cover a contiguous range of rows whenever
// the rows come in order (the usual case); their H entries are then built in
// shared memory and the warp writes the range out coalesced, skipping rows
// it does not evaluate.  Otherwise each thread writes its rows in place.
__global__ void __launch_bounds__(kBlock) k_evaluate_pairs(DevNet net, DevWork w, SolveParams sp) {
    __shared__ double sh[32];
    __shared__ double hs[kBlock / 32][kEvalSpan];
    __shared__ uint8_t hrow_id[kBlock / 32][kEvalSpan];  // row - lo of each entry; 0xFF = not evaluated
    __shared__ double wes[kBlock / 32][64];
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int gidx = u >> 5;
    const int2 grp = (u - lane) < net.n_units ? net.ev_grp[gidx] : make_int2(-1, -1);
    const int hw0 = grp.x >= 0 ? net.h_ptr[grp.x] : 0;
    const int hw1 = grp.x >= 0 ? net.h_ptr[grp.y] : 0;
    const bool staged = grp.x >= 0 && hw1 - hw0 <= kEvalSpan && grp.y - grp.x <= 64;  // warp-uniform
    if (staged) {
        for (int x = lane; x < hw1 - hw0; x += 32) {
            hs[warp][x] = 0.0;
            hrow_id[warp][x] = 0xFF;
        }
        __syncwarp();
    }
    double obj = 0.0, hub = 0.0;
    const int2 un = u < net.n_units ? net.ev_unit[u] : make_int2(-1, -1);
    bool skip = un.x < 0;
    if (!skip && net.meas_grid) {
        const uint32_t gf = w.grid_flags[net.meas_grid[un.x]];
        skip = (gf & sp.skip_flags) || (gf & sp.need_flags) != sp.need_flags;
    }
    const bool exact = sp.exact_jacobian != 0;
    // the H row of row q: in the warp's staged range or in place (zeroed)
    auto row_of = [&](int q) -> double* {
        const int base = net.h_ptr[q], nh = net.h_ptr[q + 1] - base;
        if (staged) {
            for (int x = 0; x < nh; ++x) hrow_id[warp][base - hw0 + x] = static_cast<uint8_t>(q - grp.x);
            return &hs[warp][base - hw0];
        }
        double* hrow = w.hval + base;
        for (int x = 0; x < nh; ++x) hrow[x] = 0.0;
        return hrow;
    };
    // residual, weight, outputs and objective of row q with value hv
    auto finish = [&](int q, int kind, double hv, const double* hrow) {
        const int base = net.h_ptr[q], nh = net.h_ptr[q + 1] - base;
        if (sp.mixed && !staged)
            for (int x = 0; x < nh; ++x) w.hval32[base + x] = static_cast<float>(hrow[x]);
        double rr = 0.0, we = 0.0;
        if (kind != 5) {
            rr = w.z[q] - hv;
            const double wb = net.m_w[q];
            we = wb;
            if (sp.robust) {  // kernels.cu:634-671
                const double sg = net.m_sigma[q];
                const double rn = fabs(rr / sg);
                if (!(rn <= sp.huber_gamma)) we = sp.huber_gamma / (sg * fabs(rr) + kEps);
            }
            obj += wb * rr * rr;
            if (sp.huber_objective) {  // rho(u) = u^2 / 2 inside gamma, gamma |u| - gamma^2 / 2 outside
                const double uu = fabs(rr) / fmax(net.m_sigma[q], kEps);
                hub += (uu <= sp.huber_gamma) ? 0.5 * uu * uu
                                              : sp.huber_gamma * uu - 0.5 * sp.huber_gamma * sp.huber_gamma;
            }
        } else {
            hv = 0.0;
        }
        w.h[q] = hv;
        w.r[q] = rr;
        w.w_eff[q] = we;
        w.wr[q] = we * rr;
        // weighted H entries for the gain sums G_ij = sum (w h_a) h_b
        if (staged) {
            wes[warp][q - grp.x] = we;
        } else if (sp.mixed && w.hw32) {
            for (int x = 0; x < nh; ++x) w.hw32[base + x] = static_cast<float>(we * hrow[x]);
        } else if (!sp.mixed && w.hw) {
            for (int x = 0; x < nh; ++x) w.hw[base + x] = we * hrow[x];
        }
    };
    if (!skip) {
        const int qa = un.x, qb = un.y;
        const int kind = net.m_kind[qa];
        const int ty = net.m_type[qa];
        const int loc = net.m_loc[qa];
        if (kind == 0) {  // V_MAG
            double* hrow = row_of(qa);
            hrow[0] = 1.0;
            finish(qa, kind, w.v[loc], hrow);
        } else if (kind == 1) {  // V_ANGLE
            double* hrow = row_of(qa);
            if (net.h_ptr[qa + 1] > net.h_ptr[qa]) hrow[0] = 1.0;
            finish(qa, kind, w.th[loc], hrow);
        } else if (kind == 2) {  // P/Q injection or pseudo; with its twin when qb >= 0
            // slot 0: the P row, slot 1: the Q row (either may be absent)
            const bool a_is_q = (ty == 3 || ty == 8);
            const int qp = a_is_q ? qb : qa, qq = a_is_q ? qa : qb;
            double* hp = qp >= 0 ? row_of(qp) : nullptr;
            double* hq = qq >= 0 ? row_of(qq) : nullptr;
            const double Vi = w.v[loc];
            const double2 cs_i = w.bus_cs[loc];
            double hvp = 0.0, dVip = 0.0, dTip = 0.0, hvq = 0.0, dViq = 0.0, dTiq = 0.0;
            const int e0 = net.y_ptr[loc], e1 = net.y_ptr[loc + 1];
            for (int e = e0; e < e1; ++e) {
                const int j = net.y_col[e];
                const double G = net.y_g[e], B = net.y_b[e];
                if (j == loc) {
                    hvp += Vi * Vi * G;
                    dVip += 2.0 * Vi * G;
                    if (!exact) dTip += Vi * Vi * B;
                    hvq -= Vi * Vi * B;
                    dViq -= 2.0 * Vi * B;
                    if (!exact) dTiq += Vi * Vi * G;
                } else {
                    const double Vj = w.v[j];
                    double sn, cn;
                    angle_diff(cs_i, w.bus_cs[j], &sn, &cn);
                    const double gcbs = G * cn + B * sn, gsbc = G * sn - B * cn;
                    const int pt = net.y_hpos_t[e], pv = net.y_hpos_v[e];
                    if (hp) {
                        hvp += Vi * Vj * gcbs;
                        dVip += Vj * gcbs;
                        dTip -= Vi * Vj * gsbc;
                        if (pt >= 0) hp[pt] += Vi * Vj * gsbc;
                        hp[pv] += Vi * gcbs;
                    }
                    if (hq) {
                        hvq += Vi * Vj * gsbc;
                        dViq += Vj * gsbc;
                        dTiq += Vi * Vj * gcbs;
                        if (pt >= 0) hq[pt] += -Vi * Vj * gcbs;
                        hq[pv] += Vi * gsbc;
                    }
                }
            }
            const int pt = net.y_hpos_t[e0], pv = net.y_hpos_v[e0];
            if (hp) {
                if (pt >= 0) hp[pt] += dTip;
                hp[pv] += dVip;
                finish(qp, kind, hvp, hp);
            }
            if (hq) {
                if (pt >= 0) hq[pt] += dTiq;
                hq[pv] += dViq;
                finish(qq, kind, hvq, hq);
            }
        } else if (kind == 3) {  // P/Q flow; with its twin at the same end when qb >= 0
            const bool to_end = net.m_end[qa] != 0;
            if (qb < 0) {
                double* hrow = row_of(qa);
                const FlowTerms f = flow_terms_cs(net, w.v, w.bus_cs, loc, ty == 5, to_end, exact);
                put_flow(hrow, net.m_fpos[qa], f.d);
                finish(qa, kind, f.val, hrow);
            } else {
                const bool a_is_q = ty == 5;
                const int qp = a_is_q ? qb : qa, qq = a_is_q ? qa : qb;
                double sn, cn;
                branch_angle(net, w.bus_cs, loc, &sn, &cn);
                FlowTerms fp, fq;
                flow_terms_pq(net, w.v, loc, to_end, exact, sn, cn, fp, fq);
                double* hp = row_of(qp);
                put_flow(hp, net.m_fpos[qp], fp.d);
                finish(qp, kind, fp.val, hp);
                double* hq = row_of(qq);
                put_flow(hq, net.m_fpos[qq], fq.d);
                finish(qq, kind, fq.val, hq);
            }
        } else if (kind == 4) {  // current magnitude
            double* hrow = row_of(qa);
            const bool to_end = net.m_end[qa] != 0;
            const FlowTerms fp = flow_terms_cs(net, w.v, w.bus_cs, loc, false, to_end, exact);
            const int ib = to_end ? net.br_to[loc] : net.br_from[loc];
            const double ve = w.v[ib];
            const double vs = fmax(ve, kEps);
            const double on = net.br_closed[loc] ? 1.0 : 0.0;
            double d[4];
            double hv;
            if (!exact) {  // the reference reuses the P-flow derivatives
                const FlowTerms fq = flow_terms_cs(net, w.v, w.bus_cs, loc, true, to_end, exact);
                hv = sqrt(fp.val * fp.val + fq.val * fq.val) / vs * on;
                for (int x = 0; x < 4; ++x) d[x] = fp.d[x];
            } else {
                const FlowTerms fq = flow_terms_cs(net, w.v, w.bus_cs, loc, true, to_end, exact);
                const double S = sqrt(fp.val * fp.val + fq.val * fq.val);
                hv = S / vs * on;
                for (int x = 0; x < 4; ++x)
                    d[x] = (S > 0.0) ? (fp.val * fp.d[x] + fq.val * fq.d[x]) / (S * vs) * on : 0.0;
                if (ve > kEps) d[to_end ? 3 : 1] -= S / (vs * vs) * on;
            }
            put_flow(hrow, net.m_fpos[qa], d);
            finish(qa, kind, hv, hrow);
        } else {
            double* hrow = row_of(qa);
            finish(qa, kind, 0.0, hrow);
        }
    }
    if (staged) {
        __syncwarp();
        for (int x = lane; x < hw1 - hw0; x += 32) {
            const int r = hrow_id[warp][x];
            if (r == 0xFF) continue;
            const double v = hs[warp][x];
            w.hval[hw0 + x] = v;
            if (sp.mixed) {
                w.hval32[hw0 + x] = static_cast<float>(v);
                if (w.hw32) w.hw32[hw0 + x] = static_cast<float>(wes[warp][r] * v);
            } else if (w.hw) {
                w.hw[hw0 + x] = wes[warp][r] * v;
            }
        }
    }
    const double s = block_sum(obj, sh);
    if (threadIdx.x == 0) w.part[blockIdx.x] = s;
    if (sp.huber_objective) {
        __syncthreads();  // sh is reused
        const double hs2 = block_sum(hub, sh);
        if (threadIdx.x == 0) w.hpart[blockIdx.x] = hs2;
    }
}

// a3/a6/a7/a8/a9 fused, one thread per measurement row (the form for
// evaluations with no paired rows: twice the threads of k_evaluate_pairs,
// which a small grid needs to fill the GPU).

__global__ void __launch_bounds__(kBlock) k_evaluate_rows(DevNet net, DevWork w, SolveParams sp) {
    __shared__ double sh[32];
    // A warp's rows own the contiguous H range [hw0, hw1).  When it fits,
    // each row is built in shared memory and the warp writes the range out
    // coalesced (H in FP64, FP32 and weighted), skipping rows it did not
    // evaluate; otherwise each thread writes its own row in place.
    __shared__ double hs[kBlock / 32][kEvalSpan];
    __shared__ uint16_t hlane[kBlock / 32][kEvalSpan];
    __shared__ double wes[kBlock / 32][32];
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int qw0 = q - lane;
    const int hw0 = qw0 < net.n_meas ? net.h_ptr[qw0] : 0;
    const int hw1 = qw0 < net.n_meas ? net.h_ptr[min(qw0 + 32, net.n_meas)] : 0;
    const bool staged = hw1 - hw0 <= kEvalSpan;  // warp-uniform
    if (staged) {
        for (int x = lane; x < hw1 - hw0; x += 32) {
            hs[warp][x] = 0.0;
            hlane[warp][x] = 0xFFFF;  // not evaluated: left as it is
        }
        __syncwarp();
    }
    double obj = 0.0, hub = 0.0;
    bool skip = false;
    if (q < net.n_meas && net.meas_grid) {
        const uint32_t gf = w.grid_flags[net.meas_grid[q]];
        skip = (gf & sp.skip_flags) || (gf & sp.need_flags) != sp.need_flags;
    }
    if (q < net.n_meas && !skip) {
        const int kind = net.m_kind[q];
        const int ty = net.m_type[q];
        const int loc = net.m_loc[q];
        const bool exact = sp.exact_jacobian != 0;
        const int base = net.h_ptr[q];
        const int nh = net.h_ptr[q + 1] - base;
        double* hrow = staged ? &hs[warp][base - hw0] : w.hval + base;
        if (staged) {
            for (int x = 0; x < nh; ++x) hlane[warp][base - hw0 + x] = static_cast<uint16_t>(lane);
        } else {
            for (int x = 0; x < nh; ++x) hrow[x] = 0.0;
        }
        double hv = 0.0;
        if (kind == 0) {  // V_MAG
            hv = w.v[loc];
            hrow[0] = 1.0;
        } else if (kind == 1) {  // V_ANGLE
            hv = w.th[loc];
            if (nh > 0) hrow[0] = 1.0;
        } else if (kind == 2) {  // P/Q injection or pseudo
            const bool isq = (ty == 3 || ty == 8);
            const double Vi = w.v[loc];
            const double2 cs_i = w.bus_cs[loc];
            double dVi = 0.0, dTi = 0.0;
            const int e0 = net.y_ptr[loc], e1 = net.y_ptr[loc + 1];
            for (int e = e0; e < e1; ++e) {
                const int j = net.y_col[e];
                const double G = net.y_g[e], B = net.y_b[e];
                if (j == loc) {
                    if (!isq) {
                        hv += Vi * Vi * G;
                        dVi += 2.0 * Vi * G;
                        if (!exact) dTi += Vi * Vi * B;
                    } else {
                        hv -= Vi * Vi * B;
                        dVi -= 2.0 * Vi * B;
                        if (!exact) dTi += Vi * Vi * G;
                    }
                } else {
                    const double Vj = w.v[j];
                    double s, c;
                    angle_diff(cs_i, w.bus_cs[j], &s, &c);
                    const double gcbs = G * c + B * s, gsbc = G * s - B * c;
                    double dTj, dVj;
                    if (!isq) {
                        hv += Vi * Vj * gcbs;
                        dVi += Vj * gcbs;
                        dTi -= Vi * Vj * gsbc;
                        dTj = Vi * Vj * gsbc;
                        dVj = Vi * gcbs;
                    } else {
                        hv += Vi * Vj * gsbc;
                        dVi += Vj * gsbc;
                        dTi += Vi * Vj * gcbs;
                        dTj = -Vi * Vj * gcbs;
                        dVj = Vi * gsbc;
                    }
                    const int pt = net.y_hpos_t[e];
                    if (pt >= 0) hrow[pt] += dTj;
                    hrow[net.y_hpos_v[e]] += dVj;
                }
            }
            const int pt = net.y_hpos_t[e0];
            if (pt >= 0) hrow[pt] += dTi;
            hrow[net.y_hpos_v[e0]] += dVi;
        } else if (kind == 3) {  // P/Q flow
            const bool to_end = net.m_end[q] != 0;
            const FlowTerms f = flow_terms_cs(net, w.v, w.bus_cs, loc, ty == 5, to_end, exact);
            hv = f.val;
            put_flow(hrow, net.m_fpos[q], f.d);
        } else if (kind == 4) {  // current magnitude
            const bool to_end = net.m_end[q] != 0;
            const FlowTerms fp = flow_terms_cs(net, w.v, w.bus_cs, loc, false, to_end, exact);
            const int ib = to_end ? net.br_to[loc] : net.br_from[loc];
            const double ve = w.v[ib];
            const double vs = fmax(ve, kEps);
            const double on = net.br_closed[loc] ? 1.0 : 0.0;
            double d[4];
            if (!exact) {  // the reference reuses the P-flow derivatives
                hv = 0.0;
                const FlowTerms fq = flow_terms_cs(net, w.v, w.bus_cs, loc, true, to_end, exact);
                hv = sqrt(fp.val * fp.val + fq.val * fq.val) / vs * on;
                for (int x = 0; x < 4; ++x) d[x] = fp.d[x];
            } else {
                const FlowTerms fq = flow_terms_cs(net, w.v, w.bus_cs, loc, true, to_end, exact);
                const double S = sqrt(fp.val * fp.val + fq.val * fq.val);
                hv = S / vs * on;
                for (int x = 0; x < 4; ++x)
                    d[x] = (S > 0.0) ? (fp.val * fp.d[x] + fq.val * fq.d[x]) / (S * vs) * on : 0.0;
                if (ve > kEps) d[to_end ? 3 : 1] -= S / (vs * vs) * on;
            }
            put_flow(hrow, net.m_fpos[q], d);
        }
        if (sp.mixed && !staged)
            for (int x = 0; x < nh; ++x) w.hval32[base + x] = static_cast<float>(hrow[x]);
        double rr = 0.0, we = 0.0;
        if (kind != 5) {
            rr = w.z[q] - hv;
            const double wb = net.m_w[q];
            we = wb;
            if (sp.robust) {  // kernels.cu:634-671
                const double sg = net.m_sigma[q];
                const double rn = fabs(rr / sg);
                if (!(rn <= sp.huber_gamma)) we = sp.huber_gamma / (sg * fabs(rr) + kEps);
            }
            obj = wb * rr * rr;
            if (sp.huber_objective) {  // rho(u) = u^2 / 2 inside gamma, gamma |u| - gamma^2 / 2 outside
                const double u = fabs(rr) / fmax(net.m_sigma[q], kEps);
                hub = (u <= sp.huber_gamma) ? 0.5 * u * u : sp.huber_gamma * u - 0.5 * sp.huber_gamma * sp.huber_gamma;
            }
        } else {
            hv = 0.0;
        }
        w.h[q] = hv;
        w.r[q] = rr;
        w.w_eff[q] = we;
        w.wr[q] = we * rr;
        // weighted H entries for the gain sums G_ij = sum (w h_a) h_b
        if (staged) {
            wes[warp][lane] = we;
        } else if (sp.mixed && w.hw32) {
            for (int x = 0; x < nh; ++x) w.hw32[base + x] = static_cast<float>(we * hrow[x]);
        } else if (!sp.mixed && w.hw) {
            for (int x = 0; x < nh; ++x) w.hw[base + x] = we * hrow[x];
        }
    }
    if (staged) {
        __syncwarp();
        for (int x = lane; x < hw1 - hw0; x += 32) {
            const int r = hlane[warp][x];
            if (r == 0xFFFF) continue;
            const double v = hs[warp][x];
            w.hval[hw0 + x] = v;
            if (sp.mixed) {
                w.hval32[hw0 + x] = static_cast<float>(v);
                if (w.hw32) w.hw32[hw0 + x] = static_cast<float>(wes[warp][r] * v);
            } else if (w.hw) {
                w.hw[hw0 + x] = wes[warp][r] * v;
            }
        }
    }
    const double s = block_sum(obj, sh);
    if (threadIdx.x == 0) w.part[blockIdx.x] = s;
    if (sp.huber_objective) {
        __syncthreads();  // sh is reused
        const double hs = block_sum(hub, sh);
        if (threadIdx.x == 0) w.hpart[blockIdx.x] = hs;
    }
}

// Huber objective of the last evaluation (block partials in order).
__global__ void k_huber_objective(DevWork w, int nblk) {
    __shared__ double sh[32];
    double acc = 0.0;
    for (int b = threadIdx.x; b < nblk; b += blockDim.x) acc += w.hpart[b];
    acc = block_sum(acc, sh);
    if (threadIdx.x == 0) w.status->huber_objective = acc;
}

// a11: b = H^T (w r) in permuted state order, one thread per state (gather).
__global__ void k_rhs(DevNet net, DevFactor f, DevWork w) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= f.n_state) return;
    if (f.ps_grid && (w.grid_flags[f.ps_grid[t]] & FLAG_FROZEN)) return;
    double acc = 0.0;
    for (int x = f.rhs_ptr[t]; x < f.rhs_ptr[t + 1]; ++x) {
        const int hidx = f.rhs_h[x];
        acc += w.hval[hidx] * w.wr[net.h_row[hidx]];
    }
    w.rhs[t] = acc;
}

// Mixed-precision refinement of one Gauss-Newton step (FP32 factor M ~ G):
//   dx0 = M^-1 b;  repeat: rho = b - H^T W (H dx) in FP64, dx += M^-1 rho.
__global__ void k_to_fp32(DevFactor f, DevWork w) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= f.n_state) return;
    w.rhs32[t] = static_cast<float>(w.rhs[t]);
}

__global__ void k_refine_begin(DevFactor f, DevWork w) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= f.n_state) return;
    w.b0[t] = w.rhs[t];
    w.dx[t] = static_cast<double>(w.sol32[t]);
}

__global__ void k_refine_spmv(DevNet net, DevWork w) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= net.n_meas) return;
    double acc = 0.0;
    for (int h = net.h_ptr[q]; h < net.h_ptr[q + 1]; ++h)
        acc += static_cast<double>(w.hval32[h]) * w.dx[net.h_pcol[h]];
    w.hdx[q] = w.w_eff[q] * acc;
}

__global__ void k_refine_rhs(DevNet net, DevFactor f, DevWork w) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= f.n_state) return;
    double acc = 0.0;
    for (int x = f.rhs_ptr[t]; x < f.rhs_ptr[t + 1]; ++x) {
        const int hidx = f.rhs_h[x];
        acc += static_cast<double>(w.hval32[hidx]) * w.hdx[net.h_row[hidx]];
    }
    w.rhs32[t] = static_cast<float>(w.b0[t] - acc);
}

__global__ void k_refine_accumulate(DevFactor f, DevWork w) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= f.n_state) return;
    w.dx[t] += static_cast<double>(w.sol32[t]);
}

// Objective, largest |r| (lowest index on ties) and the bad-data count
// (active rows with sigma > 0 and |r| / sigma > threshold,
// sle_engine.cu:959-977).  Two deterministic passes: per-block partials over
// the rows, then one block over the partials in block order.
__global__ void __launch_bounds__(kBlock) k_objective_part(DevNet net, DevWork w, double bad_threshold) {
    __shared__ double sb[kBlock];
    __shared__ int si[kBlock];
    __shared__ int sc[kBlock];
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    double best = -1.0;
    int bidx = 0x7fffffff, cnt = 0;
    if (q < net.n_meas && net.m_kind[q] != 5) {
        const double a = fabs(w.r[q]);
        best = a;
        bidx = q;
        const double sg = net.m_sigma[q];
        if (sg > 0.0 && a / sg > bad_threshold) cnt = 1;
    }
    sb[threadIdx.x] = best;
    si[threadIdx.x] = bidx;
    sc[threadIdx.x] = cnt;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            const double b2 = sb[threadIdx.x + o];
            const int i2 = si[threadIdx.x + o];
            if (b2 > sb[threadIdx.x] || (b2 == sb[threadIdx.x] && i2 < si[threadIdx.x])) {
                sb[threadIdx.x] = b2;
                si[threadIdx.x] = i2;
            }
            sc[threadIdx.x] += sc[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        w.opart[blockIdx.x] = sb[0];
        w.oidx[blockIdx.x] = si[0];
        w.ocnt[blockIdx.x] = sc[0];
    }
}

// nblk: blocks of k_objective_part (rows); nblk_eval: blocks of the last
// k_evaluate (evaluation units), whose objective partials are summed.
__global__ void k_objective(DevNet net, DevWork w, int nblk, int nblk_eval) {
    __shared__ double sh[32];
    __shared__ double sb[1024];
    __shared__ int si[1024];
    __shared__ int sc[1024];
    double acc = 0.0;
    for (int b = threadIdx.x; b < nblk_eval; b += blockDim.x) acc += w.part[b];
    const double tot = block_sum(acc, sh);
    double best = -1.0;
    int bidx = 0x7fffffff, cnt = 0;
    for (int b = threadIdx.x; b < nblk; b += blockDim.x) {
        const double a = w.opart[b];
        const int i = w.oidx[b];
        if (a > best || (a == best && i < bidx)) { best = a; bidx = i; }
        cnt += w.ocnt[b];
    }
    sb[threadIdx.x] = best;
    si[threadIdx.x] = bidx;
    sc[threadIdx.x] = cnt;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) {
            const double b2 = sb[threadIdx.x + o];
            const int i2 = si[threadIdx.x + o];
            if (b2 > sb[threadIdx.x] || (b2 == sb[threadIdx.x] && i2 < si[threadIdx.x])) {
                sb[threadIdx.x] = b2;
                si[threadIdx.x] = i2;
            }
            sc[threadIdx.x] += sc[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        w.status->objective = tot;
        w.status->largest_residual = sb[0] < 0.0 ? 0.0 : sb[0];
        w.status->largest_idx = si[0] == 0x7fffffff ? -1 : si[0];
        w.status->bad_count = sc[0];
    }
}

// a13: x += dx (slack angle fixed), V clamped, block maxima of |dx|.
__global__ void __launch_bounds__(kBlock) k_update(DevNet net, DevFactor f, DevWork w, SolveParams sp,
                                                   const double* step) {
    __shared__ double sh[32];
    __shared__ int bad;
    if (threadIdx.x == 0) bad = 0;
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double mx = 0.0;
    if (i < net.n_bus) {
        const int pt = f.bus_ps_theta[i];
        const double dv = step[f.bus_ps_v[i]];
        double dt = 0.0;
        if (pt >= 0) {
            dt = step[pt];
            w.th[i] += dt;
        }
        double vn = w.v[i] + dv;
        vn = fmax(vn, sp.vmin);
        vn = fmin(vn, sp.vmax);
        w.v[i] = vn;
        if (!isfinite(dt) || !isfinite(dv)) bad = 1;
        mx = fmax(fabs(dt), fabs(dv));
        if (mx != mx) mx = 0.0;
    }
    const double m = block_max(mx, sh);
    if (threadIdx.x == 0) {
        w.part[blockIdx.x] = m;
        if (bad) atomicOr(&w.status->flags, FLAG_NONFINITE);
    }
}

// A step with a non-finite entry (FLAG_NONFINITE from k_update) is never
// converged and reports a NaN max |dx|: the reference's max reduction turns
// NaN once a NaN step fills its blocks (kernels.cu:557-574,752-782), so
// "max |dx| < tol" fails and checkValidityKernel's flag decides: DIVERGED
// (wls_solver.cu:493-517, 343-352).
__global__ void k_update_finalize(DevWork w, int nblk, double tol) {
    __shared__ double sh[32];
    double m = 0.0;
    for (int b = threadIdx.x; b < nblk; b += blockDim.x) m = fmax(m, w.part[b]);
    m = block_max(m, sh);
    if (threadIdx.x == 0) {
        const bool bad = (w.status->flags & FLAG_NONFINITE) != 0;
        w.status->max_mismatch = bad ? __longlong_as_double(0x7ff8000000000000LL) : m;
        if (!bad && m < tol) atomicOr(&w.status->flags, FLAG_CONVERGED);
    }
}

// kernels.cu:799-817
__global__ void k_flat_start(DevNet net, DevWork w) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= net.n_bus) return;
    const int t = net.bus_type[i];
    w.v[i] = (t == 1 || t == 2) ? net.v_setpoint[i] : 1.0;
    w.th[i] = 0.0;
}

__global__ void k_injections(DevNet net, DevWork w) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= net.n_bus) return;
    const double Vi = w.v[i], ti = w.th[i];
    double P = 0.0, Q = 0.0;
    for (int e = net.y_ptr[i]; e < net.y_ptr[i + 1]; ++e) {
        const int j = net.y_col[e];
        const double G = net.y_g[e], B = net.y_b[e];
        double s = 0.0, c = 1.0;
        if (j != i) sincos(ti - w.th[j], &s, &c);
        const double vv = Vi * w.v[j];
        P += vv * (G * c + B * s);
        Q += vv * (G * s - B * c);
    }
    w.p_inj[i] = P;
    w.q_inj[i] = Q;
}

__global__ void k_flows(DevNet net, DevWork w) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= net.n_branch) return;
    w.pf[k] = flow_terms(net, w.v, w.th, k, false, false, true).val;
    w.qf[k] = flow_terms(net, w.v, w.th, k, true, false, true).val;
    w.pt[k] = flow_terms(net, w.v, w.th, k, false, true, true).val;
    w.qt[k] = flow_terms(net, w.v, w.th, k, true, true, true).val;
}

// Batch: one block per grid.  Clears the grid's flags (FROZEN for grids not
// in this solve) and applies a flat start where requested.
__global__ void k_batch_begin(DevNet net, DevWork w, DevBatch b) {
    const int g = blockIdx.x;
    const bool act = b.active[g] != 0;
    if (threadIdx.x == 0) {
        b.flags[g] = act ? 0u : (FLAG_FROZEN | FLAG_INACTIVE);
        b.iters[g] = 0;
        b.mismatch[g] = 0.0;
    }
    if (!act || !b.flat[g]) return;
    for (int i = b.bus_off[g] + threadIdx.x; i < b.bus_off[g + 1]; i += blockDim.x) {
        const int t = net.bus_type[i];
        w.v[i] = (t == 1 || t == 2) ? net.v_setpoint[i] : 1.0;
        w.th[i] = 0.0;
    }
}

// f2: islands of the closed-branch graph (the reference's topological check,
// sle_engine.cu:684-753, on the device).
__global__ void k_island_init(DevNet net, int32_t* parent, int32_t* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < net.n_bus) parent[i] = i;
    if (i == 0) {
        out[0] = 0;
        out[1] = 0;
        out[3] = 0;
    }
}

__device__ __forceinline__ int island_root(const int32_t* parent, int x) {
    for (int guard = 0; guard < 64 && parent[x] != x; ++guard) x = parent[x];
    return x;
}

// out[3] = 1 when some branch joined two components this round
__global__ void k_island_hook(DevNet net, int32_t* parent, int32_t* out) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= net.n_branch || !net.br_closed[k]) return;
    const int a = island_root(parent, net.br_from[k]);
    const int b = island_root(parent, net.br_to[k]);
    if (a == b) return;
    atomicMin(parent + max(a, b), min(a, b));
    out[3] = 1;
}

__global__ void k_island_jump(DevNet net, int32_t* parent) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= net.n_bus) return;
    int p = parent[i];
    for (int guard = 0; guard < 64 && parent[p] != p; ++guard) p = parent[p];
    parent[i] = p;
}

__global__ void k_island_count(DevNet net, const int32_t* parent, int32_t* out) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < net.n_bus && parent[i] == i) atomicAdd(out + 0, 1);
    if (i < net.n_meas && net.m_active[i]) atomicAdd(out + 1, 1);
}

// Stream mode: grids with active[g] join the running batch.
__global__ void k_batch_activate(DevNet net, DevWork w, DevBatch b) {
    const int g = blockIdx.x;
    if (!b.active[g]) return;
    if (threadIdx.x == 0) {
        b.flags[g] = 0u;
        b.iters[g] = 0;
        b.mismatch[g] = 0.0;
    }
    if (!b.flat[g]) return;
    for (int i = b.bus_off[g] + threadIdx.x; i < b.bus_off[g + 1]; i += blockDim.x) {
        const int t = net.bus_type[i];
        w.v[i] = (t == 1 || t == 2) ? net.v_setpoint[i] : 1.0;
        w.th[i] = 0.0;
    }
}

__global__ void k_batch_retire(DevBatch b) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g < b.n_grids && b.retire[g]) b.flags[g] = (b.flags[g] | FLAG_FROZEN | FLAG_INACTIVE) & ~FLAG_FINAL;
}

// Batch a13, spread over CTAs: each item applies the step to its buses and
// writes its max |dx| and whether a step entry was not finite; then one
// thread per grid combines its items and decides, exactly as the single-grid
// loop does after its step: a frozen grid takes no step; a grid whose
// factorisation flagged a non-positive pivot stops as singular without
// applying the step; otherwise it stops when max |dx| < tol (converged) or
// dx is not finite (diverged).
__global__ void __launch_bounds__(kBlock) k_batch_update_part(DevFactor f, DevWork w, DevBatch b, SolveParams sp,
                                                              const double* step) {
    __shared__ double sh[32];
    const int2 it = b.bus_items[blockIdx.x];
    const int g = it.x;
    const uint32_t fl = b.flags[g];
    if (fl & (FLAG_FROZEN | FLAG_SINGULAR)) return;  // the whole CTA
    const int end = min(it.y + kBatchChunk, b.bus_off[g + 1]);
    double mx = 0.0;
    int bad = 0;
    for (int i = it.y + threadIdx.x; i < end; i += blockDim.x) {
        const int pt = f.bus_ps_theta[i];
        const double dv = step[f.bus_ps_v[i]];
        double dt = 0.0;
        if (pt >= 0) {
            dt = step[pt];
            w.th[i] += dt;
        }
        double vn = w.v[i] + dv;
        vn = fmax(vn, sp.vmin);
        vn = fmin(vn, sp.vmax);
        w.v[i] = vn;
        if (!isfinite(dt) || !isfinite(dv)) bad = 1;
        double m = fmax(fabs(dt), fabs(dv));
        if (m != m) m = 0.0;
        mx = fmax(mx, m);
    }
    bad = __syncthreads_or(bad);
    const double m = block_max(mx, sh);
    if (threadIdx.x == 0) {
        b.part[blockIdx.x] = m;
        b.part_bad[blockIdx.x] = bad;
    }
}

__global__ void k_batch_update_fin(DevBatch b, double tol) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= b.n_grids) return;
    const uint32_t fl = b.flags[g];
    if (fl & FLAG_FROZEN) return;
    if (fl & FLAG_SINGULAR) {
        b.flags[g] = fl | FLAG_FROZEN;
        b.iters[g] += 1;
        return;
    }
    double m = 0.0;
    int bad = 0;
    for (int k = b.bus_item_ptr[g]; k < b.bus_item_ptr[g + 1]; ++k) {
        m = fmax(m, b.part[k]);
        bad |= b.part_bad[k];
    }
    b.mismatch[g] = bad ? __longlong_as_double(0x7ff8000000000000LL) : m;
    b.iters[g] += 1;
    if (bad) {
        b.flags[g] = fl | FLAG_NONFINITE | FLAG_FROZEN;
    } else if (m < tol) {
        b.flags[g] = fl | FLAG_CONVERGED | FLAG_FROZEN;
    } else {
        atomicAdd(b.running, 1);
    }
}

// Objective sum w r^2 of each selected grid (not inactive, flags holding
// `need`): per item in row order, then per grid over its items in order.
__global__ void __launch_bounds__(kBlock) k_batch_objective_part(DevNet net, DevWork w, DevBatch b, uint32_t need) {
    __shared__ double sh[32];
    const int2 it = b.row_items[blockIdx.x];
    const uint32_t fl = b.flags[it.x];
    if ((fl & FLAG_INACTIVE) || (fl & need) != need) return;  // the whole CTA
    const int end = min(it.y + kBatchChunk, b.meas_off[it.x + 1]);
    double acc = 0.0;
    for (int q = it.y + threadIdx.x; q < end; q += blockDim.x)
        if (net.m_kind[q] != 5) acc += net.m_w[q] * w.r[q] * w.r[q];
    const double tot = block_sum(acc, sh);
    if (threadIdx.x == 0) b.part[blockIdx.x] = tot;
}

__global__ void k_batch_objective_fin(DevBatch b, uint32_t need) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= b.n_grids) return;
    const uint32_t fl = b.flags[g];
    if ((fl & FLAG_INACTIVE) || (fl & need) != need) return;
    double t = 0.0;
    for (int k = b.row_item_ptr[g]; k < b.row_item_ptr[g + 1]; ++k) t += b.part[k];
    b.objective[g] = t;
}

__global__ void k_batch_mark_final(DevBatch b) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g < b.n_grids && b.retire[g]) b.flags[g] |= FLAG_FINAL;
}

__global__ void k_gn_loop_init(DevBatch b, int32_t limit) {
    b.loop[0] = 0;
    b.loop[1] = limit;
    b.loop[2] = 0;
}

// One thread, after the step's last kernel: the step's flags and the running
// count are final.  Same decision as the host loop of Engine::batch_solve.
__global__ void k_gn_loop_next(cudaGraphConditionalHandle h, DevBatch b, const DevStatus* st) {
    const int32_t steps = b.loop[0] + 1;
    b.loop[0] = steps;
    const bool timed_out = (st->flags & FLAG_TIMEOUT) != 0u;
    if (timed_out) b.loop[2] = 1;
    cudaGraphSetConditional(h, (!timed_out && *b.running > 0 && steps < b.loop[1]) ? 1u : 0u);
}

inline int nblocks(int n) { return (n + kBlock - 1) / kBlock; }

}  // namespace

cudaError_t launch_batch_begin(const DevNet& net, const DevWork& w, const DevBatch& b, cudaStream_t st) {
    if (b.n_grids <= 0) return cudaSuccess;
    k_batch_begin<<<b.n_grids, kBlock, 0, st>>>(net, w, b);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_batch_update(const DevNet& net, const DevFactor& f, const DevWork& w, const DevBatch& b,
                                const SolveParams& sp, const double* step, cudaStream_t st) {
    if (b.n_grids <= 0) return cudaSuccess;
    if (b.n_bus_items > 0) {
        k_batch_update_part<<<b.n_bus_items, kBlock, 0, st>>>(f, w, b, sp, step);
        count_launches(1);
    }
    k_batch_update_fin<<<nblocks(b.n_grids), kBlock, 0, st>>>(b, sp.tol);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_islands(const DevNet& net, int32_t* parent, int32_t* out, int32_t max_rounds, cudaStream_t st) {
    const int nb = nblocks(std::max(net.n_bus, 1));
    k_island_init<<<nb, kBlock, 0, st>>>(net, parent, out);
    count_launches(1);
    int32_t rounds = 0, joined = 1;
    cudaError_t e = cudaSuccess;
    while (joined && e == cudaSuccess) {
        if (rounds == max_rounds) {
            rounds = -1;
            break;
        }
        e = cudaMemsetAsync(out + 3, 0, sizeof(int32_t), st);
        if (net.n_branch > 0 && e == cudaSuccess) {
            k_island_hook<<<nblocks(net.n_branch), kBlock, 0, st>>>(net, parent, out);
            count_launches(1);
        }
        k_island_jump<<<nb, kBlock, 0, st>>>(net, parent);
        count_launches(1);
        if (e == cudaSuccess) e = cudaMemcpyAsync(&joined, out + 3, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        ++rounds;
    }
    if (e != cudaSuccess) return e;
    k_island_count<<<nblocks(std::max(std::max(net.n_bus, net.n_meas), 1)), kBlock, 0, st>>>(net, parent, out);
    count_launches(1);
    e = cudaMemcpyAsync(out + 2, &rounds, sizeof(int32_t), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e == cudaSuccess ? cudaGetLastError() : e;
}

cudaError_t launch_batch_activate(const DevNet& net, const DevWork& w, const DevBatch& b, cudaStream_t st) {
    if (b.n_grids <= 0) return cudaSuccess;
    k_batch_activate<<<b.n_grids, kBlock, 0, st>>>(net, w, b);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_batch_retire(const DevBatch& b, cudaStream_t st) {
    if (b.n_grids <= 0) return cudaSuccess;
    k_batch_retire<<<(b.n_grids + kBlock - 1) / kBlock, kBlock, 0, st>>>(b);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_gn_loop_init(const DevBatch& b, int32_t limit, cudaStream_t st) {
    k_gn_loop_init<<<1, 1, 0, st>>>(b, limit);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_gn_loop_next(cudaGraphConditionalHandle h, const DevBatch& b, const DevWork& w, cudaStream_t st) {
    k_gn_loop_next<<<1, 1, 0, st>>>(h, b, w.status);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_batch_objective(const DevNet& net, const DevWork& w, const DevBatch& b, uint32_t need,
                                   cudaStream_t st) {
    if (b.n_grids <= 0) return cudaSuccess;
    if (b.n_row_items > 0) {
        k_batch_objective_part<<<b.n_row_items, kBlock, 0, st>>>(net, w, b, need);
        count_launches(1);
    }
    k_batch_objective_fin<<<nblocks(b.n_grids), kBlock, 0, st>>>(b, need);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_batch_mark_final(const DevBatch& b, cudaStream_t st) {
    if (b.n_grids <= 0) return cudaSuccess;
    k_batch_mark_final<<<nblocks(b.n_grids), kBlock, 0, st>>>(b);
    count_launches(1);
    return cudaGetLastError();
}

std::atomic<int64_t> g_kernel_launches{0};
thread_local int64_t t_kernel_launches = 0;

cudaError_t launch_admittance_and_ybus(const DevNet& net, cudaStream_t st) {
    if (net.n_branch > 0) {
        k_admittance<<<nblocks(net.n_branch), kBlock, 0, st>>>(net);
        count_launches(1);
    }
    k_ybus<<<nblocks(net.n_bus), kBlock, 0, st>>>(net);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_evaluate(const DevNet& net, const DevWork& w, const SolveParams& sp, cudaStream_t st) {
    if (net.n_meas <= 0) return cudaSuccess;
    k_bus_trig<<<nblocks(net.n_bus), kBlock, 0, st>>>(net, w, sp);
    // the unit list has as many units as rows when no row is paired
    if (net.n_units < net.n_meas)
        k_evaluate_pairs<<<nblocks(net.n_units), kBlock, 0, st>>>(net, w, sp);
    else
        k_evaluate_rows<<<nblocks(net.n_meas), kBlock, 0, st>>>(net, w, sp);
    count_launches(2);
    if (sp.huber_objective) {
        k_huber_objective<<<1, 1024, 0, st>>>(w, nblocks(net.n_units));
        count_launches(1);
    }
    return cudaGetLastError();
}

cudaError_t launch_objective(const DevNet& net, const DevWork& w, double bad_threshold, cudaStream_t st) {
    const int nb = net.n_meas > 0 ? nblocks(net.n_meas) : 0;
    if (nb > 0) {
        k_objective_part<<<nb, kBlock, 0, st>>>(net, w, bad_threshold);
        count_launches(1);
    }
    k_objective<<<1, 1024, 0, st>>>(net, w, nb, net.n_units > 0 ? nblocks(net.n_units) : 0);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_rhs(const DevNet& net, const DevFactor& f, const DevWork& w, cudaStream_t st) {
    k_rhs<<<nblocks(f.n_state), kBlock, 0, st>>>(net, f, w);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_update(const DevNet& net, const DevFactor& f, const DevWork& w, const SolveParams& sp,
                          const double* step, cudaStream_t st) {
    const int nb = nblocks(net.n_bus);
    k_update<<<nb, kBlock, 0, st>>>(net, f, w, sp, step);
    k_update_finalize<<<1, 1024, 0, st>>>(w, nb, sp.tol);
    count_launches(2);
    return cudaGetLastError();
}

cudaError_t launch_to_fp32(const DevFactor& f, const DevWork& w, cudaStream_t st) {
    k_to_fp32<<<nblocks(f.n_state), kBlock, 0, st>>>(f, w);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_refine_begin(const DevFactor& f, const DevWork& w, cudaStream_t st) {
    k_refine_begin<<<nblocks(f.n_state), kBlock, 0, st>>>(f, w);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_refine_residual(const DevNet& net, const DevFactor& f, const DevWork& w, cudaStream_t st) {
    if (net.n_meas > 0) {
        k_refine_spmv<<<nblocks(net.n_meas), kBlock, 0, st>>>(net, w);
        count_launches(1);
    }
    k_refine_rhs<<<nblocks(f.n_state), kBlock, 0, st>>>(net, f, w);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_refine_accumulate(const DevFactor& f, const DevWork& w, cudaStream_t st) {
    k_refine_accumulate<<<nblocks(f.n_state), kBlock, 0, st>>>(f, w);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_flat_start(const DevNet& net, const DevWork& w, cudaStream_t st) {
    k_flat_start<<<nblocks(net.n_bus), kBlock, 0, st>>>(net, w);
    count_launches(1);
    return cudaGetLastError();
}

cudaError_t launch_results(const DevNet& net, const DevWork& w, cudaStream_t st) {
    k_injections<<<nblocks(net.n_bus), kBlock, 0, st>>>(net, w);
    count_launches(1);
    if (net.n_branch > 0) {
        k_flows<<<nblocks(net.n_branch), kBlock, 0, st>>>(net, w);
        count_launches(1);
    }
    return cudaGetLastError();
}

}  // namespace sle_gb300
