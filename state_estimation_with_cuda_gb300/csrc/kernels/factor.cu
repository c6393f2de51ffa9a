// Level-scheduled multifrontal Cholesky of the gain matrix G = H^T W H and the
// forward / backward solves (replaces the reference's per-call
// cusolverSp csrlsvchol, sparse_matrix.cu:793-895, and its quadratic RHS).
//
// Front s (rows R_s, nc_s pivot columns) is assembled from
//   - its gain entries, each a fixed-order sum of w_m H[m,a] H[m,b] over the
//     measurement rows m that couple the two states (gathered, no atomics), and
//   - its children's update matrices, extend-added through relative maps,
// then partially factorised: L11 = chol(F11), L21 = F21 L11^-T,
// U_s = F22 - L21 L21^T.  Fronts with f <= kSmallFrontMax live in shared memory
// (one CTA per front); larger fronts are factorised in a global workspace by a
// blocked right-looking loop whose panel, triangular-solve and trailing-update
// steps are spread over many CTAs.
#include "kernels.cuh"

namespace sle_gb300 {
namespace {

constexpr int kThreads = 256;
constexpr int kNB = 32;  // panel width of the blocked big-front path

__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ double gain_entry(const DevNet& net, const DevFactor& F, const DevWork& W, int tg) {
    double acc = 0.0;
    const int64_t p1 = F.tgt_pair_ptr[tg + 1];
    for (int64_t p = F.tgt_pair_ptr[tg]; p < p1; ++p) {
        const int a = F.pair_a[p], b = F.pair_b[p];
        acc += W.w_eff[net.h_row[a]] * W.hval[a] * W.hval[b];
    }
    return acc;
}

__device__ __forceinline__ double safe_pivot(double d, uint32_t* flags) {
    if (!(d > 0.0) || !isfinite(d)) {
        atomicOr(flags, FLAG_SINGULAR);
        return 1.0;
    }
    return sqrt(d);
}

// ---------------------------------------------------------------------------
// Small fronts: one CTA per front, front held in shared memory.
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) k_front_small(DevNet net, DevFactor F, DevWork W, const int* fronts) {
    extern __shared__ double Fm[];
    const int s = fronts[blockIdx.x];
    const int f = F.sn_f[s];
    const int nc = F.sn_c0[s + 1] - F.sn_c0[s];
    const int tid = threadIdx.x, nth = blockDim.x;
    for (int x = tid; x < f * f; x += nth) Fm[x] = 0.0;
    __syncthreads();
    for (int tg = F.sn_tgt_ptr[s] + tid; tg < F.sn_tgt_ptr[s + 1]; tg += nth) Fm[F.tgt_local[tg]] = gain_entry(net, F, W, tg);
    __syncthreads();
    for (int ci = F.sn_child_ptr[s]; ci < F.sn_child_ptr[s + 1]; ++ci) {
        const int c = F.sn_child[ci];
        const int m = F.sn_f[c] - (F.sn_c0[c + 1] - F.sn_c0[c]);
        const double* U = W.u + F.sn_u_off[c];
        const int* rel = F.sn_relmap + F.sn_su_off[c];
        for (int x = tid; x < m * m; x += nth) {
            const int i = x % m, j = x / m;
            if (i >= j) Fm[rel[i] + rel[j] * f] += U[x];
        }
        __syncthreads();
    }
    const int lane = tid & 31, warp = tid >> 5, nwarp = nth >> 5;
    for (int k = 0; k < nc; ++k) {
        if (tid == 0) Fm[k + k * f] = safe_pivot(Fm[k + k * f], &W.status->flags);
        __syncthreads();
        const double piv = Fm[k + k * f];
        for (int i = k + 1 + tid; i < f; i += nth) Fm[i + k * f] /= piv;
        __syncthreads();
        for (int j = k + 1 + warp; j < f; j += nwarp) {
            const double ljk = Fm[j + k * f];
            for (int i = j + lane; i < f; i += 32) Fm[i + j * f] -= Fm[i + k * f] * ljk;
        }
        __syncthreads();
    }
    double* L = W.lx + F.sn_lx_off[s];
    for (int x = tid; x < f * nc; x += nth) L[x] = Fm[x];
    const int m = f - nc;
    double* U = W.u + F.sn_u_off[s];
    for (int x = tid; x < m * m; x += nth) {
        const int i = x % m, j = x / m;
        U[x] = Fm[(nc + i) + (nc + j) * f];
    }
}

// ---------------------------------------------------------------------------
// Big fronts: global workspace, blocked right-looking partial factorisation.
// ---------------------------------------------------------------------------
__global__ void k_big_zero(double* B, int64_t n) {
    for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x) B[x] = 0.0;
}

__global__ void k_big_targets(DevNet net, DevFactor F, DevWork W, int s) {
    double* B = W.big + F.sn_big_off[s];
    const int t0 = F.sn_tgt_ptr[s], t1 = F.sn_tgt_ptr[s + 1];
    for (int tg = t0 + blockIdx.x * blockDim.x + threadIdx.x; tg < t1; tg += gridDim.x * blockDim.x)
        B[F.tgt_local[tg]] = gain_entry(net, F, W, tg);
}

__global__ void k_big_extend_add(DevFactor F, DevWork W, int s, int c) {
    double* B = W.big + F.sn_big_off[s];
    const int f = F.sn_f[s];
    const int m = F.sn_f[c] - (F.sn_c0[c + 1] - F.sn_c0[c]);
    const double* U = W.u + F.sn_u_off[c];
    const int* rel = F.sn_relmap + F.sn_su_off[c];
    const int64_t mm = (int64_t)m * m;
    for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < mm; x += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(x % m), j = (int)(x / m);
        if (i >= j) B[rel[i] + (int64_t)rel[j] * f] += U[x];
    }
}

// Factor the pb x pb diagonal block at column p0 (one CTA).
__global__ void k_big_potrf(DevFactor F, DevWork W, int s, int p0, int pb) {
    __shared__ double D[kNB * kNB];
    double* B = W.big + F.sn_big_off[s];
    const int f = F.sn_f[s];
    for (int x = threadIdx.x; x < pb * pb; x += blockDim.x) {
        const int i = x % pb, j = x / pb;
        D[x] = B[(p0 + i) + (int64_t)(p0 + j) * f];
    }
    __syncthreads();
    for (int k = 0; k < pb; ++k) {
        if (threadIdx.x == 0) D[k + k * pb] = safe_pivot(D[k + k * pb], &W.status->flags);
        __syncthreads();
        const double piv = D[k + k * pb];
        for (int i = k + 1 + threadIdx.x; i < pb; i += blockDim.x) D[i + k * pb] /= piv;
        __syncthreads();
        for (int x = threadIdx.x; x < pb * pb; x += blockDim.x) {
            const int i = x % pb, j = x / pb;
            if (j > k && i >= j) D[i + j * pb] -= D[i + k * pb] * D[j + k * pb];
        }
        __syncthreads();
    }
    for (int x = threadIdx.x; x < pb * pb; x += blockDim.x) {
        const int i = x % pb, j = x / pb;
        if (i >= j) B[(p0 + i) + (int64_t)(p0 + j) * f] = D[x];
    }
}

// Rows below the diagonal block: X = A L_dd^-T, 64 rows per CTA.
__global__ void k_big_trsm(DevFactor F, DevWork W, int s, int p0, int pb) {
    __shared__ double D[kNB * kNB];
    double* B = W.big + F.sn_big_off[s];
    const int f = F.sn_f[s];
    for (int x = threadIdx.x; x < pb * pb; x += blockDim.x) {
        const int i = x % pb, j = x / pb;
        D[x] = B[(p0 + i) + (int64_t)(p0 + j) * f];
    }
    __syncthreads();
    const int r = p0 + pb + blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= f) return;
    double x[kNB];
    for (int c = 0; c < pb; ++c) {
        double a = B[r + (int64_t)(p0 + c) * f];
        for (int k = 0; k < c; ++k) a -= x[k] * D[c + k * pb];
        x[c] = a / D[c + c * pb];
    }
    for (int c = 0; c < pb; ++c) B[r + (int64_t)(p0 + c) * f] = x[c];
}

// Trailing lower update C -= A A^T over rows/cols >= q0 = p0 + pb with the
// panel columns [p0, p0 + pb); 32 x 32 tiles, lower tiles only.
__global__ void __launch_bounds__(256) k_big_syrk(DevFactor F, DevWork W, int s, int p0, int pb) {
    __shared__ double Ai[32][kNB + 1];
    __shared__ double Aj[32][kNB + 1];
    double* B = W.big + F.sn_big_off[s];
    const int f = F.sn_f[s];
    const int q0 = p0 + pb;
    // map blockIdx.x -> (ti, tj), tj <= ti
    int t = blockIdx.x, ti = 0;
    while (t > ti) { t -= ti + 1; ++ti; }
    const int tj = t;
    const int r0 = q0 + ti * 32, c0 = q0 + tj * 32;
    for (int x = threadIdx.x; x < 32 * pb; x += blockDim.x) {
        const int rr = x % 32, kk = x / 32;
        Ai[rr][kk] = (r0 + rr < f) ? B[(r0 + rr) + (int64_t)(p0 + kk) * f] : 0.0;
        Aj[rr][kk] = (c0 + rr < f) ? B[(c0 + rr) + (int64_t)(p0 + kk) * f] : 0.0;
    }
    __syncthreads();
    // each thread: 4 outputs, rows (threadIdx.x % 32), cols (threadIdx.x / 32) + 8 * q
    const int rr = threadIdx.x % 32;
    for (int qq = 0; qq < 4; ++qq) {
        const int cc = threadIdx.x / 32 + 8 * qq;
        const int gr = r0 + rr, gc = c0 + cc;
        if (gr >= f || gc >= f || gr < gc) continue;
        double acc = 0.0;
        for (int k = 0; k < pb; ++k) acc += Ai[rr][k] * Aj[cc][k];
        B[gr + (int64_t)gc * f] -= acc;
    }
}

__global__ void k_big_writeout(DevFactor F, DevWork W, int s) {
    const double* Bm = W.big + F.sn_big_off[s];
    const int f = F.sn_f[s];
    const int nc = F.sn_c0[s + 1] - F.sn_c0[s];
    const int m = f - nc;
    double* L = W.lx + F.sn_lx_off[s];
    const int64_t nl = (int64_t)f * nc;
    for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < nl; x += (int64_t)gridDim.x * blockDim.x) L[x] = Bm[x];
    double* U = W.u + F.sn_u_off[s];
    const int64_t nu = (int64_t)m * m;
    for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < nu; x += (int64_t)gridDim.x * blockDim.x) {
        const int i = (int)(x % m), j = (int)(x / m);
        U[x] = Bm[(nc + i) + (int64_t)(nc + j) * f];
    }
}

// ---------------------------------------------------------------------------
// Solves.  Forward (bottom-up): v = [rhs of own columns; 0] + children's
// update vectors; y = L11^-1 v1; update vector = v2 - L21 y.
// Backward (top-down): x1 = L11^-T (y - L21^T x_rows).
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) k_fwd(DevFactor F, DevWork W, const int* fronts) {
    extern __shared__ double v[];
    const int s = fronts[blockIdx.x];
    const int f = F.sn_f[s];
    const int c0 = F.sn_c0[s];
    const int nc = F.sn_c0[s + 1] - c0;
    const int tid = threadIdx.x, nth = blockDim.x;
    for (int i = tid; i < f; i += nth) v[i] = (i < nc) ? W.rhs[c0 + i] : 0.0;
    __syncthreads();
    for (int ci = F.sn_child_ptr[s]; ci < F.sn_child_ptr[s + 1]; ++ci) {
        const int c = F.sn_child[ci];
        const int m = F.sn_f[c] - (F.sn_c0[c + 1] - F.sn_c0[c]);
        const double* su = W.su + F.sn_su_off[c];
        const int* rel = F.sn_relmap + F.sn_su_off[c];
        for (int i = tid; i < m; i += nth) v[rel[i]] += su[i];
        __syncthreads();
    }
    const double* L = W.lx + F.sn_lx_off[s];
    for (int k = 0; k < nc; ++k) {
        const double yk = v[k] / L[k + (int64_t)k * f];
        for (int i = k + 1 + tid; i < f; i += nth) v[i] -= L[i + (int64_t)k * f] * yk;
        __syncthreads();
    }
    for (int k = tid; k < nc; k += nth) W.sol[c0 + k] = v[k] / L[k + (int64_t)k * f];
    double* su = W.su + F.sn_su_off[s];
    for (int i = tid; i < f - nc; i += nth) su[i] = v[nc + i];
}

__global__ void __launch_bounds__(kThreads) k_bwd(DevFactor F, DevWork W, const int* fronts) {
    extern __shared__ double t[];
    const int s = fronts[blockIdx.x];
    const int f = F.sn_f[s];
    const int c0 = F.sn_c0[s];
    const int nc = F.sn_c0[s + 1] - c0;
    const int* rows = F.sn_rows + F.sn_rows_off[s];
    const double* L = W.lx + F.sn_lx_off[s];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    for (int k = warp; k < nc; k += nwarp) {
        double acc = 0.0;
        for (int r = nc + lane; r < f; r += 32) acc += L[r + (int64_t)k * f] * W.sol[rows[r]];
        acc = warp_sum(acc);
        if (lane == 0) t[k] = W.sol[c0 + k] - acc;
    }
    __syncthreads();
    for (int k = nc - 1; k >= 0; --k) {
        const double xk = t[k] / L[k + (int64_t)k * f];
        __syncthreads();
        for (int i = threadIdx.x; i < k; i += blockDim.x) t[i] -= L[k + (int64_t)i * f] * xk;
        if (threadIdx.x == 0) t[k] = xk;
        __syncthreads();
    }
    for (int k = threadIdx.x; k < nc; k += blockDim.x) W.sol[c0 + k] = t[k];
}

__global__ void k_gain_export(DevNet net, DevFactor F, DevWork W, int n_tgt, double* out) {
    for (int tg = blockIdx.x * blockDim.x + threadIdx.x; tg < n_tgt; tg += gridDim.x * blockDim.x)
        out[tg] = gain_entry(net, F, W, tg);
}

inline int grid_for(int64_t n, int threads) {
    int64_t g = (n + threads - 1) / threads;
    if (g > 152 * 16) g = 152 * 16;
    return (int)(g < 1 ? 1 : g);
}

}  // namespace

cudaError_t launch_factor(const DevNet& net, const DevFactor& F, const DevWork& W, const LevelSchedule& ls,
                          cudaStream_t st) {
    static bool attr_set = false;
    if (!attr_set) {
        cudaError_t e = cudaFuncSetAttribute(k_front_small, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             kSmallFrontMax * kSmallFrontMax * (int)sizeof(double));
        if (e != cudaSuccess) return e;
        attr_set = true;
    }
    for (int l = 0; l < ls.n_levels; ++l) {
        const int ns = ls.h_small_ptr[l + 1] - ls.h_small_ptr[l];
        if (ns > 0) {
            const int mf = ls.max_small_f;
            const size_t smem = (size_t)mf * mf * sizeof(double);
            k_front_small<<<ns, kThreads, smem, st>>>(net, F, W, ls.d_small + ls.h_small_ptr[l]);
            ++g_kernel_launches;
        }
        for (int b = ls.h_big_ptr[l]; b < ls.h_big_ptr[l + 1]; ++b) {
            const int s = ls.h_big[b];
            const int f = ls.h_sn_f[s];
            const int nc = ls.h_sn_c0[s + 1] - ls.h_sn_c0[s];
            double* B = W.big + ls.h_big_off[s];
            k_big_zero<<<grid_for((int64_t)f * f, 256), 256, 0, st>>>(B, (int64_t)f * f);
            ++g_kernel_launches;
            const int nt = ls.h_tgt_ptr[s + 1] - ls.h_tgt_ptr[s];
            if (nt > 0) {
                k_big_targets<<<grid_for(nt, 256), 256, 0, st>>>(net, F, W, s);
                ++g_kernel_launches;
            }
            for (int ci = ls.h_child_ptr[s]; ci < ls.h_child_ptr[s + 1]; ++ci) {
                const int c = ls.h_child[ci];
                const int64_t m = ls.h_sn_f[c] - (ls.h_sn_c0[c + 1] - ls.h_sn_c0[c]);
                if (m > 0) {
                    k_big_extend_add<<<grid_for(m * m, 256), 256, 0, st>>>(F, W, s, c);
                    ++g_kernel_launches;
                }
            }
            for (int p0 = 0; p0 < nc; p0 += kNB) {
                const int pb = (nc - p0) < kNB ? (nc - p0) : kNB;
                k_big_potrf<<<1, 256, 0, st>>>(F, W, s, p0, pb);
                ++g_kernel_launches;
                const int rows = f - p0 - pb;
                if (rows > 0) {
                    k_big_trsm<<<(rows + 63) / 64, 64, 0, st>>>(F, W, s, p0, pb);
                    const int T = (rows + 31) / 32;
                    k_big_syrk<<<T * (T + 1) / 2, 256, 0, st>>>(F, W, s, p0, pb);
                    g_kernel_launches += 2;
                }
            }
            k_big_writeout<<<grid_for((int64_t)f * f, 256), 256, 0, st>>>(F, W, s);
            ++g_kernel_launches;
        }
    }
    return cudaGetLastError();
}

cudaError_t launch_gain_export(const DevNet& net, const DevFactor& F, const DevWork& W, int32_t n_tgt, double* out,
                               cudaStream_t st) {
    if (n_tgt > 0) {
        k_gain_export<<<grid_for(n_tgt, 256), 256, 0, st>>>(net, F, W, n_tgt, out);
        ++g_kernel_launches;
    }
    return cudaGetLastError();
}

cudaError_t launch_solve(const DevFactor& F, const DevWork& W, const LevelSchedule& ls, cudaStream_t st) {
    for (int l = 0; l < ls.n_levels; ++l) {
        const int n = ls.h_all_ptr[l + 1] - ls.h_all_ptr[l];
        if (n > 0) {
            k_fwd<<<n, kThreads, (size_t)ls.h_lvl_maxf[l] * sizeof(double), st>>>(F, W, ls.d_all + ls.h_all_ptr[l]);
            ++g_kernel_launches;
        }
    }
    for (int l = ls.n_levels - 1; l >= 0; --l) {
        const int n = ls.h_all_ptr[l + 1] - ls.h_all_ptr[l];
        if (n > 0) {
            k_bwd<<<n, kThreads, (size_t)ls.h_lvl_maxf[l] * sizeof(double), st>>>(F, W, ls.d_all + ls.h_all_ptr[l]);
            ++g_kernel_launches;
        }
    }
    return cudaGetLastError();
}

}  // namespace sle_gb300
