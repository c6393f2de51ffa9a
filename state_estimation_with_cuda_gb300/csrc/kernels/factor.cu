// Level-scheduled multifrontal Cholesky of the gain matrix G = H^T W H and the
// forward / backward solves (replaces the reference's per-call
// cusolverSp csrlsvchol, sparse_matrix.cu:793-895, and its quadratic RHS
// kernel, kernels.cu:823-862).
//
// Front s (rows R_s, nc_s pivot columns, order f_s) is assembled from
//   - its gain entries, each a fixed-order sum of w_m H[m,a] H[m,b] over the
//     measurement rows m that couple the two states (gathered, no atomics), and
//   - its children's update matrices, extend-added through relative maps,
// then partially factorised: L11 = chol(F11), L21 = F21 L11^-T,
// U_s = F22 - L21 L21^T.
//
// Small fronts (little work) are one CTA each with the whole front in shared
// memory.  Big fronts live in place in an f x f region (L panel = first nc
// columns, update matrix = trailing block, both column-major with ld = f) and
// are processed for a whole level at once by tile work lists: an assembly
// kernel (one CTA per 32-column tile column, so every entry has one writer), a
// panel kernel (each CTA factors the 32 x 32 diagonal tile and solves one row
// tile against it) and a trailing-update kernel (one CTA per 32 x 32 tile).
// The factor type T is double for the FP64 pipeline and float for the
// mixed-precision one; the mixed pipeline forms the gain entries' sums in
// float (gain_acc32, the default) or in double.
#include "kernels.cuh"

#include <algorithm>
#include <mutex>

namespace sle_gb300 {
namespace {

constexpr int kThreads = 256;

// G entry = sum over its pairs (a, b) of (w h_a) h_b, the weighted entry
// hw[a] written by the evaluation (FP64: the same product, so the same sum),
// accumulated in ACC.
template <typename HV, typename ACC>
__device__ __forceinline__ ACC gain_entry(const DevFactor& F, const HV* hval, const HV* hw, int tg) {
    ACC acc = ACC(0);
    const int64_t p1 = F.tgt_pair_ptr[tg + 1];
    for (int64_t p = F.tgt_pair_ptr[tg]; p < p1; ++p) {
        const int a = F.pair_a[p], b = F.pair_b[p];
        acc += static_cast<ACC>(hw[a]) * static_cast<ACC>(hval[b]);
    }
    return acc;
}

// All gain entries of the factorisation at once: fully parallel, so the
// dependent gathers are hidden by occupancy instead of sitting on the
// elimination tree's critical path.
template <typename T, typename HV, typename ACC = double>
__global__ void k_gain_values(DevFactor F, DevWork W, const HV* hval, const HV* hw, T* gv, int n_tgt) {
    for (int tg = blockIdx.x * blockDim.x + threadIdx.x; tg < n_tgt; tg += gridDim.x * blockDim.x) {
        if (F.tgt_grid && (W.grid_flags[F.tgt_grid[tg]] & FLAG_FROZEN)) continue;
        gv[tg] = static_cast<T>(gain_entry<HV, ACC>(F, hval, hw, tg));
    }
}

// Where a non-positive pivot of front s is reported: the grid's own flags in
// a batch, the engine status otherwise.
__device__ __forceinline__ uint32_t* singular_flags(const DevFactor& F, const DevWork& W, int s) {
    return W.grid_flags ? W.grid_flags + F.sn_grid[s] : &W.status->flags;
}
// Batch: fronts of grids that take no further step are skipped.
__device__ __forceinline__ bool front_frozen(const DevFactor& F, const DevWork& W, int s) {
    return W.grid_flags && (W.grid_flags[F.sn_grid[s]] & FLAG_FROZEN);
}

// Pivot: L_kk = sqrt(d) and 1 / L_kk for a positive finite d (the callers
// flag a non-positive or non-finite d as a matrix that is not positive
// definite and go on with 1).  FP64: a reciprocal square root seeded in FP32
// and refined by two Newton-Raphson steps y <- y (3 - d y^2) / 2 (each step
// doubles the correct bits: ~24 -> 48 -> 96), which keeps serial FP64 work
// short on a GPU with few FP64 units; the library routines are used outside
// the FP32 range.
__device__ __forceinline__ void pivot_value(float d, float* sq, float* inv) {
    const float y = rsqrtf(d);  // the FP32 factor is a preconditioner of FP64 steps
    *sq = d * y;
    *inv = y;
}
__device__ __forceinline__ void pivot_value(double d, double* sq, double* inv) {
    if (d > 1e-30 && d < 1e30) {
        double y = static_cast<double>(rsqrtf(static_cast<float>(d)));
        y = y * (1.5 - 0.5 * d * y * y);
        y = y * (1.5 - 0.5 * d * y * y);
        *sq = d * y;
        *inv = y;
    } else {
        *sq = sqrt(d);
        *inv = 1.0 / *sq;
    }
}

// Extend-add child c's update matrix (lower triangle) into a front buffer.
template <typename T>
__device__ __forceinline__ const T* update_of(const DevFactor& F, const T* lx, const T* ub, int c) {
    return (F.sn_u_big[c] ? lx : ub) + F.sn_u_off[c];
}

// Extend-add of every child of front s with no barrier between children:
// warp w owns the front's target columns t with t % nwarp == w and walks the
// children in order, adding only into its own columns, so no two warps touch
// the same entry and each entry's additions keep the children's order.  Per
// child, the warp selects its columns 32 at a time (ballot over the relative
// map), then loads up to four of them (four rows per lane each) before it
// scatters them.  The caller follows with a block barrier.
template <typename T>
__device__ __forceinline__ void extend_add_children(const DevFactor& F, const T* lx, const T* ubase, int s, T* dst,
                                                    int ldd) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    for (int ci = F.sn_child_ptr[s]; ci < F.sn_child_ptr[s + 1]; ++ci) {
        const int c = F.sn_child[ci];
        const int m = F.sn_f[c] - (F.sn_c0[c + 1] - F.sn_c0[c]);
        const T* U = update_of<T>(F, lx, ubase, c);
        const int uld = F.sn_u_ld[c];
        const int* rel = F.sn_relmap + F.sn_su_off[c];
        for (int j0 = 0; j0 < m; j0 += 32) {
            const int jl = j0 + lane;
            const int tj = (jl < m) ? rel[jl] : -1;
            unsigned own = __ballot_sync(0xffffffffu, tj >= 0 && (tj % nwarp) == warp);
            while (own) {
                int js[4];
                int cnt = 0;
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    js[q] = -1;
                    if (own) {
                        const int b = __ffs(own) - 1;
                        own &= own - 1;
                        js[q] = j0 + b;
                        ++cnt;
                    }
                }
                const int jmin = js[0];  // the smallest column has the most rows
                for (int ib = 0;; ib += 128) {
                    T u[4][4];
                    int ri[4][4];
#pragma unroll
                    for (int q = 0; q < 4; ++q)
#pragma unroll
                        for (int t = 0; t < 4; ++t) {
                            const int j = js[q];
                            const int i = j + ib + lane + 32 * t;
                            const bool ok = j >= 0 && i < m;
                            u[q][t] = ok ? __ldcg(U + (int64_t)j * uld + i) : T(0);
                            ri[q][t] = ok ? rel[i] : -1;
                        }
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const int j = js[q];
                        if (j < 0) continue;
                        const int pj = __shfl_sync(0xffffffffu, tj, j - j0) * ldd;
#pragma unroll
                        for (int t = 0; t < 4; ++t)
                            if (ri[q][t] >= 0) dst[ri[q][t] + pj] += u[q][t];
                    }
                    if (jmin + ib + 128 >= m) break;
                }
                (void)cnt;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Small fronts: one CTA per front, front held in shared memory.
//
// Layout: column-major with a leading dimension padded to 16 bytes
// (front_ld), so four consecutive rows of a column are one or two aligned
// vector loads.  The partial factorisation runs over 32-column panels:
//   (1) warp 0 factors the diagonal block in registers (lane i holds row i,
//       columns broadcast by shuffles) and leaves L11^T and 1/diag in shared
//       memory;
//   (2) every thread solves one row of the panel below the block,
//       x = a L11^-T, by forward substitution in registers;
//   (3) the trailing lower triangle is updated by 4x4 register tiles,
//       A22 -= X X^T, two vector loads and sixteen FMAs per panel column.
// ---------------------------------------------------------------------------
constexpr int kPanel = 32;  // widest panel of the in-shared-memory factorisation
static_assert(kThreads - 32 >= kSmallFrontMax32, "one thread per front row besides warp 0");

template <typename T>
__device__ __forceinline__ void load4(const T* p, T (&v)[4]);
template <>
__device__ __forceinline__ void load4<float>(const float* p, float (&v)[4]) {
    const float4 q = *reinterpret_cast<const float4*>(p);
    v[0] = q.x; v[1] = q.y; v[2] = q.z; v[3] = q.w;
}
template <>
__device__ __forceinline__ void load4<double>(const double* p, double (&v)[4]) {
    const double2 q0 = reinterpret_cast<const double2*>(p)[0];
    const double2 q1 = reinterpret_cast<const double2*>(p)[1];
    v[0] = q0.x; v[1] = q0.y; v[2] = q1.x; v[3] = q1.y;
}
template <typename T>
__device__ __forceinline__ void store4(T* p, const T (&v)[4]);
template <>
__device__ __forceinline__ void store4<float>(float* p, const float (&v)[4]) {
    *reinterpret_cast<float4*>(p) = make_float4(v[0], v[1], v[2], v[3]);
}
template <>
__device__ __forceinline__ void store4<double>(double* p, const double (&v)[4]) {
    reinterpret_cast<double2*>(p)[0] = make_double2(v[0], v[1]);
    reinterpret_cast<double2*>(p)[1] = make_double2(v[2], v[3]);
}

// FP32 factors store L11^-1 in each diagonal block's slot, so that the solves
// multiply by it (independent dot products) instead of sweeping the triangle
// one column at a time.  FP64 keeps L11 there: at this GPU's FP64 rate the
// inversion costs the factorisation more than the solves save.
template <typename T>
constexpr bool kInvDiag = sizeof(T) == 4;

// Diagonal blocks in one warp's registers.  warp_potrf_bcast eliminates the
// first kb columns of the rows the warp holds: lane i owns row i in a[]
// (entries j <= i; zeros elsewhere); the remaining columns receive the Schur
// complement update.  Per pivot k the pivot comes by shuffle, lanes below
// scale their entry by 1 / L_kk, and every entry a_ij, k < j <= i, gets
// a_ij -= l_ik l_jk, the column l_jk broadcast through the 16-byte-aligned
// shared buffer col[] (four FP32 or two FP64 entries per load).  Entries
// above the diagonal are left unmasked: a lane reads col[j] only for j > k,
// written by lane j, whose value there is an entry of L, and the entries
// above the diagonal are never written out.  Fully unrolled and branch-free
// (a branch per column, even one always taken, keeps the next step's loads
// from overlapping the pivot chain).  On return a[] is row i of L and
// *inv_out = 1 / L_ii; returns true if a pivot was not positive and finite
// (then replaced by 1).  warp_trinv_v4 forms L^-1 one column per lane
// (L^-1 e_j by right-looking substitution, its rows read four at a time) and
// writes rows i >= j to dst[i + j * ld].
template <int KP>
__device__ __forceinline__ bool warp_potrf_bcast(float (&a)[KP], int kb, int lane, float* inv_out, float* col) {
    static_assert(KP % 4 == 0, "whole float4 groups");
    bool bad = false;
    float my_inv = 0.f;
#pragma unroll
    for (int k = 0; k < KP; ++k) {
        if (k < kb) {
            float d = __shfl_sync(0xffffffffu, a[k], k);
            bad |= !(d > 0.f) || !isfinite(d);
            d = (d > 0.f && isfinite(d)) ? d : 1.f;
            float sq, inv;
            pivot_value(d, &sq, &inv);
            const float lk = (lane == k) ? sq : (lane > k ? a[k] * inv : a[k]);
            a[k] = lk;
            my_inv = (lane == k) ? inv : my_inv;
            if (k + 1 < KP) {
                col[lane] = lk;
                __syncwarp();
#pragma unroll
                for (int g = (k + 1) / 4; g < KP / 4; ++g) {
                    const float4 v = reinterpret_cast<const float4*>(col)[g];
                    const float w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                        if (4 * g + q > k) a[4 * g + q] = a[4 * g + q] - lk * w[q];
                }
                __syncwarp();
            }
        }
    }
    *inv_out = my_inv;
    return bad;
}

// lt rows 16-byte aligned (LTLD % 4 == 0): each row of L is read four
// entries per broadcast load.
template <int KP, int LTLD>
__device__ __forceinline__ void warp_trinv_v4(const float (*lt)[LTLD], const float* rinv, int kb, int lane, float* dst,
                                              int ld) {
    static_assert(KP % 4 == 0 && LTLD % 4 == 0, "whole, aligned float4 groups");
    float x[KP];
#pragma unroll
    for (int i = 0; i < KP; ++i) x[i] = (i == lane) ? 1.f : 0.f;
#pragma unroll
    for (int c = 0; c < KP; ++c) {
        if (c < kb) {
            x[c] *= rinv[c];
#pragma unroll
            for (int g = (c + 1) / 4; g < KP / 4; ++g) {
                const float4 v = reinterpret_cast<const float4*>(lt[c])[g];
                const float w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
                for (int q = 0; q < 4; ++q)
                    if (4 * g + q > c) x[4 * g + q] -= x[c] * w[q];
            }
        }
    }
    if (lane < kb) {
#pragma unroll
        for (int i = 0; i < KP; ++i)
            if (i >= lane && i < kb) dst[i + lane * ld] = x[i];
    }
}

// FP64 form of warp_potrf_bcast (two entries per 16-byte load).
template <int KP>
__device__ __forceinline__ bool warp_potrf_bcast(double (&a)[KP], int kb, int lane, double* inv_out, double* col) {
    static_assert(KP % 2 == 0, "whole double2 groups");
    bool bad = false;
    double my_inv = 0.0;
#pragma unroll
    for (int k = 0; k < KP; ++k) {
        if (k < kb) {
            double d = __shfl_sync(0xffffffffu, a[k], k);
            bad |= !(d > 0.0) || !isfinite(d);
            d = (d > 0.0 && isfinite(d)) ? d : 1.0;
            double sq, inv;
            pivot_value(d, &sq, &inv);
            const double lk = (lane == k) ? sq : (lane > k ? a[k] * inv : a[k]);
            a[k] = lk;
            my_inv = (lane == k) ? inv : my_inv;
            if (k + 1 < KP) {
                col[lane] = lk;
                __syncwarp();
#pragma unroll
                for (int g = (k + 1) / 2; g < KP / 2; ++g) {
                    const double2 v = reinterpret_cast<const double2*>(col)[g];
                    const double w[2] = {v.x, v.y};
#pragma unroll
                    for (int q = 0; q < 2; ++q)
                        if (2 * g + q > k) a[2 * g + q] = a[2 * g + q] - lk * w[q];
                }
                __syncwarp();
            }
        }
    }
    *inv_out = my_inv;
    return bad;
}

constexpr int kWarpsPerCta = kThreads / 32;
constexpr int kWtLd = kWarpFrontMax + 1;

template <typename T>
struct WarpTile {
    T a[kWarpFrontMax * kWtLd];  // a[c * kWtLd + r] = front entry (r, c)
    T rinv[kWarpFrontMax];
};

__device__ __forceinline__ int warp_claim(int* counter) {
    int item = 0;
    if ((threadIdx.x & 31) == 0) item = atomicAdd(counter, 1);
    return __shfl_sync(0xffffffffu, item, 0);
}

// Lane 0 counts finished front s into its parent when the parent belongs to
// the same phase; returns the parent when this completed its last child.
__device__ __forceinline__ int warp_continue_up(const DevFactor& F, const int8_t* phase, int ph, const int32_t* nchild,
                                                int* cnt, int s) {
    __syncwarp();
    int nxt = -1;
    if ((threadIdx.x & 31) == 0) {
        const int p = F.sn_parent[s];
        if (p >= 0 && phase[p] == ph) {
            __threadfence();
            if (atomicAdd(cnt + p, 1) + 1 == nchild[p]) {
                __threadfence();
                nxt = p;
            }
        }
    }
    nxt = __shfl_sync(0xffffffffu, nxt, 0);
    __syncwarp();
    return nxt;
}

template <typename T>
__device__ void warp_front_factor(const DevFactor& F, const DevWork& W, const T* gv, T* lx, T* ub, int s,
                                  WarpTile<T>& t) {
    const int lane = threadIdx.x & 31;
    const int f = F.sn_f[s];
    const int c0 = F.sn_c0[s];
    const int nc = F.sn_c0[s + 1] - c0;
    for (int c = 0; c < f; ++c) t.a[c * kWtLd + lane] = T(0);
    __syncwarp();
    {
        // original entries, four per lane in flight
        const int tg0 = F.sn_tgt_ptr[s], tg1 = F.sn_tgt_ptr[s + 1];
        for (int tb = tg0; tb < tg1; tb += 128) {
            T g[4];
            int l[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int tg = tb + lane + 32 * q;
                l[q] = tg < tg1 ? F.tgt_local[tg] : -1;  // row + col * f
                g[q] = tg < tg1 ? gv[tg] : T(0);
            }
#pragma unroll
            for (int q = 0; q < 4; ++q)
                if (l[q] >= 0) {
                    const int c = l[q] / f;
                    t.a[c * kWtLd + (l[q] - c * f)] = g[q];
                }
        }
    }
    __syncwarp();
    for (int ci = F.sn_child_ptr[s]; ci < F.sn_child_ptr[s + 1]; ++ci) {
        const int ch = F.sn_child[ci];
        const int m = F.sn_f[ch] - (F.sn_c0[ch + 1] - F.sn_c0[ch]);  // < kWarpFrontMax: the parent holds m rows
        const T* U = update_of<T>(F, lx, ub, ch);
        const int uld = F.sn_u_ld[ch];
        const int ri = lane < m ? F.sn_relmap[F.sn_su_off[ch] + lane] : 0;
        for (int j = 0; j < m; j += 4) {
            T u[4];
#pragma unroll
            for (int q = 0; q < 4; ++q)
                u[q] = (j + q < m && lane >= j + q && lane < m) ? __ldcg(U + lane + (int64_t)(j + q) * uld) : T(0);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int rj = __shfl_sync(0xffffffffu, ri, (j + q) & 31);
                if (j + q < m && lane >= j + q && lane < m) t.a[rj * kWtLd + ri] += u[q];
            }
        }
        __syncwarp();
    }
    // Right-looking elimination of the first nc columns in the tile, lane i
    // owning row i; the trailing columns receive the Schur complement.  The
    // loops are bounded by the front's own size (warp fronts are narrow:
    // median 16 rows, 4 columns), which keeps the kernel small enough for the
    // instruction cache.
    T my_inv = T(0);
    bool bad = false;
    for (int k = 0; k < nc; ++k) {
        T d = t.a[k * kWtLd + k];
        const bool badk = !(d > T(0)) || !isfinite(d);
        bad |= badk;
        d = badk ? T(1) : d;
        T sq, inv;
        pivot_value(d, &sq, &inv);
        const bool below = lane > k && lane < f;
        const T lik = below ? t.a[k * kWtLd + lane] * inv : T(0);
        __syncwarp();  // column k read by every lane before it is overwritten
        if (lane == k) {
            t.a[k * kWtLd + k] = sq;
            my_inv = inv;
        }
        if (below) t.a[k * kWtLd + lane] = lik;
        __syncwarp();
        if (below)
            for (int j = k + 1; j <= lane; ++j) t.a[j * kWtLd + lane] -= lik * t.a[k * kWtLd + j];
        __syncwarp();
    }
    if (bad && lane == 0) atomicOr(singular_flags(F, W, s), FLAG_SINGULAR);
    if (lane < nc) reinterpret_cast<T*>(W.rdiag)[c0 + lane] = my_inv;
    T* L = lx + F.sn_lx_off[s];
    const int row0 = kInvDiag<T> ? nc : 0;  // FP32 writes its diagonal block as L11^-1 below
    if (lane < f)
        for (int c = 0; c < nc; ++c)
            if (lane >= c && lane >= row0) L[lane + c * f] = t.a[c * kWtLd + lane];
    const int m = f - nc;
    T* Uo = ub + F.sn_u_off[s];
    for (int j = nc; j < f; ++j)
        if (lane >= j && lane < f) Uo[(lane - nc) + (j - nc) * m] = t.a[j * kWtLd + lane];
    if constexpr (kInvDiag<T>) {
        // column j of L11^-1 by forward substitution, lane j; its entries
        // x_i (i > j) are kept transposed in the tile's free upper triangle,
        // at (row j, column i)
        if (lane < nc) t.rinv[lane] = my_inv;
        __syncwarp();
        if (lane < nc) {
            const int j = lane;
            for (int i = j + 1; i < nc; ++i) {
                T acc = -t.a[j * kWtLd + i] * my_inv;  // L_ij x_j with x_j = 1 / L_jj
                for (int k = j + 1; k < i; ++k) acc -= t.a[k * kWtLd + i] * t.a[k * kWtLd + j];
                t.a[i * kWtLd + j] = acc * t.rinv[i];
            }
        }
        __syncwarp();
        // L11^-1 into the diagonal block: lane i writes row i
        if (lane < nc)
            for (int j = 0; j <= lane; ++j)
                L[lane + j * f] = (j == lane) ? my_inv : t.a[lane * kWtLd + j];
    }
}

// Shared-memory scratch of one front besides the front itself.
template <typename T>
struct FrontSmem {
    __align__(16) T lt[kPanel][kPanel + 4];  // lt[c][r] = L11[r][c] of the current panel (16-byte aligned rows)
    __align__(16) T col[kPanel];             // pivot column broadcast of warp_potrf_bcast
    T rinv[kPanel];                          // 1 / L11[c][c]
};

// Assembles and partially factorises front s in shared memory (Fm holds
// front_ld(f) x f values) with panels of KP <= kPanel columns.
template <typename T, int KP>
__device__ void front_factor(const DevFactor& F, const DevWork& W, const T* gv, T* lx, T* ub, int s, T* Fm,
                             FrontSmem<T>& sm) {
    static_assert(KP <= kPanel && KP <= 32, "panel wider than a warp");
    const int f = F.sn_f[s];
    const int ldf = front_ld<T>(f);
    const int nc = F.sn_c0[s + 1] - F.sn_c0[s];
    const int tid = threadIdx.x, nth = blockDim.x;
    const int lane = tid & 31, warp = tid >> 5;
    for (int x = tid; x < ldf * f; x += nth) Fm[x] = T(0);
    __syncthreads();
    if (ldf == f) {
        for (int tg = F.sn_tgt_ptr[s] + tid; tg < F.sn_tgt_ptr[s + 1]; tg += nth) Fm[F.tgt_local[tg]] = gv[tg];
    } else {
        for (int tg = F.sn_tgt_ptr[s] + tid; tg < F.sn_tgt_ptr[s + 1]; tg += nth) {
            const int l = F.tgt_local[tg];  // row + col * f
            const int c = l / f;
            Fm[(l - c * f) + c * ldf] = gv[tg];
        }
    }
    __syncthreads();
    extend_add_children<T>(F, lx, ub, s, Fm, ldf);
    __syncthreads();
    T* rdg = reinterpret_cast<T*>(W.rdiag) + F.sn_c0[s];
#pragma unroll 1
    for (int k0 = 0; k0 < nc; k0 += KP) {
        const int kb = min(KP, nc - k0);
        // (1) diagonal block, one warp, in registers.  The loop over the
        // block's columns stays rolled (compact code for a single warp); the
        // current column is picked out of the row registers by selects.
        if (warp == 0) {
            T a[KP];
            const int i = k0 + lane;
#pragma unroll
            for (int j = 0; j < KP; ++j) a[j] = (lane < kb && j <= lane) ? Fm[i + (k0 + j) * ldf] : T(0);
            T my_inv;
            const bool bad = warp_potrf_bcast<KP>(a, kb, lane, &my_inv, sm.col);
            if (lane < kb) {
                sm.rinv[lane] = my_inv;
                rdg[k0 + lane] = my_inv;
            }
            if (bad && lane == 0) atomicOr(singular_flags(F, W, s), FLAG_SINGULAR);
#pragma unroll
            for (int j = 0; j < KP; ++j)
                if (lane < kb && j <= lane) {
                    Fm[i + (k0 + j) * ldf] = a[j];
                    sm.lt[j][lane] = a[j];
                }
        }
        __syncthreads();
        // (2) FP32: warp 0 writes the inverse of the diagonal block into its
        // slot.  The other threads (FP64: all): rows below the block,
        // x = a L11^-T, one row per thread (f - q0 < kThreads - 32)
        const int q0 = k0 + kb;
        constexpr int kInvThreads = kInvDiag<T> ? 32 : 0;
        if (kInvDiag<T> && warp == 0) {
            if constexpr (sizeof(T) == 4)
                warp_trinv_v4<KP, kPanel + 4>(sm.lt, sm.rinv, kb, lane, Fm + k0 + k0 * ldf, ldf);
        } else {
            const int r = q0 + tid - kInvThreads;
            if (r < f) {
                T x[KP];
#pragma unroll
                for (int c = 0; c < KP; ++c) x[c] = (c < kb) ? Fm[r + (k0 + c) * ldf] : T(0);
#pragma unroll
                for (int c = 0; c < KP; ++c) {
                    if (c < kb) {
                        x[c] *= sm.rinv[c];
#pragma unroll
                        for (int c2 = c + 1; c2 < KP; ++c2) x[c2] -= x[c] * sm.lt[c][c2];
                    }
                }
#pragma unroll
                for (int c = 0; c < KP; ++c)
                    if (c < kb) Fm[r + (k0 + c) * ldf] = x[c];
            }
        }
        __syncthreads();
        // (3) trailing update of the lower triangle, 4x4 tiles on 4-aligned
        // rows; tiles are numbered down each tile column so that neighbouring
        // threads touch neighbouring rows (conflict-free vector accesses)
        if (q0 < f) {
            const int R0 = q0 & ~3;
            const int nt = (f - R0 + 3) >> 2;
            const int ntiles = nt * (nt + 1) / 2;
            const float b2 = 2.f * nt + 1.f;
#pragma unroll 1
            for (int t = tid; t < ntiles; t += nth) {
                // column bj holds tiles bi = bj..nt-1 and starts at bj*nt - bj*(bj-1)/2
                int bj = static_cast<int>((b2 - sqrtf(b2 * b2 - 8.f * t)) * 0.5f);
                bj = max(0, min(bj, nt - 1));
                while (bj > 0 && bj * nt - bj * (bj - 1) / 2 > t) --bj;
                while (bj + 1 < nt && (bj + 1) * nt - (bj + 1) * bj / 2 <= t) ++bj;
                const int bi = bj + (t - (bj * nt - bj * (bj - 1) / 2));
                const int i0 = R0 + 4 * bi, j0 = R0 + 4 * bj;
                T acc[4][4];
#pragma unroll
                for (int u = 0; u < 4; ++u)
#pragma unroll
                    for (int v = 0; v < 4; ++v) acc[u][v] = T(0);
#pragma unroll 2
                for (int c = 0; c < kb; ++c) {
                    const T* col = Fm + (k0 + c) * ldf;
                    T av[4], bv[4];
                    load4<T>(col + i0, av);
                    load4<T>(col + j0, bv);
#pragma unroll
                    for (int u = 0; u < 4; ++u)
#pragma unroll
                        for (int v = 0; v < 4; ++v) acc[u][v] += av[u] * bv[v];
                }
#pragma unroll
                for (int v = 0; v < 4; ++v) {
                    const int j = j0 + v;
                    if (j < q0 || j >= f) continue;
                    T* dst = Fm + i0 + j * ldf;
                    T cur[4];
                    load4<T>(dst, cur);
#pragma unroll
                    for (int u = 0; u < 4; ++u)
                        if (i0 + u >= j && i0 + u < f) cur[u] -= acc[u][v];
                    store4<T>(dst, cur);
                }
            }
        }
        __syncthreads();
    }
    T* L = lx + F.sn_lx_off[s];
    for (int x = tid; x < f * nc; x += nth) {
        const int c = x / f;
        L[x] = Fm[(x - c * f) + c * ldf];
    }
    const int m = f - nc;
    T* U = ub + F.sn_u_off[s];
    const int nwarp = nth >> 5;
    for (int j = warp; j < m; j += nwarp)
        for (int i = lane; i < m; i += 32) U[i + (int64_t)j * m] = Fm[(nc + i) + (nc + j) * ldf];
}

// Panel widths: fronts of the high-occupancy dataflow phase (f <= 64) use
// 16-column panels and a register budget for several CTAs per SM; the rest
// use 32-column panels and the full register file (one CTA per SM anyway).
constexpr int kPanelSmall = kPanelFlowA;
template <typename T>
constexpr int kMinBlocksA = sizeof(T) == 4 ? 3 : 2;

template <typename T>
__global__ void __launch_bounds__(kThreads, 1) k_front_small(DevFactor F, DevWork W, const T* gv, T* lx, T* ub,
                                                             const int* fronts) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ FrontSmem<T> sm;
    const int s = fronts[blockIdx.x];
    if (front_frozen(F, W, s)) return;
    front_factor<T, kPanel>(F, W, gv, lx, ub, s, reinterpret_cast<T*>(smem_raw), sm);
}

// ---------------------------------------------------------------------------
// Dataflow scheduling: a persistent grid claims work items in order from an
// atomic counter; an item waits (bounded) until the items it depends on have
// published their completion flag.  Items are ordered so that every
// dependency is claimed earlier, and a CTA only waits on items already
// claimed by running CTAs, so progress never depends on CTAs that have not
// started.  Data produced inside the pass is read with L1-bypassing loads.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void wait_done(const int* flag, uint32_t* status, long long limit) {
    long long spins = 0;
    while (atomicAdd(const_cast<int*>(flag), 0) == 0) {
        if (++spins > limit) {
            atomicOr(status, FLAG_TIMEOUT);
            return;
        }
        __nanosleep(64);
    }
    __threadfence();
}

__device__ __forceinline__ void publish_done(int* flag) {
    __threadfence();
    atomicExch(flag, 1);
}

// Thread 0 alone claims, waits and publishes; each such step is followed by
// __syncwarp() so that warp 0 is converged again before the block barrier
// (the single-warp phases of a front rely on a converged warp 0).
__device__ __forceinline__ int claim(int* counter, int* slot) {
    __syncthreads();
    if (threadIdx.x == 0) *slot = atomicAdd(counter, 1);
    __syncwarp();
    __syncthreads();
    return *slot;
}

// After front s is complete (all threads past a barrier): thread 0 counts s
// into its parent's completed children; the CTA that completes the last child
// of a parent handled by the same sweep (phase[p] == ph, or every front when
// phase is null) continues with that parent.  Returns the next front or -1.
__device__ __forceinline__ int continue_up(const DevFactor& F, const int8_t* phase, int ph, const int32_t* nchild,
                                           int* cnt, int s, int* slot) {
    if (threadIdx.x == 0) {
        int nxt = -1;
        const int p = F.sn_parent[s];
        if (p >= 0 && (phase == nullptr || phase[p] == ph)) {
            __threadfence();
            if (atomicAdd(cnt + p, 1) + 1 == nchild[p]) {
                __threadfence();
                nxt = p;
            }
        }
        *slot = nxt;
    }
    __syncwarp();
    __syncthreads();
    return *slot;
}

template <typename T, int KP, int kMinBlocks>
__global__ void __launch_bounds__(kThreads, kMinBlocks) k_front_flow(DevFactor F, DevWork W, const T* gv, T* lx,
                                                                     T* ub, const int* ready, const int* n_ready,
                                                                     const int8_t* phase, int ph,
                                                                     const int32_t* nchild, int* counter, int* cnt) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ FrontSmem<T> sm;
    __shared__ int slot;
    const int nr = *n_ready;
    for (;;) {
        const int item = claim(counter, &slot);
        if (item >= nr) break;
        int s = ready[item];
        while (s >= 0) {
            if (!front_frozen(F, W, s))
                front_factor<T, KP>(F, W, gv, lx, ub, s, reinterpret_cast<T*>(smem_raw), sm);
            __syncthreads();
            s = continue_up(F, phase, ph, nchild, cnt, s, &slot);
        }
    }
}

// ---------------------------------------------------------------------------
// Big fronts, in place (L panel and update matrix share the f x f region at
// sn_lx_off with ld = f).  Work lists hold int4 (front, a, b, 0).
// ---------------------------------------------------------------------------
__device__ __forceinline__ int lower_bound_i32(const int* a, int lo, int hi, int key) {
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (a[mid] < key) lo = mid + 1; else hi = mid;
    }
    return lo;
}

// Assembly of a tiled front, one CTA per (tile column tj, block rb of
// kAsmRows rows from the tile's first column down): zero the block's lower
// part, write its G entries, then add the update-matrix entries of the
// children that land in it, child by child (a barrier between children keeps
// every entry's sum in child order, as in the single-CTA fronts).  The
// block's target range and its contributing children with their column and
// row ranges come from the host schedule (AsmItem / AsmChild).
template <typename T>
__global__ void __launch_bounds__(kThreads) k_big_assemble(DevFactor F, DevWork W, const T* gv, T* lx, T* ub,
                                                           const AsmItem* work, const AsmChild* kids) {
    const AsmItem wk = work[blockIdx.x];
    const int s = wk.s, tj = wk.tj, rb = wk.rb;
    if (front_frozen(F, W, s)) return;  // the whole CTA, before any barrier
    const int f = F.sn_f[s];
    T* B = lx + F.sn_lx_off[s];
    const int c0 = tj * kTile, c1 = min(c0 + kTile, f);
    const int R0 = c0 + rb * kAsmRows, R1 = min(R0 + kAsmRows, f);
    const int tid = threadIdx.x, nth = blockDim.x;
    for (int x = tid; x < (c1 - c0) * (R1 - R0); x += nth) {
        const int c = c0 + x / (R1 - R0), r = R0 + x % (R1 - R0);
        if (r >= c) B[r + (int64_t)c * f] = T(0);
    }
    __syncthreads();
    for (int tg = wk.tg_lo + tid; tg < wk.tg_hi; tg += nth) {
        const int l = F.tgt_local[tg];
        const int r = l % f;
        if (r >= R0 && r < R1) B[l] = gv[tg];
    }
    __syncthreads();
    for (int ci = wk.ch_lo; ci < wk.ch_hi; ++ci) {
        const AsmChild ch = kids[ci];
        const int c = ch.c;
        const int* rel = F.sn_relmap + F.sn_su_off[c];
        const T* U = update_of<T>(F, lx, ub, c);
        const int uld = F.sn_u_ld[c];
        const int lane = tid & 31, warp = tid >> 5, nwarp = nth >> 5;
        for (int j = ch.j0 + warp; j < ch.j1; j += nwarp) {
            const int64_t pj = (int64_t)rel[j] * f;
            const T* Uj = U + (int64_t)j * uld;
            for (int i0 = max(j, ch.ilo) + lane; i0 < ch.ihi; i0 += 128) {
                T u[4];
                int r[4];
#pragma unroll
                for (int t = 0; t < 4; ++t) {
                    const int i = i0 + 32 * t;
                    u[t] = (i < ch.ihi) ? Uj[i] : T(0);
                    r[t] = (i < ch.ihi) ? rel[i] : 0;
                }
#pragma unroll
                for (int t = 0; t < 4; ++t)
                    if (i0 + 32 * t < ch.ihi) B[r[t] + pj] += u[t];
            }
        }
        __syncthreads();
    }
}

// FP64 panel step p, part 1 (one CTA per front): warp 0 factors the diagonal
// tile with a row per lane in registers (warp_potrf_bcast) and writes L_dd
// back; the other warps solve the rows of tile p below the block (only a last
// block narrower than a tile has any: x = a L_dd^-T by forward substitution in
// registers; volatile reads keep the compiler from hoisting the factor into
// registers across rows).  k_big_trsm takes the row tiles below on many CTAs;
// then the trailing update.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_big_potrf(DevFactor F, DevWork W, T* lx, const int4* work, int p) {
    static_assert(sizeof(T) == 8, "FP32 panels use k_big_panel32");
    constexpr int ld = kTile + 1;
    __shared__ T D[kTile * ld];
    __shared__ T rdiag[kTile];
    __shared__ __align__(16) T colbuf[kTile];
    const int s = work[blockIdx.x].x;
    if (front_frozen(F, W, s)) return;  // the whole CTA, before any barrier
    const int f = F.sn_f[s];
    const int nc = F.sn_c0[s + 1] - F.sn_c0[s];
    T* B = lx + F.sn_lx_off[s];
    const int p0 = p * kTile;
    const int pb = min(kTile, nc - p0);
    if (threadIdx.x < 32) {
        // warp 0: the diagonal block, row i in lane i's registers
        const int i = threadIdx.x;
        T a[kTile];
#pragma unroll
        for (int j = 0; j < kTile; ++j) a[j] = (i < pb && j <= i) ? B[(p0 + i) + (int64_t)(p0 + j) * f] : T(0);
        T inv;
        const bool bad = warp_potrf_bcast<kTile>(a, pb, i, &inv, colbuf);
        if (bad && i == 0) atomicOr(singular_flags(F, W, s), FLAG_SINGULAR);
#pragma unroll
        for (int j = 0; j < kTile; ++j)
            if (i < pb && j <= i) {
                D[i + j * ld] = a[j];
                B[(p0 + i) + (int64_t)(p0 + j) * f] = a[j];
            }
        if (i < pb) {
            rdiag[i] = inv;
            reinterpret_cast<T*>(W.rdiag)[F.sn_c0[s] + p0 + i] = inv;
        }
    }
    __syncthreads();
    if (threadIdx.x >= 32) {
        // the rows of tile p below the block (a last block narrower than a
        // tile): x = a L_dd^-T by forward substitution in registers
        const volatile T* Dv = D;
        const int r_end = min(p0 + kTile, f);
#pragma unroll 1
        for (int r = p0 + pb + threadIdx.x - 32; r < r_end; r += blockDim.x - 32) {
            T x[kTile];
#pragma unroll
            for (int c = 0; c < kTile; ++c) x[c] = (c < pb) ? B[r + (int64_t)(p0 + c) * f] : T(0);
#pragma unroll
            for (int c = 0; c < kTile; ++c) {
                if (c < pb) {
                    x[c] *= rdiag[c];
#pragma unroll
                    for (int c2 = c + 1; c2 < kTile; ++c2) x[c2] -= x[c] * Dv[c2 + c * ld];
                }
            }
#pragma unroll
            for (int c = 0; c < kTile; ++c)
                if (c < pb) B[r + (int64_t)(p0 + c) * f] = x[c];
        }
    }
}

// Loads of front entries in the tiled-front kernels.  kL2: the entry may have
// been written by another CTA of the same launch (the dataflow kernel), so
// the load bypasses L1.
template <bool kL2, typename T>
__device__ __forceinline__ T ld_entry(const T* p) {
    if constexpr (kL2) return __ldcg(p);
    else return *p;
}

// FP32 panel step p of the tiled fronts.  The rows below the diagonal block
// are cut into chunks of kPanelRows, one CTA each.  Every CTA
// factors the 32 x 32 diagonal block itself (warp 0, in registers) and
// inverts it while the other warps stage the chunk's rows of the panel; then
// it solves the chunk as X = A L_dd^-T = A (L_dd^-1)^T, a register-tiled
// product with 4 x 4 outputs per thread.  The CTA that reads the diagonal
// tile last (a counter per front and step) writes L_dd^-1 into it for the
// solves: no CTA reads an overwritten tile, and none waits for another.
template <bool kL2>
__device__ __forceinline__ void big_panel32_item(const DevFactor& F, const DevWork& W, float* lx, int s, int p,
                                                 int chunk, int nchunk, int pair, int* step_cnt) {
    static_assert(kThreads == 256 && kPanelRows == 128 && kTile == 32, "thread tiling below");
    constexpr int ld = kTile + 4;          // 16-byte aligned rows
    constexpr int lt_ld = kTile + 4;       // 16-byte aligned rows
    constexpr int as_ld = kPanelRows + 4;  // 16-byte aligned rows
    __shared__ __align__(16) float D[kTile * ld];  // D[i + j * ld] = L_dd[i][j]
    __shared__ __align__(16) float colbuf[kTile];
    __shared__ float rdiag[kTile];
    __shared__ __align__(16) float Lt[kTile * lt_ld];  // Lt[k][c] = L_dd^-1[c][k]
    __shared__ __align__(16) float As[kTile * as_ld];  // As[k][r] = A[r0 + r][k], then X
    __shared__ int last;
    const int f = F.sn_f[s];
    const int nc = F.sn_c0[s + 1] - F.sn_c0[s];
    float* B = lx + F.sn_lx_off[s];
    const int p0 = p * kTile;
    const int pb = min(kTile, nc - p0);
    const int r0 = p0 + pb + chunk * kPanelRows;    // first row of the chunk
    const int nr = max(0, min(kPanelRows, f - r0));  // its rows
    const int tid = threadIdx.x;
    // From the second step on, the previous step's trailing update has already
    // factored and inverted this diagonal block (look-ahead in k_big_update):
    // its slot holds L_dd^-1, the pivots are checked and rdiag is written.
    const bool pre = p > 0;
    {
        // all staging loads in flight before the first shared-memory store:
        // thread (j, i) with i = tid % 32 reads column j = tid / 32 + 8 q of
        // the diagonal tile and rows i + 32 u of the chunk's column
        constexpr int kQ = kTile / (kThreads / 32);  // columns per thread
        const int i = tid & 31, j0 = tid >> 5;
        float dv[kQ], av[kQ][kPanelRows / 32];
#pragma unroll
        for (int q = 0; q < kQ; ++q) {
            const int j = j0 + q * (kThreads / 32);
            const float* col = B + (int64_t)(p0 + j) * f;
            dv[q] = (j < pb && i < pb && i >= j) ? ld_entry<kL2>(col + p0 + i) : 0.f;
#pragma unroll
            for (int u = 0; u < kPanelRows / 32; ++u) {
                const int r = i + 32 * u;
                av[q][u] = (j < pb && r < nr) ? ld_entry<kL2>(col + r0 + r) : 0.f;
            }
        }
#pragma unroll
        for (int q = 0; q < kQ; ++q) {
            const int j = j0 + q * (kThreads / 32);
            D[i + j * ld] = pre ? 0.f : dv[q];
            Lt[j * lt_ld + i] = pre ? dv[q] : 0.f;  // Lt[j][i] = L_dd^-1[i][j]
#pragma unroll
            for (int u = 0; u < kPanelRows / 32; ++u) As[j * as_ld + i + 32 * u] = av[q][u];
        }
    }
    __syncthreads();
    if (tid == 0) last = !pre && (atomicAdd(step_cnt + pair, 1) == nchunk - 1);  // this CTA's tile reads are done
    if (tid < 32 && !pre) {
        const int i = tid;
        float a[kTile];
#pragma unroll
        for (int j = 0; j < kTile; ++j) a[j] = (i < pb && j <= i) ? D[i + j * ld] : 0.f;
        float inv;
        const bool bad = warp_potrf_bcast<kTile>(a, pb, i, &inv, colbuf);
        if (bad && i == 0 && chunk == 0) atomicOr(singular_flags(F, W, s), FLAG_SINGULAR);
#pragma unroll
        for (int j = 0; j < kTile; ++j)
            if (i < pb && j <= i) D[i + j * ld] = a[j];
        if (i < pb) rdiag[i] = inv;
        if (chunk == 0 && i < pb) reinterpret_cast<float*>(W.rdiag)[F.sn_c0[s] + p0 + i] = inv;
        __syncwarp();
        warp_trinv_v4<kTile, ld>(reinterpret_cast<const float (*)[ld]>(D), rdiag, pb, i, Lt, lt_ld);
    }
    __syncthreads();
    {
        // thread (rg, cg): rows 4rg..4rg+3, columns 4cg..4cg+3 of the chunk
        const int cg = tid & 7, rg = tid >> 3;
        float acc[4][4];
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int v = 0; v < 4; ++v) acc[u][v] = 0.f;
#pragma unroll 8
        for (int k = 0; k < kTile; ++k) {
            const float4 a4 = *reinterpret_cast<const float4*>(&As[k * as_ld + 4 * rg]);
            const float4 l4 = *reinterpret_cast<const float4*>(&Lt[k * lt_ld + 4 * cg]);
            const float av[4] = {a4.x, a4.y, a4.z, a4.w}, lv[4] = {l4.x, l4.y, l4.z, l4.w};
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int v = 0; v < 4; ++v) acc[u][v] += av[u] * lv[v];
        }
        __syncthreads();  // every read of A is done
#pragma unroll
        for (int v = 0; v < 4; ++v)
            *reinterpret_cast<float4*>(&As[(4 * cg + v) * as_ld + 4 * rg]) =
                make_float4(acc[0][v], acc[1][v], acc[2][v], acc[3][v]);
    }
    __syncthreads();
    for (int x = tid; x < kTile * kPanelRows; x += kThreads) {
        const int r = x % kPanelRows, k = x / kPanelRows;
        if (r < nr && k < pb) B[(r0 + r) + (int64_t)(p0 + k) * f] = As[k * as_ld + r];
    }
    if (last) {
        for (int x = tid; x < kTile * kTile; x += kThreads) {
            const int i = x % kTile, j = x / kTile;
            if (i < pb && j <= i) B[(p0 + i) + (int64_t)(p0 + j) * f] = Lt[j * lt_ld + i];
        }
    }
}

__global__ void __launch_bounds__(kThreads) k_big_panel32(DevFactor F, DevWork W, float* lx, const int4* work, int p,
                                                          int* step_cnt) {
    const int4 wk = work[blockIdx.x];
    if (front_frozen(F, W, wk.x)) return;  // the whole CTA, before any barrier
    big_panel32_item<false>(F, W, lx, wk.x, p, wk.y, wk.z, wk.w, step_cnt);
}

// FP64 panel step p, part 2: X = A L_dd^-T for the row tiles ti > p, spread
// over CTAs (one SM's FP64 rate cannot carry a whole panel).  One warp per
// row tile and one lane per row, forward substitution in registers against
// the diagonal tile staged in shared memory.
template <typename T>
constexpr int kTrsmWarps = sizeof(T) == 4 ? 8 : 4;

template <typename T>
__global__ void __launch_bounds__(32 * kTrsmWarps<T>) k_big_trsm(DevFactor F, DevWork W, T* lx, const int4* work,
                                                                 int n_work, int p) {
    __shared__ T lt[kTrsmWarps<T>][kTile][kTile + 1];  // lt[w][c][r] = L_dd[r][c]
    __shared__ T rinv[kTrsmWarps<T>][kTile];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int item = blockIdx.x * kTrsmWarps<T> + warp;
    if (item >= n_work) return;  // the whole warp; no block barrier follows
    const int4 wk = work[item];
    const int s = wk.x, ti = wk.y;
    if (front_frozen(F, W, s)) return;  // the whole warp
    const int f = F.sn_f[s];
    const int nc = F.sn_c0[s + 1] - F.sn_c0[s];
    T* B = lx + F.sn_lx_off[s];
    const int p0 = p * kTile;
    const int pb = min(kTile, nc - p0);
    for (int c = 0; c < pb; ++c)
        lt[warp][c][lane] = (lane < pb && lane > c) ? B[(p0 + lane) + (int64_t)(p0 + c) * f] : T(0);
    if (lane < pb) rinv[warp][lane] = reinterpret_cast<const T*>(W.rdiag)[F.sn_c0[s] + p0 + lane];
    __syncwarp();
    const int r = ti * kTile + lane;
    if (r < f) {
        T x[kTile];
#pragma unroll
        for (int c = 0; c < kTile; ++c) x[c] = (c < pb) ? B[r + (int64_t)(p0 + c) * f] : T(0);
#pragma unroll
        for (int c = 0; c < kTile; ++c) {
            if (c < pb) {
                x[c] *= rinv[warp][c];
#pragma unroll
                for (int c2 = c + 1; c2 < kTile; ++c2) x[c2] -= x[c] * lt[warp][c][c2];
            }
        }
#pragma unroll
        for (int c = 0; c < kTile; ++c)
            if (c < pb) B[r + (int64_t)(p0 + c) * f] = x[c];
    }
}

// Trailing update of step p: the kUpdTile x kUpdTile tile (ti, tj) -= A_i A_j^T
// over the panel's columns, restricted to rows >= cols >= p0 + pb.  The two
// row blocks of the panel are staged k-major in shared memory; thread
// (tr, tc) accumulates rows tr + 16u and columns tc + 16v (u, v < 2) in
// registers, four shared loads per four FMAs (a thread per output needed
// two per FMA), and its read-modify-writes of a column touch 16 consecutive
// rows per half warp.
template <typename T, bool kL2>
__device__ __forceinline__ void big_update_item(const DevFactor& F, const DevWork& W, T* lx, int s, int p, int ti,
                                                int tj) {
    static_assert(kThreads == 256 && kUpdTile == 32, "thread tiling below");
    constexpr int ld = kUpdTile + 1;
    __shared__ T Ai[kTile * ld];  // Ai[k * ld + r] = A(R0 + r, p0 + k)
    __shared__ T Aj[kTile * ld];
    const int f = F.sn_f[s];
    const int nc = F.sn_c0[s + 1] - F.sn_c0[s];
    T* B = lx + F.sn_lx_off[s];
    const int p0 = p * kTile;
    const int pb = min(kTile, nc - p0);
    const int q0 = p0 + pb;
    const int R0 = ti * kUpdTile, C0 = tj * kUpdTile;
    for (int x = threadIdx.x; x < kUpdTile * kTile; x += kThreads) {
        const int r = x % kUpdTile, k = x / kUpdTile;
        const T* col = B + (int64_t)(p0 + k) * f;
        Ai[k * ld + r] = (k < pb && R0 + r < f) ? ld_entry<kL2>(col + R0 + r) : T(0);
        Aj[k * ld + r] = (k < pb && C0 + r < f) ? ld_entry<kL2>(col + C0 + r) : T(0);
    }
    __syncthreads();
    const int tr = threadIdx.x & 15, tc = threadIdx.x >> 4;
    T acc[2][2] = {{T(0), T(0)}, {T(0), T(0)}};
#pragma unroll 4
    for (int k = 0; k < pb; ++k) {
        const T a0 = Ai[k * ld + tr], a1 = Ai[k * ld + tr + 16];
        const T b0 = Aj[k * ld + tc], b1 = Aj[k * ld + tc + 16];
        acc[0][0] += a0 * b0;
        acc[0][1] += a0 * b1;
        acc[1][0] += a1 * b0;
        acc[1][1] += a1 * b1;
    }
#pragma unroll
    for (int v = 0; v < 2; ++v) {
        const int gc = C0 + tc + 16 * v;
        if (gc < q0 || gc >= f) continue;
        T* dst = B + (int64_t)gc * f;
#pragma unroll
        for (int u = 0; u < 2; ++u) {
            const int gr = R0 + tr + 16 * u;
            if (gr >= gc && gr < f) dst[gr] = ld_entry<kL2>(dst + gr) - acc[u][v];
        }
    }
    if constexpr (sizeof(T) == 4) {
        // Look-ahead (FP32 tiled fronts): the tile that is the next step's
        // diagonal block comes first in the step's work list; after its own
        // update its CTA factors the block (L_dd) and inverts it in warp 0
        // while the step's other tiles are still updating, and leaves L_dd^-1
        // in the block's slot, the pivots' reciprocals in rdiag and the pivot
        // check done, so that the next panel step only applies L_dd^-1.  The
        // arithmetic is that of the panel kernel's own factorisation.
        if (ti == tj && R0 == q0 && q0 < nc) {
            constexpr int dld = kTile + 4, lt_ld = kTile + 4;  // 16-byte aligned rows
            __shared__ __align__(16) float D[kTile * dld];
            __shared__ float rdiag[kTile];
            __shared__ float Lt[kTile * lt_ld];
            __shared__ __align__(16) float colbuf[kTile];
            __syncthreads();  // every update of this tile is written
            const int pb2 = min(kTile, nc - q0);
            if (threadIdx.x < 32) {
                const int i = threadIdx.x;
                float a[kTile];
#pragma unroll
                for (int j = 0; j < kTile; ++j)
                    a[j] = (i < pb2 && j <= i) ? ld_entry<kL2>(B + (q0 + i) + (int64_t)(q0 + j) * f) : 0.f;
                float inv;
                const bool bad = warp_potrf_bcast<kTile>(a, pb2, i, &inv, colbuf);
                if (bad && i == 0) atomicOr(singular_flags(F, W, s), FLAG_SINGULAR);
#pragma unroll
                for (int j = 0; j < kTile; ++j) D[i + j * dld] = (i < pb2 && j <= i) ? a[j] : 0.f;
                if (i < pb2) {
                    rdiag[i] = inv;
                    reinterpret_cast<float*>(W.rdiag)[F.sn_c0[s] + q0 + i] = inv;
                }
                __syncwarp();
                warp_trinv_v4<kTile, dld>(reinterpret_cast<const float (*)[dld]>(D), rdiag, pb2, i, Lt, lt_ld);
                __syncwarp();
                for (int c = 0; c < pb2; ++c)
                    if (i >= c && i < pb2) B[(q0 + i) + (int64_t)(q0 + c) * f] = Lt[c * lt_ld + i];
            }
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(kThreads) k_big_update(DevFactor F, DevWork W, T* lx, const int4* work, int p) {
    const int4 wk = work[blockIdx.x];
    if (front_frozen(F, W, wk.x)) return;  // the whole CTA, before any barrier
    big_update_item<T, false>(F, W, lx, wk.x, p, wk.y, wk.z);
}

// Bounded wait of the tiled-front dataflow (one lane per dependency): true
// once the flag is set; false when the wait runs out (it then raises
// FLAG_TIMEOUT) or when another wait of the pass has run out, so that a
// failed pass ends in about one spin limit instead of one per item.
__device__ __forceinline__ bool wait_tile(const int* flag, uint32_t* status, long long limit) {
    long long spins = 0;
    for (;;) {
        int v;
        asm volatile("ld.acquire.gpu.global.b32 %0, [%1];" : "=r"(v) : "l"(flag) : "memory");
        if (v != 0) return true;
        if (++spins > limit) {
            atomicOr(status, FLAG_TIMEOUT);
            return false;
        }
        if ((spins & 63) == 0 && (atomicOr(status, 0u) & FLAG_TIMEOUT)) return false;
        __nanosleep(32);
    }
}

// FP32 tiled fronts of one synchronous level in one launch: a persistent grid
// claims the level's TileTask items in order, waits (bounded) for each
// item's dependencies and publishes its completion; the items run the same
// arithmetic as the per-step kernels.  Dependencies are always claimed
// earlier, so the smallest unfinished item is always running and progress
// never depends on CTAs that have not started (the grid need not be
// co-resident; a CTA holds at most the item it runs and the next one it has
// claimed).  Per item: the next claim and its 64-byte task load are issued
// while the current item runs, and warp 0 polls the dependencies in
// parallel, one lane each.  Entries written during the launch are read past
// L1 (ld_entry<true>).  Items of frozen grids, and every item once a wait has
// timed out, publish without computing.
constexpr int kTileFlowBlocks = 3;
__global__ void __launch_bounds__(kThreads, kTileFlowBlocks)
    k_big_flow32(DevFactor F, DevWork W, float* lx, const TileTask* tasks, int n, int* done, int* counter,
                 int* step_cnt) {
    constexpr int kWords = sizeof(TileTask) / sizeof(int);
    static_assert(kWords <= 32, "one lane per task word");
    __shared__ TileTask task[2];
    __shared__ int next[2];
    __shared__ int skip;
    const int tid = threadIdx.x, lane = tid & 31;
    uint32_t* status = &W.status->flags;
    int buf = 0;
    if (tid < 32) {
        int item = 0;
        if (lane == 0) item = atomicAdd(counter, 1);
        item = __shfl_sync(0xffffffffu, item, 0);
        if (lane == 0) next[0] = item;
        if (item < n && lane < kWords)
            reinterpret_cast<int*>(&task[0])[lane] = __ldg(reinterpret_cast<const int*>(tasks + item) + lane);
    }
    __syncthreads();
    for (;;) {
        const int item = next[buf];
        if (item >= n) break;
        // warp 1 claims and loads the next item; warp 0 waits for this one's inputs
        if (tid >= 32 && tid < 64) {
            int nx = 0;
            if (lane == 0) nx = atomicAdd(counter, 1);
            nx = __shfl_sync(0xffffffffu, nx, 0);
            if (lane == 0) next[buf ^ 1] = nx;
            if (nx < n && lane < kWords)
                reinterpret_cast<int*>(&task[buf ^ 1])[lane] =
                    __ldg(reinterpret_cast<const int*>(tasks + nx) + lane);
        }
        const TileTask& t = task[buf];
        if (tid < 32) {
            const bool ok = lane < t.ndep ? wait_tile(done + t.dep[lane], status, W.spin_limit) : true;
            const bool all = __all_sync(0xffffffffu, ok);
            if (lane == 0) skip = !all || front_frozen(F, W, t.s) || (atomicOr(status, 0u) & FLAG_TIMEOUT) != 0u;
            __syncwarp();
        }
        __syncthreads();
        if (!skip) {
            if (t.kind == 0)
                big_panel32_item<true>(F, W, lx, t.s, t.p, t.a, t.b, t.aux, step_cnt);
            else
                big_update_item<float, true>(F, W, lx, t.s, t.p, t.a, t.b);
        }
        __syncthreads();
        if (tid == 0) publish_done(done + item);
        __syncwarp();
        buf ^= 1;
    }
}

// ---------------------------------------------------------------------------
// Solves.  Forward (bottom-up): v = [b of own columns; 0] + children's update
// vectors; y = L11^-1 v1; update vector = v2 - L21 y.
// Backward (top-down): x1 = L11^-T (y - L21^T x_rows).
// Blocked by columns: each diagonal block is staged in shared memory and
// applied by one warp (FP32: a mat-vec with the stored L11^-1, one lane per
// row; FP64: a column sweep); the rectangular update below (forward) or the
// dot products against the solved rows (backward) use every thread with
// coalesced reads of the column-major panel.
// ---------------------------------------------------------------------------
struct SolveVecs {
    const void* rhs;  // [n_state] right-hand side, permuted (V)
    void* sol;        // [n_state] solution, permuted (V)
    void* su;         // solve update vectors (V)
};

// Forward step of a warp front: v = [b of own columns; 0] + children's update
// vectors (in child order), y = L11^-1 v1, update vector v2 - L21 y.
template <typename T, typename V>
__device__ void warp_front_fwd(const DevFactor& F, const T* lx, const T* rdiag, const SolveVecs& sv, int s, V* v) {
    const V* rhs = reinterpret_cast<const V*>(sv.rhs);
    V* sol = reinterpret_cast<V*>(sv.sol);
    V* sub = reinterpret_cast<V*>(sv.su);
    const int lane = threadIdx.x & 31;
    const int f = F.sn_f[s];
    const int c0 = F.sn_c0[s];
    const int nc = F.sn_c0[s + 1] - c0;
    const T* L = lx + F.sn_lx_off[s];
    const V rd = (!kInvDiag<T> && lane < nc) ? static_cast<V>(rdiag[c0 + lane]) : V(0);
    v[lane] = (lane < nc) ? rhs[c0 + lane] : V(0);
    __syncwarp();
    const int cp0 = F.sn_child_ptr[s], cp1 = F.sn_child_ptr[s + 1];
    for (int cb = cp0; cb < cp1; cb += 8) {
        V val[8];
        int row[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            row[u] = -1;
            val[u] = V(0);
            if (cb + u < cp1) {
                const int c = F.sn_child[cb + u];
                const int m = F.sn_f[c] - (F.sn_c0[c + 1] - F.sn_c0[c]);
                if (lane < m) {
                    const int64_t o = F.sn_su_off[c];
                    val[u] = __ldcg(sub + o + lane);
                    row[u] = F.sn_relmap[o + lane];
                }
            }
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            if (row[u] >= 0) v[row[u]] += val[u];
            __syncwarp();
        }
    }
    V y = V(0);
    if constexpr (kInvDiag<T>) {
        if (lane < nc)
            for (int j = 0; j <= lane; ++j) y += static_cast<V>(L[lane + j * f]) * v[j];
        __syncwarp();
        if (lane < nc) v[lane] = y;
    } else {
        for (int k = 0; k < nc; ++k) {
            const V yk = v[k] * __shfl_sync(0xffffffffu, rd, k);
            __syncwarp();
            if (lane > k && lane < nc) v[lane] -= static_cast<V>(L[lane + k * f]) * yk;
            if (lane == 0) v[k] = yk;
            __syncwarp();
        }
        y = lane < nc ? v[lane] : V(0);
    }
    __syncwarp();
    if (lane < nc) {
        sol[c0 + lane] = y;
    } else if (lane < f) {
        V acc = v[lane];
        for (int k = 0; k < nc; ++k) acc -= static_cast<V>(L[lane + k * f]) * v[k];
        sub[F.sn_su_off[s] + (lane - nc)] = acc;
    }
    __syncwarp();
}

// Backward step of a warp front: t = y - L21^T x2, x1 = L11^-T t (lane c
// computes column c).
template <typename T, typename V>
__device__ void warp_front_bwd(const DevFactor& F, const T* lx, const T* rdiag, const SolveVecs& sv, int s, V* x) {
    V* sol = reinterpret_cast<V*>(sv.sol);
    const int lane = threadIdx.x & 31;
    const int f = F.sn_f[s];
    const int c0 = F.sn_c0[s];
    const int nc = F.sn_c0[s + 1] - c0;
    const int* rows = F.sn_rows + F.sn_rows_off[s];
    const T* L = lx + F.sn_lx_off[s];
    const V rd = (!kInvDiag<T> && lane < nc) ? static_cast<V>(rdiag[c0 + lane]) : V(0);
    x[lane] = lane < f ? (lane < nc ? __ldcg(sol + c0 + lane) : __ldcg(sol + rows[lane])) : V(0);
    __syncwarp();
    V t = V(0);
    if (lane < nc) {
        t = x[lane];
        for (int r = nc; r < f; ++r) t -= static_cast<V>(L[r + lane * f]) * x[r];
    }
    __syncwarp();
    if (lane < nc) x[lane] = t;
    __syncwarp();
    if constexpr (kInvDiag<T>) {
        V val = V(0);
        if (lane < nc)
            for (int i = lane; i < nc; ++i) val += static_cast<V>(L[i + lane * f]) * x[i];
        __syncwarp();
        if (lane < nc) x[lane] = val;
    } else {
        for (int k = nc - 1; k >= 0; --k) {
            const V xk = x[k] * __shfl_sync(0xffffffffu, rd, k);
            __syncwarp();
            if (lane < k) x[lane] -= static_cast<V>(L[k + lane * f]) * xk;
            if (lane == 0) x[k] = xk;
            __syncwarp();
        }
    }
    __syncwarp();
    if (lane < nc) sol[c0 + lane] = x[lane];
    __syncwarp();
}

template <typename T, typename V>
__device__ void front_fwd(const DevFactor& F, const T* lx, const T* rdiag, const SolveVecs& sv, int s, V* v, T* D) {
    const V* rhs = reinterpret_cast<const V*>(sv.rhs);
    V* sol = reinterpret_cast<V*>(sv.sol);
    V* sub = reinterpret_cast<V*>(sv.su);
    const int f = F.sn_f[s];
    const int c0 = F.sn_c0[s];
    const int nc = F.sn_c0[s + 1] - c0;
    const int tid = threadIdx.x, nth = blockDim.x;
    const T* L = lx + F.sn_lx_off[s];
    for (int i = tid; i < f; i += nth) v[i] = (i < nc) ? rhs[c0 + i] : V(0);
    __syncthreads();
    // children's update vectors, eight children at a time: every thread issues
    // its loads for all eight before the ordered adds (one barrier per child
    // keeps the sum order fixed)
    const int cp0 = F.sn_child_ptr[s], cp1 = F.sn_child_ptr[s + 1];
    for (int cb = cp0; cb < cp1; cb += 8) {
        V val[8];
        int row[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            row[u] = -1;
            val[u] = V(0);
            if (cb + u < cp1) {
                const int c = F.sn_child[cb + u];
                const int m = F.sn_f[c] - (F.sn_c0[c + 1] - F.sn_c0[c]);
                if (tid < m) {
                    const int64_t o = F.sn_su_off[c];
                    val[u] = __ldcg(sub + o + tid);
                    row[u] = F.sn_relmap[o + tid];
                }
            }
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            if (cb + u < cp1) {
                if (row[u] >= 0) v[row[u]] += val[u];
                const int c = F.sn_child[cb + u];
                const int m = F.sn_f[c] - (F.sn_c0[c + 1] - F.sn_c0[c]);
                const int64_t o = F.sn_su_off[c];
                for (int i = tid + nth; i < m; i += nth) v[F.sn_relmap[o + i]] += __ldcg(sub + o + i);
                __syncthreads();
            }
        }
    }
    // blocks of the factor's panel width (FP32: the diagonal slots hold
    // L11^-1) or of kTile (FP64: L11 with its reciprocal diagonal)
    const int bw = kInvDiag<T> ? (F.sn_pw ? F.sn_pw[s] : kTile) : kTile;
    constexpr int ld = kTile + 1;
    for (int k0 = 0; k0 < nc; k0 += bw) {
        const int kb = min(bw, nc - k0);
        for (int x = tid; x < kb * kb; x += nth) {
            const int i = x % kb, j = x / kb;
            if constexpr (kInvDiag<T>)
                D[i + j * ld] = (i >= j) ? L[(k0 + i) + (int64_t)(k0 + j) * f] : T(0);
            else
                D[i + j * ld] = (i == j) ? rdiag[c0 + k0 + i] : L[(k0 + i) + (int64_t)(k0 + j) * f];
        }
        __syncthreads();
        if (tid < 32) {
            if constexpr (kInvDiag<T>) {
                // y = L11^-1 v: one lane per row, independent dot products
                V y = V(0);
                if (tid < kb)
                    for (int j = 0; j <= tid; ++j) y += static_cast<V>(D[tid + j * ld]) * v[k0 + j];
                __syncwarp();
                if (tid < kb) v[k0 + tid] = y;
            } else {
                // column sweep, lane i updating row k + 1 + i
                for (int k = 0; k < kb; ++k) {
                    const V yk = v[k0 + k] * static_cast<V>(D[k + k * ld]);
                    __syncwarp();
                    const int i = k + 1 + tid;
                    if (i < kb) v[k0 + i] -= static_cast<V>(D[i + k * ld]) * yk;
                    if (tid == 0) v[k0 + k] = yk;
                    __syncwarp();
                }
            }
        }
        __syncthreads();
        for (int i = k0 + kb + tid; i < f; i += nth) {
            V acc = v[i];
            for (int k = 0; k < kb; ++k) acc -= static_cast<V>(L[i + (int64_t)(k0 + k) * f]) * v[k0 + k];
            v[i] = acc;
        }
        __syncthreads();
    }
    for (int k = tid; k < nc; k += nth) sol[c0 + k] = v[k];
    V* su = sub + F.sn_su_off[s];
    for (int i = tid; i < f - nc; i += nth) su[i] = v[nc + i];
}

template <typename V>
__device__ __forceinline__ V warp_sum_v(V v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Column entries a lane of the backward CTA sweep loads ahead of their use.
template <typename T>
constexpr int kSolveBatch = sizeof(T) == 4 ? 16 : 8;

template <typename T, typename V>
__device__ void front_bwd(const DevFactor& F, const T* lx, const T* rdiag, const SolveVecs& sv, int s, V* x, T* D) {
    V* sol = reinterpret_cast<V*>(sv.sol);
    const int f = F.sn_f[s];
    const int c0 = F.sn_c0[s];
    const int nc = F.sn_c0[s + 1] - c0;
    const int* rows = F.sn_rows + F.sn_rows_off[s];
    const T* L = lx + F.sn_lx_off[s];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    for (int r = threadIdx.x; r < f; r += blockDim.x) x[r] = (r < nc) ? __ldcg(sol + c0 + r) : __ldcg(sol + rows[r]);
    __syncthreads();
    // blocks as in the forward sweep, last first; x1 = L11^-T t
    const int bw = kInvDiag<T> ? (F.sn_pw ? F.sn_pw[s] : kTile) : kTile;
    constexpr int ld = kTile + 1;
    const int nblk = (nc + bw - 1) / bw;
    for (int b = nblk - 1; b >= 0; --b) {
        const int k0 = b * bw, kb = min(bw, nc - k0);
        // t_k = x_k - sum over the rows below of L[r][k] x_r, rows in order;
        // long columns load kSolveBatch entries per lane ahead of their use
        // (the same additions, a load latency per batch instead of per entry)
        for (int k = k0 + warp; k < k0 + kb; k += nwarp) {
            V acc = V(0);
            const T* Lk = L + (int64_t)k * f;
            int r = k0 + kb + lane;
            for (; r + 32 * (kSolveBatch<T> - 1) < f; r += 32 * kSolveBatch<T>) {
                T l[kSolveBatch<T>];
#pragma unroll
                for (int u = 0; u < kSolveBatch<T>; ++u) l[u] = Lk[r + 32 * u];
#pragma unroll
                for (int u = 0; u < kSolveBatch<T>; ++u) acc += static_cast<V>(l[u]) * x[r + 32 * u];
            }
            for (; r < f; r += 32) acc += static_cast<V>(Lk[r]) * x[r];
            acc = warp_sum_v(acc);
            if (lane == 0) x[k] -= acc;
        }
        for (int q = threadIdx.x; q < kb * kb; q += blockDim.x) {
            const int i = q % kb, j = q / kb;
            if constexpr (kInvDiag<T>)
                D[i + j * ld] = (i >= j) ? L[(k0 + i) + (int64_t)(k0 + j) * f] : T(0);
            else
                D[i + j * ld] = (i == j) ? rdiag[c0 + k0 + i] : L[(k0 + i) + (int64_t)(k0 + j) * f];
        }
        __syncthreads();
        if (threadIdx.x < 32) {
            if constexpr (kInvDiag<T>) {
                // x = (L11^-1)^T t: one lane per column of L11^-1
                const int c = threadIdx.x;
                V val = V(0);
                if (c < kb)
                    for (int i = c; i < kb; ++i) val += static_cast<V>(D[i + c * ld]) * x[k0 + i];
                __syncwarp();
                if (c < kb) x[k0 + c] = val;
            } else {
                // column sweep from the last, lane i updating row i < k
                for (int k = kb - 1; k >= 0; --k) {
                    const V xk = x[k0 + k] * static_cast<V>(D[k + k * ld]);
                    __syncwarp();
                    const int i = threadIdx.x;
                    if (i < k) x[k0 + i] -= static_cast<V>(D[k + i * ld]) * xk;
                    if (threadIdx.x == 0) x[k0 + k] = xk;
                    __syncwarp();
                }
            }
        }
        __syncthreads();
    }
    for (int k = threadIdx.x; k < nc; k += blockDim.x) sol[c0 + k] = x[k];
}

template <typename T, typename V>
__global__ void __launch_bounds__(kThreads) k_fwd(DevFactor F, const T* lx, const T* rdiag, SolveVecs sv,
                                                  const int* fronts) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ T D[kTile * (kTile + 1)];
    front_fwd<T, V>(F, lx, rdiag, sv, fronts[blockIdx.x], reinterpret_cast<V*>(smem_raw), D);
}

template <typename T, typename V>
__global__ void __launch_bounds__(kThreads) k_bwd(DevFactor F, const T* lx, const T* rdiag, SolveVecs sv,
                                                  const int* fronts) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ T D[kTile * (kTile + 1)];
    front_bwd<T, V>(F, lx, rdiag, sv, fronts[blockIdx.x], reinterpret_cast<V*>(smem_raw), D);
}

// Forward sweep by continuation from the leaves (see continue_up).
template <typename T, typename V>
__global__ void __launch_bounds__(kThreads) k_fwd_flow(DevFactor F, DevWork W, const T* lx, const T* rdiag,
                                                       SolveVecs sv, const int* ready, const int* n_ready,
                                                       const int32_t* nchild, int* counter, int* cnt) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ T D[kTile * (kTile + 1)];
    __shared__ int slot;
    const int nr = *n_ready;
    for (;;) {
        const int item = claim(counter, &slot);
        if (item >= nr) break;
        int s = ready[item];
        while (s >= 0) {
            if (!front_frozen(F, W, s)) front_fwd<T, V>(F, lx, rdiag, sv, s, reinterpret_cast<V*>(smem_raw), D);
            __syncthreads();
            s = continue_up(F, nullptr, 0, nchild, cnt, s, &slot);
        }
    }
}

// Backward sweep as dataflow: order = fronts top-down, waits on the parent.
template <typename T, typename V>
__global__ void __launch_bounds__(kThreads) k_bwd_flow(DevFactor F, DevWork W, const T* lx, const T* rdiag,
                                                       SolveVecs sv, const int* order, const int* n_items,
                                                       int* counter, int* done) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ T D[kTile * (kTile + 1)];
    __shared__ int slot;
    const int ni = *n_items;
    for (;;) {
        const int item = claim(counter, &slot);
        if (item >= ni) break;
        const int s = order[item];
        if (front_frozen(F, W, s)) {
            if (threadIdx.x == 0) publish_done(done + s);
            __syncwarp();
            continue;
        }
        if (threadIdx.x == 0 && F.sn_parent[s] >= 0)
            wait_done(done + F.sn_parent[s], &W.status->flags, W.spin_limit);
        __syncwarp();
        __syncthreads();
        front_bwd<T, V>(F, lx, rdiag, sv, s, reinterpret_cast<V*>(smem_raw), D);
        __syncthreads();
        if (threadIdx.x == 0 && s != W.hold_front) publish_done(done + s);
    }
}

// ---------------------------------------------------------------------------
// Warp fronts: a front whose whole subtree is at most kWarpFrontMax wide is
// handled by one warp (eight fronts per CTA, no block barriers).  Factor: the
// front is assembled in the warp's tile in shared memory (original entries,
// then the children's update matrices in child order), loaded row per lane
// into registers and partially factorised there (the first nc pivots, which
// also leave the Schur complement in the trailing columns), then L (FP32:
// with L11^-1 in its diagonal block) and the update matrix are written out.
// Solves: the forward and backward steps of the same fronts, a lane per row.
// A warp continues with the parent when it completes the parent's last child
// in the same phase, as the CTA sweeps do.
// ---------------------------------------------------------------------------
template <typename T>
constexpr int kMinBlocksW = sizeof(T) == 4 ? 4 : 2;

template <typename T>
__global__ void __launch_bounds__(kThreads, kMinBlocksW<T>) k_front_warp(DevFactor F, DevWork W, const T* gv, T* lx,
                                                                         T* ub, const int* ready, const int* n_ready,
                                                                         const int8_t* phase, int ph,
                                                                         const int32_t* nchild, int* counter,
                                                                         int* cnt) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    WarpTile<T>& t = reinterpret_cast<WarpTile<T>*>(smem_raw)[threadIdx.x >> 5];
    const int nr = *n_ready;
    for (;;) {
        const int item = warp_claim(counter);
        if (item >= nr) break;
        int s = ready[item];
        while (s >= 0) {
            if (!front_frozen(F, W, s)) warp_front_factor<T>(F, W, gv, lx, ub, s, t);
            s = warp_continue_up(F, phase, ph, nchild, cnt, s);
        }
    }
}

template <typename T, typename V>
__global__ void __launch_bounds__(kThreads) k_fwd_warp(DevFactor F, DevWork W, const T* lx, const T* rdiag,
                                                       SolveVecs sv, const int* ready, const int* n_ready,
                                                       const int8_t* phase, int ph, const int32_t* nchild,
                                                       int* counter, int* cnt) {
    __shared__ V vw[kWarpsPerCta][kWarpFrontMax];
    V* v = vw[threadIdx.x >> 5];
    const int nr = *n_ready;
    for (;;) {
        const int item = warp_claim(counter);
        if (item >= nr) break;
        int s = ready[item];
        while (s >= 0) {
            if (!front_frozen(F, W, s)) warp_front_fwd<T, V>(F, lx, rdiag, sv, s, v);
            s = warp_continue_up(F, phase, ph, nchild, cnt, s);
        }
    }
}

// Backward steps of the warp fronts in top-down order, each waiting (bounded)
// on its parent's flag; parents outside the warp phase finished in the CTA
// sweep before this launch.
template <typename T, typename V>
__global__ void __launch_bounds__(kThreads) k_bwd_warp(DevFactor F, DevWork W, const T* lx, const T* rdiag,
                                                       SolveVecs sv, const int* order, const int* n_items,
                                                       int* counter, int* done) {
    __shared__ V xw[kWarpsPerCta][kWarpFrontMax];
    V* x = xw[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const int ni = *n_items;
    for (;;) {
        const int item = warp_claim(counter);
        if (item >= ni) break;
        const int s = order[item];
        if (!front_frozen(F, W, s)) {
            if (lane == 0 && F.sn_parent[s] >= 0) wait_done(done + F.sn_parent[s], &W.status->flags, W.spin_limit);
            __syncwarp();
            warp_front_bwd<T, V>(F, lx, rdiag, sv, s, x);
        }
        if (lane == 0 && s != W.hold_front) publish_done(done + s);
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// Claim-list compaction for a batch.  The lists (phase A, phase B, forward
// leaves, backward order, warp phase, warp backward order) are cut into chunks of kCompactChunk
// entries, one CTA each.  Pass 1 counts each chunk's fronts whose grid is not
// frozen; pass 2 offsets a chunk by the counts of the chunks before it in
// the same list and writes its kept entries in their original order (the
// claim order carries the critical-path priority and, for the backward
// sweep, parents before children).  A frozen grid's fronts form whole trees
// of their own, so no kept front has a dropped child or parent.
// ---------------------------------------------------------------------------
struct ReadyLists {
    const int* src[kReadyLists];
    int* dst[kReadyLists];
    int n[kReadyLists];
    int chunk0[kReadyLists + 1];  // first chunk of each list; the last entry = all chunks
};

__device__ __forceinline__ int list_of_chunk(const ReadyLists& R, int b) {
    int l = 0;
    while (l < kReadyLists - 1 && b >= R.chunk0[l + 1]) ++l;
    return l;
}

__device__ __forceinline__ bool claim_kept(const DevFactor& F, const DevWork& W, const ReadyLists& R, int l, int i) {
    return i < R.n[l] && !(W.grid_flags[F.sn_grid[R.src[l][i]]] & FLAG_FROZEN);
}

constexpr int kCompactThreads = 256;
static_assert(kCompactChunk % kCompactThreads == 0, "whole rounds per chunk");

__global__ void __launch_bounds__(kCompactThreads) k_ready_count(DevFactor F, DevWork W, ReadyLists R, int* chunk_cnt) {
    const int b = blockIdx.x;
    const int l = list_of_chunk(R, b);
    const int base = (b - R.chunk0[l]) * kCompactChunk;
    int total = 0;
    for (int r = 0; r < kCompactChunk; r += kCompactThreads)
        total += __syncthreads_count(claim_kept(F, W, R, l, base + r + threadIdx.x));
    if (threadIdx.x == 0) chunk_cnt[b] = total;
}

__global__ void __launch_bounds__(kCompactThreads) k_ready_compact(DevFactor F, DevWork W, ReadyLists R,
                                                                    const int* chunk_cnt, int* counts) {
    __shared__ int warp_n[kCompactThreads / 32];
    __shared__ int s_off;
    const int b = blockIdx.x;
    const int l = list_of_chunk(R, b);
    const int base = (b - R.chunk0[l]) * kCompactChunk;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // offset of this chunk: kept entries of the list's earlier chunks
    int part = 0;
    for (int q = R.chunk0[l] + threadIdx.x; q < b; q += kCompactThreads) part += chunk_cnt[q];
    for (int o = 16; o > 0; o >>= 1) part += __shfl_down_sync(0xffffffffu, part, o);
    if (lane == 0) warp_n[warp] = part;
    __syncthreads();
    if (threadIdx.x == 0) {
        int t = 0;
        for (int w = 0; w < kCompactThreads / 32; ++w) t += warp_n[w];
        s_off = t;
    }
    __syncthreads();
    int off = s_off;
    for (int r = 0; r < kCompactChunk; r += kCompactThreads) {
        const int i = base + r + threadIdx.x;
        const bool keep = claim_kept(F, W, R, l, i);
        const unsigned m = __ballot_sync(0xffffffffu, keep);
        __syncthreads();  // warp_n of the previous round has been read
        if (lane == 0) warp_n[warp] = __popc(m);
        __syncthreads();
        int before = 0, all = 0;
        for (int w = 0; w < kCompactThreads / 32; ++w) {
            before += (w < warp) ? warp_n[w] : 0;
            all += warp_n[w];
        }
        if (keep) R.dst[l][off + before + __popc(m & ((1u << lane) - 1u))] = R.src[l][i];
        off += all;
    }
    if (threadIdx.x == 0 && b == R.chunk0[l + 1] - 1) counts[l] = off;
}


template <typename HV>
__global__ void k_gain_export(DevFactor F, const HV* hval, const HV* hw, int n_tgt, double* out) {
    for (int tg = blockIdx.x * blockDim.x + threadIdx.x; tg < n_tgt; tg += gridDim.x * blockDim.x)
        out[tg] = gain_entry<HV, double>(F, hval, hw, tg);
}

inline int grid_for(int64_t n, int threads) {
    int64_t g = (n + threads - 1) / threads;
    if (g > 152 * 16) g = 152 * 16;
    return (int)(g < 1 ? 1 : g);
}

template <typename V>
size_t solve_smem(int maxf) {
    return (size_t)(maxf + 2) * sizeof(V);
}

template <typename T, typename HV>
cudaError_t prepare_impl() {
    cudaError_t e = cudaFuncSetAttribute(k_front_small<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)front_smem<T>(small_front_max<T>()));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_front_flow<T, kPanel, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)front_smem<T>(small_front_max<T>()));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_front_flow<T, kPanelSmall, kMinBlocksA<T>>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)front_smem<T>(kFlowSmallFMax));
    const int mx = (int)solve_smem<double>(16384);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_fwd<T, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_bwd<T, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_fwd_flow<T, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_bwd_flow<T, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, mx);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_front_warp<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)(sizeof(WarpTile<T>) * kWarpsPerCta));

    return e;
}

template <typename T, typename HV>
cudaError_t factor_impl(const DevNet& net, const DevFactor& F, const DevWork& W, const LevelSchedule& ls, const HV* hval,
                        const HV* hw,
                        T* lx, T* ub, cudaStream_t st) {
    T* gv = reinterpret_cast<T*>(W.gvals);
    if (ls.n_tgt > 0) {
        if (sizeof(T) == 4 && ls.gain_acc32)
            k_gain_values<T, HV, float><<<grid_for(ls.n_tgt, 256), 256, 0, st>>>(F, W, hval, hw, gv, ls.n_tgt);
        else
            k_gain_values<T, HV, double><<<grid_for(ls.n_tgt, 256), 256, 0, st>>>(F, W, hval, hw, gv, ls.n_tgt);
        count_launches(1);
    }
    if (ls.flow_a_n + ls.flow_b_n + ls.flow_w_n > 0) {
        cudaError_t e = cudaMemsetAsync(W.flow, 0, sizeof(int) * (size_t)(F.n_super + 8), st);
        if (e != cudaSuccess) return e;
        int* counters = W.flow + F.n_super;
        if (ls.flow_w_n > 0) {
            k_front_warp<T><<<ls.flow_w_grid, kThreads, sizeof(WarpTile<T>) * kWarpsPerCta, st>>>(
                F, W, gv, lx, ub, ls.d_flow_w, ls.d_ready_n + 4, ls.d_phase, 3, ls.d_phase_nchild, counters + 2,
                W.flow);
            count_launches(1);
        }
        if (ls.flow_a_n > 0) {
            const int mf = ls.flow_a_maxf;
            k_front_flow<T, kPanelSmall, kMinBlocksA<T>><<<ls.flow_a_grid, kThreads, front_smem<T>(mf), st>>>(
                F, W, gv, lx, ub, ls.d_flow_a, ls.d_ready_n + 0, ls.d_phase, 1, ls.d_phase_nchild, counters + 0, W.flow);
            count_launches(1);
        }
        if (ls.flow_b_n > 0) {
            const int mf = ls.flow_b_maxf;
            k_front_flow<T, kPanel, 1><<<ls.flow_b_grid, kThreads, front_smem<T>(mf), st>>>(
                F, W, gv, lx, ub, ls.d_flow_b, ls.d_ready_n + 1, ls.d_phase, 2, ls.d_phase_nchild, counters + 1, W.flow);
            count_launches(1);
        }
    }
    if (sizeof(T) == 4 && ls.n_pot_pairs > 0) {
        cudaError_t e = cudaMemsetAsync(ls.d_pot_cnt, 0, sizeof(int) * (size_t)ls.n_pot_pairs, st);
        if (e != cudaSuccess) return e;
    }
    const bool tile_flow = sizeof(T) == 4 && ls.n_tt > 0;
    if (tile_flow) {
        cudaError_t e = cudaMemsetAsync(ls.d_tt_done, 0, sizeof(int) * (size_t)(ls.n_tt + ls.n_levels), st);
        if (e != cudaSuccess) return e;
    }
    for (int l = 0; l < ls.n_levels; ++l) {
        const int ns = ls.h_small_ptr[l + 1] - ls.h_small_ptr[l];
        if (ns > 0) {
            const int mf = ls.h_small_maxf[l];
            k_front_small<T><<<ns, kThreads, front_smem<T>(mf), st>>>(F, W, gv, lx, ub,
                                                                                  ls.d_small + ls.h_small_ptr[l]);
            count_launches(1);
        }
        const int na = ls.h_asm_ptr[l + 1] - ls.h_asm_ptr[l];
        if (na > 0) {
            k_big_assemble<T><<<na, kThreads, 0, st>>>(F, W, gv, lx, ub, ls.d_asm + ls.h_asm_ptr[l], ls.d_asm_child);
            count_launches(1);
            const int nt = tile_flow ? ls.h_tt_ptr[l + 1] - ls.h_tt_ptr[l] : 0;
            if constexpr (sizeof(T) == 4) {
                if (nt > 0) {
                    k_big_flow32<<<std::min(nt, ls.tt_grid), kThreads, 0, st>>>(
                        F, W, lx, ls.d_tt + ls.h_tt_ptr[l], nt, ls.d_tt_done + ls.h_tt_ptr[l],
                        ls.d_tt_done + ls.n_tt + l, ls.d_pot_cnt);
                    count_launches(1);
                }
            }
            for (int p = 0; nt == 0 && p < ls.h_lvl_panels[l]; ++p) {
                const int slot = ls.h_step_ptr[l] + p;
                const int npot = ls.h_pot_ptr[slot + 1] - ls.h_pot_ptr[slot];
                const int nupd = ls.h_upd_ptr[slot + 1] - ls.h_upd_ptr[slot];
                if (npot > 0) {
                    if constexpr (sizeof(T) == 4)
                        k_big_panel32<<<npot, kThreads, 0, st>>>(F, W, lx, ls.d_pot + ls.h_pot_ptr[slot], p,
                                                                 ls.d_pot_cnt);
                    else
                        k_big_potrf<T><<<npot, kThreads, 0, st>>>(F, W, lx, ls.d_pot + ls.h_pot_ptr[slot], p);
                    count_launches(1);
                }
                if constexpr (sizeof(T) == 8) {
                    const int npan = ls.h_pan_ptr[slot + 1] - ls.h_pan_ptr[slot];
                    if (npan > 0) {
                        k_big_trsm<T><<<(npan + kTrsmWarps<T> - 1) / kTrsmWarps<T>, 32 * kTrsmWarps<T>, 0, st>>>(
                            F, W, lx, ls.d_pan + ls.h_pan_ptr[slot], npan, p);
                        count_launches(1);
                    }
                }
                if (nupd > 0) {
                    k_big_update<T><<<nupd, kThreads, 0, st>>>(F, W, lx, ls.d_upd + ls.h_upd_ptr[slot], p);
                    count_launches(1);
                }
            }
        }
    }
    return cudaGetLastError();
}

template <typename T>
cudaError_t solve_impl(const DevFactor& F, const DevWork& W, const LevelSchedule& ls, const T* lx, const T* rdiag,
                       SolveVecs sv, cudaStream_t st) {
    if (ls.solve_flow) {
        // flags: [0, n_super) forward, [n_super, 2 n_super) backward, then counters
        const int ns = F.n_super;
        int* fwd_done = W.flow + ns + 8;
        int* bwd_done = fwd_done + ns;
        int* counters = bwd_done + ns;
        cudaError_t e = cudaMemsetAsync(fwd_done, 0, sizeof(int) * (size_t)(2 * ns + 8), st);
        if (e != cudaSuccess) return e;
        const size_t smem = solve_smem<T>(ls.solve_maxf);
        // warp fronts first going up, last coming down
        if (ls.flow_w_n > 0) {
            k_fwd_warp<T, T><<<ls.solve_w_grid, kThreads, 0, st>>>(F, W, lx, rdiag, sv, ls.d_flow_w, ls.d_ready_n + 4,
                                                                   ls.d_phase, 3, ls.d_phase_nchild, counters + 2,
                                                                   fwd_done);
            count_launches(1);
        }
        if (ls.up_n > 0) {
            k_fwd_flow<T, T><<<ls.up_grid, kThreads, smem, st>>>(F, W, lx, rdiag, sv, ls.d_up, ls.d_ready_n + 2,
                                                                 ls.d_nchild, counters + 0, fwd_done);
            k_bwd_flow<T, T><<<ls.solve_grid, kThreads, smem, st>>>(F, W, lx, rdiag, sv, ls.d_down, ls.d_ready_n + 3,
                                                                    counters + 1, bwd_done);
            count_launches(2);
        }
        if (ls.down_w_n > 0) {
            k_bwd_warp<T, T><<<ls.solve_w_grid, kThreads, 0, st>>>(F, W, lx, rdiag, sv, ls.d_down_w, ls.d_ready_n + 5,
                                                                   counters + 3, bwd_done);
            count_launches(1);
        }
        return cudaGetLastError();
    }
    for (int l = 0; l < ls.n_levels; ++l) {
        const int n = ls.h_all_ptr[l + 1] - ls.h_all_ptr[l];
        if (n > 0) {
            k_fwd<T, T><<<n, kThreads, solve_smem<T>(ls.h_lvl_maxf[l]), st>>>(F, lx, rdiag, sv,
                                                                               ls.d_all + ls.h_all_ptr[l]);
            count_launches(1);
        }
    }
    for (int l = ls.n_levels - 1; l >= 0; --l) {
        const int n = ls.h_all_ptr[l + 1] - ls.h_all_ptr[l];
        if (n > 0) {
            k_bwd<T, T><<<n, kThreads, solve_smem<T>(ls.h_lvl_maxf[l]), st>>>(F, lx, rdiag, sv,
                                                                               ls.d_all + ls.h_all_ptr[l]);
            count_launches(1);
        }
    }
    return cudaGetLastError();
}

template <typename T>
FlowGrids flow_grids_impl(int32_t maxf_a, int32_t maxf_b, int32_t solve_maxf) {
    FlowGrids g{0, 0, 0, 0, 0, 0};
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return g;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return g;
    auto resident = [&](const void* fn, size_t smem) {
        int per_sm = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kThreads, smem) != cudaSuccess) return 0;
        return per_sm * sms;
    };
    g.a = resident((const void*)k_front_flow<T, kPanelSmall, kMinBlocksA<T>>, front_smem<T>(maxf_a));
    g.b = resident((const void*)k_front_flow<T, kPanel, 1>, front_smem<T>(maxf_b));
    if (solve_maxf <= 16384) g.solve = resident((const void*)k_fwd_flow<T, T>, solve_smem<T>(solve_maxf));
    g.w = resident((const void*)k_front_warp<T>, sizeof(WarpTile<T>) * kWarpsPerCta);
    g.wsolve = std::min(resident((const void*)k_fwd_warp<T, T>, 0), resident((const void*)k_bwd_warp<T, T>, 0));
    g.tile = sizeof(T) == 4 ? resident((const void*)k_big_flow32, 0) : 0;
    cudaGetLastError();
    return g;
}

}  // namespace

cudaError_t launch_ready_compact(const DevFactor& F, const DevWork& W, const LevelSchedule& ls, cudaStream_t st) {
    ReadyLists R;
    R.chunk0[0] = 0;
    for (int l = 0; l < kReadyLists; ++l) {
        R.src[l] = ls.src_lists[l];
        R.dst[l] = ls.cmp_lists[l];
        R.n[l] = ls.src_n[l];
        R.chunk0[l + 1] = R.chunk0[l] + (R.n[l] + kCompactChunk - 1) / kCompactChunk;
    }
    const int nb = R.chunk0[kReadyLists];
    if (nb == 0 || !W.grid_flags) return cudaSuccess;
    k_ready_count<<<nb, kCompactThreads, 0, st>>>(F, W, R, ls.d_chunk_cnt);
    k_ready_compact<<<nb, kCompactThreads, 0, st>>>(F, W, R, ls.d_chunk_cnt, ls.d_ready_n);
    count_launches(2);
    return cudaGetLastError();
}

FlowGrids flow_grids(bool mixed, int32_t maxf_a, int32_t maxf_b, int32_t solve_maxf) {
    return mixed ? flow_grids_impl<float>(maxf_a, maxf_b, solve_maxf)
                 : flow_grids_impl<double>(maxf_a, maxf_b, solve_maxf);
}

cudaError_t prepare_factor_kernels() {
    cudaError_t e = prepare_impl<double, double>();
    if (e == cudaSuccess) e = prepare_impl<float, float>();
    return e;
}

cudaError_t launch_factor32(const DevNet& net, const DevFactor& F, const DevWork& W, const LevelSchedule& ls,
                            cudaStream_t st) {
    return factor_impl<float, float>(net, F, W, ls, W.hval32, W.hw32, W.lx32, W.u32, st);
}

cudaError_t launch_solve32(const DevFactor& F, const DevWork& W, const LevelSchedule& ls, cudaStream_t st) {
    return solve_impl<float>(F, W, ls, W.lx32, reinterpret_cast<const float*>(W.rdiag),
                             SolveVecs{W.rhs32, W.sol32, W.su32}, st);
}

cudaError_t launch_factor(const DevNet& net, const DevFactor& F, const DevWork& W, const LevelSchedule& ls,
                          cudaStream_t st) {
    return factor_impl<double, double>(net, F, W, ls, W.hval, W.hw, W.lx, W.u, st);
}

cudaError_t launch_solve(const DevFactor& F, const DevWork& W, const LevelSchedule& ls, cudaStream_t st) {
    return solve_impl<double>(F, W, ls, W.lx, reinterpret_cast<const double*>(W.rdiag),
                              SolveVecs{W.rhs, W.sol, W.su}, st);
}

cudaError_t launch_gain_export(const DevNet& net, const DevFactor& F, const DevWork& W, int32_t n_tgt, double* out,
                               cudaStream_t st) {
    if (n_tgt > 0) {
        k_gain_export<double><<<grid_for(n_tgt, 256), 256, 0, st>>>(F, W.hval, W.hw, n_tgt, out);
        count_launches(1);
    }
    return cudaGetLastError();
}


// ---------------------------------------------------------------------------
// Allocation-free factor/solve.  One call's scratch -- right-hand side and
// solution staging in state order, the dataflow flags, the solve update
// vectors and the small fronts' update matrices -- lives in one file-scope
// device array of kNoAllocScratchBytes.  The address is looked up once per
// device (cudaGetSymbolAddress, with that device current); every call on a
// device shares the array, so calls that overlap in time race.
// ---------------------------------------------------------------------------
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {
constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
unsigned char* g_noalloc_ptr[kNoAllocMaxDevices] = {};

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

struct NoAllocLayout {
    size_t rhs, x, flow, su, u, total;  // byte offsets into the scratch array
};

NoAllocLayout noalloc_layout(const NoAllocShape& sh) {
    NoAllocLayout l{};
    size_t off = 0;
    l.rhs = off;
    off = align256(off + sizeof(double) * (size_t)sh.n_state);
    l.x = off;
    off = align256(off + sizeof(double) * (size_t)sh.n_state);
    l.flow = off;
    off = align256(off + sizeof(int) * (3 * (size_t)sh.n_super + 16));
    l.su = off;
    off = align256(off + sizeof(double) * (size_t)sh.su_elems);
    l.u = off;
    off = align256(off + sizeof(double) * (size_t)sh.u_elems);
    l.total = off;
    return l;
}

// state index -> permuted position (theta of every bus but the slack, then |V|)
__device__ __forceinline__ int ps_of_state(const DevNet& net, const DevFactor& F, int st) {
    const int nth = net.n_bus - 1;
    if (st < nth) return F.bus_ps_theta[st < net.slack ? st : st + 1];
    return F.bus_ps_v[st - nth];
}

__global__ void k_state_to_ps(DevNet net, DevFactor F, const double* in, double* out) {
    const int st = blockIdx.x * blockDim.x + threadIdx.x;
    if (st < F.n_state) out[ps_of_state(net, F, st)] = in[st];
}

__global__ void k_ps_to_state(DevNet net, DevFactor F, const double* in, double* out) {
    const int st = blockIdx.x * blockDim.x + threadIdx.x;
    if (st < F.n_state) out[st] = in[ps_of_state(net, F, st)];
}
}  // namespace

size_t noalloc_scratch_need(const NoAllocShape& sh) { return noalloc_layout(sh).total; }

cudaError_t noalloc_scratch_setup(void** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= kNoAllocMaxDevices) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_noalloc_ptr[dev] = static_cast<unsigned char*>(p);
    }
    *out = g_noalloc_ptr[dev];
    return cudaSuccess;
}

cudaError_t launch_factor_solve_noalloc(const DevNet& net, const DevFactor& F, const DevWork& W,
                                        const LevelSchedule& ls, const NoAllocShape& sh, const double* rhs_host,
                                        double* x_host, cudaStream_t st) {
    const NoAllocLayout l = noalloc_layout(sh);
    if (l.total > kNoAllocScratchBytes) return cudaErrorInvalidValue;  // callers check the size first
    void* base = nullptr;
    cudaError_t e = noalloc_scratch_setup(&base);
    if (e != cudaSuccess) return e;
    unsigned char* b = static_cast<unsigned char*>(base);
    double* d_rhs = reinterpret_cast<double*>(b + l.rhs);
    double* d_x = reinterpret_cast<double*>(b + l.x);
    DevWork W2 = W;
    W2.flow = reinterpret_cast<int*>(b + l.flow);  // cleared at the start of each pass
    W2.su = reinterpret_cast<double*>(b + l.su);
    W2.u = reinterpret_cast<double*>(b + l.u);
    const int n = F.n_state;
    e = cudaMemcpyAsync(d_rhs, rhs_host, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) return e;
    if (n > 0) {
        k_state_to_ps<<<grid_for(n, 256), 256, 0, st>>>(net, F, d_rhs, W2.rhs);
        count_launches(1);
    }
    e = factor_impl<double, double>(net, F, W2, ls, W2.hval, W2.hw, W2.lx, W2.u, st);
    if (e == cudaSuccess)
        e = solve_impl<double>(F, W2, ls, W2.lx, reinterpret_cast<const double*>(W2.rdiag),
                               SolveVecs{W2.rhs, W2.sol, W2.su}, st);
    if (e != cudaSuccess) return e;
    if (n > 0) {
        k_ps_to_state<<<grid_for(n, 256), 256, 0, st>>>(net, F, W2.sol, d_x);
        count_launches(1);
    }
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(x_host, d_x, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, st);
    return e;
}

}  // namespace sle_gb300
