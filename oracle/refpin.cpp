// Reference-kernel harness: runs the reference's own element kernels, built
// unchanged from its sources into cubins (oracle/build_ref.py), on the GPU.
//
// TEST INFRASTRUCTURE ONLY: the parity tests use it to pin the CPU oracle's
// restatement of Ybus, h(x) and the reference-formula Jacobian to the
// reference's code; the product never links or calls it.
//
// The host orchestration follows the reference's launch code step by step:
//   Ybus     SparseMatrixManager::buildYbus (sparse_matrix.cu:498-626):
//            computeBranchAdmittanceKernel, row counts = 1 + countYbus-
//            NonzerosKernel, exclusive scan, initYbusDiagonalKernel,
//            fillYbusKernel (atomic slot claims, so off-diagonal order is
//            arrival order)
//   h(x)     launchPowerFlowKernels (kernels.cu:955-1057) for grids below
//            its size switches (<= 10,000 branches, <= 16 neighbours a bus):
//            computePowerInjectionsKernel, computeBranchFlowsKernel,
//            computeBranchCurrentsKernel; then
//            launchMeasurementFunctionKernel (kernels.cu:1059-1091)
//   H        analyzeJacobianPattern (sparse_matrix.cu:1552-1616: 10 slots a
//            row, columns -1) and computeJacobianValuesKernel
//            (sparse_matrix.cu:1627-2147)
// with 256-thread blocks (BLOCK_SIZE_STANDARD, sle_types.cuh:500-510).
// Kernels are found in the loaded modules by their identifier (the
// enumerated function names of a module, cuModuleEnumerateFunctions).
#include <cuda.h>

#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

namespace {

std::string g_err;
CUcontext g_ctx = nullptr;
CUmodule g_mk = nullptr, g_ms = nullptr;

enum Fn { F_ADMIT, F_COUNT, F_DIAG, F_FILL, F_INJ, F_FLOW, F_CUR, F_MEAS, F_JAC, F_N };
const char* kIdent[F_N] = {"computeBranchAdmittanceKernel", "countYbusNonzerosKernel", "initYbusDiagonalKernel",
                           "fillYbusKernel", "computePowerInjectionsKernel", "computeBranchFlowsKernel",
                           "computeBranchCurrentsKernel", "computeMeasurementFunctionKernel",
                           "computeJacobianValuesKernel"};
CUfunction g_fn[F_N] = {};

bool ok(CUresult r, const char* what) {
    if (r == CUDA_SUCCESS) return true;
    const char* s = nullptr;
    cuGetErrorString(r, &s);
    g_err = std::string(what) + ": " + (s ? s : "CUDA driver error");
    return false;
}

// The reference's kernels live in namespace sle: their Itanium-mangled names
// start with "_ZN3sle<length><identifier>E".
CUfunction find_fn(CUmodule m, const char* ident) {
    unsigned n = 0;
    if (cuModuleGetFunctionCount(&n, m) != CUDA_SUCCESS || n == 0) return nullptr;
    std::vector<CUfunction> fs(n);
    if (cuModuleEnumerateFunctions(fs.data(), n, m) != CUDA_SUCCESS) return nullptr;
    const std::string prefix = "_ZN3sle" + std::to_string(std::strlen(ident)) + ident + "E";
    for (CUfunction f : fs) {
        const char* name = nullptr;
        if (cuFuncGetName(&name, f) == CUDA_SUCCESS && name && std::strncmp(name, prefix.c_str(), prefix.size()) == 0)
            return f;
    }
    return nullptr;
}

struct Buf {
    CUdeviceptr p = 0;
    ~Buf() {
        if (p) cuMemFree(p);
    }
};

template <typename T>
bool put(Buf& b, const T* src, size_t n) {
    if (!ok(cuMemAlloc(&b.p, sizeof(T) * (n ? n : 1)), "cuMemAlloc")) return false;
    if (n && src) return ok(cuMemcpyHtoD(b.p, src, sizeof(T) * n), "cuMemcpyHtoD");
    if (n) return ok(cuMemsetD8(b.p, 0, sizeof(T) * n), "cuMemsetD8");
    return true;
}

bool launch(Fn f, int n, std::vector<void*> args) {
    if (n <= 0) return true;
    const unsigned grid = static_cast<unsigned>((n + 255) / 256);
    return ok(cuLaunchKernel(g_fn[f], grid, 1, 1, 256, 1, 1, 0, nullptr, args.data(), nullptr), kIdent[f]);
}

// Branch arrays on the device, admittances computed by the reference kernel.
struct Branches {
    Buf from, to, r, x, b, tap, shift, status, gs, bs, bsf, bst;
    int32_t n = 0;
    bool load(int32_t nbr, const int32_t* f, const int32_t* t, const float* rr, const float* xx, const float* bb,
              const float* tp, const float* sh, const uint8_t* st) {
        n = nbr;
        return put(from, f, nbr) && put(to, t, nbr) && put(r, rr, nbr) && put(x, xx, nbr) && put(b, bb, nbr) &&
               put(tap, tp, nbr) && put(shift, sh, nbr) && put(status, st, nbr) && put<float>(gs, nullptr, nbr) &&
               put<float>(bs, nullptr, nbr) && put<float>(bsf, nullptr, nbr) && put<float>(bst, nullptr, nbr) &&
               launch(F_ADMIT, n, {&gs.p, &bs.p, &bsf.p, &bst.p, &r.p, &x.p, &b.p, &tap.p, &n});
    }
};

struct Ybus {
    Buf ptr, col, g, b;
    int32_t nnz = 0;
    std::vector<int32_t> h_ptr;
};

bool build_ybus(int32_t nb, Branches& br, Ybus& y) {
    std::vector<int32_t> ones(nb, 1);
    Buf counts, offs;
    if (!put(counts, ones.data(), nb)) return false;
    int32_t nbr = br.n;
    if (!launch(F_COUNT, nbr, {&counts.p, &br.from.p, &br.to.p, &br.status.p, &nbr, &nb})) return false;
    std::vector<int32_t> c(nb);
    if (!ok(cuMemcpyDtoH(c.data(), counts.p, sizeof(int32_t) * nb), "row counts")) return false;
    y.h_ptr.assign(nb + 1, 0);
    for (int32_t i = 0; i < nb; ++i) y.h_ptr[i + 1] = y.h_ptr[i] + c[i];
    y.nnz = y.h_ptr[nb];
    if (!put(y.ptr, y.h_ptr.data(), nb + 1) || !put<int32_t>(y.col, nullptr, y.nnz) || !put<float>(y.g, nullptr, y.nnz) ||
        !put<float>(y.b, nullptr, y.nnz) || !put<int32_t>(offs, nullptr, nb))
        return false;
    if (!launch(F_DIAG, nb, {&y.g.p, &y.b.p, &y.col.p, &y.ptr.p, &nb})) return false;
    return launch(F_FILL, nbr, {&y.g.p, &y.b.p, &y.col.p, &offs.p, &y.ptr.p, &br.from.p, &br.to.p, &br.gs.p, &br.bs.p,
                                &br.bsf.p, &br.bst.p, &br.tap.p, &br.shift.p, &br.status.p, &nbr, &nb});
}

}  // namespace

extern "C" {

const char* rp_error(void) { return g_err.c_str(); }

// Loads the reference cubins from `dir` (kernels.cubin, sparse_matrix.cubin)
// on device 0's primary context.  0 on success.
int32_t rp_open(const char* dir) {
    if (g_mk && g_ms) return 0;
    CUdevice dev;
    if (!ok(cuInit(0), "cuInit") || !ok(cuDeviceGet(&dev, 0), "cuDeviceGet") ||
        !ok(cuDevicePrimaryCtxRetain(&g_ctx, dev), "primary context") || !ok(cuCtxSetCurrent(g_ctx), "cuCtxSetCurrent"))
        return -1;
    const std::string d = dir;
    if (!ok(cuModuleLoad(&g_mk, (d + "/kernels.cubin").c_str()), "load kernels.cubin") ||
        !ok(cuModuleLoad(&g_ms, (d + "/sparse_matrix.cubin").c_str()), "load sparse_matrix.cubin"))
        return -1;
    for (int f = 0; f < F_N; ++f) {
        g_fn[f] = find_fn(f <= F_FILL || f == F_JAC ? g_ms : g_mk, kIdent[f]);
        if (!g_fn[f]) {
            g_err = std::string("kernel not found in the reference modules: ") + kIdent[f];
            return -1;
        }
    }
    return 0;
}

// Ybus by the reference's buildYbus steps: row_ptr[n_bus+1]; col, g, b of
// length cap (>= nnz).  Returns nnz, or -1.
int32_t rp_ybus(int32_t n_bus, int32_t n_br, const int32_t* from, const int32_t* to, const float* r, const float* x,
                const float* b, const float* tap, const float* shift, const uint8_t* status, int32_t* row_ptr,
                int32_t* col, float* g, float* bv, int32_t cap) {
    if (cuCtxSetCurrent(g_ctx) != CUDA_SUCCESS) return -1;
    Branches br;
    Ybus y;
    if (!br.load(n_br, from, to, r, x, b, tap, shift, status) || !build_ybus(n_bus, br, y)) return -1;
    if (y.nnz > cap) {
        g_err = "output capacity below nnz";
        return -1;
    }
    std::memcpy(row_ptr, y.h_ptr.data(), sizeof(int32_t) * (n_bus + 1));
    if (!ok(cuMemcpyDtoH(col, y.col.p, sizeof(int32_t) * y.nnz), "ybus col") ||
        !ok(cuMemcpyDtoH(g, y.g.p, sizeof(float) * y.nnz), "ybus g") ||
        !ok(cuMemcpyDtoH(bv, y.b.p, sizeof(float) * y.nnz), "ybus b") || !ok(cuCtxSynchronize(), "sync"))
        return -1;
    return y.nnz;
}

// h(x) and the reference-formula Jacobian at (v, th): h[n_meas];
// hcol / hval [10 n_meas] in the kernel's write order, -1 / 0 padding.
int32_t rp_evaluate(int32_t n_bus, int32_t slack, int32_t n_br, const int32_t* from, const int32_t* to,
                    const float* r, const float* x, const float* b, const float* tap, const float* shift,
                    const uint8_t* status, int32_t n_meas, const uint8_t* mtype, const int32_t* mloc,
                    const uint8_t* mend, const float* v, const float* th, float* h, int32_t* hcol, float* hval) {
    if (cuCtxSetCurrent(g_ctx) != CUDA_SUCCESS) return -1;
    Branches br;
    Ybus y;
    if (!br.load(n_br, from, to, r, x, b, tap, shift, status) || !build_ybus(n_bus, br, y)) return -1;
    std::vector<float> ones(n_meas, 1.0f);
    std::vector<uint8_t> active(n_meas, 1);
    Buf dv, dth, pinj, qinj, pf, qf, pt, qt, ifr, ito, dtype, dloc, dend, dpt, dct, dact, dh, hptr, hc, hv;
    const int32_t slots = 10;  // 2 * avg_degree + 2 (sparse_matrix.cu:1574-1595)
    std::vector<int32_t> hp(n_meas + 1);
    for (int32_t q = 0; q <= n_meas; ++q) hp[q] = q * slots;
    std::vector<int32_t> minus1(static_cast<size_t>(n_meas) * slots, -1);
    if (!put(dv, v, n_bus) || !put(dth, th, n_bus) || !put<float>(pinj, nullptr, n_bus) ||
        !put<float>(qinj, nullptr, n_bus) || !put<float>(pf, nullptr, n_br) || !put<float>(qf, nullptr, n_br) ||
        !put<float>(pt, nullptr, n_br) || !put<float>(qt, nullptr, n_br) || !put<float>(ifr, nullptr, n_br) ||
        !put<float>(ito, nullptr, n_br) || !put(dtype, mtype, n_meas) || !put(dloc, mloc, n_meas) ||
        !put(dend, mend, n_meas) || !put(dpt, ones.data(), n_meas) || !put(dct, ones.data(), n_meas) ||
        !put(dact, active.data(), n_meas) || !put<float>(dh, nullptr, n_meas) || !put(hptr, hp.data(), n_meas + 1) ||
        !put(hc, minus1.data(), minus1.size()) || !put<float>(hv, nullptr, minus1.size()))
        return -1;
    int32_t nb = n_bus, nbr = n_br, m = n_meas, sl = slack;
    if (!launch(F_INJ, nb, {&pinj.p, &qinj.p, &dv.p, &dth.p, &y.ptr.p, &y.col.p, &y.g.p, &y.b.p, &nb}) ||
        !launch(F_FLOW, nbr, {&pf.p, &qf.p, &pt.p, &qt.p, &dv.p, &dth.p, &br.from.p, &br.to.p, &br.gs.p, &br.bs.p,
                              &br.bsf.p, &br.bst.p, &br.tap.p, &br.shift.p, &br.status.p, &nbr}) ||
        !launch(F_CUR, nbr, {&ifr.p, &ito.p, &pf.p, &qf.p, &pt.p, &qt.p, &dv.p, &br.from.p, &br.to.p, &br.status.p,
                             &nbr}) ||
        !launch(F_MEAS, m, {&dh.p, &dtype.p, &dloc.p, &dend.p, &dpt.p, &dct.p, &dact.p, &dv.p, &dth.p, &pinj.p,
                            &qinj.p, &pf.p, &qf.p, &pt.p, &qt.p, &ifr.p, &ito.p, &m}) ||
        !launch(F_JAC, m, {&hv.p, &hc.p, &hptr.p, &dtype.p, &dloc.p, &dend.p, &dpt.p, &dct.p, &dact.p, &dv.p, &dth.p,
                           &y.ptr.p, &y.col.p, &y.g.p, &y.b.p, &br.from.p, &br.to.p, &br.gs.p, &br.bs.p, &br.tap.p,
                           &br.shift.p, &sl, &nb, &m}))
        return -1;
    if (!ok(cuMemcpyDtoH(h, dh.p, sizeof(float) * n_meas), "h") ||
        !ok(cuMemcpyDtoH(hcol, hc.p, sizeof(int32_t) * minus1.size()), "H columns") ||
        !ok(cuMemcpyDtoH(hval, hv.p, sizeof(float) * minus1.size()), "H values") || !ok(cuCtxSynchronize(), "sync"))
        return -1;
    return 0;
}

}  // extern "C"
