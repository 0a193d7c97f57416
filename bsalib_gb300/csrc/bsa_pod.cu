// bsa_pod.cu -- truncated POD of the nodal cross-PSD for the Mesher functions.
//
// getFM_full_tm_scalar_msh_POD_ (functionsImpl.F90:474-1019) expands S(f1), S(f2) and
// S(f1 + f2) of every point in their eigenpairs (dsyev) and sums the BFM over the kept ones:
// with S_t(f) = sum_{kept p} lambda_p v_p v_p^T the result is exactly the direct form with
// every S(f) replaced by S_t(f), i.e. A(f) = S(f) L replaced by A_t(f) = V_t Lambda_t V_t^T L.
// With every POD mode kept (the reference's default) S_t = S and the direct form is used
// unchanged; when bsa_setPODTruncationThreshold / bsa_setPODNOfModesKept drop modes, this file
// builds the A table of the Mesher's frequencies from the truncated expansions, so every Mesher
// path (FP64 points and zones, split-precision zones) evaluates the truncated form.
//
// Per (frequency, component): S(f) is formed in FP64 on the device, decomposed by cuSOLVER's
// dsyevd (eigenvalues ascending, as dsyev's), the kept count chosen on the device
// (getNPODModesByThreshold_, :203-230, as the reference builds it by default -- see pod_count),
// and A_t(f) = V_t Lambda_t (V_t^T L) written into the FP64 or FP32 A table.  cuSOLVER is
// loaded on first use (dlopen), so the library loads without it when no truncation is asked.
#include <cuda_runtime.h>
#include <cusolverDn.h>
#include <dlfcn.h>

#include <cmath>
#include <vector>

#include "../../include/bsa_gpu.h"
#include "bsa_engine.cuh"

namespace bsa {
namespace pod {

// S_ij(f) = c_ij^|f| sqrt(S_i S_j), column-major n x n (symmetric).
__global__ void k_pod_smat(int n, double af, const double *__restrict__ logc, const double *__restrict__ Sn,
                           double *__restrict__ M) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n * n) return;
    const int i = (int)(t % n), j = (int)(t / n);
    const double g = (af == 0.0) ? 1.0 : exp(af * logc[(size_t)i * n + j]);  // c^0 = 1
    M[t] = g * sqrt(Sn[i]) * sqrt(Sn[j]);
}

// Kept count of one expansion, eigenvalues W ascending.  mode 1: getNPODModesByThreshold_ as
// built with dsyev (the count starts at 2 and walks down over the smallest eigenvalues, so it
// is 1 when W[1] < lim W[n-1], else 0; where W[0] reaches the limit too the reference reads
// outside the array, taken as 0 here); mode 2: the fixed count nfix.
__global__ void k_pod_count(int n, int mode, double lim, int nfix, const double *__restrict__ W,
                            const int *__restrict__ info, int *__restrict__ cnt, int *__restrict__ bad) {
    if (threadIdx.x != 0) return;
    if (*info != 0) atomicExch(bad, *info);
    int c = n;
    if (mode == 2) {
        c = nfix;
    } else if (mode == 1) {
        bool same = true;
        for (int k = 0; k < n; ++k) same = same && (W[k] == W[n - 1]);
        if (same) {
            c = 1;
        } else {
            const double limval = lim * W[n - 1];
            int p = 2;  // 1-based, as the reference
            while (p >= 1 && W[p - 1] >= limval) --p;
            c = p - 1 > 0 ? p - 1 : 0;
        }
    }
    *cnt = c < 0 ? 0 : (c > n ? n : c);
}

// G[p][m] = lambda_p sum_i V[i][p] L[i][m] for the kept p (the top cnt eigenpairs).
__global__ void k_pod_g(int n, int nm, const double *__restrict__ V, const double *__restrict__ W,
                        const double *__restrict__ L, const int *__restrict__ cnt, double *__restrict__ G) {
    const int p = blockIdx.x;
    if (p < n - *cnt) return;
    const double *v = V + (size_t)p * n;
    for (int m = threadIdx.x; m < nm; m += blockDim.x) {
        double s = 0.0;
        for (int i = 0; i < n; ++i) s = fma(v[i], L[(size_t)i * nm + m], s);
        G[(size_t)p * nm + m] = W[p] * s;
    }
}

// A_t[i][m] = sum_{kept p} V[i][p] G[p][m], written in FP64 or FP32.
template <class T>
__global__ void k_pod_a(int n, int nm, const double *__restrict__ V, const double *__restrict__ G,
                        const int *__restrict__ cnt, T *__restrict__ A) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)n * nm) return;
    const int i = (int)(t / nm), m = (int)(t % nm);
    double s = 0.0;
    for (int p = n - *cnt; p < n; ++p) s = fma(V[(size_t)p * n + i], G[(size_t)p * nm + m], s);
    A[(size_t)i * nm + m] = (T)s;
}

// cuSOLVER entry points, resolved on first use.
struct Solver {
    bool tried = false;
    void *lib = nullptr;
    decltype(&cusolverDnCreate) create = nullptr;
    decltype(&cusolverDnDestroy) destroy = nullptr;
    decltype(&cusolverDnSetStream) set_stream = nullptr;
    decltype(&cusolverDnDsyevd_bufferSize) buffer_size = nullptr;
    decltype(&cusolverDnDsyevd) syevd = nullptr;
    cusolverDnHandle_t h = nullptr;
    bool load() {
        if (tried) return syevd != nullptr;
        tried = true;
        for (const char *name : {"libcusolver.so.12", "libcusolver.so.13", "libcusolver.so"}) {
            lib = dlopen(name, RTLD_NOW | RTLD_LOCAL);
            if (lib) break;
        }
        if (!lib) return false;
        create = (decltype(create))dlsym(lib, "cusolverDnCreate");
        destroy = (decltype(destroy))dlsym(lib, "cusolverDnDestroy");
        set_stream = (decltype(set_stream))dlsym(lib, "cusolverDnSetStream");
        buffer_size = (decltype(buffer_size))dlsym(lib, "cusolverDnDsyevd_bufferSize");
        syevd = (decltype(syevd))dlsym(lib, "cusolverDnDsyevd");
        if (!create || !destroy || !set_stream || !buffer_size || !syevd) {
            syevd = nullptr;
            return false;
        }
        if (create(&h) != CUSOLVER_STATUS_SUCCESS) {
            syevd = nullptr;
            return false;
        }
        return true;
    }
};

Solver &solver() {
    static Solver s;
    return s;
}

}  // namespace pod

int Engine::pod_atable(const std::vector<double> &freqs, bool fp32) {
    using namespace pod;
    const int nf = (int)freqs.size(), ntc = (int)set.tc.size(), n = in.nnl, nm = nme;
    Solver &sv = solver();
    if (!sv.load()) return fail(BSA_ERR_UNSUPPORTED, "truncated POD needs cuSOLVER (libcusolver), which could not be loaded");
    int rc = build_psd(freqs);  // nodal PSD table S[f][comp][node] into dS
    if (rc) return rc;
    cudaError_t e;
    if (sv.set_stream(sv.h, stream) != CUSOLVER_STATUS_SUCCESS) return fail(BSA_ERR_CUDA, "cusolverDnSetStream failed");
    int lwork = 0;
    if (sv.buffer_size(sv.h, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, nullptr, n, nullptr, &lwork) !=
        CUSOLVER_STATUS_SUCCESS)
        return fail(BSA_ERR_CUDA, "cusolverDnDsyevd_bufferSize failed");
    const size_t nn = (size_t)n * n;
    // scratch: matrix / eigenvectors, eigenvalues, G, workspace, info, count, failure flag
    const size_t bytes = sizeof(double) * (nn + n + (size_t)n * nm + (size_t)lwork) + 4 * sizeof(int) + 256;
    if ((e = dPod.reserve(bytes))) return cuda_fail(e, "allocating POD scratch");
    double *M = dPod.as<double>(), *W = M + nn, *G = W + n, *work = G + (size_t)n * nm;
    int *info = (int *)(work + lwork), *cnt = info + 1, *bad = info + 2;
    if (fp32) {
        if ((e = dA32.reserve(sizeof(float) * (size_t)nf * K * nm))) return cuda_fail(e, "allocating A");
    } else {
        if ((e = dA.reserve(sizeof(double) * (size_t)nf * K * nm))) return cuda_fail(e, "allocating A");
    }
    if ((e = cudaMemsetAsync(bad, 0, sizeof(int), stream))) return cuda_fail(e, "memset");
    const bool thr = pod_trunc_lim > 0.0 && pod_trunc_lim != 1.0;  // BsaLibImpl.F90:479-481
    const int mode = thr ? 1 : 2;
    for (int fi = 0; fi < nf; ++fi)
        for (int itc = 0; itc < ntc; ++itc) {
            const double af = std::fabs(freqs[fi]);
            const double *Sn = dS.as<double>() + ((size_t)fi * ntc + itc) * n;
            k_pod_smat<<<(unsigned)((nn + 255) / 256), 256, 0, stream>>>(n, af, dLogc.as<double>() + (size_t)itc * nn,
                                                                          Sn, M);
            if (sv.syevd(sv.h, CUSOLVER_EIG_MODE_VECTOR, CUBLAS_FILL_MODE_LOWER, n, M, n, W, work, lwork, info) !=
                CUSOLVER_STATUS_SUCCESS)
                return fail(BSA_ERR_CUDA, "cusolverDnDsyevd failed");
            k_pod_count<<<1, 32, 0, stream>>>(n, mode, pod_trunc_lim, pod_nmodes, W, info, cnt, bad);
            const double *Lt = dL.as<double>() + (size_t)itc * n * nm;
            k_pod_g<<<n, 64, 0, stream>>>(n, nm, M, W, Lt, cnt, G);
            const size_t arow = ((size_t)fi * ntc + itc) * n * nm;
            const unsigned ga = (unsigned)(((size_t)n * nm + 255) / 256);
            if (fp32)
                k_pod_a<float><<<ga, 256, 0, stream>>>(n, nm, M, G, cnt, dA32.as<float>() + arow);
            else
                k_pod_a<double><<<ga, 256, 0, stream>>>(n, nm, M, G, cnt, dA.as<double>() + arow);
            if ((e = cudaGetLastError())) return cuda_fail(e, "POD kernels");
            kernels += 4;
        }
    int hbad = 0;
    if ((e = cudaMemcpyAsync(&hbad, bad, sizeof(int), cudaMemcpyDeviceToHost, stream)) ||
        (e = cudaStreamSynchronize(stream)))
        return cuda_fail(e, "POD expansion");
    if (hbad) return fail(BSA_ERR_CUDA, "dsyevd did not converge (info %d)", hbad);
    return BSA_OK;
}

}  // namespace bsa
