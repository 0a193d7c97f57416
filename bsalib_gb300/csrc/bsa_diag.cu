// bsa_diag.cu -- diagonal-only spectra (same node, same mode; settings i_only_diag_ = 1,
// bound at src/bsa/BsaLibImpl.F90:313-336), FP64 on the CUDA cores.
//
// With the same loaded node on all three ends the coherence is 1 and the nodal triple sum
// collapses to one sum over k = (component, node):
//   B_m(f1,f2) = 2 sum_k W_km g_k(f1,f2),   W_km = Q_km L_km^2
//   Classic (getFM_diag_tnlm_vect_cls_, functionsImpl.F90:1747-1968; scalar form :2460-2560):
//       g_k = S_k(f1) S_k(f2) + S_k(f1+f2) S_k(f2) + S_k(f1) S_k(f1+f2)
//   Mesher (getFM_diag_tnm_scalar_msh_, :1123-1210, which evaluates S(f1+f2) but reads
//   S(f1) S(f2) in its place):
//       g_k = S_k(f1) S_k(f2) + S_k(f1) S_k(f2)^2 + S_k(f1)^2 S_k(f2)
// Q_km L_km^2 is the product of the three per-node sums over the loaded DOFs that the
// reference forms as its triple loop over DOFs.  Per point this is one length-K dot product
// per mode, i.e. a [points x K] x [K x nm] product whose left factor is generated on the
// fly; O(K nm) flops per point against O(K nm^3) for the full tensor, so it stays FP64.
// B_R = B_F Re[H_m(w1) H_m(w2) conj H_m(w1+w2)] (getRM_diag_vect_cls_ :1974-2101,
// getRM_diag_scalar_cls_ :2562-2637, getRM_diag_scalar_msh_ :1212-1286); the force PSD is
// psd[f][m] = sum_k L_km^2 S_k(f) (functionsImpl.F90:1924-1947).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "../../include/bsa_gpu.h"
#include "bsa_engine.cuh"
#include "bsa_kernels.cuh"

namespace bsa {
namespace diag {

constexpr int kPts = 64;   // points per tile
constexpr int kKC = 32;    // k per shared-memory chunk
constexpr int kMG = 4;     // threads per point (mode groups)
constexpr int kMT = 16;    // modes per thread: nm <= kMG * kMT
constexpr int kMaxModes = kMG * kMT;
constexpr int kBuf = kKC * kMaxModes + kKC * (kPts + 1);

// One block per group of point tiles (grid-stride); thread t owns point t % 64 of the tile
// and modes m = t / 64 + 4 u.  Per-block moment partials part[block][m] in FP64.
__global__ __launch_bounds__(256) void k_diag_fp64(const double *__restrict__ S, const double *__restrict__ W,
                                                   int K, int nm, PointSrc ps, long long npts, int msh_form,
                                                   FrfPar frf, double *__restrict__ part_mf,
                                                   double *__restrict__ part_mr, double *__restrict__ bf_out,
                                                   double *__restrict__ br_out) {
    __shared__ double buf[kBuf];
    __shared__ int pix[kPts], piy[kPts], piz[kPts];
    __shared__ double pw[kPts], pf1[kPts], pf2[kPts];
    double(*Ws)[kMaxModes] = (double(*)[kMaxModes])buf;
    double(*Gs)[kPts + 1] = (double(*)[kPts + 1])(buf + kKC * kMaxModes);
    const int t = threadIdx.x, pl = t % kPts, mg = t / kPts;
    double smf[kMT], smr[kMT];
#pragma unroll
    for (int u = 0; u < kMT; ++u) smf[u] = smr[u] = 0.0;
    const long long ntiles = (npts + kPts - 1) / kPts;
    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const long long p0 = tile * kPts;
        __syncthreads();
        if (t < kPts) {
            int ix = 0, iy = 0, iz = -1;
            double w = 0.0, f1 = 0.0, f2 = 0.0;
            if (p0 + t < npts) get_point(ps, p0 + t, ix, iy, iz, w, f1, f2);
            pix[t] = ix; piy[t] = iy; piz[t] = iz;
            pw[t] = w; pf1[t] = f1; pf2[t] = f2;
        }
        __syncthreads();
        double acc[kMT];
#pragma unroll
        for (int u = 0; u < kMT; ++u) acc[u] = 0.0;
        for (int k0 = 0; k0 < K; k0 += kKC) {
            const int kc = min(kKC, K - k0);
            for (int e = t; e < kKC * kMaxModes; e += 256) {
                const int kk = e / kMaxModes, m = e % kMaxModes;
                Ws[kk][m] = (kk < kc && m < nm) ? W[(size_t)(k0 + kk) * nm + m] : 0.0;
            }
            // one warp reads 32 consecutive k of one point
            for (int e = t; e < kKC * kPts; e += 256) {
                const int kk = e % kKC, q = e / kKC;
                double g = 0.0;
                if (kk < kc && p0 + q < npts) {
                    const size_t k = (size_t)(k0 + kk);
                    const double s1 = S[(size_t)pix[q] * K + k], s2 = S[(size_t)piy[q] * K + k];
                    if (msh_form) {
                        g = s1 * s2 + s1 * s2 * s2 + s1 * s1 * s2;
                    } else {
                        const double s12 = piz[q] >= 0 ? S[(size_t)piz[q] * K + k] : 0.0;
                        g = s1 * s2 + s12 * s2 + s1 * s12;
                    }
                }
                Gs[kk][q] = g;
            }
            __syncthreads();
            for (int kk = 0; kk < kc; ++kk) {
                const double g = Gs[kk][pl];
#pragma unroll
                for (int u = 0; u < kMT; ++u) acc[u] = fma(Ws[kk][mg + kMG * u], g, acc[u]);
            }
            __syncthreads();
        }
        const long long p = p0 + pl;
        if (p >= npts) continue;
        const double w = pw[pl], w1 = pf1[pl] * kPi2, w2 = pf2[pl] * kPi2;
        const ZoneDev *z = ps.zones ? ps.zones + ps.zid[p] : nullptr;
#pragma unroll
        for (int u = 0; u < kMT; ++u) {
            const int m = mg + kMG * u;
            if (m >= nm) continue;
            const double bfv = 2.0 * acc[u];
            const double M = frf.M[m], Kk = frf.K[m], C = frf.C[m];
            double F;
            if (ps.cptr) {
                // listed BRM points (triangular zones), each with its coefficient
                F = 0.0;
                const long long e1 = ps.cptr[p + 1];
                for (long long e = ps.cptr[p]; e < e1; ++e) {
                    const double v1 = ps.cq[3 * e] * kPi2, v2 = ps.cq[3 * e + 1] * kPi2;
                    double h1r, h1i, h2r, h2i, h3r, h3i;
                    frf_eval(M, Kk, C, v1, h1r, h1i);
                    frf_eval(M, Kk, C, v2, h2r, h2i);
                    frf_eval(M, Kk, C, v1 + v2, h3r, h3i);
                    F = fma(ps.cq[3 * e + 2], (h1r * h2r - h1i * h2i) * h3r + (h1r * h2i + h1i * h2r) * h3i, F);
                }
                smf[u] = fma(w, bfv, smf[u]);
                smr[u] = fma(F, bfv, smr[u]);
                continue;
            }
            if (z) {
                // Mesher zone point: this BFM lattice point enters every BRM lattice point of
                // its bilinear support with weight lambda (the full-tensor kernel's rule).
                const int li = ps.zi[p], lj = ps.zj[p];
                const int NI = (z->ni - 1) * z->Fi, NJ = (z->nj - 1) * z->Fj;
                F = 0.0;
                for (int di = 1 - z->Fi; di < z->Fi; ++di) {
                    const int qi = li * z->Fi + di;
                    if (qi < 0 || qi > NI) continue;
                    for (int dj = 1 - z->Fj; dj < z->Fj; ++dj) {
                        const int qj = lj * z->Fj + dj;
                        if (qj < 0 || qj > NJ) continue;
                        const double lam = (1.0 - (double)abs(di) / z->Fi) * (1.0 - (double)abs(dj) / z->Fj);
                        const double ti = (qi == 0 || qi == NI) ? 0.5 : 1.0, tj = (qj == 0 || qj == NJ) ? 0.5 : 1.0;
                        const double wq = z->sym * (z->wI / z->Fi) * (z->wJ / z->Fj) * ti * tj * lam;
                        const double a = (double)qi / z->Fi, bq = (double)qj / z->Fj;
                        const double v1 = (z->fi0 + a * z->dIi + bq * z->dJi) * kPi2;
                        const double v2 = (z->fj0 + a * z->dIj + bq * z->dJj) * kPi2;
                        double h1r, h1i, h2r, h2i, h3r, h3i;
                        frf_eval(M, Kk, C, v1, h1r, h1i);
                        frf_eval(M, Kk, C, v2, h2r, h2i);
                        frf_eval(M, Kk, C, v1 + v2, h3r, h3i);
                        F = fma(wq, (h1r * h2r - h1i * h2i) * h3r + (h1r * h2i + h1i * h2r) * h3i, F);
                    }
                }
                smf[u] = fma(w, bfv, smf[u]);
                smr[u] = fma(F, bfv, smr[u]);
                continue;
            }
            double h1r, h1i, h2r, h2i, h3r, h3i;
            frf_eval(M, Kk, C, w1, h1r, h1i);
            frf_eval(M, Kk, C, w2, h2r, h2i);
            frf_eval(M, Kk, C, w1 + w2, h3r, h3i);
            F = (h1r * h2r - h1i * h2i) * h3r + (h1r * h2i + h1i * h2r) * h3i;
            const double brv = bfv * F;
            smf[u] = fma(w, bfv, smf[u]);
            smr[u] = fma(w, brv, smr[u]);
            if (bf_out) bf_out[(size_t)p * nm + m] = bfv;
            if (br_out) br_out[(size_t)p * nm + m] = brv;
        }
    }
    // Fixed-order reduction over the 64 point lanes of each mode.
    double *red = buf;  // [kMaxModes][kPts]
    for (int pass = 0; pass < 2; ++pass) {
        __syncthreads();
#pragma unroll
        for (int u = 0; u < kMT; ++u) red[(mg + kMG * u) * kPts + pl] = pass == 0 ? smf[u] : smr[u];
        __syncthreads();
        if (t < nm) {
            double s = 0.0;
            for (int q = 0; q < kPts; ++q) s += red[t * kPts + q];
            (pass == 0 ? part_mf : part_mr)[(size_t)blockIdx.x * nm + t] = s;
        }
    }
}

// psd[f][m] = sum_k W2[k][m] S[f][k], W2 = L^2.
__global__ void k_force_psd_diag(int nf, int K, int nm, const double *__restrict__ S, const double *__restrict__ W2,
                                 double *__restrict__ psd) {
    const int f = blockIdx.x, m = threadIdx.x;
    if (f >= nf || m >= nm) return;
    double s = 0.0;
    for (int k = 0; k < K; ++k) s = fma(W2[(size_t)k * nm + m], S[(size_t)f * K + k], s);
    psd[(size_t)f * nm + m] = s;
}

int groups(long long npts) {
    static int nsm = 0;
    if (nsm == 0) {
        int dev = 0;
        if (cudaGetDevice(&dev) != cudaSuccess ||
            cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || nsm <= 0)
            nsm = 132;
    }
    const long long ntiles = (npts + kPts - 1) / kPts;
    return (int)std::max(1LL, std::min(ntiles, 4LL * nsm));
}

}  // namespace diag

cudaError_t launch_force_psd_diag(cudaStream_t st, int nf, int K, int nm, const double *S, const double *W2,
                                  double *psd) {
    diag::k_force_psd_diag<<<nf, 64, 0, st>>>(nf, K, nm, S, W2, psd);
    return cudaGetLastError();
}

// Diagonal-only contraction + FRF + weighted reduction over a point source; dS holds every
// S-table row the source names.  msh_form selects the Mesher products.  bf/br host buffers
// (optional) receive (nm, npts).
int Engine::contract_diag(const PointSrc &ps, long long npts, int msh_form, double *m3mf, double *m3mr,
                          double *bf_host, double *br_host) {
    if (nme > diag::kMaxModes) return fail(BSA_ERR_UNSUPPORTED, "diagonal-only spectra support at most 64 kept modes");
    cudaError_t e;
    const int G = diag::groups(npts);
    if ((e = dPartF.reserve(sizeof(double) * (size_t)G * nme)) || (e = dPartR.reserve(sizeof(double) * (size_t)G * nme)))
        return cuda_fail(e, "allocating partial sums");
    if ((e = dOut.reserve(sizeof(double) * 5 * (size_t)nme))) return cuda_fail(e, "out");
    double *bfd = nullptr, *brd = nullptr;
    if (bf_host || br_host) {
        if ((e = dBF.reserve(sizeof(double) * (size_t)npts * nme)) || (e = dBR.reserve(sizeof(double) * (size_t)npts * nme)))
            return cuda_fail(e, "allocating bispectra");
        bfd = dBF.as<double>();
        brd = dBR.as<double>();
    }
    if ((e = cudaEventRecord(ev2, stream)) || (e = cudaEventRecord(evg0, stream))) return cuda_fail(e, "event");
    diag::k_diag_fp64<<<G, 256, 0, stream>>>(dS.as<double>(), dWd3.as<double>(), K, nme, ps, npts, msh_form, frf(),
                                             dPartF.as<double>(), dPartR.as<double>(), bfd, brd);
    if ((e = cudaGetLastError())) return cuda_fail(e, "diagonal contraction kernel");
    if ((e = cudaEventRecord(evg1, stream))) return cuda_fail(e, "event");
    double *o = dOut.as<double>() + 3 * (size_t)nme;
    if ((e = launch_reduce_groups(stream, G, nme, dPartF.as<double>(), o, dPartR.as<double>(), o + nme)))
        return cuda_fail(e, "reduction kernel");
    kernels += 2;
    std::vector<double> h(2 * (size_t)nme);
    if ((e = cudaMemcpyAsync(h.data(), o, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, stream)))
        return cuda_fail(e, "moment copy");
    if (bf_host && (e = cudaMemcpyAsync(bf_host, bfd, sizeof(double) * (size_t)npts * nme, cudaMemcpyDeviceToHost, stream)))
        return cuda_fail(e, "bispectrum copy");
    if (br_host && (e = cudaMemcpyAsync(br_host, brd, sizeof(double) * (size_t)npts * nme, cudaMemcpyDeviceToHost, stream)))
        return cuda_fail(e, "bispectrum copy");
    if ((e = cudaEventRecord(ev1, stream)) || (e = cudaStreamSynchronize(stream))) return cuda_fail(e, "sync");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ev2, ev1);
    last_ms_contraction = ms;
    cudaEventElapsedTime(&ms, evg0, evg1);
    last_ms_gemm = ms;
    d2h += (double)sizeof(double) * h.size() + (bf_host ? 8.0 * npts * nme : 0.0) + (br_host ? 8.0 * npts * nme : 0.0);
    if (m3mf) std::memcpy(m3mf, h.data(), sizeof(double) * nme);
    if (m3mr) std::memcpy(m3mr, h.data() + nme, sizeof(double) * nme);
    return BSA_OK;
}

}  // namespace bsa
