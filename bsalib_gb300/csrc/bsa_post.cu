// bsa_post.cu -- second-order post-processing of the path: the background / resonant
// decomposition of the modal response variances (bsa_computeBRdecomp,
// src/bsa/BsaLibImpl.F90:1292-1420) and the Gaussian / non-Gaussian peak factors
// (bsa_computePeakFactors, :1428-1517).
//
// The resonant part needs each kept mode's force PSD at its own natural frequency,
//   S_Fm(f_m) = sum_tc sum_{k,j} sum_{l1,l2} phi_j(l1,m) phi_k(l2,m) a_k(l1) a_j(l2) S_jk(f_m)
// (getBR_SFm_val_, functionsImpl.F90:2650-2745).  The reference pairs the DOF index of node j's
// mode shape with node k's force coefficient; with one loaded DOF per node this is
// L_m(j) L_m(k) S_jk; with several loaded DOFs the pairing is kept as written.  One block per kept mode,
// the (component, k, j) pairs strided over its threads, a fixed-order tree reduction.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/bsa_gpu.h"
#include "bsa_engine.cuh"
#include "bsa_kernels.cuh"

namespace bsa {

namespace post {

// S[im][itc*nnl + node] at f = fm[im]; logc[itc][i][j]; aw[itc][node][l] linear force
// coefficients (DOF id order); ph[node][l][im] mode shapes of the loaded DOFs.
__global__ void k_br_sfm(int nme, int ntc, int nnl, int nl, const double *__restrict__ fm,
                         const double *__restrict__ S, const double *__restrict__ logc,
                         const double *__restrict__ aw, const double *__restrict__ ph, double *__restrict__ out) {
    const int im = blockIdx.x;
    const double fa = fabs(fm[im]);
    const int K = ntc * nnl;
    const long long tot = (long long)ntc * nnl * nnl;
    double s = 0.0;
    for (long long x = threadIdx.x; x < tot; x += blockDim.x) {
        const int j = (int)(x % nnl);
        const long long r = x / nnl;
        const int k = (int)(r % nnl), itc = (int)(r / nnl);
        const double Sj = S[(size_t)im * K + itc * nnl + j], Sk = S[(size_t)im * K + itc * nnl + k];
        const double c = fa == 0.0 ? 1.0 : exp(fa * logc[((size_t)itc * nnl + j) * nnl + k]);
        const double Sjk = c * sqrt(Sj * Sk);
        double t = 0.0;
        for (int l2 = 0; l2 < nl; ++l2)
            for (int l1 = 0; l1 < nl; ++l1) {
                const double phs = ph[((size_t)j * nl + l1) * nme + im] * ph[((size_t)k * nl + l2) * nme + im];
                const double a = aw[((size_t)itc * nnl + k) * nl + l1] * aw[((size_t)itc * nnl + j) * nl + l2];
                t += phs * (a * Sjk);
            }
        s += t;
    }
    __shared__ double red[256];
    red[threadIdx.x] = s;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[im] = red[0];
}

}  // namespace post

int Engine::br_decomp(const double *m2mf, double *bkg, double *res) {
    kernels = 0;
    h2d = d2h = 0;
    int rc = upload_problem();
    if (rc) return rc;
    if (in.ext_phitc) return fail(BSA_ERR_UNSUPPORTED, "BR decomposition needs the modal matrix and force coefficients");
    if (!in.natf || !in.xsi) return fail(BSA_ERR_STATE, "natural frequencies / damping not set");
    const int ntc = (int)set.tc.size(), nnl = in.nnl, nl = in.nlibsl, nd = in.wfc_nd;
    const int ndofs = in.ndofs ? in.ndofs : in.nn * in.nlibs;
    std::vector<double> fm(nme), aw((size_t)ntc * nnl * nl), ph((size_t)nnl * nl * nme);
    for (int im = 0; im < nme; ++im) fm[im] = in.natf[modes[im] - 1];
    for (int l = 0; l < nl; ++l)
        if (in.libs_load[l] > nl) return fail(BSA_ERR_ARG, "loaded DOF id %d exceeds the force-coefficient rows", in.libs_load[l]);
    for (int itc = 0; itc < ntc; ++itc)
        for (int i = 0; i < nnl; ++i)
            for (int l = 0; l < nl; ++l)
                aw[((size_t)itc * nnl + i) * nl + l] =
                    in.wfc[(size_t)(in.libs_load[l] - 1) + (size_t)nl * ((size_t)(set.tc[itc] - 1) + (size_t)nd * i)];
    for (int i = 0; i < nnl; ++i) {
        const int skip = (in.n_load[i] - 1) * in.nlibs;
        for (int l = 0; l < nl; ++l)
            for (int im = 0; im < nme; ++im)
                ph[((size_t)i * nl + l) * nme + im] =
                    in.phi[(size_t)(skip + in.libs_load[l] - 1) + (size_t)ndofs * (modes[im] - 1)];
    }
    cudaError_t e;
    if ((rc = build_psd(fm))) return rc;
    if ((e = upload(dMixA, aw, stream)) || (e = upload(dMixB, ph, stream)) || (e = dOut.reserve(sizeof(double) * nme)))
        return cuda_fail(e, "BR decomposition upload");
    post::k_br_sfm<<<nme, 256, 0, stream>>>(nme, ntc, nnl, nl, dFreq.as<double>(), dS.as<double>(), dLogc.as<double>(),
                                           dMixA.as<double>(), dMixB.as<double>(), dOut.as<double>());
    if ((e = cudaGetLastError())) return cuda_fail(e, "BR decomposition kernel");
    kernels += 1;
    std::vector<double> sfm(nme);
    if ((e = cudaMemcpyAsync(sfm.data(), dOut.p, sizeof(double) * nme, cudaMemcpyDeviceToHost, stream)) ||
        (e = cudaStreamSynchronize(stream)))
        return cuda_fail(e, "BR decomposition copy");
    d2h += sizeof(double) * nme;
    const bool diag = set.onlyd != 0;
    for (int im = 0; im < nme; ++im) {
        const int m = modes[im] - 1;
        const double km2 = in.Kg[m] * in.Kg[m];
        bkg[im] = m2mf[diag ? im : (size_t)im * nme + im] / km2;
        res[im] = kPi * kPi2 * fm[im] * sfm[im] / (2 * in.xsi[m] * km2);
    }
    return BSA_OK;
}

}  // namespace bsa

using bsa::eng;

extern "C" {

int bsa_computeBRdecomp(const double *m2mf, double *bkg, double *res) {
    bsa::Engine &E = eng();
    if (E.halted) return BSA_ERR_STATE;
    if (!m2mf || !bkg || !res) return E.fail(BSA_ERR_ARG, "null argument");
    return E.br_decomp(m2mf, bkg, res);
}

int bsa_computePeakFactors(int n, const double *m2, const double *m2o2, double obs_time, double *peak_g,
                           const double *sk, double *peak_ng_pos, double *peak_ng_neg) {
    bsa::Engine &E = eng();
    if (n <= 0 || !m2 || !m2o2 || !peak_g || (sk && !peak_ng_pos)) return E.fail(BSA_ERR_ARG, "invalid argument");
    bool any = false;
    for (int i = 0; i < n; ++i) any = any || m2o2[i] != 0.0;
    if (!any) {
        E.last_error = "\"m2_ord2\" is null: cannot compute extremes";  // a warning: not sticky
        return BSA_SKIPPED;
    }
    const double gamma = 0.5772, pi2 = bsa::kPi * bsa::kPi;
    std::vector<double> beta(n);
    for (int i = 0; i < n; ++i) {
        beta[i] = std::sqrt(m2o2[i] / m2[i]) / bsa::kPi2 * obs_time;
        if (beta[i] < 1.0) {
            E.last_error = "observation time too short for the zero-crossing rate";  // a warning: not sticky
            return BSA_SKIPPED;
        }
    }
    for (int i = 0; i < n; ++i) {
        const double b = std::sqrt(2 * std::log(beta[i]));
        peak_g[i] = gamma / b + b;
        if (!sk) continue;
        // Kwon & Kareem (2014) Hermite model, excess kurtosis from the skewness (g4 = 3/2 sk^2).
        const double r = sk[i] * sk[i], g4 = 1.5 * r;
        const double h40 = std::sqrt(1.0 + 1.5 * g4);
        const double h3 = sk[i] / (4.0 + 2.0 * h40), h4 = (h40 - 1.0) / 18.0;
        const double k = 1.0 / std::sqrt(1 + 2.0 * h3 * h3 + 6.0 * h4 * h4);
        const double b2 = b * b, b3 = b2 * b;
        double pos = 5.44 / b3;
        pos = pos + (3.0 / b * (pi2 / 6.0 - gamma + gamma * gamma));
        pos = pos + (b3 + 3 * b * (gamma - 1));
        pos = pos * h4;
        double neg = pos;
        const double t = h3 * (b2 + 2.0 * gamma - 1. + 1.98 / b2);
        pos = pos + t;
        neg = neg - t;
        peak_ng_pos[i] = (pos + peak_g[i]) * k;
        if (peak_ng_neg) peak_ng_neg[i] = (neg + peak_g[i]) * k;
    }
    return BSA_OK;
}

}  // extern "C"
