// bsa_post.cu -- post-processing of the path: the background / resonant decomposition of the
// modal response variances (bsa_computeBRdecomp, src/bsa/BsaLibImpl.F90:1292-1420), the
// Gaussian / non-Gaussian peak factors (bsa_computePeakFactors, :1428-1517) and the nodal
// response moments by modal recombination (bsa_modalRecombination, app/bsa.F90:935-1053).
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

// Modal recombination, one block per DOF d with the kept modes' shape values ph[d][im] in
// shared memory (modalRecombination, app/bsa.F90:935-1053): rows of out ([6][ndofs])
//   0 m2 diag  = sum_m m2(m, m) phi_m^2          3 m2 CCC  = sum_{j,k} m2(j, k) phi_j phi_k
//   1 m3 diag  = sum_m m3(m, m, m) phi_m^3       4 m3 CCC  = sum_{i,j,k} m3(i, j, k) phi_i phi_j phi_k
//   2 m2o2 diag (as m2, from m2o2)               5 m2o2 CCC (as m2 CCC)
// diag_only: the spectra have one entry per mode (m2(m), m3(m)); rows 3-5 are not formed.  The
// index sums are strided over the threads and reduced in a fixed-order tree.
__global__ void k_recomb(int ndofs, int nme, int diag_only, const double *__restrict__ ph,
                         const double *__restrict__ m2, const double *__restrict__ m3,
                         const double *__restrict__ m2o2, double *__restrict__ out) {
    const int d = blockIdx.x;
    extern __shared__ double sph[];
    double *red = sph + nme;
    for (int im = threadIdx.x; im < nme; im += blockDim.x) sph[im] = ph[(size_t)d * nme + im];
    __syncthreads();
    double acc[6] = {0, 0, 0, 0, 0, 0};
    for (int m = threadIdx.x; m < nme; m += blockDim.x) {
        const double p = sph[m], p2 = p * p;
        const int i2 = diag_only ? m : m * nme + m;
        const int i3 = diag_only ? m : (m * nme + m) * nme + m;
        acc[0] += m2[i2] * p2;
        acc[1] += m3[i3] * (p2 * p);
        if (m2o2) acc[2] += m2o2[i2] * p2;
    }
    if (!diag_only) {
        const long long n2 = (long long)nme * nme, n3 = n2 * nme;
        for (long long x = threadIdx.x; x < n2; x += blockDim.x) {
            const double pp = sph[x % nme] * sph[x / nme];
            acc[3] += m2[x] * pp;
            if (m2o2) acc[5] += m2o2[x] * pp;
        }
        for (long long x = threadIdx.x; x < n3; x += blockDim.x) {
            const int i = (int)(x % nme), j = (int)((x / nme) % nme), k = (int)(x / n2);
            acc[4] += m3[x] * (sph[i] * sph[j] * sph[k]);
        }
    }
    for (int r = 0; r < 6; ++r) {
        red[threadIdx.x] = acc[r];
        __syncthreads();
        for (int h = blockDim.x / 2; h > 0; h >>= 1) {
            if ((int)threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
            __syncthreads();
        }
        if (threadIdx.x == 0) out[(size_t)r * ndofs + d] = red[0];
        __syncthreads();
    }
}

}  // namespace post

// bsa_modalRecombination: the kept modes' shapes over every DOF (r_modm(:, modes_), as the
// standalone driver passes them, app/bsa.F90:158-165), the modal moments on the device, one
// recombination kernel; skewness on the host as the reference writes it, m3 / m2^(3/2).
int Engine::modal_recomb(const double *m2mr, const double *m3mr, const double *m2o2mr, double *const *outs) {
    kernels = 0;
    graph_launches = 0;
    h2d = d2h = 0;
    int rc = validate();
    if (rc) return rc;
    if (in.ext_phitc || !in.phi) return fail(BSA_ERR_UNSUPPORTED, "modal recombination needs the modal matrix");
    if ((rc = ensure_stream())) return rc;
    const int ndofs = in.phi_ndofs;
    if (ndofs <= 0) return fail(BSA_ERR_STATE, "modal matrix not set");
    const bool diag_only = set.onlyd != 0;
    const size_t n2 = (size_t)dim_psd(), n3 = (size_t)dim_bisp();
    std::vector<double> ph((size_t)ndofs * nme);
    for (int d = 0; d < ndofs; ++d)
        for (int im = 0; im < nme; ++im) ph[(size_t)d * nme + im] = in.phi[(size_t)d + (size_t)ndofs * (modes[im] - 1)];
    std::vector<double> mom(2 * n2 + n3);
    std::memcpy(mom.data(), m2mr, sizeof(double) * n2);
    std::memcpy(mom.data() + n2, m3mr, sizeof(double) * n3);
    if (m2o2mr) std::memcpy(mom.data() + n2 + n3, m2o2mr, sizeof(double) * n2);
    cudaError_t e;
    if ((e = upload(dMixA, ph, stream)) || (e = upload(dMixB, mom, stream)) ||
        (e = dOut.reserve(sizeof(double) * 6 * (size_t)ndofs)))
        return cuda_fail(e, "modal recombination upload");
    const double *dm = dMixB.as<double>();
    const int threads = 256;
    post::k_recomb<<<ndofs, threads, sizeof(double) * (nme + threads), stream>>>(
        ndofs, nme, diag_only ? 1 : 0, dMixA.as<double>(), dm, dm + n2, m2o2mr ? dm + n2 + n3 : nullptr,
        dOut.as<double>());
    if ((e = cudaGetLastError())) return cuda_fail(e, "modal recombination kernel");
    kernels += 1;
    std::vector<double> h(6 * (size_t)ndofs);
    if ((e = cudaMemcpyAsync(h.data(), dOut.p, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, stream)) ||
        (e = cudaStreamSynchronize(stream)))
        return cuda_fail(e, "modal recombination copy");
    d2h += sizeof(double) * h.size();
    // outs: m2, m3, m2o2, sk (diag), then m2, m3, m2o2, sk (CCC)
    for (int br = 0; br < 2; ++br) {
        if (br == 1 && diag_only) break;  // the reference forms no CCC for diagonal-only spectra
        const double *m2 = h.data() + (size_t)(3 * br) * ndofs, *m3 = m2 + ndofs, *mo = m3 + ndofs;
        if (outs[4 * br + 0]) std::memcpy(outs[4 * br + 0], m2, sizeof(double) * ndofs);
        if (outs[4 * br + 1]) std::memcpy(outs[4 * br + 1], m3, sizeof(double) * ndofs);
        if (outs[4 * br + 2]) std::memcpy(outs[4 * br + 2], mo, sizeof(double) * ndofs);
        if (outs[4 * br + 3])
            for (int d = 0; d < ndofs; ++d) outs[4 * br + 3][d] = m3[d] / std::pow(m2[d], 1.5);
    }
    return BSA_OK;
}

int Engine::br_decomp(const double *m2mf, double *bkg, double *res) {
    kernels = 0;
    graph_launches = 0;
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

int bsa_modalRecombination(const double *m2mr, const double *m3mr, const double *m2o2mr, double *m2_diag,
                           double *m3_diag, double *m2o2_diag, double *sk_diag, double *m2_ccc, double *m3_ccc,
                           double *m2o2_ccc, double *sk_ccc) {
    bsa::Engine &E = eng();
    if (E.halted) return BSA_ERR_STATE;
    if (!m2mr || !m3mr) return E.fail(BSA_ERR_ARG, "null modal moments");
    double *const outs[8] = {m2_diag, m3_diag, m2o2_diag, sk_diag, m2_ccc, m3_ccc, m2o2_ccc, sk_ccc};
    return E.modal_recomb(m2mr, m3mr, m2o2mr, outs);
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
