// bsa_kernels.cu -- FP64 kernels of the BFM hot path (nodal spectra, per-frequency
// factor A(f), force PSD / second-order moments, and the plain FP64 contraction with the
// FRF product and the weighted moment reduction fused into its epilogue).
#include "bsa_kernels.cuh"

#include <algorithm>

namespace bsa {

// ------------------------------------------------------------------------------------
// Stage (a): nodal turbulence PSD.  One thread per (f, itc, node), node fastest so the
// stores are coalesced.  Model formulas: vonKarmanPSD_ (WindPSDImpl.F90:149-226, u form
// for tc == 1, v/w form otherwise), kaimalPSD_ (:231-243, identically zero),
// davenportPSD_Greisch_ (:249-277), davenportPSD_Uliege_ (:283-316); divided by 4 pi
// under the circular-frequency convention (:142-143).  R = double for the FP64 paths; the
// split-precision paths, whose A(f) tables take sqrt(S) in FP32, evaluate the same formulas
// in FP32 (R = float: relative error ~1e-7, where FP64's pow costs ~100 FP64 instructions).
// ------------------------------------------------------------------------------------
template <typename R>
__global__ void k_nodal_psd(int nf, const double *__restrict__ f, int ntc, int4 tcs, int nnl,
                            const PsdNode *__restrict__ par, int psd_type, int scaling,
                            double *__restrict__ S) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long tot = (long long)nf * ntc * nnl;
    if (t >= tot) return;
    const int i = (int)(t % nnl);
    const long long r = t / nnl;
    const int itc = (int)(r % ntc);
    const int fi = (int)(r / ntc);
    const int tc = itc == 0 ? tcs.x : (itc == 1 ? tcs.y : tcs.z);
    const PsdNode p = par[itc * nnl + i];
    const R fr = (R)f[fi], Ls = (R)p.Ls, U = (R)p.U, Uref = (R)p.Uref, sg = (R)p.sigma;
    const R sig2 = sg * sg;
    R v = 0;
    switch (psd_type) {
    case 1:
        if (tc == 1) {
            const R rt = Ls / U;
            R x = fabs(fr) * rt;
            x = x * x;
            x = pow(R(1) + R(70.7) * x, R(5.0 / 6.0));
            v = R(4) * (rt * sig2) / x;
        } else {
            R d = R(2) * (fr * (Ls / U));
            d = d * d;
            const R r2 = pow(R(1) + R(70.7) * d, R(11.0 / 6.0)) * U;
            const R r3 = Ls * (R(1) + R(188.4) * d) / r2 * sig2;
            const R a = r3 + r3;
            v = a + a;
        }
        break;
    case 2:
        v = 0;
        break;
    case 3: {
        const R cst1 = R(0.65 * 1200.0);
        const R x = cst1 * fr / Uref;
        v = cst1 * sig2 / Uref / pow(R(1) + x * x, R(5.0 / 6.0));
    } break;
    case 5: {
        const R clu = Ls / U;
        const R cf = fabs(fr) * clu;
        v = ((R(2.0 / 3.0)) * cf * clu * sig2) / pow(R(1) + cf * cf, R(4.0 / 3.0));
    } break;
    default:
        v = 0;
    }
    if (scaling == 1) v = v / R(kPi4);
    S[t] = (double)v;
}

cudaError_t launch_nodal_psd(cudaStream_t st, int nf, const double *f, int ntc, const int *tcs_host,
                             int nnl, const PsdNode *par, int psd_type, int scaling, double *S, bool fp32) {
    const long long tot = (long long)nf * ntc * nnl;
    if (tot == 0) return cudaSuccess;
    int4 tcs = make_int4(tcs_host[0], ntc > 1 ? tcs_host[1] : 0, ntc > 2 ? tcs_host[2] : 0, 0);
    const int blk = 256;
    const unsigned grid = (unsigned)((tot + blk - 1) / blk);
    if (fp32)
        k_nodal_psd<float><<<grid, blk, 0, st>>>(nf, f, ntc, tcs, nnl, par, psd_type, scaling, S);
    else
        k_nodal_psd<double><<<grid, blk, 0, st>>>(nf, f, ntc, tcs, nnl, par, psd_type, scaling, S);
    return cudaGetLastError();
}

// ------------------------------------------------------------------------------------
// Stage (a)+(b) factor: A(f)[(itc,i)][m] = sqrt(S_i) sum_j c_ij^|f| sqrt(S_j) L[(itc,j)][m].
// The coherent cross-PSD c_ij^|f| sqrt(S_i S_j) (functionsImpl.F90:1450-1477,
// getFullNodalPSD WindPSDImpl.F90:76-108) is generated on the fly from log c_ij and never
// stored as an NNL^2 x NF tensor.  Block: 32 rows i x all modes, j streamed in tiles of
// 32 through shared memory.  c^0 = 1 for every c (Fortran 0**0 = 1).
// ------------------------------------------------------------------------------------
__global__ __launch_bounds__(256) void k_atable(int nf, const double *__restrict__ f, int ntc, int nnl,
                                                int nm, const double *__restrict__ logc,
                                                const double *__restrict__ S,
                                                const double *__restrict__ L, double *__restrict__ A) {
    const int fi = blockIdx.x / ntc, itc = blockIdx.x % ntc;
    const int i0 = blockIdx.y * 32;
    __shared__ double Gs[32][33];
    __shared__ double Ls[32][64];
    const double af = fabs(f[fi]);
    const double *Sf = S + ((size_t)fi * ntc + itc) * nnl;
    const double *lc = logc + (size_t)itc * nnl * nnl;
    const double *Lt = L + (size_t)itc * nnl * nm;
    const int t = threadIdx.x, il = t >> 3, mg = t & 7;
    double acc[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) acc[u] = 0.0;
    for (int j0 = 0; j0 < nnl; j0 += 32) {
        for (int e = t; e < 32 * 32; e += 256) {
            const int ii = e >> 5, jj = e & 31, gi = i0 + ii, gj = j0 + jj;
            double g = 0.0;
            if (gi < nnl && gj < nnl) {
                const double l = lc[(size_t)gi * nnl + gj];
                g = (af == 0.0) ? 1.0 : exp(af * l);
            }
            Gs[ii][jj] = g;
        }
        for (int e = t; e < 32 * nm; e += 256) {
            const int jj = e / nm, m = e % nm, gj = j0 + jj;
            Ls[jj][m] = gj < nnl ? sqrt(Sf[gj]) * Lt[(size_t)gj * nm + m] : 0.0;
        }
        __syncthreads();
#pragma unroll 4
        for (int jj = 0; jj < 32; ++jj) {
            const double g = Gs[il][jj];
#pragma unroll
            for (int u = 0; u < 8; ++u) {
                const int m = mg + 8 * u;
                if (m < nm) acc[u] = fma(g, Ls[jj][m], acc[u]);
            }
        }
        __syncthreads();
    }
    const int gi = i0 + il;
    if (gi < nnl) {
        const double si = sqrt(Sf[gi]);
        double *out = A + (((size_t)fi * ntc + itc) * nnl + gi) * nm;
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int m = mg + 8 * u;
            if (m < nm) out[m] = si * acc[u];
        }
    }
}

__global__ void k_log_coh(size_t n, double *__restrict__ lc, float *__restrict__ lc32) {
    const size_t x = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= n) return;
    const double v = log(lc[x]);
    lc[x] = v;
    lc32[x] = (float)v;
}

cudaError_t launch_log_coh(cudaStream_t st, size_t n, double *lc, float *lc32) {
    if (n == 0) return cudaSuccess;
    k_log_coh<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(n, lc, lc32);
    return cudaGetLastError();
}

cudaError_t launch_atable(cudaStream_t st, int nf, const double *f, int ntc, int nnl, int nm,
                          const double *logc, const double *S, const double *L, double *A) {
    if (nf == 0) return cudaSuccess;
    if (nm > 64) return cudaErrorInvalidValue;
    dim3 grid((unsigned)nf * ntc, (unsigned)((nnl + 31) / 32));
    k_atable<<<grid, 256, 0, st>>>(nf, f, ntc, nnl, nm, logc, S, L, A);
    return cudaGetLastError();
}

// ------------------------------------------------------------------------------------
// Second-order path: force PSD and m2 moments (functionsImpl.F90:1548-1560, 1653-1676;
// BsaClassicImpl.F90:149-154, 197-210).
// ------------------------------------------------------------------------------------
template <class TA>
__global__ void k_force_psd(int ntc, int nnl, int nm, const double *__restrict__ L, const TA *__restrict__ A,
                            double *__restrict__ psd) {
    const int fi = blockIdx.x;
    const int nm2 = nm * nm, K = ntc * nnl;
    const TA *Af = A + (size_t)fi * K * nm;
    for (int pr = threadIdx.x; pr < nm2; pr += blockDim.x) {
        const int n = pr % nm, o = pr / nm;
        double s = 0.0;
        for (int k = 0; k < K; ++k) s = fma(L[(size_t)k * nm + o], (double)Af[(size_t)k * nm + n], s);
        psd[(size_t)fi * nm2 + pr] = s;
    }
}

cudaError_t launch_force_psd(cudaStream_t st, int nf, int ntc, int nnl, int nm, const double *L,
                             const double *A, double *psd) {
    if (nf == 0) return cudaSuccess;
    k_force_psd<double><<<nf, 256, 0, st>>>(ntc, nnl, nm, L, A, psd);
    return cudaGetLastError();
}

// The same from the FP32 tables of the split path: FP32 products summed in FP32 over runs of
// 32 k and the runs in FP64 (GB300's FP64 rate makes the all-FP64 form the slow one; the
// operands are FP32-rounded anyway, and the runs keep the sum to ~1e-7).
__global__ void k_force_psd32(int ntc, int nnl, int nm, const float *__restrict__ L, const float *__restrict__ A,
                              double *__restrict__ psd) {
    const int fi = blockIdx.x;
    const int nm2 = nm * nm, K = ntc * nnl;
    const float *Af = A + (size_t)fi * K * nm;
    for (int pr = threadIdx.x; pr < nm2; pr += blockDim.x) {
        const int n = pr % nm, o = pr / nm;
        double s = 0.0;
        for (int k0 = 0; k0 < K; k0 += 32) {
            const int k1 = min(K, k0 + 32);
            float r = 0.f;
            for (int k = k0; k < k1; ++k) r = fmaf(L[(size_t)k * nm + o], Af[(size_t)k * nm + n], r);
            s += (double)r;
        }
        psd[(size_t)fi * nm2 + pr] = s;
    }
}

cudaError_t launch_force_psd32(cudaStream_t st, int nf, int ntc, int nnl, int nm, const float *L,
                               const float *A, double *psd) {
    if (nf == 0) return cudaSuccess;
    k_force_psd32<<<nf, 256, 0, st>>>(ntc, nnl, nm, L, A, psd);
    return cudaGetLastError();
}

// One block per (n, o) pair; threads stride over frequencies, fixed-order tree reduction.
// diag != 0: psd[f][m] holds the same-mode spectra (length nm), pair (n, o) = (m, m).
__global__ void k_m2(int k0, int k1, int nm, int diag, const double *__restrict__ f, const double *__restrict__ wf,
                     const double *__restrict__ psd, FrfPar frf, double *m2mf, double *m2mr,
                     double *m2o2mr) {
    const int nm2 = diag ? nm : nm * nm;
    const int pr = blockIdx.x;
    const int n = diag ? pr : pr % nm, o = diag ? pr : pr / nm;
    double sf = 0.0, sr = 0.0, so = 0.0;
    for (int k = k0 + threadIdx.x; k < k1; k += blockDim.x) {
        const double w = f[k] * kPi2;
        double hnr, hni, hor, hoi;
        frf_eval(frf.M[n], frf.K[n], frf.C[n], w, hnr, hni);
        frf_eval(frf.M[o], frf.K[o], frf.C[o], w, hor, hoi);
        const double p = psd[(size_t)k * nm2 + pr];
        const double pr_ = p * (hor * hnr + hoi * hni);
        sf += wf[k] * p;
        sr += wf[k] * pr_;
        so += wf[k] * (pr_ * w * w);
    }
    __shared__ double red[3][256];
    red[0][threadIdx.x] = sf;
    red[1][threadIdx.x] = sr;
    red[2][threadIdx.x] = so;
    __syncthreads();
    for (int h = blockDim.x / 2; h > 0; h >>= 1) {
        if ((int)threadIdx.x < h)
            for (int q = 0; q < 3; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + h];
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        if (m2mf) m2mf[pr] = red[0][0];
        if (m2mr) m2mr[pr] = red[1][0];
        if (m2o2mr) m2o2mr[pr] = red[2][0];
    }
}

cudaError_t launch_m2(cudaStream_t st, int k0, int k1, int nm, int diag, const double *f, const double *wf,
                      const double *psd, FrfPar frf, double *m2mf, double *m2mr, double *m2o2mr) {
    k_m2<<<diag ? nm : nm * nm, 256, 0, st>>>(k0, k1, nm, diag, f, wf, psd, frf, m2mf, m2mr, m2o2mr);
    return cudaGetLastError();
}

// ------------------------------------------------------------------------------------
// Stages (b)+(c) in FP64, one block per (point group, tile of NOT (n,o) pairs).
// ------------------------------------------------------------------------------------
constexpr int KC = 32;

template <int NOT, int MT>
__global__ __launch_bounds__(256) void k_bfm_fp64(const double *__restrict__ A,
                                                  const double *__restrict__ Q, int K, int nm,
                                                  PointSrc ps, long long npts, FrfPar frf,
                                                  double *__restrict__ part_mf,
                                                  double *__restrict__ part_mr,
                                                  double *__restrict__ bf_out,
                                                  double *__restrict__ br_out) {
    constexpr int MG = 256 / NOT;  // m-groups; thread owns m = mg + MG * u, u < MT
    const int tile = blockIdx.x, pg = blockIdx.y, G = gridDim.y;
    const int t = threadIdx.x, nol = t % NOT, mg = t / NOT;
    const int nm2 = nm * nm;
    const long long nm3 = (long long)nm2 * nm;
    const int no = tile * NOT + nol;
    const bool ok = no < nm2;
    const int n = ok ? no % nm : 0, o = ok ? no / nm : 0;
    extern __shared__ double sm[];
    double *Qs = sm;
    double *Zs = Qs + KC * nm;
    double *Ps = Zs + KC * nm;
    double *Rs = Ps + KC * NOT;
    double *Hs = Rs + KC * NOT;  // [3][nm][2]
    double smf[MT], smr[MT];
#pragma unroll
    for (int u = 0; u < MT; ++u) smf[u] = smr[u] = 0.0;
    const size_t tab = (size_t)K * nm;
    for (long long p = pg; p < npts; p += G) {
        int ix, iy, iz;
        double w, f1, f2;
        get_point(ps, p, ix, iy, iz, w, f1, f2);
        const double *X = A + (size_t)ix * tab;
        const double *Y = A + (size_t)iy * tab;
        const double *Z = iz >= 0 ? A + (size_t)iz * tab : nullptr;
        double acc[MT];
#pragma unroll
        for (int u = 0; u < MT; ++u) acc[u] = 0.0;
        for (int k0 = 0; k0 < K; k0 += KC) {
            const int kc = min(KC, K - k0);
            for (int e = t; e < kc * nm; e += 256) {
                Qs[e] = Q[(size_t)k0 * nm + e];
                Zs[e] = Z ? Z[(size_t)k0 * nm + e] : 0.0;
            }
            for (int e = t; e < kc * NOT; e += 256) {
                const int kk = e / NOT, jl = e % NOT, pr = tile * NOT + jl;
                double pv = 0.0, rv = 0.0;
                if (pr < nm2) {
                    const int nn = pr % nm, oo = pr / nm;
                    const size_t r = (size_t)(k0 + kk) * nm;
                    const double x = X[r + nn], y = Y[r + oo], qn = Q[r + nn], qo = Q[r + oo];
                    pv = x * y;
                    rv = fma(qn, y, x * qo);
                }
                Ps[e] = pv;
                Rs[e] = rv;
            }
            __syncthreads();
            if (ok) {
                for (int kk = 0; kk < kc; ++kk) {
                    const double pv = Ps[kk * NOT + nol], rv = Rs[kk * NOT + nol];
                    const double *qr = Qs + kk * nm, *zr = Zs + kk * nm;
#pragma unroll
                    for (int u = 0; u < MT; ++u) {
                        const int m = mg + MG * u;
                        if (m < nm) acc[u] = fma(qr[m], pv, fma(zr[m], rv, acc[u]));
                    }
                }
            }
            __syncthreads();
        }
        if (ps.cptr) {
            // listed BRM points (triangular zones): G = sum_e c_e Re[H_m(w1_e) H_n(w2_e) conj H_o(w1_e + w2_e)]
            double g[MT];
#pragma unroll
            for (int u = 0; u < MT; ++u) g[u] = 0.0;
            const long long e1 = ps.cptr[p + 1];
            for (long long e = ps.cptr[p]; e < e1; ++e) {
                const double v1 = ps.cq[3 * e] * kPi2, v2 = ps.cq[3 * e + 1] * kPi2, ce = ps.cq[3 * e + 2];
                if (t < nm) {
                    frf_eval(frf.M[t], frf.K[t], frf.C[t], v1, Hs[2 * t], Hs[2 * t + 1]);
                    frf_eval(frf.M[t], frf.K[t], frf.C[t], v2, Hs[2 * nm + 2 * t], Hs[2 * nm + 2 * t + 1]);
                    frf_eval(frf.M[t], frf.K[t], frf.C[t], v1 + v2, Hs[4 * nm + 2 * t], Hs[4 * nm + 2 * t + 1]);
                }
                __syncthreads();
                if (ok) {
                    const double h2r = Hs[2 * nm + 2 * n], h2i = Hs[2 * nm + 2 * n + 1];
                    const double h3r = Hs[4 * nm + 2 * o], h3i = Hs[4 * nm + 2 * o + 1];
                    const double cr = h2r * h3r + h2i * h3i, ci = h2i * h3r - h2r * h3i;
#pragma unroll
                    for (int u = 0; u < MT; ++u) {
                        const int m = mg + MG * u;
                        if (m < nm) g[u] = fma(ce, Hs[2 * m] * cr - Hs[2 * m + 1] * ci, g[u]);
                    }
                }
                __syncthreads();
            }
            if (ok) {
#pragma unroll
                for (int u = 0; u < MT; ++u) {
                    const int m = mg + MG * u;
                    if (m < nm) {
                        const double bfv = 2.0 * acc[u];
                        smf[u] = fma(w, bfv, smf[u]);
                        smr[u] = fma(g[u], bfv, smr[u]);
                    }
                }
            }
            continue;
        }
        if (ps.zones) {
            // Mesher zone point: the force bispectrum of this BFM lattice point enters every
            // BRM lattice point of its bilinear support with weight lambda; accumulate
            // G = sum_q lambda_q w_q Re[H_m(w1_q) H_n(w2_q) conj H_o(w1_q + w2_q)].
            const ZoneDev z = ps.zones[ps.zid[p]];
            const int li = ps.zi[p], lj = ps.zj[p];
            const int NI = (z.ni - 1) * z.Fi, NJ = (z.nj - 1) * z.Fj;  // last BRM index
            double g[MT];
#pragma unroll
            for (int u = 0; u < MT; ++u) g[u] = 0.0;
            for (int di = 1 - z.Fi; di < z.Fi; ++di) {
                const int qi = li * z.Fi + di;
                if (qi < 0 || qi > NI) continue;
                for (int dj = 1 - z.Fj; dj < z.Fj; ++dj) {
                    const int qj = lj * z.Fj + dj;
                    if (qj < 0 || qj > NJ) continue;
                    const double lam = (1.0 - (double)abs(di) / z.Fi) * (1.0 - (double)abs(dj) / z.Fj);
                    const double ti = (qi == 0 || qi == NI) ? 0.5 : 1.0, tj = (qj == 0 || qj == NJ) ? 0.5 : 1.0;
                    const double wq = z.sym * (z.wI / z.Fi) * (z.wJ / z.Fj) * ti * tj * lam;
                    const double a = (double)qi / z.Fi, bq = (double)qj / z.Fj;
                    const double q1 = z.fi0 + a * z.dIi + bq * z.dJi, q2 = z.fj0 + a * z.dIj + bq * z.dJj;
                    const double v1 = q1 * kPi2, v2 = q2 * kPi2;
                    if (t < nm) {
                        frf_eval(frf.M[t], frf.K[t], frf.C[t], v1, Hs[2 * t], Hs[2 * t + 1]);
                        frf_eval(frf.M[t], frf.K[t], frf.C[t], v2, Hs[2 * nm + 2 * t], Hs[2 * nm + 2 * t + 1]);
                        frf_eval(frf.M[t], frf.K[t], frf.C[t], v1 + v2, Hs[4 * nm + 2 * t], Hs[4 * nm + 2 * t + 1]);
                    }
                    __syncthreads();
                    if (ok) {
                        const double h2r = Hs[2 * nm + 2 * n], h2i = Hs[2 * nm + 2 * n + 1];
                        const double h3r = Hs[4 * nm + 2 * o], h3i = Hs[4 * nm + 2 * o + 1];
                        const double cr = h2r * h3r + h2i * h3i, ci = h2i * h3r - h2r * h3i;
#pragma unroll
                        for (int u = 0; u < MT; ++u) {
                            const int m = mg + MG * u;
                            if (m < nm) g[u] = fma(wq, Hs[2 * m] * cr - Hs[2 * m + 1] * ci, g[u]);
                        }
                    }
                    __syncthreads();
                }
            }
            if (ok) {
#pragma unroll
                for (int u = 0; u < MT; ++u) {
                    const int m = mg + MG * u;
                    if (m < nm) {
                        const double bfv = 2.0 * acc[u];
                        smf[u] = fma(w, bfv, smf[u]);
                        smr[u] = fma(g[u], bfv, smr[u]);
                    }
                }
            }
            continue;
        }
        const double w1 = f1 * kPi2, w2 = f2 * kPi2;
        if (t < nm) {
            frf_eval(frf.M[t], frf.K[t], frf.C[t], w1, Hs[2 * t], Hs[2 * t + 1]);
            frf_eval(frf.M[t], frf.K[t], frf.C[t], w2, Hs[2 * nm + 2 * t], Hs[2 * nm + 2 * t + 1]);
            frf_eval(frf.M[t], frf.K[t], frf.C[t], w1 + w2, Hs[4 * nm + 2 * t], Hs[4 * nm + 2 * t + 1]);
        }
        __syncthreads();
        if (ok) {
            const double h2r = Hs[2 * nm + 2 * n], h2i = Hs[2 * nm + 2 * n + 1];
            const double h3r = Hs[4 * nm + 2 * o], h3i = Hs[4 * nm + 2 * o + 1];
            // H_n(w2) conj(H_o(w1+w2))
            const double cr = h2r * h3r + h2i * h3i, ci = h2i * h3r - h2r * h3i;
#pragma unroll
            for (int u = 0; u < MT; ++u) {
                const int m = mg + MG * u;
                if (m < nm) {
                    const double F = Hs[2 * m] * cr - Hs[2 * m + 1] * ci;
                    const double bfv = 2.0 * acc[u];
                    const double brv = bfv * F;
                    smf[u] = fma(w, bfv, smf[u]);
                    smr[u] = fma(w, brv, smr[u]);
                    const size_t idx = (size_t)p * nm3 + m + (size_t)nm * no;
                    if (bf_out) bf_out[idx] = bfv;
                    if (br_out) br_out[idx] = brv;
                }
            }
        }
        __syncthreads();
    }
    if (ok) {
#pragma unroll
        for (int u = 0; u < MT; ++u) {
            const int m = mg + MG * u;
            if (m < nm) {
                const size_t idx = (size_t)pg * nm3 + m + (size_t)nm * no;
                part_mf[idx] = smf[u];
                part_mr[idx] = smr[u];
            }
        }
    }
}

static int not_for(int nm) {
    const int nm2 = nm * nm;
    return nm2 >= 64 ? 64 : (nm2 > 16 ? 32 : 16);
}

int bfm_fp64_groups(long long npts, int nm) {
    const int NOT = not_for(nm);
    const int tiles = (nm * nm + NOT - 1) / NOT;
    long long g = (1216 + tiles - 1) / tiles;  // about 8 blocks per SM on 152 SMs
    g = std::min<long long>(g, npts);
    g = std::min<long long>(g, 65535);
    return (int)std::max<long long>(g, 1);
}

template <int NOT, int MT>
static cudaError_t launch_bfm_t(cudaStream_t st, const double *A, const double *Q, int K, int nm,
                                const PointSrc &ps, long long npts, FrfPar frf, int n_groups,
                                double *part_mf, double *part_mr, double *bf_out, double *br_out) {
    const size_t smem = sizeof(double) * (2 * KC * nm + 2 * KC * NOT + 6 * nm);
    cudaError_t e = cudaFuncSetAttribute(k_bfm_fp64<NOT, MT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid((unsigned)((nm * nm + NOT - 1) / NOT), (unsigned)n_groups);
    k_bfm_fp64<NOT, MT><<<grid, 256, smem, st>>>(A, Q, K, nm, ps, npts, frf, part_mf, part_mr, bf_out, br_out);
    return cudaGetLastError();
}

// MT = smallest supported count >= ceil(nm / MG), so no thread carries idle mode slots.
template <int NOT>
static cudaError_t launch_bfm_n(cudaStream_t st, const double *A, const double *Q, int K, int nm,
                                const PointSrc &ps, long long npts, FrfPar frf, int n_groups,
                                double *part_mf, double *part_mr, double *bf_out, double *br_out) {
    constexpr int MG = 256 / NOT;
    const int need = (nm + MG - 1) / MG;
#define BSA_MT_CASE(V)                                                                                   \
    if (need <= V)                                                                                       \
        return launch_bfm_t<NOT, V>(st, A, Q, K, nm, ps, npts, frf, n_groups, part_mf, part_mr, bf_out, br_out);
    BSA_MT_CASE(1)
    BSA_MT_CASE(2)
    BSA_MT_CASE(4)
    BSA_MT_CASE(6)
    BSA_MT_CASE(8)
    BSA_MT_CASE(12)
    BSA_MT_CASE(16)
#undef BSA_MT_CASE
    return cudaErrorInvalidValue;
}

cudaError_t launch_bfm_fp64(cudaStream_t st, const double *A, const double *Q, int K, int nm,
                            const PointSrc &ps, long long npts, FrfPar frf, int n_groups,
                            double *part_mf, double *part_mr, double *bf_out, double *br_out) {
    if (nm > 64 || nm < 1) return cudaErrorInvalidValue;
    if (npts == 0) return cudaSuccess;
    switch (not_for(nm)) {
    case 64:
        return launch_bfm_n<64>(st, A, Q, K, nm, ps, npts, frf, n_groups, part_mf, part_mr, bf_out, br_out);
    case 32:
        return launch_bfm_n<32>(st, A, Q, K, nm, ps, npts, frf, n_groups, part_mf, part_mr, bf_out, br_out);
    default:
        return launch_bfm_n<16>(st, A, Q, K, nm, ps, npts, frf, n_groups, part_mf, part_mr, bf_out, br_out);
    }
}

__global__ void k_reduce_groups(int n_groups, long long len, const double *__restrict__ part,
                                double *__restrict__ out, const double *__restrict__ part2,
                                double *__restrict__ out2) {
    const long long x = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= len) return;
    double s = 0.0, s2 = 0.0;
    for (int g = 0; g < n_groups; ++g) {
        s += part[(size_t)g * len + x];
        if (part2) s2 += part2[(size_t)g * len + x];
    }
    out[x] = s;
    if (out2) out2[x] = s2;
}

cudaError_t launch_reduce_groups(cudaStream_t st, int n_groups, long long len, const double *part,
                                 double *out, const double *part2, double *out2) {
    if (len == 0) return cudaSuccess;
    k_reduce_groups<<<(unsigned)((len + 255) / 256), 256, 0, st>>>(n_groups, len, part, out, part2, out2);
    return cudaGetLastError();
}

}  // namespace bsa
