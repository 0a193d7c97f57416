/*
 * bsa_oracle.c -- TEST INFRASTRUCTURE ONLY (the parity oracle).
 *
 * A plain-C, FP64 restatement of BsaLib's bispectral-force-model (BFM) hot path, written
 * to follow the reference's loop order and quirks so that the CUDA path can be checked
 * against it.  Nothing in the product links or calls this file: only the tests, the
 * smoke check and the CPU-baseline leg of the benchmark load it.
 *
 * Parity status: the reference's Fortran cannot be built in this environment (no Fortran
 * compiler, no LAPACK) and ships no tests or golden vectors.  Its GPU offload kernel
 * (BsaCL/src/bsacl.cl, OpenCL C) is compiled for the host by oracle/bsacl_ref.py: this
 * oracle's Classic force / response bispectra over frequency pairs and its nodal PSD are
 * PINNED against that reference code (tests/test_oracle_bsacl_pin.py, 2e-7; fixtures in
 * tests/golden/bsacl_ref.npz).  The rest (grid weights, Mesher zones, POD) is cross-checked
 * by independent numpy restatements (tests/golden/make_golden.py).
 *
 * Array conventions follow the Fortran reference: every multi-dimensional array is
 * column-major, node / mode / lib / zone identifiers passed in are 1-based.
 *
 * Reference files cited below are relative to the BsaLib project root.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define PI_ 3.14159265358979323846264338327950288
#define PIt2 (2.0 * PI_)
#define PIt4 (4.0 * PI_)

typedef struct {
    int nn, nlibs, nnl, nlibsl;
    const int *n_load;        /* (nnl) 1-based node ids               */
    const int *libs_load;     /* (nlibsl) 1-based nodal DOF ids        */
    int psd_type;             /* 1 von Karman, 2 Kaimal, 3 Davenport (Greisch), 5 Davenport (Uliege) */
    int scaling;              /* i_def_scaling_: 1 circular freq., 2 freq. */
    int idir;                 /* wind direction (1 = X)                */
    int ntc;
    const int *tc;            /* (ntc) turbulent components 1..3       */
    int nz;
    const double *u_mean_ref; /* (nz)                                  */
    const double *L;          /* (3,3,nz) turbulence length scales     */
    const double *sigma;      /* (3,nz) turbulence std                  */
    const double *u_node;     /* (nn) nodal mean speed                 */
    const int *wz_node;       /* (nn) 1-based wind zone of each node   */
    const double *nod_corr;   /* ((nn*nn+nn)/2, 3) packed coherence    */
    const double *wfc;        /* (nlibsl, ndegw3, nnl) force coeffs    */
    int ndegw3;
    int ndofs, nm;
    const double *phi;        /* (ndofs, nm) modal matrix              */
    const double *Mm, *Km;    /* (nm) generalised mass / stiffness     */
    const double *Cm;         /* (nm, nm) generalised damping          */
    int nm_eff;
    const int *modes;         /* (nm_eff) 1-based kept modes           */
    const double *phitc;      /* (nm_eff, nnl, ndegw3) projected coeffs */
} orc_problem;

#define I2(i, j, ld) ((size_t)(i) + (size_t)(ld) * (size_t)(j))
#define I3(i, j, k, ld1, ld2) ((size_t)(i) + (size_t)(ld1) * ((size_t)(j) + (size_t)(ld2) * (size_t)(k)))

/* util_getCorrVectIndex, src/utils/utility.F90:60-71 (1-based in, 1-based out). */
long orc_corr_index(int ni, int nj, int tot)
{
    if (nj >= ni) return (long)(ni - 1) * tot + nj - (long)(((long)ni * ni - ni) / 2);
    return (long)(nj - 1) * tot + ni - (long)(((long)nj * nj - nj) / 2);
}

static double corr_of(const orc_problem *P, int ni, int nj, int tc)
{
    long id = orc_corr_index(ni, nj, P->nn);
    long ncorr = ((long)P->nn * P->nn + P->nn) / 2;
    return P->nod_corr[(size_t)(id - 1) + (size_t)ncorr * (size_t)(tc - 1)];
}

/*
 * evalPSD_ (src/wind/WindPSDImpl.F90:123-144) with the model functions
 * vonKarmanPSD_ (:149-226), kaimalPSD_ (:231-243), davenportPSD_Greisch_ (:249-277) and
 * davenportPSD_Uliege_ (:283-316).  out(nf, nnl) column-major.  Returns 0, or -1 for a
 * PSD id the reference has no function for (id 4, or out of range).
 */
int orc_eval_psd(const orc_problem *P, int nf, const double *f, int itc, double *out)
{
    const int idir = P->idir;
    for (int in = 0; in < P->nnl; ++in) {
        const int n = P->n_load[in];
        const int wz = P->wz_node[n - 1];
        const double U = P->u_node[n - 1];
        const double sig = P->sigma[I2(itc - 1, wz - 1, 3)];
        double *col = out + (size_t)nf * in;
        switch (P->psd_type) {
        case 1: {
            if (itc == 1) {
                const double Lv = P->L[I3(0, idir - 1, wz - 1, 3, 3)];
                const double rt = Lv / U;
                const double rs = rt * sig * sig;
                for (int k = 0; k < nf; ++k) {
                    double x = fabs(f[k]) * rt;
                    x = x * x;
                    x = pow(1.0 + 70.7 * x, 5.0 / 6.0);
                    col[k] = 4.0 * rs / x;
                }
            } else {
                const double Lv = P->L[I3(itc - 1, idir - 1, wz - 1, 3, 3)];
                for (int k = 0; k < nf; ++k) {
                    double d = 2.0 * (f[k] * (Lv / U));
                    d = d * d;
                    double r1 = 1.0 + 70.7 * d;
                    double r2 = pow(r1, 11.0 / 6.0) * U;
                    double r3 = Lv * (1.0 + 188.4 * d) / r2 * (sig * sig);
                    double a = r3 + r3;
                    col[k] = a + a;
                }
            }
        } break;
        case 2:
            for (int k = 0; k < nf; ++k) col[k] = 0.0;
            break;
        case 3: {
            const double cst1 = 0.65 * 1200.0;
            const double Ur = P->u_mean_ref[wz - 1];
            for (int k = 0; k < nf; ++k) {
                double x = cst1 * f[k] / Ur;
                col[k] = cst1 * (sig * sig) / Ur / pow(1.0 + pow(x, 2.0), 5.0 / 6.0);
            }
        } break;
        case 5: {
            const double Lv = P->L[I3(itc - 1, idir - 1, wz - 1, 3, 3)];
            const double clu = Lv / U;
            for (int k = 0; k < nf; ++k) {
                double cf = fabs(f[k]) * clu;
                col[k] = ((2.0 / 3.0) * cf * clu * (sig * sig)) / pow(1.0 + cf * cf, 4.0 / 3.0);
            }
        } break;
        default:
            return -1;
        }
        if (P->scaling == 1)
            for (int k = 0; k < nf; ++k) col[k] = col[k] / PIt4;
    }
    return 0;
}

/*
 * validateModalInfo_ (src/bsa/BsaLibImpl.F90:545-599): a mode is kept only when
 * max|Phi(:,m)| == 1 exactly.  Writes the kept 1-based mode ids, returns their count.
 */
int orc_validate_modes(int ndofs, int nm, const double *phi, int *modes_out)
{
    int nk = 0;
    for (int m = 0; m < nm; ++m) {
        double mx = 0.0;
        for (int d = 0; d < ndofs; ++d) {
            double a = fabs(phi[I2(d, m, ndofs)]);
            if (a > mx) mx = a;
        }
        if (mx == 1.0) modes_out[nk++] = m + 1;
    }
    return nk;
}

/*
 * setPhitimesCLocalInstance_ (src/bsa/BsaLibImpl.F90:611-671):
 * out(im, in, id) = sum_l wfc(l, id, in) * Phi((n-1)*nlibs + libs_load(l), modes(im)).
 */
void orc_phitimesc(const orc_problem *P, double *out)
{
    const int nme = P->nm_eff, nnl = P->nnl, nd = P->ndegw3;
    for (size_t x = 0; x < (size_t)nme * nnl * nd; ++x) out[x] = 0.0;
    for (int in = 0; in < nnl; ++in) {
        const int n = P->n_load[in];
        const int skip = (n - 1) * P->nlibs;
        for (int id = 0; id < nd; ++id)
            for (int im = 0; im < nme; ++im) {
                const int m = P->modes[im];
                double s = 0.0;
                for (int l = 0; l < P->nlibsl; ++l)
                    s += P->wfc[I3(l, id, in, P->nlibsl, nd)] *
                         P->phi[I2(skip + P->libs_load[l] - 1, m - 1, P->ndofs)];
                out[I3(im, in, id, nme, nnl)] += s;
            }
    }
}

/*
 * computeFreqsVect_ (src/bsa/classic/BsaClassicImpl.F90:443-560).  res_peak_width = xsi*natf
 * (StructureImpl.F90 ComputeResPeakWidths).  Writes the grid into f_out (capacity cap) and
 * the possibly-overridden df into *df_out.  Returns the number of frequencies, or -1
 * (zero input / capacity), -2 (even count under scaling 1).
 */
int orc_compute_freqs(int nfreqs, double df, int scaling, int test_mode, int nm,
                      const double *natf, const double *xsi, double *f_out, int cap,
                      double *df_out)
{
    if (nfreqs == 0 || df == 0.0) return -1;
    double df_ref = INFINITY, max_ref = -INFINITY;
    for (int m = 0; m < nm; ++m) {
        double w = xsi[m] * natf[m];
        if (w < df_ref) df_ref = w;
        if (natf[m] > max_ref) max_ref = natf[m];
    }
    df_ref = df_ref / 5.0;
    int l_df_big = df > df_ref;
    int nf1 = nfreqs - 1;
    if (test_mode == 0) {
        double max_freq = df * nf1;
        if (max_freq < max_ref) {
            if (l_df_big) {
                max_freq = df_ref * nf1;
                if (max_freq < max_ref) nf1 = (int)ceil(max_ref / df_ref);
                df = df_ref;
            } else {
                nf1 = (int)ceil(max_ref / df);
            }
        }
    }
    int nf, n0;
    if (scaling == 1) {
        nf = nf1 * 2 + 1;
        if (nf % 2 == 0) return -2;
        n0 = -nf1;
    } else {
        if (nf1 % 2 != 0) nf1 += 1;
        nf = nf1 + 1;
        n0 = 0;
    }
    if (nf > cap) return -1;
    for (int i = n0; i <= nf1; ++i) f_out[i - n0] = (double)i;
    for (int i = 0; i < nf; ++i) f_out[i] = f_out[i] * df;
    *df_out = df;
    return nf;
}

static inline double ipow(double c, double e) { return pow(c, e); }

/*
 * getFM_full_tnm_vect_cls_ (src/bsa/functions/functionsImpl.F90:1312-1587): Classic
 * vectorised BFM.  Loop order tc -> k -> j -> i (nodes) -> f2 column (OpenMP, as the
 * reference's `parallel do` over ifrj) -> modes k, j, i -> vector over f1.
 * Suvw(nf, nnl*ntc); psd(nf, nm^2); bisp(nf, nf, nm^3) with f1 fastest.
 * The padded S(f1+f2) arrays are zero-initialised (the reference leaves the padding
 * uninitialised, functionsImpl.F90:1409-1413): |f1+f2| beyond the grid reads 0.
 * bisp may be NULL when compute_bisp == 0.  nthreads <= 0 uses the OpenMP default.
 */
void orc_cls_vect_bfm(const orc_problem *P, int nf, const double *f, const double *Suvw,
                      int compute_bisp, double *psd, double *bisp, int nthreads)
{
    const int nnl = P->nnl, nme = P->nm_eff, nd = P->ndegw3;
    const size_t nm2 = (size_t)nme * nme, nm3 = nm2 * nme;
    const int n_pad = (nf - 1) / 2;
    const int pad_len = (nf - 1) + nf;
    const int iin = n_pad; /* 0-based start of the centre */

    double *fabs_ = malloc(sizeof(double) * nf);
    double *SJK = malloc(sizeof(double) * nf);
    double *SIK = malloc(sizeof(double) * nf);
    double *SIJ = malloc(sizeof(double) * nf);
    double *SIKp = calloc((size_t)pad_len, sizeof(double));
    double *SIJp = calloc((size_t)pad_len, sizeof(double));
    for (int k = 0; k < nf; ++k) fabs_[k] = fabs(f[k]);
    for (size_t x = 0; x < (size_t)nf * nm2; ++x) psd[x] = 0.0;
    if (compute_bisp)
        for (size_t x = 0; x < (size_t)nf * nf * nm3; ++x) bisp[x] = 0.0;
#ifdef _OPENMP
    int nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#endif

    for (int itc = 0; itc < P->ntc; ++itc) {
        const int tc = P->tc[itc];
        const int tcl = tc - 1, tcq = tc + 2; /* 0-based coeff index: linear, quadratic */
        const int posN = itc * nnl;
        for (int ink = 0; ink < nnl; ++ink) {
            const int nk = P->n_load[ink];
            const double *Sk = Suvw + (size_t)nf * (posN + ink);
            for (int inj = 0; inj < nnl; ++inj) {
                const int nj = P->n_load[inj];
                const double *Sj = Suvw + (size_t)nf * (posN + inj);
                const double cJK = corr_of(P, nj, nk, tc);
                for (int k = 0; k < nf; ++k) SJK[k] = ipow(cJK, fabs_[k]) * sqrt(Sk[k] * Sj[k]);

                if (compute_bisp) {
                    for (int ini = 0; ini < nnl; ++ini) {
                        const int ni = P->n_load[ini];
                        const double *Si = Suvw + (size_t)nf * (posN + ini);
                        const double cIK = corr_of(P, ni, nk, tc);
                        const double cIJ = corr_of(P, ni, nj, tc);
                        for (int k = 0; k < nf; ++k) {
                            SIK[k] = ipow(cIK, fabs_[k]) * sqrt(Si[k] * Sk[k]);
                            SIKp[iin + k] = SIK[k];
                            SIJ[k] = ipow(cIJ, fabs_[k]) * sqrt(Si[k] * Sj[k]);
                            SIJp[iin + k] = SIJ[k];
                        }
#ifdef _OPENMP
#pragma omp parallel for num_threads(nt) schedule(static)
#endif
                        for (int ifrj = 0; ifrj < nf; ++ifrj) {
                            const double sikj = SIK[ifrj], sjkj = SJK[ifrj];
                            const double *sijp = SIJp + ifrj, *sikp = SIKp + ifrj;
                            size_t posm = 0;
                            for (int imk = 0; imk < nme; ++imk) {
                                const double kUb = P->phitc[I3(imk, ink, tcl, nme, nnl)];
                                const double ku = P->phitc[I3(imk, ink, tcq, nme, nnl)];
                                for (int imj = 0; imj < nme; ++imj) {
                                    const double jUb = P->phitc[I3(imj, inj, tcl, nme, nnl)];
                                    const double ju = P->phitc[I3(imj, inj, tcq, nme, nnl)];
                                    for (int imi = 0; imi < nme; ++imi) {
                                        const double iUb = P->phitc[I3(imi, ini, tcl, nme, nnl)];
                                        const double iu = P->phitc[I3(imi, ini, tcq, nme, nnl)];
                                        const double c1 = iu * jUb * kUb;
                                        const double c2 = iUb * ju * kUb;
                                        const double c3 = iUb * jUb * ku;
                                        double *b = bisp + (size_t)nf * ((size_t)ifrj + (size_t)nf * posm);
                                        for (int k = 0; k < nf; ++k) {
                                            const double t1 = SIJ[k] * sikj;
                                            const double t2 = sijp[k] * sjkj;
                                            const double t3 = SJK[k] * sikp[k];
                                            b[k] = b[k] + 2.0 * ((c1 * t1) + (c2 * t2) + (c3 * t3));
                                        }
                                        ++posm;
                                    }
                                }
                            }
                        }
                    }
                }
                /* force PSD: psd(:, posm) += phik(imk,1)*phij(imj,1)*S_JK, posm = imj + (imk-1)*nm */
                size_t posm = 0;
                for (int imk = 0; imk < nme; ++imk) {
                    const double kUb = P->phitc[I3(imk, ink, tcl, nme, nnl)];
                    for (int imj = 0; imj < nme; ++imj) {
                        const double jUb = P->phitc[I3(imj, inj, tcl, nme, nnl)];
                        double *p = psd + (size_t)nf * posm;
                        for (int k = 0; k < nf; ++k) p[k] = p[k] + (kUb * jUb * SJK[k]);
                        ++posm;
                    }
                }
            }
        }
    }
    (void)nd;
    free(fabs_); free(SJK); free(SIK); free(SIJ); free(SIKp); free(SIJp);
}

/* Frequency-response tables: H(w) = 1 / (K - w^2 M + i w C), stored as (Hr, Hi). */
static inline void frf(const orc_problem *P, int im, double w, double *hr, double *hi)
{
    const int m = P->modes[im] - 1;
    const double r = -(w * w * P->Mm[m]) + P->Km[m];
    const double ip = P->Cm[I2(m, m, P->nm)] * w;
    const double h = r * r + ip * ip;
    *hr = r / h;
    *hi = -ip / h;
}

/*
 * getRM_full_vect_cls_ (functionsImpl.F90:1598-1738), in place on psd(nf, nm^2) and
 * bisp(nf, nf, nm^3):  psd(:, j+(k-1)nm) *= Re[H_k conj(H_j)],
 * bisp(:, :, i+(j-1)nm+(k-1)nm^2) *= Re[H_i(w1) H_j(w2) conj(H_k(w1+w2))].
 * The reference's posm counters carry implicit SAVE (a second call in one process
 * mis-indexes); this restatement indexes from 1 on every call, i.e. a first call.
 */
void orc_cls_vect_brm(const orc_problem *P, int nf, const double *f, int compute_bisp,
                      double *psd, double *bisp)
{
    const int nme = P->nm_eff;
    double *Hr = malloc(sizeof(double) * nf * nme), *Hi = malloc(sizeof(double) * nf * nme);
    for (int im = 0; im < nme; ++im)
        for (int k = 0; k < nf; ++k) frf(P, im, f[k] * PIt2, &Hr[I2(k, im, nf)], &Hi[I2(k, im, nf)]);
    size_t pp = 0, pb = 0;
    for (int imk = 0; imk < nme; ++imk) {
        for (int imj = 0; imj < nme; ++imj) {
            double *p = psd + (size_t)nf * pp;
            for (int k = 0; k < nf; ++k)
                p[k] = p[k] * (Hr[I2(k, imk, nf)] * Hr[I2(k, imj, nf)] + Hi[I2(k, imk, nf)] * Hi[I2(k, imj, nf)]);
            if (compute_bisp) {
                for (int imi = 0; imi < nme; ++imi) {
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
                    for (int j = 0; j < nf; ++j) {
                        double *b = bisp + (size_t)nf * ((size_t)j + (size_t)nf * pb);
                        const double wj = f[j] * PIt2;
                        for (int i = 0; i < nf; ++i) {
                            double h12r, h12i;
                            frf(P, imk, f[i] * PIt2 + wj, &h12r, &h12i);
                            b[i] = b[i] * (Hr[I2(i, imi, nf)] * Hr[I2(j, imj, nf)] * h12r +
                                           Hr[I2(i, imi, nf)] * Hi[I2(j, imj, nf)] * h12i +
                                           Hi[I2(i, imi, nf)] * Hr[I2(j, imj, nf)] * h12i -
                                           Hi[I2(i, imi, nf)] * Hi[I2(j, imj, nf)] * h12r);
                        }
                    }
                    ++pb;
                }
            }
            ++pp;
        }
    }
    free(Hr); free(Hi);
}

/*
 * intgSpectraVect_ (src/bsa/classic/BsaClassicImpl.F90:567-633).  m2: trapezoid over f;
 * m3: full sum * d^2 minus d^2/2 on the four borders and 3/2 d^2 on the four vertices
 * (net vertex weight -d^2/2).  d = df * 2pi under scaling 1.  psd/bisp may be NULL.
 */
void orc_intg_vect(int nf, const double *f, int scaling, int dim2, const double *psd, double *m2,
                   int dim3, const double *bisp, double *m3)
{
    double delta = f[1] - f[0];
    if (scaling == 1) delta = delta * PIt2;
    const double d_2 = delta / 2.0;
    if (psd && m2) {
        for (int c = 0; c < dim2; ++c) {
            const double *p = psd + (size_t)nf * c;
            double s = 0.0;
            for (int k = 0; k < nf; ++k) s += p[k];
            m2[c] = s * delta;
            m2[c] = m2[c] - ((p[0] + p[nf - 1]) * d_2);
        }
    }
    if (bisp && m3) {
        const double d2 = delta * delta, rt = 1.5 * d2, d2_2 = d2 / 2.0;
        const int nf_1 = nf - 1;
        for (int c = 0; c < dim3; ++c) {
            const double *b = bisp + (size_t)nf * nf * c;
#define B_(i, j) b[(size_t)(i) + (size_t)nf * (j)]
            double s = 0.0;
            for (int j = 0; j < nf; ++j) {
                double cs = 0.0;
                for (int i = 0; i < nf; ++i) cs += B_(i, j);
                s += cs;
            }
            double v = s * d2;
            v = v - B_(0, 0) * rt;
            double side = 0.0;
            for (int i = 1; i < nf_1; ++i) side += B_(i, 0) * d2_2;
            v = v - side;
            v = v - B_(nf - 1, 0) * rt;
            for (int i = 1; i < nf_1; ++i) {
                v = v - B_(0, i) * d2_2;
                v = v - B_(nf - 1, i) * d2_2;
            }
            v = v - B_(0, nf - 1) * rt;
            side = 0.0;
            for (int i = 1; i < nf_1; ++i) side += B_(i, nf - 1) * d2_2;
            v = v - side;
            v = v - B_(nf - 1, nf - 1) * rt;
            m3[c] = v;
#undef B_
        }
    }
}

/*
 * Classic driver, vectorised branch (BsaClassicImpl.F90:39-376 with 141-213): nodal PSD
 * table, BFM, integration, BRM, integration, omega^2-weighted response PSD.
 * Outputs m2mf/m2mr/m2o2mr (nm^2) and m3mf/m3mr (nm^3); any may be NULL.
 * Optionally returns the force and response bispectra (nf, nf, nm^3) when bf/br != NULL.
 */
int orc_classic_vect(const orc_problem *P, int nf, const double *f, double *m2mf, double *m2mr,
                     double *m2o2mr, double *m3mf, double *m3mr, double *bf, double *br, int nthreads)
{
    const int nnl = P->nnl, nme = P->nm_eff;
    const size_t nm2 = (size_t)nme * nme, nm3 = nm2 * nme;
    double *S = malloc(sizeof(double) * (size_t)nf * nnl * P->ntc);
    for (int itc = 0; itc < P->ntc; ++itc)
        if (orc_eval_psd(P, nf, f, P->tc[itc], S + (size_t)nf * nnl * itc)) { free(S); return -1; }
    double *psd = malloc(sizeof(double) * (size_t)nf * nm2);
    double *bisp = malloc(sizeof(double) * (size_t)nf * nf * nm3);
    if (!psd || !bisp) { free(S); free(psd); free(bisp); return -3; }
    orc_cls_vect_bfm(P, nf, f, S, 1, psd, bisp, nthreads);
    orc_intg_vect(nf, f, P->scaling, (int)nm2, m2mf ? psd : NULL, m2mf, (int)nm3, m3mf ? bisp : NULL, m3mf);
    if (bf) memcpy(bf, bisp, sizeof(double) * (size_t)nf * nf * nm3);
    orc_cls_vect_brm(P, nf, f, 1, psd, bisp);
    orc_intg_vect(nf, f, P->scaling, (int)nm2, m2mr ? psd : NULL, m2mr, (int)nm3, m3mr ? bisp : NULL, m3mr);
    if (br) memcpy(br, bisp, sizeof(double) * (size_t)nf * nf * nm3);
    if (m2o2mr) {
        for (size_t c = 0; c < nm2; ++c)
            for (int k = 0; k < nf; ++k) {
                const double w = f[k] * PIt2;
                psd[k + (size_t)nf * c] = psd[k + (size_t)nf * c] * w * w;
            }
        orc_intg_vect(nf, f, P->scaling, (int)nm2, psd, m2o2mr, 0, NULL, NULL);
    }
    free(S); free(psd); free(bisp);
    return 0;
}

/*
 * getFM_full_tnm_scalar_cls_ (functionsImpl.F90:2122-2318) for one grid pair (ii, ij),
 * 0-based.  Suvw(nf, nnl*ntc); Suvw_pad(nnl*ntc) is the padded S at f1+f2 (zero beyond
 * the grid).  psd(nm^2) is filled only when ij == 0, as in the reference.
 * k_lo/k_hi bound the outer k-node loop (0, nnl for the full routine); the benchmark's
 * CPU leg times a slice of it.
 */
void orc_cls_scalar_pair(const orc_problem *P, int nf, int ii, int ij, double fi, double fj,
                         const double *Suvw, const double *Suvw_pad, int compute_bisp,
                         double *psd, double *bisp, int k_lo, int k_hi)
{
    const int nnl = P->nnl, nme = P->nm_eff;
    const size_t nm2 = (size_t)nme * nme, nm3 = nm2 * nme;
    for (size_t x = 0; x < nm2; ++x) psd[x] = 0.0;
    if (compute_bisp) for (size_t x = 0; x < nm3; ++x) bisp[x] = 0.0;
    const double fia = fabs(fi), fja = fabs(fj), fija = fabs(fi + fj);
    for (int itc = 0; itc < P->ntc; ++itc) {
        const int posN = itc * nnl, tc = P->tc[itc];
        const int tcl = tc - 1, tcq = tc + 2;
        for (int ink = k_lo; ink < k_hi; ++ink) {
            const int nk = P->n_load[ink], pk = posN + ink;
            const double Ski = Suvw[I2(ii, pk, nf)], Skj = Suvw[I2(ij, pk, nf)], Skij = Suvw_pad[pk];
            for (int inj = 0; inj < nnl; ++inj) {
                const int nj = P->n_load[inj], pj = posN + inj;
                const double cJK = corr_of(P, nj, nk, tc);
                const double Sji = Suvw[I2(ii, pj, nf)], Sjj = Suvw[I2(ij, pj, nf)], Sjij = Suvw_pad[pj];
                const double SJKi = pow(cJK, fia) * sqrt(Sji * Ski);
                const double SJKj = pow(cJK, fja) * sqrt(Sjj * Skj);
                if (compute_bisp) {
                    for (int ini = 0; ini < nnl; ++ini) {
                        const int ni = P->n_load[ini], pi_ = posN + ini;
                        const double cIK = corr_of(P, ni, nk, tc), cIJ = corr_of(P, ni, nj, tc);
                        const double Sii = Suvw[I2(ii, pi_, nf)], Sij = Suvw[I2(ij, pi_, nf)], Siij = Suvw_pad[pi_];
                        const double SIKj = pow(cIK, fja) * sqrt(Sij * Skj);
                        const double SIKij = pow(cIK, fija) * sqrt(Siij * Skij);
                        const double SIJi = pow(cIJ, fia) * sqrt(Sii * Sji);
                        const double SIJij = pow(cIJ, fija) * sqrt(Siij * Sjij);
                        const double t1 = SIJi * SIKj, t2 = SIJij * SJKj, t3 = SJKi * SIKij;
                        size_t posm = 0;
                        for (int imk = 0; imk < nme; ++imk) {
                            const double kUb = P->phitc[I3(imk, ink, tcl, nme, nnl)];
                            const double ku = P->phitc[I3(imk, ink, tcq, nme, nnl)];
                            for (int imj = 0; imj < nme; ++imj) {
                                const double jUb = P->phitc[I3(imj, inj, tcl, nme, nnl)];
                                const double ju = P->phitc[I3(imj, inj, tcq, nme, nnl)];
                                for (int imi = 0; imi < nme; ++imi) {
                                    const double iUb = P->phitc[I3(imi, ini, tcl, nme, nnl)];
                                    const double iu = P->phitc[I3(imi, ini, tcq, nme, nnl)];
                                    bisp[posm] = bisp[posm] + 2.0 * ((iu * jUb * kUb * t1) + (iUb * ju * kUb * t2) +
                                                                     (iUb * jUb * ku * t3));
                                    ++posm;
                                }
                            }
                        }
                    }
                }
                if (ij == 0) {
                    size_t posm = 0;
                    for (int imk = 0; imk < nme; ++imk) {
                        const double kUb = P->phitc[I3(imk, ink, tcl, nme, nnl)];
                        for (int imj = 0; imj < nme; ++imj) {
                            psd[posm] = psd[posm] + (kUb * P->phitc[I3(imj, inj, tcl, nme, nnl)] * SJKi);
                            ++posm;
                        }
                    }
                }
            }
        }
    }
}

/*
 * getRM_full_scalar_cls_ (functionsImpl.F90:2329-2442): response PSD (only when ij == 0)
 * and response bispectrum at one pair.
 */
void orc_cls_scalar_brm(const orc_problem *P, int ij, double fi, double fj, const double *psdin,
                        double *psdout, const double *bispin, double *bispout, int compute_bisp)
{
    const int nme = P->nm_eff;
    double H1r[256], H1i[256], H2r[256], H2i[256], H3r[256], H3i[256];
    const double wi = fi * PIt2, wj = fj * PIt2;
    for (int m = 0; m < nme; ++m) {
        frf(P, m, wi, &H1r[m], &H1i[m]);
        frf(P, m, wj, &H2r[m], &H2i[m]);
        frf(P, m, wi + wj, &H3r[m], &H3i[m]);
    }
    if (ij == 0) {
        size_t posm = 0;
        for (int k = 0; k < nme; ++k)
            for (int j = 0; j < nme; ++j) {
                psdout[posm] = psdin[posm] * (H1r[j] * H1r[k] + H1i[j] * H1i[k]);
                ++posm;
            }
        if (!compute_bisp) return;
    }
    size_t posm = 0;
    for (int k = 0; k < nme; ++k)
        for (int j = 0; j < nme; ++j) {
            const double t1 = H2r[j] * H3r[k], t2 = H2i[j] * H3i[k], t3 = H2r[j] * H3i[k], t4 = H2i[j] * H3r[k];
            for (int i = 0; i < nme; ++i) {
                bispout[posm] = bispin[posm] * (H1r[i] * t1 + H1r[i] * t2 + H1i[i] * t3 - H1i[i] * t4);
                ++posm;
            }
        }
}

/*
 * Classic driver, scalar branch (BsaClassicImpl.F90:255-363): every pair with a uniform
 * dw^2 weight (no edge correction), m2 by a rectangle rule dw.
 */
int orc_classic_scalar(const orc_problem *P, int nf, const double *f, double *m2mf, double *m2mr,
                       double *m2o2mr, double *m3mf, double *m3mr)
{
    const int nnl = P->nnl, nme = P->nm_eff, npsd = nnl * P->ntc;
    const size_t nm2 = (size_t)nme * nme, nm3 = nm2 * nme;
    if (nme > 256) return -1;
    double *S = malloc(sizeof(double) * (size_t)nf * npsd);
    for (int itc = 0; itc < P->ntc; ++itc)
        if (orc_eval_psd(P, nf, f, P->tc[itc], S + (size_t)nf * nnl * itc)) { free(S); return -1; }
    const int lp = (nf - 1) / 2, lpad = 2 * lp + nf;
    double *Spad = calloc((size_t)npsd * lpad, sizeof(double)); /* (npsd, lpad) */
    for (int c = 0; c < npsd; ++c)
        for (int k = 0; k < nf; ++k) Spad[I2(c, lp + k, npsd)] = S[I2(k, c, nf)];
    const double dw = (f[1] - f[0]) * PIt2, dw2 = dw * dw;
    for (size_t x = 0; x < nm2; ++x) { m2mf[x] = 0; m2mr[x] = 0; m2o2mr[x] = 0; }
    for (size_t x = 0; x < nm3; ++x) { m3mf[x] = 0; m3mr[x] = 0; }
    double *psdfm = calloc(nm2, sizeof(double)), *psdrm = calloc(nm2, sizeof(double));
    for (int ifr = 0; ifr < nf; ++ifr) {
        const double fi = f[ifr], omg = fi * PIt2;
#ifdef _OPENMP
#pragma omp parallel
#endif
        {
            double *bf = malloc(sizeof(double) * nm3), *br = malloc(sizeof(double) * nm3);
            double *pf = malloc(sizeof(double) * nm2), *pr = malloc(sizeof(double) * nm2);
#ifdef _OPENMP
#pragma omp for ordered schedule(static, 1)
#endif
            for (int jfr = 0; jfr < nf; ++jfr) {
                const double fj = f[jfr];
                orc_cls_scalar_pair(P, nf, ifr, jfr, fi, fj, S, Spad + (size_t)npsd * (ifr + jfr), 1, pf, bf, 0, nnl);
                orc_cls_scalar_brm(P, jfr, fi, fj, pf, pr, bf, br, 1);
#ifdef _OPENMP
#pragma omp ordered
#endif
                {
                    for (size_t x = 0; x < nm3; ++x) m3mf[x] = m3mf[x] + bf[x] * dw2;
                    for (size_t x = 0; x < nm3; ++x) m3mr[x] = m3mr[x] + br[x] * dw2;
                    if (jfr == 0) { memcpy(psdfm, pf, sizeof(double) * nm2); memcpy(psdrm, pr, sizeof(double) * nm2); }
                }
            }
            free(bf); free(br); free(pf); free(pr);
        }
        for (size_t x = 0; x < nm2; ++x) {
            m2mf[x] = m2mf[x] + psdfm[x] * dw;
            const double r = psdrm[x] * dw;
            m2mr[x] = m2mr[x] + r;
            m2o2mr[x] = m2o2mr[x] + r * omg * omg;
        }
    }
    free(S); free(Spad); free(psdfm); free(psdrm);
    return 0;
}

/*
 * getFM_full_tnm_scalar_msh_ (functionsImpl.F90:247-465): Mesher direct BFM at one point
 * (fi, fj) with analytic S(fi+fj); generic in the number of loaded nodal DOFs.  The
 * reference reads wfc(libs_load(l), ...) (first dimension indexed by the DOF id) and
 * Phi((n-1)*nlibs + libs_load(l), mode); both are kept.  Returns -1 when a DOF id exceeds
 * the first extent of wfc (the reference would read out of bounds there).
 */
int orc_msh_bfm_direct(const orc_problem *P, double fi, double fj, double *bfm)
{
    const int nnl = P->nnl, nme = P->nm_eff, nl = P->nlibsl, nd = P->ndegw3;
    const size_t nm3 = (size_t)nme * nme * nme;
    for (int l = 0; l < nl; ++l)
        if (P->libs_load[l] > nl) return -1;
    for (size_t x = 0; x < nm3; ++x) bfm[x] = 0.0;
    const double fij = fi + fj, afi = fabs(fi), afj = fabs(fj), afij = fabs(fij);
    double *Sfi = malloc(sizeof(double) * nnl), *Sfj = malloc(sizeof(double) * nnl), *Sfij = malloc(sizeof(double) * nnl);
    double BF[16 * 16];
    if (nl > 16) { free(Sfi); free(Sfj); free(Sfij); return -2; }
#define WFC(l, c, in) P->wfc[I3(P->libs_load[l] - 1, (c), (in), nl, nd)]
#define PHI(row, m) P->phi[I2((row)-1, (m)-1, P->ndofs)]
    for (int itc = 0; itc < P->ntc; ++itc) {
        const int tc = P->tc[itc];
        orc_eval_psd(P, 1, &fi, tc, Sfi);
        orc_eval_psd(P, 1, &fj, tc, Sfj);
        orc_eval_psd(P, 1, &fij, tc, Sfij);
        for (int ink = 0; ink < nnl; ++ink) {
            const int nk = P->n_load[ink], posK = (nk - 1) * P->nlibs;
            for (int inj = 0; inj < nnl; ++inj) {
                const int nj = P->n_load[inj], posJ = (nj - 1) * P->nlibs;
                const double cJK = corr_of(P, nj, nk, tc);
                const double SJKfi = pow(cJK, afi) * sqrt(Sfi[inj] * Sfi[ink]);
                const double SJKfj = pow(cJK, afj) * sqrt(Sfj[inj] * Sfj[ink]);
                for (int ini = 0; ini < nnl; ++ini) {
                    const int ni = P->n_load[ini], posI = (ni - 1) * P->nlibs;
                    const double cIJ = corr_of(P, ni, nj, tc), cIK = corr_of(P, ni, nk, tc);
                    double term1 = pow(cIJ, afi) * sqrt(Sfi[ini] * Sfi[inj]);
                    term1 = pow(cIK, afj) * sqrt(Sfj[ini] * Sfj[ink]) * term1;
                    double term2 = pow(cIJ, afij) * sqrt(Sfij[ini] * Sfij[inj]);
                    term2 = SJKfj * term2;
                    double term3 = pow(cIK, afij) * sqrt(Sfij[ini] * Sfij[ink]);
                    term3 = SJKfi * term3;
                    for (int lk = 0; lk < nl; ++lk) {
                        const double akU = WFC(lk, tc - 1, ink), ak = WFC(lk, tc + 2, ink);
                        for (int lj = 0; lj < nl; ++lj)
                            for (int li = 0; li < nl; ++li) {
                                const double tmp1 = WFC(li, tc + 2, ini) * WFC(lj, tc - 1, inj) * term1;
                                const double tmp2 = WFC(li, tc - 1, ini) * WFC(lj, tc + 2, inj) * term2;
                                const double tmp3 = WFC(li, tc - 1, ini) * WFC(lj, tc - 1, inj) * term3;
                                BF[li + 16 * lj] = 2.0 * ((tmp1 * akU) + (tmp2 * akU) + (tmp3 * ak));
                            }
                        size_t posm = 0;
                        for (int imk = 0; imk < nme; ++imk) {
                            const double phiK = PHI(posK + P->libs_load[lk], P->modes[imk]);
                            for (int imj = 0; imj < nme; ++imj)
                                for (int imi = 0; imi < nme; ++imi) {
                                    double s = 0.0;
                                    for (int lj = 0; lj < nl; ++lj)
                                        for (int li = 0; li < nl; ++li)
                                            s += BF[li + 16 * lj] * (PHI(posI + P->libs_load[li], P->modes[imi]) *
                                                                    PHI(posJ + P->libs_load[lj], P->modes[imj]) * phiK);
                                    bfm[posm] = bfm[posm] + s;
                                    ++posm;
                                }
                        }
                    }
                }
            }
        }
    }
#undef WFC
#undef PHI
    free(Sfi); free(Sfj); free(Sfij);
    return 0;
}

/*
 * getRM_full_scalar_msh_ (functionsImpl.F90:1031-1115): BRM on the outer product fi x fj
 * (posf runs with fj fastest).  bfm/brm are (nm^3, nfi*nfj).
 */
void orc_msh_brm(const orc_problem *P, int nfi, const double *fi, int nfj, const double *fj,
                 const double *bfm, double *brm)
{
    const int nme = P->nm_eff;
    const size_t nm3 = (size_t)nme * nme * nme;
    double H1r[256], H1i[256], H2r[256], H2i[256], H3r[256], H3i[256];
    size_t posf = 0;
    for (int i = 0; i < nfi; ++i) {
        const double wi = fi[i] * PIt2;
        for (int j = 0; j < nfj; ++j) {
            const double wj = fj[j] * PIt2;
            for (int m = 0; m < nme && m < 256; ++m) {
                frf(P, m, wi, &H1r[m], &H1i[m]);
                frf(P, m, wj, &H2r[m], &H2i[m]);
                frf(P, m, wi + wj, &H3r[m], &H3i[m]);
            }
            size_t posm = 0;
            for (int k = 0; k < nme; ++k)
                for (int jj = 0; jj < nme; ++jj)
                    for (int ii = 0; ii < nme; ++ii) {
                        brm[posm + nm3 * posf] = bfm[posm + nm3 * posf] *
                            (H1r[ii] * H2r[jj] * H3r[k] + H1r[ii] * H2i[jj] * H3i[k] +
                             H1i[ii] * H2r[jj] * H3i[k] - H1i[ii] * H2i[jj] * H3r[k]);
                        ++posm;
                    }
            ++posf;
        }
    }
}

/* computeSkewness_ (src/bsa/BsaLibImpl.F90:1630-1707), full (non-diagonal) branch. */
void orc_skewness(int dim, const double *m2, const double *m3, double *sk)
{
    size_t pm3 = 0;
    int ik = 0;
    for (int k = 1; k <= dim; ++k) {
        const double denK = sqrt(m2[ik]);
        int ij = 0;
        for (int j = 1; j <= dim; ++j) {
            const double denJ = denK * sqrt(m2[ij]);
            int ii = 0;
            for (int i = 1; i <= dim; ++i) {
                sk[pm3] = m3[pm3] / (denJ * sqrt(m2[ii]));
                ++pm3;
                ii = i * dim + i;
            }
            ij = j * dim + j;
        }
        ik = k * dim + k;
    }
}

/*
 * modalRecombination, CCC branch (app/bsa.F90:935-1053): nodal m2, m3 and skewness from
 * modal moments.  phi(ndofs, nmodes).
 */
void orc_modal_recomb(int ndofs, int nmodes, const double *phi, const double *m2mr,
                      const double *m3mr, double *m2_r, double *m3_r, double *sk_r)
{
    for (int d = 0; d < ndofs; ++d) { m2_r[d] = 0; m3_r[d] = 0; }
    for (int k = 0; k < nmodes; ++k)
        for (int j = 0; j < nmodes; ++j) {
            const size_t p2 = (size_t)k * nmodes + j;
            for (int d = 0; d < ndofs; ++d)
                m2_r[d] = m2_r[d] + m2mr[p2] * phi[I2(d, j, ndofs)] * phi[I2(d, k, ndofs)];
            for (int i = 0; i < nmodes; ++i) {
                const size_t p3 = ((size_t)k * nmodes + j) * nmodes + i;
                for (int d = 0; d < ndofs; ++d)
                    m3_r[d] = m3_r[d] + m3mr[p3] * phi[I2(d, i, ndofs)] * phi[I2(d, j, ndofs)] * phi[I2(d, k, ndofs)];
            }
        }
    for (int d = 0; d < ndofs; ++d) sk_r[d] = m3_r[d] / pow(m2_r[d], 1.5);
}

/*
 * modalRecombination, both branches (app/bsa.F90:935-1053), in the routine's loop order:
 * out[0..5][ndofs] = m2 diag, m3 diag, m2o2 diag, m2 CCC, m3 CCC, m2o2 CCC; sk[0..1][ndofs] =
 * diag and CCC skewness m3 / m2^(3/2).  is_diag: the spectra have one entry per mode (then the
 * CCC rows are not formed).  m2o2mr may be NULL (its rows stay zero).  phi(ndofs, nmodes).
 */
void orc_modal_recomb_all(int ndofs, int nmodes, int is_diag, const double *phi, const double *m2mr,
                          const double *m3mr, const double *m2o2mr, double *out, double *sk)
{
    for (int r = 0; r < 6 * ndofs; ++r) out[r] = 0.0;
    double *m2d = out, *m3d = out + ndofs, *mod = out + 2 * ndofs;
    double *m2f = out + 3 * ndofs, *m3f = out + 4 * ndofs, *mof = out + 5 * ndofs;
    for (int im = 0; im < nmodes; ++im) {
        size_t p2, p3;
        if (is_diag) {
            p2 = (size_t)im;
            p3 = (size_t)im;
        } else {
            const size_t t = (size_t)im * nmodes;
            p2 = t + im;
            p3 = t * nmodes + p2;
        }
        for (int d = 0; d < ndofs; ++d) {
            const double p1 = phi[I2(d, im, ndofs)];
            double r = p1 * p1;
            m2d[d] = m2d[d] + m2mr[p2] * r;
            if (m2o2mr) mod[d] = mod[d] + m2o2mr[p2] * r;
            r = r * p1;
            m3d[d] = m3d[d] + m3mr[p3] * r;
        }
    }
    for (int d = 0; d < ndofs; ++d) sk[d] = m3d[d] / pow(m2d[d], 1.5);
    if (is_diag) return;
    for (int k = 0; k < nmodes; ++k) {
        const size_t t12 = (size_t)k * nmodes, t13 = t12 * nmodes;
        for (int j = 0; j < nmodes; ++j) {
            const size_t t23 = (size_t)j * nmodes, p2 = t12 + j;
            for (int d = 0; d < ndofs; ++d) {
                m2f[d] = m2f[d] + m2mr[p2] * phi[I2(d, j, ndofs)] * phi[I2(d, k, ndofs)];
                if (m2o2mr) mof[d] = mof[d] + m2o2mr[p2] * phi[I2(d, j, ndofs)] * phi[I2(d, k, ndofs)];
            }
            for (int i = 0; i < nmodes; ++i) {
                const size_t p3 = t13 + t23 + i;
                for (int d = 0; d < ndofs; ++d)
                    m3f[d] = m3f[d] + m3mr[p3] * phi[I2(d, i, ndofs)] * phi[I2(d, j, ndofs)] * phi[I2(d, k, ndofs)];
            }
        }
    }
    for (int d = 0; d < ndofs; ++d) sk[ndofs + d] = m3f[d] / pow(m2f[d], 1.5);
}

int orc_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/*
 * One rectangular Mesher zone, post-mesh (compute_rz_ and interpolateRZ_HTPC_v3,
 * src/bsa/meshing/zones/_shared_poly2d.fi:40-454 and 470-2166, with the BFM multi-level
 * refinement off): the direct BFM (getFM_full_tnm_scalar_msh_) on the ni x nj lattice
 * (f1, f2) = (fi0, fj0) + i (dIi, dIj) + j (dJi, dJj); the BFM integral with the lattice's
 * trapezoid weights (vertex dwI dwJ / 4, border / 2, centre 1); the BRM lattice refined by
 * (Fi, Fj), the BFM interpolated linearly along J then along I between lattice points, the
 * BRM (getRM_full_scalar_msh_) at every BRM point and its trapezoid weights with
 * (dwI / Fi)(dwJ / Fj).  Both integrals times sym are added to m3mf / m3mr (nm^3).
 */
int orc_msh_bfm_diag(const orc_problem *P, double fi, double fj, double *bfm);
void orc_msh_brm_diag(const orc_problem *P, int nfi, const double *fi, int nfj, const double *fj,
                      const double *bfm, double *brm);

static int rect_zone_impl(const orc_problem *P, double fi0, double fj0, double dIi, double dIj, double dJi,
                          double dJj, int ni, int nj, int Fi, int Fj, double sym, int diag, double *m3mf,
                          double *m3mr)
{
    const int nme = P->nm_eff;
    /* per-point tensor length: nm^3, or nm for the diagonal-only spectra */
    const size_t nm3 = diag ? (size_t)nme : (size_t)nme * nme * nme;
    if (ni < 2 || nj < 2 || Fi < 1 || Fj < 1 || nme > 256) return -1;
    double *bfm = malloc(sizeof(double) * nm3 * (size_t)ni * nj);
    double *tmp = malloc(sizeof(double) * nm3), *brm = malloc(sizeof(double) * nm3);
    if (!bfm || !tmp || !brm) { free(bfm); free(tmp); free(brm); return -3; }
    for (int i = 0; i < ni; ++i)
        for (int j = 0; j < nj; ++j) {
            const double f1 = fi0 + i * dIi + j * dJi, f2 = fj0 + i * dIj + j * dJj;
            int rc = diag ? orc_msh_bfm_diag(P, f1, f2, bfm + nm3 * ((size_t)i * nj + j))
                          : orc_msh_bfm_direct(P, f1, f2, bfm + nm3 * ((size_t)i * nj + j));
            if (rc) { free(bfm); free(tmp); free(brm); return rc; }
        }
    const double dwI = sqrt(dIi * dIi + dIj * dIj) * PIt2, dwJ = sqrt(dJi * dJi + dJj * dJj) * PIt2;
    for (int i = 0; i < ni; ++i)
        for (int j = 0; j < nj; ++j) {
            const double w = sym * dwI * dwJ * ((i == 0 || i == ni - 1) ? 0.5 : 1.0) * ((j == 0 || j == nj - 1) ? 0.5 : 1.0);
            const double *b = bfm + nm3 * ((size_t)i * nj + j);
            for (size_t x = 0; x < nm3; ++x) m3mf[x] += w * b[x];
        }
    const int NI = (ni - 1) * Fi, NJ = (nj - 1) * Fj;
    for (int qi = 0; qi <= NI; ++qi)
        for (int qj = 0; qj <= NJ; ++qj) {
            const int i0 = qi / Fi < ni - 1 ? qi / Fi : ni - 2, j0 = qj / Fj < nj - 1 ? qj / Fj : nj - 2;
            const double ti = (double)(qi - i0 * Fi) / Fi, tj = (double)(qj - j0 * Fj) / Fj;
            const double *b00 = bfm + nm3 * ((size_t)i0 * nj + j0), *b01 = bfm + nm3 * ((size_t)i0 * nj + j0 + 1);
            const double *b10 = bfm + nm3 * ((size_t)(i0 + 1) * nj + j0), *b11 = bfm + nm3 * ((size_t)(i0 + 1) * nj + j0 + 1);
            for (size_t x = 0; x < nm3; ++x) {
                const double left = b00[x] * (1.0 - tj) + b01[x] * tj;     /* along J, column i0   */
                const double right = b10[x] * (1.0 - tj) + b11[x] * tj;    /* along J, column i0+1 */
                tmp[x] = left * (1.0 - ti) + right * ti;                    /* along I              */
            }
            const double a = (double)qi / Fi, bq = (double)qj / Fj;
            const double f1 = fi0 + a * dIi + bq * dJi, f2 = fj0 + a * dIj + bq * dJj;
            if (diag)
                orc_msh_brm_diag(P, 1, &f1, 1, &f2, tmp, brm);
            else
                orc_msh_brm(P, 1, &f1, 1, &f2, tmp, brm);
            const double w = sym * (dwI / Fi) * (dwJ / Fj) * ((qi == 0 || qi == NI) ? 0.5 : 1.0) *
                             ((qj == 0 || qj == NJ) ? 0.5 : 1.0);
            for (size_t x = 0; x < nm3; ++x) m3mr[x] += w * brm[x];
        }
    free(bfm); free(tmp); free(brm);
    return 0;
}

int orc_rect_zone(const orc_problem *P, double fi0, double fj0, double dIi, double dIj, double dJi, double dJj,
                  int ni, int nj, int Fi, int Fj, double sym, double *m3mf, double *m3mr)
{
    return rect_zone_impl(P, fi0, fj0, dIi, dIj, dJi, dJj, ni, nj, Fi, Fj, sym, 0, m3mf, m3mr);
}

/* The same zone with the diagonal-only Mesher functions (m3mf / m3mr of length nm). */
int orc_rect_zone_diag(const orc_problem *P, double fi0, double fj0, double dIi, double dIj, double dJi,
                       double dJj, int ni, int nj, int Fi, int Fj, double sym, double *m3mf, double *m3mr)
{
    return rect_zone_impl(P, fi0, fj0, dIi, dIj, dJi, dJj, ni, nj, Fi, Fj, sym, 1, m3mf, m3mr);
}

/* ======================================================================================
 * Diagonal-only spectra (settings i_only_diag_ = 1, bound at src/bsa/BsaLibImpl.F90:313-336):
 * same-node, same-mode tensors, dimM_psd_ = dimM_bisp_ = nm.  These follow the reference's
 * loops over the loaded-DOF triple with the raw force coefficients and modal matrix.
 * ====================================================================================== */
#define WFCR(l, c, in) P->wfc[I3(P->libs_load[l] - 1, (c), (in), P->nlibsl, P->ndegw3)]
#define PHIR(row, m) P->phi[I2((row)-1, (m)-1, P->ndofs)]

/*
 * getFM_diag_tnlm_vect_cls_ (functionsImpl.F90:1747-1968).  Per (tc, node): the padded
 * S(f1+f2) (zero beyond the grid), tmp1 = S(f1+f2) S(f2), tmp2 = S(f1+f2) S(f1),
 * tmp3 = S(f1) S(f2); BF = 2 (q_i l_j l_k tmp3 + l_i q_j l_k tmp1 + l_i l_j q_k tmp2) over
 * the DOF triple (k, j, i), times phi_k phi_j phi_i of each kept mode.
 * psd(nf, nm) += phi_j phi_k l_j l_k S(f); bisp(nf, nf, nm) with f1 fastest.
 */
int orc_cls_vect_bfm_diag(const orc_problem *P, int nf, const double *f, const double *Suvw, int compute_bisp,
                          double *psd, double *bisp)
{
    const int nnl = P->nnl, nme = P->nm_eff, nl = P->nlibsl;
    const int n_pad = (nf - 1) / 2, pad_len = (nf - 1) + nf;
    (void)f;
    double *Spad = calloc((size_t)pad_len, sizeof(double));
    double *t1 = malloc(sizeof(double) * (size_t)nf * nf), *t2 = malloc(sizeof(double) * (size_t)nf * nf);
    double *t3 = malloc(sizeof(double) * (size_t)nf * nf);
    if (!Spad || !t1 || !t2 || !t3) { free(Spad); free(t1); free(t2); free(t3); return -3; }
    for (size_t x = 0; x < (size_t)nf * nme; ++x) psd[x] = 0.0;
    if (compute_bisp)
        for (size_t x = 0; x < (size_t)nf * nf * nme; ++x) bisp[x] = 0.0;
    for (int itc = 0; itc < P->ntc; ++itc) {
        const int tc = P->tc[itc], tcl = tc - 1, tcq = tc + 2;
        for (int in = 0; in < nnl; ++in) {
            const int posN = (P->n_load[in] - 1) * P->nlibs;
            const double *S = Suvw + (size_t)nf * ((size_t)itc * nnl + in);
            if (compute_bisp) {
                for (int k = 0; k < nf; ++k) Spad[n_pad + k] = S[k];
                for (int j = 0; j < nf; ++j)
                    for (int i = 0; i < nf; ++i) {
                        const double s12 = Spad[i + j];
                        t1[I2(i, j, nf)] = s12 * S[j];
                        t2[I2(i, j, nf)] = s12 * S[i];
                        t3[I2(i, j, nf)] = S[i] * S[j];
                    }
                for (int lk = 0; lk < nl; ++lk) {
                    const int posk = posN + P->libs_load[lk];
                    const double akU = WFCR(lk, tcl, in), ak = WFCR(lk, tcq, in);
                    for (int lj = 0; lj < nl; ++lj) {
                        const int posj = posN + P->libs_load[lj];
                        const double ajU = WFCR(lj, tcl, in), aj = WFCR(lj, tcq, in);
                        for (int li = 0; li < nl; ++li) {
                            const int posi = posN + P->libs_load[li];
                            const double aiU = WFCR(li, tcl, in), ai = WFCR(li, tcq, in);
                            const double c3 = ai * ajU * akU, c1 = aiU * aj * akU, c2 = aiU * ajU * ak;
                            for (int im = 0; im < nme; ++im) {
                                const int m = P->modes[im];
                                const double ph = PHIR(posk, m) * PHIR(posj, m) * PHIR(posi, m);
                                double *b = bisp + (size_t)nf * nf * im;
                                for (size_t x = 0; x < (size_t)nf * nf; ++x) {
                                    const double bf = 2.0 * ((c3 * t3[x]) + (c1 * t1[x]) + (c2 * t2[x]));
                                    b[x] = b[x] + ph * bf;
                                }
                            }
                        }
                    }
                }
            }
            for (int lk = 0; lk < nl; ++lk) {
                const int posk = posN + P->libs_load[lk];
                const double akU = WFCR(lk, tcl, in);
                for (int lj = 0; lj < nl; ++lj) {
                    const int posj = posN + P->libs_load[lj];
                    const double ajU = WFCR(lj, tcl, in);
                    for (int im = 0; im < nme; ++im) {
                        const int m = P->modes[im];
                        const double ph = PHIR(posj, m) * PHIR(posk, m);
                        double *p = psd + (size_t)nf * im;
                        for (int k = 0; k < nf; ++k) p[k] = p[k] + ph * (ajU * akU * S[k]);
                    }
                }
            }
        }
    }
    free(Spad); free(t1); free(t2); free(t3);
    return 0;
}

/*
 * getRM_diag_vect_cls_ (functionsImpl.F90:1974-2101), in place: psd(:, m) *= |H_m|^2,
 * bisp(:, :, m) *= Re[H_m(w1) H_m(w2) conj H_m(w1 + w2)].
 */
void orc_cls_vect_brm_diag(const orc_problem *P, int nf, const double *f, int compute_bisp, double *psd,
                           double *bisp)
{
    const int nme = P->nm_eff;
    double *Hr = malloc(sizeof(double) * nf), *Hi = malloc(sizeof(double) * nf);
    for (int im = 0; im < nme; ++im) {
        for (int k = 0; k < nf; ++k) frf(P, im, f[k] * PIt2, &Hr[k], &Hi[k]);
        double *p = psd + (size_t)nf * im;
        for (int k = 0; k < nf; ++k) p[k] = p[k] * (Hr[k] * Hr[k] + Hi[k] * Hi[k]);
        if (!compute_bisp) continue;
        double *b = bisp + (size_t)nf * nf * im;
        for (int j = 0; j < nf; ++j)
            for (int i = 0; i < nf; ++i) {
                double h12r, h12i;
                frf(P, im, f[i] * PIt2 + f[j] * PIt2, &h12r, &h12i);
                b[I2(i, j, nf)] = b[I2(i, j, nf)] * (Hr[i] * Hr[j] * h12r + Hr[i] * Hi[j] * h12i +
                                                     Hi[i] * Hr[j] * h12i - Hi[i] * Hi[j] * h12r);
            }
    }
    free(Hr); free(Hi);
}

/* Classic driver, vectorised branch, diagonal-only (m2* and m3* of length nm). */
int orc_classic_vect_diag(const orc_problem *P, int nf, const double *f, double *m2mf, double *m2mr,
                          double *m2o2mr, double *m3mf, double *m3mr, double *bf, double *br)
{
    const int nnl = P->nnl, nme = P->nm_eff;
    double *S = malloc(sizeof(double) * (size_t)nf * nnl * P->ntc);
    double *psd = malloc(sizeof(double) * (size_t)nf * nme);
    double *bisp = malloc(sizeof(double) * (size_t)nf * nf * nme);
    if (!S || !psd || !bisp) { free(S); free(psd); free(bisp); return -3; }
    for (int itc = 0; itc < P->ntc; ++itc)
        if (orc_eval_psd(P, nf, f, P->tc[itc], S + (size_t)nf * nnl * itc)) { free(S); free(psd); free(bisp); return -1; }
    int rc = orc_cls_vect_bfm_diag(P, nf, f, S, 1, psd, bisp);
    if (rc) { free(S); free(psd); free(bisp); return rc; }
    orc_intg_vect(nf, f, P->scaling, nme, m2mf ? psd : NULL, m2mf, nme, m3mf ? bisp : NULL, m3mf);
    if (bf) memcpy(bf, bisp, sizeof(double) * (size_t)nf * nf * nme);
    orc_cls_vect_brm_diag(P, nf, f, 1, psd, bisp);
    orc_intg_vect(nf, f, P->scaling, nme, m2mr ? psd : NULL, m2mr, nme, m3mr ? bisp : NULL, m3mr);
    if (br) memcpy(br, bisp, sizeof(double) * (size_t)nf * nf * nme);
    if (m2o2mr) {
        for (int c = 0; c < nme; ++c)
            for (int k = 0; k < nf; ++k) {
                const double w = f[k] * PIt2;
                psd[k + (size_t)nf * c] = psd[k + (size_t)nf * c] * w * w;
            }
        orc_intg_vect(nf, f, P->scaling, nme, psd, m2o2mr, 0, NULL, NULL);
    }
    free(S); free(psd); free(bisp);
    return 0;
}

/*
 * getFM_diag_tnlm_scalar_cls_ (functionsImpl.F90:2460-2560) at one grid pair (ii, ij),
 * 0-based: psd(nm) only when ij == 0; Suvw_pad(nnl*ntc) is S at f1+f2 (zero beyond the grid).
 */
void orc_cls_scalar_pair_diag(const orc_problem *P, int nf, int ii, int ij, const double *Suvw,
                              const double *Suvw_pad, int compute_bisp, double *psd, double *bisp)
{
    const int nnl = P->nnl, nme = P->nm_eff, nl = P->nlibsl;
    for (int m = 0; m < nme; ++m) { psd[m] = 0.0; bisp[m] = 0.0; }
    int iposN = 0;
    for (int itc = 0; itc < P->ntc; ++itc) {
        const int tc = P->tc[itc], tcl = tc - 1, tcq = tc + 2;
        for (int in = 0; in < nnl; ++in, ++iposN) {
            const int posNi = (P->n_load[in] - 1) * P->nlibs;
            const double Si = Suvw[I2(ii, iposN, nf)];
            if (ij == 0) {
                for (int im = 0; im < nme; ++im) {
                    const int m = P->modes[im];
                    double s = 0.0;
                    for (int l2 = 0; l2 < nl; ++l2)
                        for (int l1 = 0; l1 < nl; ++l1) {
                            const double phij = PHIR(posNi + P->libs_load[l1], m) * PHIR(posNi + P->libs_load[l2], m);
                            s += phij * ((WFCR(l1, tcl, in) * WFCR(l2, tcl, in)) * Si);
                        }
                    psd[im] = psd[im] + s;
                }
            }
            if (!compute_bisp) continue;
            const double Sj = Suvw[I2(ij, iposN, nf)], Sij = Suvw_pad[iposN];
            for (int lk = 0; lk < nl; ++lk) {
                const double akU = WFCR(lk, tcl, in), ak = WFCR(lk, tcq, in);
                for (int im = 0; im < nme; ++im) {
                    const int m = P->modes[im];
                    const double phik = PHIR(posNi + P->libs_load[lk], m);
                    double s = 0.0;
                    for (int l2 = 0; l2 < nl; ++l2)
                        for (int l1 = 0; l1 < nl; ++l1) {
                            const double tmp1 = (WFCR(l1, tcq, in) * WFCR(l2, tcl, in)) * (Si * Sj);
                            const double tmp2 = (WFCR(l1, tcl, in) * WFCR(l2, tcq, in)) * (Sij * Sj);
                            const double tmp3 = (WFCR(l1, tcl, in) * WFCR(l2, tcl, in)) * (Sij * Si);
                            const double bf = 2.0 * ((tmp1 * akU) + (tmp2 * akU) + (tmp3 * ak));
                            const double phij = PHIR(posNi + P->libs_load[l1], m) * PHIR(posNi + P->libs_load[l2], m);
                            s += (phij * bf) * phik;
                        }
                    bisp[im] = bisp[im] + s;
                }
            }
        }
    }
}

/* getRM_diag_scalar_cls_ (functionsImpl.F90:2562-2637). */
void orc_cls_scalar_brm_diag(const orc_problem *P, int ij, double fi, double fj, const double *psdin,
                             double *psdout, const double *bispin, double *bispout)
{
    const int nme = P->nm_eff;
    const double wi = fi * PIt2, wj = fj * PIt2;
    for (int m = 0; m < nme; ++m) {
        double h1r, h1i, h2r, h2i, h3r, h3i;
        frf(P, m, wi, &h1r, &h1i);
        frf(P, m, wj, &h2r, &h2i);
        frf(P, m, wi + wj, &h3r, &h3i);
        if (ij == 0) psdout[m] = psdin[m] * (h1r * h1r + h1i * h1i);
        bispout[m] = bispin[m] * (h1r * h2r * h3r + h1r * h2i * h3i + h1i * h2r * h3i - h1i * h2i * h3r);
    }
}

/* Classic driver, scalar branch, diagonal-only (uniform dw^2 weights, rectangle m2). */
int orc_classic_scalar_diag(const orc_problem *P, int nf, const double *f, double *m2mf, double *m2mr,
                            double *m2o2mr, double *m3mf, double *m3mr)
{
    const int nnl = P->nnl, nme = P->nm_eff, npsd = nnl * P->ntc;
    double *S = malloc(sizeof(double) * (size_t)nf * npsd);
    for (int itc = 0; itc < P->ntc; ++itc)
        if (orc_eval_psd(P, nf, f, P->tc[itc], S + (size_t)nf * nnl * itc)) { free(S); return -1; }
    const int lp = (nf - 1) / 2, lpad = 2 * lp + nf;
    double *Spad = calloc((size_t)npsd * lpad, sizeof(double));
    for (int c = 0; c < npsd; ++c)
        for (int k = 0; k < nf; ++k) Spad[I2(c, lp + k, npsd)] = S[I2(k, c, nf)];
    const double dw = (f[1] - f[0]) * PIt2, dw2 = dw * dw;
    double *bf = malloc(sizeof(double) * nme), *br = malloc(sizeof(double) * nme);
    double *pf = malloc(sizeof(double) * nme), *pr = malloc(sizeof(double) * nme);
    double *psdfm = calloc(nme, sizeof(double)), *psdrm = calloc(nme, sizeof(double));
    for (int m = 0; m < nme; ++m) { m2mf[m] = 0; m2mr[m] = 0; m2o2mr[m] = 0; m3mf[m] = 0; m3mr[m] = 0; }
    for (int ifr = 0; ifr < nf; ++ifr) {
        const double fi = f[ifr], omg = fi * PIt2;
        for (int jfr = 0; jfr < nf; ++jfr) {
            orc_cls_scalar_pair_diag(P, nf, ifr, jfr, S, Spad + (size_t)npsd * (ifr + jfr), 1, pf, bf);
            orc_cls_scalar_brm_diag(P, jfr, fi, f[jfr], pf, pr, bf, br);
            for (int m = 0; m < nme; ++m) {
                m3mf[m] = m3mf[m] + bf[m] * dw2;
                m3mr[m] = m3mr[m] + br[m] * dw2;
            }
            if (jfr == 0) { memcpy(psdfm, pf, sizeof(double) * nme); memcpy(psdrm, pr, sizeof(double) * nme); }
        }
        for (int m = 0; m < nme; ++m) {
            m2mf[m] = m2mf[m] + psdfm[m] * dw;
            const double r = psdrm[m] * dw;
            m2mr[m] = m2mr[m] + r;
            m2o2mr[m] = m2o2mr[m] + r * omg * omg;
        }
    }
    free(S); free(Spad); free(bf); free(br); free(pf); free(pr); free(psdfm); free(psdrm);
    return 0;
}

/*
 * getFM_diag_tnm_scalar_msh_ (functionsImpl.F90:1123-1210): diagonal-only Mesher BFM at
 * one point.  The reference evaluates S(fi+fj) but never reads it: its products are
 * S_IJ = S(fi) S(fj), S_IJJ = S_IJ S(fj), S_IJI = S_IJ S(fi), with
 * BF = 2 (q_i l_j S_IJ l_k + l_i q_j S_IJJ l_k + l_i l_j S_IJI q_k).  Kept as written.
 */
int orc_msh_bfm_diag(const orc_problem *P, double fi, double fj, double *bfm)
{
    const int nnl = P->nnl, nme = P->nm_eff, nl = P->nlibsl;
    for (int l = 0; l < nl; ++l)
        if (P->libs_load[l] > nl) return -1;
    for (int m = 0; m < nme; ++m) bfm[m] = 0.0;
    double *Sfi = malloc(sizeof(double) * nnl), *Sfj = malloc(sizeof(double) * nnl);
    for (int itc = 0; itc < P->ntc; ++itc) {
        const int tc = P->tc[itc], tcl = tc - 1, tcq = tc + 2;
        orc_eval_psd(P, 1, &fi, tc, Sfi);
        orc_eval_psd(P, 1, &fj, tc, Sfj);
        for (int in = 0; in < nnl; ++in) {
            const int posi = (P->n_load[in] - 1) * P->nlibs;
            const double sij = Sfi[in] * Sfj[in];
            const double sijj = sij * Sfj[in], siji = sij * Sfi[in];
            for (int lk = 0; lk < nl; ++lk) {
                const double akU = WFCR(lk, tcl, in), ak = WFCR(lk, tcq, in);
                for (int im = 0; im < nme; ++im) {
                    const int m = P->modes[im];
                    const double phik = PHIR(posi + P->libs_load[lk], m);
                    double s = 0.0;
                    for (int l2 = 0; l2 < nl; ++l2)
                        for (int l1 = 0; l1 < nl; ++l1) {
                            const double tmp1 = sij * (WFCR(l1, tcq, in) * WFCR(l2, tcl, in));
                            const double tmp2 = sijj * (WFCR(l1, tcl, in) * WFCR(l2, tcq, in));
                            const double tmp3 = siji * (WFCR(l1, tcl, in) * WFCR(l2, tcl, in));
                            const double bf = 2.0 * ((tmp1 * akU) + (tmp2 * akU) + (tmp3 * ak));
                            const double ph = (PHIR(posi + P->libs_load[l1], m) * PHIR(posi + P->libs_load[l2], m)) * phik;
                            s += bf * ph;
                        }
                    bfm[im] = bfm[im] + s;
                }
            }
        }
    }
    free(Sfi); free(Sfj);
    return 0;
}

/* getRM_diag_scalar_msh_ (functionsImpl.F90:1212-1286): bfm/brm are (nm, nfi*nfj), fj fastest. */
void orc_msh_brm_diag(const orc_problem *P, int nfi, const double *fi, int nfj, const double *fj,
                      const double *bfm, double *brm)
{
    const int nme = P->nm_eff;
    size_t posf = 0;
    for (int i = 0; i < nfi; ++i) {
        const double wi = fi[i] * PIt2;
        for (int j = 0; j < nfj; ++j, ++posf) {
            const double wj = fj[j] * PIt2;
            for (int m = 0; m < nme; ++m) {
                double h1r, h1i, h2r, h2i, h3r, h3i;
                frf(P, m, wi, &h1r, &h1i);
                frf(P, m, wj, &h2r, &h2i);
                frf(P, m, wi + wj, &h3r, &h3i);
                brm[m + nme * posf] = bfm[m + nme * posf] *
                                      (h1r * h2r * h3r + h1r * h2i * h3i + h1i * h2r * h3i - h1i * h2i * h3r);
            }
        }
    }
}

/* computeSkewness_ (BsaLibImpl.F90:1641-1644), diagonal branch: sk = m3 / m2^(3/2). */
void orc_skewness_diag(int dim, const double *m2, const double *m3, double *sk)
{
    for (int i = 0; i < dim; ++i) sk[i] = m3[i] / pow(m2[i], 1.5);
}
#undef WFCR
#undef PHIR

/* ======================================================================================
 * Second-order post-processing.
 * ====================================================================================== */

/*
 * getBR_SFm_val_ (functionsImpl.F90:2650-2745): force PSD of kept mode im (mode id m) at the
 * frequency fnat; Suvw(nm, nnl*ntc) holds the nodal PSDs at every kept mode's frequency.
 * The DOF index of node j's mode shape pairs with node k's coefficient, as written.
 */
static double br_sfm(const orc_problem *P, int nme, const double *Suvw, double fnat, int im, int m)
{
    const int nnl = P->nnl, nl = P->nlibsl, nd = P->ndegw3;
    const double fiabs = fabs(fnat);
    double psd = 0.0;
    for (int itc = 0; itc < P->ntc; ++itc) {
        const int tc = P->tc[itc], posN = itc * nnl;
        for (int ink = 0; ink < nnl; ++ink) {
            const int nk = P->n_load[ink], pos_nk = (nk - 1) * P->nlibs;
            const double Sk = Suvw[I2(im, posN + ink, nme)];
            for (int inj = 0; inj < nnl; ++inj) {
                const int nj = P->n_load[inj], pos_nj = (nj - 1) * P->nlibs;
                const double corrJK = corr_of(P, nj, nk, tc);
                const double Sj = Suvw[I2(im, posN + inj, nme)];
                const double SJK = pow(corrJK, fiabs) * sqrt(Sj * Sk);
                double s = 0.0;
                for (int l2 = 0; l2 < nl; ++l2)
                    for (int l1 = 0; l1 < nl; ++l1) {
                        const double akU = P->wfc[I3(P->libs_load[l1] - 1, tc - 1, ink, nl, nd)];
                        const double ajU = P->wfc[I3(P->libs_load[l2] - 1, tc - 1, inj, nl, nd)];
                        const double phj = P->phi[I2(pos_nj + P->libs_load[l1] - 1, m - 1, P->ndofs)];
                        const double phk = P->phi[I2(pos_nk + P->libs_load[l2] - 1, m - 1, P->ndofs)];
                        s += (phj * phk) * ((akU * ajU) * SJK);
                    }
                psd = psd + s;
            }
        }
    }
    return psd;
}

/*
 * bsa_computeBRdecomp (src/bsa/BsaLibImpl.F90:1292-1420): bkg(m) = m2mf(m,m) / K_m^2,
 * res(m) = pi * 2pi * f_m * S_Fm(f_m) / (2 xsi_m K_m^2).  natf, xsi indexed by mode id;
 * m2mf of length nm (diag != 0) or nm^2.
 */
int orc_br_decomp(const orc_problem *P, const double *natf, const double *xsi, int diag, const double *m2mf,
                  double *bkg, double *res)
{
    const int nme = P->nm_eff, nnl = P->nnl;
    double *fm = malloc(sizeof(double) * nme), *col = malloc(sizeof(double) * nme * nnl);
    double *Suvw = malloc(sizeof(double) * (size_t)nme * nnl * P->ntc);
    for (int im = 0; im < nme; ++im) fm[im] = natf[P->modes[im] - 1];
    for (int itc = 0; itc < P->ntc; ++itc) {
        if (orc_eval_psd(P, nme, fm, P->tc[itc], col)) { free(fm); free(col); free(Suvw); return -1; }
        memcpy(Suvw + (size_t)nme * nnl * itc, col, sizeof(double) * nme * nnl);
    }
    for (int im = 0; im < nme; ++im) {
        const int m = P->modes[im];
        double km2 = P->Km[m - 1];
        km2 = km2 * km2;
        bkg[im] = m2mf[diag ? im : im * nme + im] / km2;
        const double sfm = br_sfm(P, nme, Suvw, fm[im], im, m);
        res[im] = PI_ * PIt2 * fm[im] * sfm / (2 * xsi[m - 1] * km2);
    }
    free(fm); free(col); free(Suvw);
    return 0;
}

/*
 * bsa_computePeakFactors (BsaLibImpl.F90:1428-1517).  Returns 1 (m2o2 all zero) or 2
 * (observation time too short) where the reference warns and returns.  sk may be NULL.
 */
int orc_peak_factors(int n, const double *m2, const double *m2o2, double obs_time, const double *sk,
                     double *peak_g, double *pos, double *neg)
{
    const double gamma_ = 0.5772, PI2 = PI_ * PI_;
    int any = 0;
    for (int i = 0; i < n; ++i) any |= (m2o2[i] != 0.0);
    if (!any) return 1;
    double *beta = malloc(sizeof(double) * n);
    for (int i = 0; i < n; ++i) {
        beta[i] = sqrt(m2o2[i] / m2[i]) / PIt2 * obs_time;
        if (beta[i] < 1.0) { free(beta); return 2; }
    }
    for (int i = 0; i < n; ++i) {
        beta[i] = sqrt(2 * log(beta[i]));
        peak_g[i] = gamma_ / beta[i];
        peak_g[i] = peak_g[i] + beta[i];
    }
    if (sk) {
        for (int i = 0; i < n; ++i) {
            const double rtmp = sk[i] * sk[i], g4 = 1.5 * rtmp;
            const double h40 = sqrt(1.0 + 1.5 * g4);
            const double h3 = sk[i] / (4.0 + 2.0 * h40);
            const double h4 = (h40 - 1.0) / 18.0;
            const double k = 1.0 / (sqrt(1 + 2.0 * h3 * h3 + 6.0 * h4 * h4));
            const double b = beta[i], b2 = b * b, b3 = b2 * b;
            double p = 5.44 / b3;
            p = p + (3.0 / b * (PI2 / 6.0 - gamma_ + (gamma_ * gamma_)));
            p = p + (b3 + 3 * b * (gamma_ - 1));
            p = p * h4;
            double q = p;
            const double r = h3 * (b2 + 2.0 * gamma_ - 1. + 1.98 / b2);
            p = p + r;
            q = q - r;
            p = p + peak_g[i];
            pos[i] = p * k;
            if (neg) neg[i] = (q + peak_g[i]) * k;
        }
    }
    free(beta);
    return 0;
}
