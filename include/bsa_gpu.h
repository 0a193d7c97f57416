/*
 * bsa_gpu.h -- C-ABI of libbsagpu, a GB300 (sm_103a) implementation of BsaLib's
 * bispectral-force-model (BFM) hot path.
 *
 * Three groups of entry points, all plain C (pointers and sizes; arrays in the Fortran
 * column-major layouts the reference uses; ids 1-based as in the reference):
 *
 *  1. The BsaLib public API for the path (module BsaLib, src/BsaLib.F90): bsa_Init, the
 *     setters the standalone driver calls (app/bsa.F90:525-606), bsa_Run, bsa_Finalise.
 *     Setters BORROW the caller's arrays, exactly like the reference (which keeps Fortran
 *     pointers to them): they must stay alive until bsa_Finalise.  bsa_Run writes into
 *     caller-owned buffers (the reference allocates them; here the caller sizes them with
 *     bsa_getSpectraDims: nm^2 for m2*, nm^3 for m3*, nm for both with diagonal-only spectra).
 *
 *  2. The reference's device offload ABI, BsaCL (BsaCL/include/bsacl.h:28-55), with the
 *     same names and argument meaning, so a Fortran host built with BSA_USE_GPU can link
 *     this library in place of BsaCL.
 *
 *  3. Plugin-level batched entries standing in for the procedure pointers the hot path
 *     sits behind (getBFMClsVect / getBRMClsVect / getMshBFM / getMshBRM,
 *     src/bsa/data/BsaLibData.F90:166-185, 295-309), plus precision control.
 *
 * Error convention: every int-returning function returns BSA_OK (0) or a negative code
 * and never exits the process (the reference's bsa_Abort ends in `error stop`).  After a
 * failure the library is halted (sticky, as BsaCL's has_halted__) until bsa_Finalise;
 * bsa_lastError() describes the first failure.  Not re-entrant: one host thread.
 */
#ifndef BSA_GPU_H_
#define BSA_GPU_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BSA_OK 0
#define BSA_ERR_ARG -1        /* invalid argument or size mismatch                  */
#define BSA_ERR_STATE -2      /* call out of order, missing input, or halted        */
#define BSA_ERR_CUDA -3       /* CUDA runtime error (message in bsa_lastError)      */
#define BSA_ERR_UNSUPPORTED -4 /* valid in the reference but not on this path       */
#define BSA_ERR_TIMEOUT -5    /* a device-side wait ran out of its iteration budget */
#define BSA_ERR_NOMEM -6      /* device allocation failed                           */
#define BSA_SKIPPED 1         /* the reference warns and returns: outputs untouched, not sticky */

#define BSA_PREC_FP64 0       /* plain FP64 contraction (parity path)               */
#define BSA_PREC_BF16X3 1     /* split BF16x3 tensor-core contraction, FP32 accum.   */

/* ---------------------------------------------------------------------------------- */
/* 1. BsaLib API (src/BsaLib.F90, src/bsa/BsaLibImpl.F90)                              */
/* ---------------------------------------------------------------------------------- */

/* bsa_Init, src/BsaLib.F90:294 (BsaLibImpl.F90:61-85): reset state, select the device. */
int bsa_Init(void);

/* Settings (src/bsa/BsaLibImpl.F90:750-980, src/settings/SettingsImpl.F90). */
int bsa_setAnalysisType(int isuban);           /* BsaLibImpl.F90:909, 1 classic 2 mesher 3 both */
int bsa_setVersion(int ivers);                 /* BsaLibImpl.F90:923                          */
int bsa_setScalingConv(int iconv);             /* BsaLibImpl.F90:930, 1 circular 2 frequency  */
int bsa_setSpectraComputation(int ipsd, int ibisp); /* BsaLibImpl.F90:937                     */
int bsa_setSpectraExtension(int ionlydiag);    /* BsaLibImpl.F90:945, 1 = diagonal-only spectra */
int bsa_setSpatialSymmetry(int isym);          /* BsaLibImpl.F90:750                          */
int bsa_setSpectraSymmetries(int isym);        /* BsaLibImpl.F90:771                          */
int bsa_setTestMode(int itest);                /* BsaLibImpl.F90:951                          */
int bsa_setupClassic(int nfreqs, double df);   /* BsaLibImpl.F90:959                          */
int bsa_setClassicMode(int imode);             /* BsaLibImpl.F90:916, 0 vectorised 1 scalar   */
int bsa_setupMesher(int isvd, int bkgrfmt, double bkgaext, double genpaext, double maxaext,
                    int ifcov, int idumpmod);  /* BsaLibImpl.F90:966                          */
/* POD truncation of the Mesher's POD form (BsaLibImpl.F90:97-115, functionsImpl.F90:203-230,
 * 474-1019).  The default keeps every POD mode, where the POD form equals the direct form.
 * A request that drops modes makes the Mesher functions evaluate every nodal cross-PSD from
 * its kept eigenpairs (cuSOLVER dsyevd, loaded on first use); the threshold count follows the
 * reference's dsyev build (one mode, or none where the second smallest eigenvalue reaches the
 * limit). */
int bsa_setPODTruncationThreshold(double rval);  /* percent of the largest eigenvalue */
int bsa_setPODNOfModesKept(int nmodes);
/* Mesher controls (BsaLibImpl.F90:90-93, 789-810, 840-843; defaults BsaLibData.F90:219-233,
 * 273): validation of each zone's post-mesh BFM step against the narrowest peak of its interest
 * modes (default on), BFM multi-level refinement by the zone policies (default on), background
 * peak width from the first turbulence direction only (default off), pre-mesh scheme
 * (0 = without diagonal crests, the default; 1 = with diagonal crests and triangular zones,
 * which the Mesher functions refuse with BSA_ERR_UNSUPPORTED) and pre-mesh mode (used by
 * scheme 1 only).  bsa_loadInputFiles applies the standalone driver's choices
 * (app/bsa.F90:544-552): no validation, no multi-level refinement, restricted peak. */
int bsa_doValidateZoneDeltas(int on);
int bsa_setBfmMLR(int on);
int bsa_setMaxBkgPeakRestriction(int on);
int bsa_setPremeshScheme(int itype);
int bsa_setPremeshMode(int imode);
int bsa_setWindDirections(const int *dirs, int ndirs);  /* BsaLibImpl.F90:983                 */
int bsa_setWindTurbComps(const int *tc, int ntc);       /* BsaLibImpl.F90:991                 */

/* Structure (src/structure/StructureImpl.F90). */
int bsa_setTotalNOfNodes(int nn);                       /* BsaLibImpl.F90:1180           */
int bsa_setNumOfNodalDOFs(int nlibs);                   /* BsaLibImpl.F90:1172           */
int bsa_setTotalNumOfDOFs(int ndofs);                   /* BsaLibImpl.F90:1163           */
int bsa_setLoadedNodes(const int *nodes_l, int nn_l);   /* BsaLibImpl.F90:1208           */
int bsa_setLoadedNodalDOFs(const int *libs_l, int nlibs_l); /* BsaLibImpl.F90:1188       */
int bsa_setNodalCoords(int nn, const double *coords);   /* BsaLibImpl.F90:1154, (3, nn)  */
int bsa_setModalInfo(int ndofs, int nm, const double *phi, const double *natf); /* BsaLibImpl.F90:1238 */
int bsa_setModalMatrices(int nm, const double *Mgen, const double *Kgen, const double *Cgen); /* BsaLibImpl.F90:1247, C (nm,nm) */
int bsa_setTotDamping(const double *xsi, int nm);       /* BsaLibImpl.F90:1264           */

/* Wind (src/wind/WindSetImpl.F90). */
int bsa_setPSDType(int ipsd);                           /* BsaLibImpl.F90:1006, ids 1,2,3,5 */
int bsa_setWindVertProf(int iwprof);                    /* BsaLibImpl.F90:1000 (stored)  */
int bsa_setWindAltDir(int ivert);                       /* BsaLibImpl.F90:1013 (stored)  */
int bsa_setAirDensity(double aird);                     /* BsaLibImpl.F90:1033 (stored)  */
int bsa_setWZMeanWindVel(const double *ubref, int nz);  /* BsaLibImpl.F90:1047           */
int bsa_setWZRefAlt(const double *zref, int nz);        /* BsaLibImpl.F90:1054 (stored)  */
int bsa_setTurbWindScales(const double *L, int nz);     /* BsaLibImpl.F90:1061, (3,3,nz) */
int bsa_setTurbWindSDT(const double *sigma, int nz);    /* BsaLibImpl.F90:1068, (3,nz)   */
int bsa_setNodalVel(const double *unod, int nn);        /* BsaLibImpl.F90:1104           */
int bsa_setNodalWindZones(const int *wz, int nn);       /* BsaLibImpl.F90:1111           */
int bsa_setNodalWindAltitudes(const double *walt, int nn); /* BsaLibImpl.F90:1118 (stored) */
int bsa_setSpatialNodalCorr(const double *corr, int64_t ncorr); /* BsaLibImpl.F90:1125, (ncorr,3) */
int bsa_setWindFCoeffs(const double *wfc, int nlibs_l, int ndegw3, int nn_l); /* BsaLibImpl.F90:1133, (nlibs_l,ndegw+3,nn_l) */

/* The standalone driver's inputs read natively: bsa.bsadata (getBsaData, app/bsa.F90:877-930)
 * and bsa.extdata (getExtData, app/bsa.F90:696-871; the files generateBSAInputFiles_,
 * BsaLibImpl.F90:2065-2155, writes) from directory dir, followed by the driver's setter
 * sequence (app/bsa.F90:525-606).  Call after bsa_Init; the library owns the arrays until
 * bsa_Finalise. */
int bsa_loadInputFiles(const char *dir);

/* Validates the inputs (validateAll_, BsaLibImpl.F90:469-535: mode validation
 * validateModalInfo_ :545-599, projection setPhitimesCLocalInstance_ :611-671) and returns
 * the number of kept modes, which sizes bsa_Run's outputs. */
int bsa_getNModesEff(int *nm_eff);

/* Lengths of one PSD and one bispectrum tensor, dimM_psd_ / dimM_bisp_
 * (src/bsa/data/BsaLibData.F90:60-64, set at BsaLibImpl.F90:313-355): nm^2 / nm^3, or nm / nm
 * with the diagonal-only spectra (bsa_setSpectraExtension(1)).  These size bsa_Run's
 * outputs and every per-point tensor below. */
int bsa_getSpectraDims(int *dim_psd, int *dim_bisp);

/* bsa_Run, src/BsaLib.F90:372-399 (BsaLibImpl.F90:153-462).  Classic outputs m2mf_cls,
 * m2mr_cls, m2o2mr_cls (dim_psd), m3mf_cls, m3mr_cls (dim_bisp); Mesher outputs m3mf_msh,
 * m3mr_msh (dim_bisp).  Any pointer may be NULL when not wanted.  The diagonal-only
 * spectra always run in FP64, whatever bsa_gpu_setPrecision says. */
int bsa_Run(double *m2mf_cls, double *m2mr_cls, double *m2o2mr_cls, double *m3mf_msh,
            double *m3mr_msh, double *m3mf_cls, double *m3mr_cls);

/* bsa_Finalise, src/BsaLib.F90:401 (cleanBSAData_): drop borrowed pointers, free device memory. */
int bsa_Finalise(void);

/* computeSkewness_ (BsaLibImpl.F90:1630-1707): sk = m3_mno / (sig_m sig_n sig_o); with the
 * diagonal-only spectra selected (bsa_setSpectraExtension(1)) m2, m3 and sk have length nm
 * and sk = m3 / m2^(3/2), as the reference's module state selects. */
int bsa_computeSkewness(int nm, const double *m2, const double *m3, double *sk);

const char *bsa_lastError(void);

/* bsa_setBispExportCallback (src/bsa/BsaLibImpl.F90:1809-1816, called from the Classic
 * analysis at BsaClassicImpl.F90:175-191 and from the Mesher's post-mesh interpolation at
 * zones/_shared_poly2d.fi:1040-1210): fn receives response bispectra, npts points at a time,
 * brm laid out [npts][dim_bisp].  Classic: the grid, f1 fastest then f2 (the reference's loop
 * order); with a callback set, bsa_Run evaluates the Classic bispectra in FP64 in column blocks
 * of the grid (whatever bsa_gpu_setPrecision says), streams each block to fn and sums the third
 * moments over the blocks.  Mesher: after the zone integration (moments in the selected
 * precision), one call per zone with every point of its BRM lattice (i fastest, then j): the
 * bilinear interpolation of the zone's FP64 force bispectra at its BFM lattice times
 * Re[H_m(w1) H_n(w2) conj H_o(w1 + w2)].  NULL switches the export off. */
typedef void (*bsa_brm_export_fn)(int npts, const double *f1, const double *f2, const double *brm, void *user);
int bsa_setBispExportCallback(bsa_brm_export_fn fn, void *user);

/* bsa_computeBRdecomp (src/bsa/BsaLibImpl.F90:1292-1420): background part
 * bkg[m] = m2mf(m,m) / K_m^2 and resonant part res[m] = pi 2pi f_m S_Fm(f_m) / (2 xsi_m K_m^2)
 * of each kept mode's response variance, S_Fm(f_m) the modal force PSD at the mode's own
 * natural frequency (getBR_SFm_val_, functionsImpl.F90:2650-2745, evaluated on the GPU).
 * m2mf is bsa_Run's m2mf_cls (dim_psd); bkg, res have nm entries. */
int bsa_computeBRdecomp(const double *m2mf, double *bkg, double *res);

/* Nodal response moments by modal recombination (modalRecombination, app/bsa.F90:935-1053, the
 * standalone driver's post-processing, which passes the kept modes' shapes over every DOF): for
 * each DOF d of the modal matrix (bsa_setModalInfo's ndofs entries per output)
 *   diag: m2 = sum_m m2mr(m, m) phi_dm^2, m3 = sum_m m3mr(m, m, m) phi_dm^3, m2o2 as m2;
 *   CCC (complete cubic combination): m2 = sum_{j,k} m2mr(j, k) phi_dj phi_dk,
 *         m3 = sum_{i,j,k} m3mr(i, j, k) phi_di phi_dj phi_dk, m2o2 as m2;
 *   sk = m3 / m2^(3/2) for each.
 * m2mr, m3mr (and m2o2mr, which may be NULL: its outputs are then zero) are bsa_Run's modal
 * moments (dim_psd, dim_bisp).  Any output may be NULL.  With the diagonal-only spectra only
 * the diag outputs are formed (the reference returns before the CCC). */
int bsa_modalRecombination(const double *m2mr, const double *m3mr, const double *m2o2mr, double *m2_diag,
                           double *m3_diag, double *m2o2_diag, double *sk_diag, double *m2_ccc, double *m3_ccc,
                           double *m2o2_ccc, double *sk_ccc);

/* bsa_computePeakFactors (BsaLibImpl.F90:1428-1517): Gaussian peak factor
 * g = gamma / beta + beta, beta = sqrt(2 ln(sqrt(m2o2 / m2) / 2pi * T)), and, when sk is
 * given, the non-Gaussian (Hermite model) positive / negative peak factors.  n entries.
 * Returns BSA_SKIPPED (outputs untouched) where the reference warns and returns: m2o2 all
 * zero, or an observation time T too short (beta < 1).  peak_ng_neg may be NULL. */
int bsa_computePeakFactors(int n, const double *m2, const double *m2o2, double obs_time, double *peak_g,
                           const double *sk, double *peak_ng_pos, double *peak_ng_neg);

/* ---------------------------------------------------------------------------------- */
/* 2. BsaCL device ABI (BsaCL/include/bsacl.h:28-55; bodies in BsaCL/src/bsacl.c)       */
/*    bsaclRun computes the response third moments m3mr (nm^3) over the outer product  */
/*    of the acquired fi x fj lists with the uniform influence dfi*dfj*4*pi^2, as      */
/*    bsacl.c:1544-1572 does; S(fi+fj) is analytic (bsacl.cl).                         */
/* ---------------------------------------------------------------------------------- */
int bsaclInit(unsigned n_threads);                                        /* bsacl.c:1032 */
int bsaclInitDeviceMemory(void);                                          /* bsacl.c:1099 */
int bsaclRun(unsigned i_thread, size_t dim, double *h_res);               /* bsacl.c:1307 */
int bsaclSetKernelID(unsigned kid);                                       /* bsacl.c:1597 */
void bsaclAcquirePSDId(uint32_t psdid);                                   /* bsacl.c:1614 */
void bsaclAcquireStructModMat(double *modmat, double *natf, uint32_t ndofs, uint32_t nmodes); /* bsacl.c:1633 */
void bsaclAcquireModalMatrices(double *Mg, double *Cg, double *Kg);       /* bsacl.c:1653 */
void bsaclAcquireLoadedNodesList(int *nodes_load, uint32_t nnodes_l);     /* bsacl.c:1672 */
void bsaclAcquireTotalNOfNodes(uint32_t nnodes_tot);                      /* bsacl.c:1687 */
void bsaclAcquireUsedModesList(int *modes, uint32_t nmodes_eff);          /* bsacl.c:1702 */
void bsaclAcquireWindCoeffs(double *wfc, uint32_t nnodes_l, uint32_t nlibs, uint32_t ndegw); /* bsacl.c:1724 */
void bsaclAcquireTurbComponentsList(int *tc, uint32_t ntc);               /* bsacl.c:1747 */
void bsaclAcquirePhiTimesCMat(double *phi_T_c, uint32_t nmodes_eff, uint32_t nnodes_l, uint32_t ndegw); /* bsacl.c:1763 */
void bsaclAcquireNodalCorrelation(double *nod_corr, uint32_t nnod_corr);  /* bsacl.c:1782 */
void bsaclAcquireWindNodalVelocities(double *nod_vel);                    /* bsacl.c:1791 */
void bsaclAcquireWindNodalWindZones(int *nod_wz);                         /* bsacl.c:1797 */
void bsaclAcquireWindTurbScales(double *wt_scl, uint32_t nwz);            /* bsacl.c:1803 */
void bsaclAcquireWindTurbStd(double *wt_std, uint32_t nwz);               /* bsacl.c:1810 */
void bsaclAcquireComputationFreqs(unsigned i_thread, uint32_t nfi, double *fi, uint32_t nfj, double *fj); /* bsacl.c:1870 */
void bsaclAcquireBaseWindTurbPSD(double *S_uvw);                          /* bsacl.c:1895 */
void bsaclSetDeviceType(uint32_t itype);                                  /* bsacl.c:1914 */
void bsaclVerifyMaxAllocCondition(size_t idim, unsigned int *ican);       /* bsacl.c:1946 */
void bsaclAbort(int ierr);                                                /* bsacl.c:1965 */
void bsaclFinalise(void);                                                 /* bsacl.c:1975 */

/* ---------------------------------------------------------------------------------- */
/* 3. Plugin-level entries and controls                                                */
/* ---------------------------------------------------------------------------------- */

/* Contraction precision for the Classic grid (BSA_PREC_FP64 default, or BSA_PREC_BF16X3). */
int bsa_gpu_setPrecision(int prec);

/* Classic S(f1+f2) beyond the grid: 1 (default) reads zero, as the reference's padded
 * copy (functionsImpl.F90:1358-1363, 1409-1413); 0 evaluates it analytically. */
int bsa_gpu_setClassicTruncation(int on);

/* Restrict the Classic analysis to grid rows (f1 index, 0-based) in [r_begin, r_end);
 * r_end = -1 runs to the last row.  The moments returned by the shards of a partition of
 * the rows sum to the full grid's (multi-GPU / multi-process sharding, one host sum). */
int bsa_gpu_setClassicRows(int r_begin, int r_end);

/* Shard rank of nshards of the Classic analysis (no counterpart in the reference; multi-GPU or
 * multi-process runs, one host sum): the second-order moments take the shard's contiguous block
 * of grid rows (f1 index, sizes differing by at most one); the bispectrum moments take the same
 * block, except in the split precision's E form, which forms each product E(f_p, f_q), q >= p,
 * once for the whole grid and so takes the product rows p = rank + nshards l (interleaved, for
 * balance).  Either way the moments of the nshards shards sum to the full grid's.  Overrides
 * bsa_gpu_setClassicRows; (0, 1) is the whole analysis.  Reset by bsa_Finalise. */
int bsa_gpu_setClassicShard(int rank, int nshards);

/* No counterpart in the reference.  on != 0: on the symmetric Classic grid f = -N..N
 * (circular-frequency scaling, the reference's default) every factor of the path is even in
 * f, so B(f1, f2) = B(-f1, -f2); bsa_Run then evaluates the rows f1 <= 0 only, the rows f1 < 0
 * with twice their integration weight.  The third moments equal the full grid's up to the
 * summation order; materialised or exported bispectra always cover the full grid. */
int bsa_gpu_setClassicSymmetry(int on);

/* Batched Classic sweep: many independent analyses (structures, wind cases) evaluated by one
 * split-precision tensor-core launch per group of cases.  The reference runs one analysis per
 * process (app/bsa.F90:72-110: setup, bsa_Run, finalise); a parametric study repeats that.
 *
 * bsa_gpu_batchAdd snapshots the current inputs as case *case_id (validated as by bsa_Run;
 * full-tensor spectra, at most 64 kept modes); the caller may then change any input and add
 * the next case.  bsa_gpu_batchRun evaluates every case added since the last
 * bsa_gpu_batchClear on its full Classic grid (the split precision of bsa_gpu_setPrecision's
 * BSA_PREC_BF16X3, whatever the current precision) and writes, concatenated in case order,
 * m3mf / m3mr (nm_c^3 each) and m2mr (nm_c^2 each); case_ms[c] is the time from the start of
 * the contraction launch of the case's group to the completion of case c, total_ms the
 * device time of the whole sweep.  Any output may be NULL.  The current inputs are left as
 * they were.  bsa_gpu_batchCase reports a case's kept modes and grid size. */
int bsa_gpu_batchAdd(int *case_id);
int bsa_gpu_batchCase(int case_id, int *nm, int *nf);
int bsa_gpu_batchRun(double *m3mf, double *m3mr, double *m2mr, double *case_ms, double *total_ms);
int bsa_gpu_batchClear(void);

/* getBFMClsVect + getBRMClsVect materialised (functionsImpl.F90:1312-1738): force and
 * response bispectra on the classic grid, (nf, nf, dim_bisp) with f1 fastest, and the grid.
 * Runs validation and the grid set-up of bsa_Run; for small grids (tests). */
int bsa_gpu_clsBispectra(double *f_out, int nf_cap, int *nf, double *bisp_f, double *bisp_r);

/* getBFMClsVect + getBRMClsVect at listed points of the Classic grid (functionsImpl.F90:1494-1538
 * for B_F, :1598-1738 for B_R): grid point p is (f[i1[p]], f[i2[p]]), 0-based indices into the
 * grid bsa_gpu_clsBispectra reports; bisp_f, bisp_r are (dim_bisp, npts), either may be NULL.
 * Computed in the precision of bsa_gpu_setPrecision: BSA_PREC_FP64 evaluates the points with
 * the FP64 kernel; BSA_PREC_BF16X3 returns the split-precision analysis's own per-point values
 * -- the E-form tensor-core products of the whole grid, with the epilogue writing the listed
 * points' bispectra instead of the moments (needs the truncated S(f1+f2), an odd grid and at
 * most 48 kept modes; BSA_ERR_UNSUPPORTED otherwise).  Runs validation and the grid set-up of
 * bsa_Run.  For measuring the split path's per-point error against the FP64 path. */
int bsa_gpu_clsBispectraAt(const int *i1, const int *i2, int npts, double *bisp_f, double *bisp_r);

/* getMshBFM / getMshBRM batched over npts arbitrary points (getFM_full_tnm_scalar_msh_,
 * functionsImpl.F90:247-465; getRM_full_scalar_msh_, :1031-1115, point-wise): bfm and brm
 * are (dim_bisp, npts); either may be NULL.  With the diagonal-only spectra these are the
 * Mesher's diagonal functions (getFM_diag_tnm_scalar_msh_, :1123-1210, whose products read
 * S(fi) S(fj) where the Classic form reads S(fi+fj); kept as written). */
int bsa_gpu_mshBispectra(const double *fi, const double *fj, int npts, double *bfm, double *brm);

/* Weighted moments over an arbitrary point set (the Mesher's zone integration,
 * _shared_poly2d.fi:2091-2119): m3mf += sum_p w_p B_F(p), m3mr += sum_p w_p B_R(p). */
int bsa_gpu_mshMoments(const double *fi, const double *fj, const double *w, int npts,
                       double *m3mf, double *m3mr);

/* No counterpart in the reference.  For callers that cannot allocate device memory (a host
 * that passes buffers from its own pool or arena and forbids allocation behind its back):
 * the weighted third moments of bsa_gpu_mshMoments over a point set, with every argument a
 * caller-owned DEVICE pointer and no cudaMalloc / cudaFree or other allocating call inside.
 *   A   [rows][K][nm]  per-frequency factors A(f) = S(f) L  (k = itc*nnl + loaded node)
 *   Q   [K][nm]        projected quadratic coefficients
 *   ix, iy, iz [npts]  rows of A at f1, f2, f1+f2 (iz < 0: S(f1+f2) taken as zero)
 *   f1, f2, w [npts]   point frequencies [Hz] and integration weights
 *   Mm, Km, Cm [nm]    generalised mass, stiffness, damping of the kept modes
 *   m3mf, m3mr [nm^3]  outputs (m fastest); stream: a cudaStream_t (NULL = legacy stream).
 * Its scratch (per-group partial sums) is a fixed 4 MiB device array held by every GPU
 * that loads the library until the process exits; nm is limited to 64, where 2*nm^3
 * doubles fill it.  The array bounds the contraction's point groups to
 * G = min(bsa_gpu_mshMoments' group count, 2^18 / nm^3): the same parallelism up to about
 * 20 kept modes, fewer CTAs above (nm = 32: 128 instead of about 1200; nm = 64: 64), where
 * bsa_gpu_mshMoments is the faster choice for large point sets.  The first call on each
 * device resolves the array's device address (cudaGetSymbolAddress) and should be made
 * before any stream capture.  All calls share the array: calls that overlap on the GPU race
 * and must be serialised by the caller.  Returns BSA_OK, BSA_ERR_ARG, BSA_ERR_CUDA, or
 * BSA_ERR_UNSUPPORTED for a device ordinal of 64 or more (message in bsa_lastError). */
int bsa_gpu_pointMomentsNoAlloc(const double *A, int K, int nm, const double *Q, const int *ix,
                                const int *iy, const int *iz, const double *f1, const double *f2,
                                const double *w, int npts, const double *Mm, const double *Km,
                                const double *Cm, double *m3mf, double *m3mr, void *stream);

/* A rectangular Mesher zone (MRectZone_t, src/bsa/meshing/zones/MRectZoneImpl.F90): BFM
 * lattice point (i, j), 0 <= i < ni, 0 <= j < nj, at (f1, f2) = (fi0, fj0) + i (dIi, dIj)
 * + j (dJi, dJj) [Hz]; the response bispectrum is integrated on the BRM lattice refined by
 * (Fi, Fj) with the force bispectrum interpolated bilinearly (interpolateRZ_HTPC_v3,
 * _shared_poly2d.fi:470-2166) and trapezoid weights; sym multiplies the zone's integrals
 * (settings i_bisp_sym_, 1 for the full plane). */
typedef struct {
    double fi0, fj0;
    double dIi, dIj;
    double dJi, dJj;
    int ni, nj;
    int Fi, Fj;
    double sym;
    int policy;   /* MPolicy id of the zone (src/bsa/meshing/policy/MPolicy.F90:34-43) */
} bsa_zone;

/* Third moments over a list of zones in one batched device pass (the post-mesh zone loop,
 * Mesh / interpolate, BsaMesherImpl.F90:1416-1553, _shared_poly2d.fi:2091-2119):
 * m3mf = sum over zones of the BFM-lattice integral, m3mr = of the BRM-lattice integral.
 * npts (optional, 2 doubles): BFM and BRM lattice point counts. */
int bsa_gpu_mshZones(const bsa_zone *zones, int nz, double *m3mf, double *m3mr, double *npts);

/* bsa_gpu_mshZones in the split precision, plus each zone's own mode-diagonal response
 * moments zdiag[z * nm + m] = m3mr(m, m, m) of zone z (the quantity the zone-refinement
 * criterion compares between lattice levels).  Needs bsa_gpu_setPrecision(BSA_PREC_BF16X3)
 * and axis-aligned zones; no counterpart in the reference (its zones are not refined by an
 * error criterion). */
int bsa_gpu_mshZonesDiag(const bsa_zone *zones, int nz, double *m3mf, double *m3mr, double *zdiag);

/* The zone-refinement proposer (no counterpart in the reference): an MLP
 * din -> width -> width -> width (ReLU) -> 1 logit, BF16 weights, FP32 accumulation, trained on
 * the device (weighted binary cross-entropy with hard or soft targets, Adam on FP32 master
 * weights).  Parameters, flattened: W1[width][din] b1 W2[width][width] b2 W3[width][width] b3
 * w4[width] b4.  bsa_mlp_create returns a handle (>= 0) or an error code; din, width <= 128. */
int bsa_mlp_create(int din, int width, unsigned long long seed);
int bsa_mlp_destroy(int h);
long long bsa_mlp_num_params(int h);
int bsa_mlp_get_params(int h, float *params, int bf16);  /* FP32 master, or the BF16 copy as floats */
int bsa_mlp_set_params(int h, const float *params);
int bsa_mlp_forward(int h, const float *x, int n, float *prob);  /* x[n][din] -> P(refine)[n] */
int bsa_mlp_gradients(int h, const float *x, const float *y, const float *sw, int n, float *loss, float *grads);
int bsa_mlp_train(int h, const float *x, const float *y, const float *sw, int n, int epochs, int batch, float lr,
                  unsigned long long seed, float *loss_out);
const char *bsa_mlp_lastError(void);

/* The zone layout the Mesher analysis (bsa_Run with analysis type 2) evaluates: restates
 * prefetchZoneLimits_ (BsaMesherImpl.F90:1638-1859) and PreMesh (:266-1393) in the scheme
 * bsa_setPremeshScheme selected, and returns its rectangular zones as the lattices the walk
 * evaluates (for rotations in [pi/2, pi) and [3 pi/2, 2 pi) the walk starts from the init
 * point with its coordinates exchanged, _shared_poly2d.fi:196-212, 873-900).  Writes at most
 * cap zones, *nz receives the full count.  The diagonal-crest scheme also lays triangles:
 * bsa_gpu_mshGenerateTriangles. */
int bsa_gpu_mshGenerateZones(bsa_zone *zones, int cap, int *nz);

/* A triangular Mesher zone (MTriangZone_t, src/bsa/meshing/zones/MTriangZoneImpl.F90) as
 * dumpTZ / DumpZone record it: corner C, A at the end of the J side CA, B, rotation rot (of CA
 * from the +f2 axis), refinements ni = nj = n; its policy's factors (BFM refinement i / j and
 * levels, after bsa_setBfmMLR; BRM factors) and the spatial-symmetry weight; seq is its
 * position in the layout's dump order (rectangles fill the other positions in order). */
typedef struct {
    double Ci, Cj, Ai, Aj, Bi, Bj;
    double rot, sym;
    int n, policy;
    int bfm_i, bfm_j, bfm_levels, brm_i, brm_j;
    int seq;
} bsa_triangle;

/* The triangles of the Mesher layout (the diagonal-crest scheme's only).  Writes at most cap
 * triangles, *nt receives the full count. */
int bsa_gpu_mshGenerateTriangles(bsa_triangle *tris, int cap, int *nt);

/* Third moments over a list of triangles (interpolateTZ_HTPC_v3, _shared_poly2d.fi:470-2166):
 * the BFM at every BFM point of each triangle's post-mesh lattice in one FP64 device pass, the
 * BRM points each feeds, with their weights and interpolation shares, in its epilogue.  npts
 * (optional, 2 doubles): BFM and BRM point counts. */
int bsa_gpu_mshTriangles(const bsa_triangle *tris, int nt, double *m3mf, double *m3mr, double *npts);

/* The post-mesh lattice of one triangle, host only (what bsa_gpu_mshTriangles evaluates):
 * counts[6] = BFM points, BRM points, interpolation terms, export records, and the point
 * counts the reference adds to msh_bfmpts_post_ / msh_brmpts_post_; *oob = 1 where the
 * reference's walk indexes its work arrays past their sizes.  Arrays (each may be NULL):
 * bfm[3 * nb] (f1, f2, m3mf weight without sym), brm[3 * nq] (f1, f2, m3mr weight), qptr[nq + 1],
 * qsrc[nnz], qc[nnz] (BRM point r interpolates sum_k qc[k] BFM(qsrc[k]), k in
 * [qptr[r], qptr[r + 1])), exp[2 * ne] (written f1, f2), eq[ne] (BRM point, -1 for zero);
 * visual != 0: the lattice of the visual mode (no BFM refinement). */
int bsa_gpu_mshTriangLattice(const bsa_triangle *t, int visual, long long *counts, int *oob, double *bfm,
                             double *brm, int *qptr, int *qsrc, double *qc, double *exp, int *eq);

/* Timing and counters of the last run. */
typedef struct {
    double ms_total;          /* device time of the last run (CUDA events)           */
    double ms_contraction;    /* device time of the contraction kernels               */
    double ms_gemm;           /* device time of the dominant contraction kernel alone  */
    double points;            /* (f1,f2) points at which B_R was produced             */
    double h2d_bytes;         /* host-to-device bytes copied by the last run          */
    double d2h_bytes;         /* device-to-host bytes copied by the last run          */
    int kernels;              /* kernels launched by the last run                     */
    int precision;            /* BSA_PREC_* used                                      */
    int graphs;               /* CUDA graphs launched by the last run (kernels counts  */
                              /* the kernels inside them too)                          */
} bsa_gpu_stats;
int bsa_gpu_getStats(bsa_gpu_stats *st);

/* Form of the split-precision Classic contraction: 1 (default) the E form -- one GEMM family
 * over half the grid pairs, each product feeding the three terms at up to six grid points --
 * where it applies (whole odd grid, truncated S(f1 + f2), at most 48 kept modes; central
 * symmetry is then not applied); 0 the D1 / D3 form everywhere.  Both give the same moments to
 * FP32 rounding.  Also read by bsa_gpu_batchRun.  No reference counterpart (reset by
 * bsa_Finalise). */
int bsa_gpu_setClassicForm(int form);

/* Tile plans of the split-precision contractions (no counterpart in the reference): the shape
 * choices the project's autotuner (python -m bsalib_gb300.autotune) searches per range of kept
 * modes nm, of K (turbulence components x loaded nodes) and of Classic grid points per axis nf.
 *   BSA_PLAN_CLS_FORM     1: the E form of the Classic contraction where it applies, 0: D1 / D3
 *   BSA_PLAN_CLS_E_WIDTH  E form FRF-table width: 8, 16, 24, 32 (2 x 16) or 48 (2 x 24)
 *   BSA_PLAN_CLS_D_WIDTH  D1 / D3 form width: 8, 16, 24, 32 or 64 (2 x 32)
 *   BSA_PLAN_MSH_WIDTH    Mesher kernel mode width: a multiple of 8 from nm to 64 (nf ignored)
 *   BSA_PLAN_CLS_E_SPLIT  E form mode passes per unit: 1, or 2 (width 16 as 2 x 8 modes, 24 as
 *                         2 x 12: half the epilogue's accumulators per pass); widths 32 and 48 are
 *                         always 2 passes, width 8 one
 * The table is read on first use from data/tile_plans.txt beside the library (or the file the
 * environment variable BSA_TILE_PLANS names): lines "family nm_lo nm_hi k_lo k_hi nf_lo nf_hi
 * value" with family cls_form | cls_e_width | cls_d_width | msh_width | cls_e_split.  The first matching plan
 * wins; a value that does not fit the case (narrower than nm, not a built width) falls back to
 * the default rule (narrowest width holding nm, E form wherever it applies).  The plans are
 * process-wide and survive bsa_Finalise.  setTilePlan adds a plan ahead of the table,
 * clearTilePlans empties it (defaults only), loadTilePlans(path) replaces it (NULL: the default
 * file again), getTilePlan reports the value the library would use. */
#define BSA_PLAN_CLS_FORM 1
#define BSA_PLAN_CLS_E_WIDTH 2
#define BSA_PLAN_CLS_D_WIDTH 3
#define BSA_PLAN_MSH_WIDTH 4
#define BSA_PLAN_CLS_E_SPLIT 5
int bsa_gpu_setTilePlan(int family, int nm_lo, int nm_hi, int k_lo, int k_hi, int nf_lo, int nf_hi, int value);
int bsa_gpu_clearTilePlans(void);
int bsa_gpu_loadTilePlans(const char *path);
int bsa_gpu_getTilePlan(int family, int nm, int K, int nf, int *value);

/* Diagnostics, no counterpart in the reference: exercises the bounded device waits.  Every
 * mbarrier wait of the tensor-core kernels gives up after 2 s (or at once when another role of the
 * launch has already given up), lets its in-flight copies and MMAs land, frees its TMEM and
 * returns; the host then reports BSA_ERR_TIMEOUT and halts until bsa_Finalise.  tile >= 0 makes
 * the next split-precision Classic analysis in the E form omit, in CTA 0, the MMA warp's
 * accumulator-ready signal of that CTA's accumulator tile, so the epilogue's wait runs out (no
 * fault, no copy left in flight); -1 switches it off.  Applies to one analysis. */
int bsa_gpu_setWaitTest(int tile);

/* No counterpart in the reference.  on != 0 (default): each split-precision Mesher zone pass
 * (every refinement level of an adaptive refinement) runs its device work -- operand rows, the
 * tcgen05 contraction, FRF rows, zone integration, reductions -- as one CUDA graph captured from
 * the library's stream; 0 launches the same kernels one by one.  Same results either way. */
int bsa_gpu_setMesherGraphs(int on);

/* No counterpart in the reference.  on_device != 0 (default): each split-precision Mesher zone
 * pass is expanded on the device from its zone list -- distinct frequencies through hash tables
 * (A-table rows, U blocks), the point and column index tables, the tasks and the work queue of
 * the contraction; 0 builds the same tables on the host and uploads them.  The A rows' order
 * differs (hash order), the moments agree to FP32 rounding. */
int bsa_gpu_setMesherExpansion(int on_device);

/* No counterpart in the reference.  Device bytes one split-precision Mesher zone pass may use
 * (operand blocks, term tensors, FRF rows, A rows); bytes <= 0 (default): 40 % of the device
 * memory, at least 4 GB.  Zones too large for a quarter of a pass run as blocks of columns and
 * strips of lines that share their boundary lattice lines (the same integrals).  A host sharing
 * the device with other allocations sets a smaller figure. */
int bsa_gpu_setMesherPassBytes(double bytes);

/* Device memory.  Blocks the library releases (bsa_Finalise, buffer growth) are kept for reuse
 * by the next analysis, up to a quarter of the device memory, so repeated bsa_Init ...
 * bsa_Finalise cycles do not pay cudaMalloc / cudaFree of the operand tables each time.  This
 * frees them (no reference counterpart: the reference holds no device memory). */
int bsa_gpu_releaseDeviceCache(void);

#ifdef __cplusplus
}
#endif
#endif /* BSA_GPU_H_ */
