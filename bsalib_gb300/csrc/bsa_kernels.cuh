// bsa_kernels.cuh -- launchers of the FP64 kernels (internal C++ interface of libbsagpu).
#pragma once
#include "bsa_common.cuh"

namespace bsa {

// Nodal PSD S[f][itc][i] for nf frequencies (evalPSD_ and the model functions,
// src/wind/WindPSDImpl.F90:123-316).  tcs: turbulent component ids (1..3) per itc.
cudaError_t launch_nodal_psd(cudaStream_t st, int nf, const double *f, int ntc, const int *tcs_host,
                             int nnl, const PsdNode *par, int psd_type, int scaling, double *S, bool fp32 = false);

// A[f][k][m] = sqrt(S_i(f)) sum_j c_ij^|f| sqrt(S_j(f)) L[(itc,j)][m]  (FP64).
// lc[x] = log(lc[x]) in place (FP64) and lc32[x] = (float)lc[x]: the coherence table log c.
cudaError_t launch_log_coh(cudaStream_t st, size_t n, double *lc, float *lc32);

cudaError_t launch_atable(cudaStream_t st, int nf, const double *f, int ntc, int nnl, int nm,
                          const double *logc, const double *S, const double *L, double *A);


// The FP32 table on the tensor cores (bsa_atable_tc.cu): tf32 hi/lo split, FP32 accumulation;
// err receives a nonzero code if a pipeline wait ran out of its budget.  nm <= 64.
// scratch: atable_tc_scratch(ntc, nnl, nm) bytes (the split B tables).
size_t atable_tc_scratch(int ntc, int nnl, int nm);
cudaError_t launch_atable_tc(cudaStream_t st, int nf, const double *f, int ntc, int nnl, int nm,
                             const float *logc, const double *S, const float *L, float *A, void *scratch, int *err);

// Force PSD on the grid psd[f][n + nm*o] = sum_k L[k][o] A[f][k][n]
// (functionsImpl.F90:1548-1560), then the second-order moments
// m2mf, m2mr (x Re[H_o conj H_n]), m2o2mr (x w^2) with per-frequency weights wf.
cudaError_t launch_force_psd(cudaStream_t st, int nf, int ntc, int nnl, int nm, const double *L,
                             const double *A, double *psd);
cudaError_t launch_force_psd32(cudaStream_t st, int nf, int ntc, int nnl, int nm, const float *L,
                               const float *A, double *psd);
// Second-order moments over the grid frequencies k in [k0, k1); diag != 0 for the
// same-mode spectra psd[f][m].
cudaError_t launch_m2(cudaStream_t st, int k0, int k1, int nm, int diag, const double *f, const double *wf,
                      const double *psd, FrfPar frf, double *m2mf, double *m2mr, double *m2o2mr);

// Diagonal-only force PSD psd[f][m] = sum_k W2[k][m] S[f][k], W2 = L^2 (functionsImpl.F90:1924-1947).
cudaError_t launch_force_psd_diag(cudaStream_t st, int nf, int K, int nm, const double *S, const double *W2,
                                  double *psd);

// FP64 BFM contraction + FRF + weighted reduction over a point set.
//   B_F[m,n,o](p) = 2 sum_k ( Q_km X_kn Y_ko + Z_km (Q_kn Y_ko + X_kn Q_ko) ),
//   X = A(f1), Y = A(f2), Z = A(f1+f2)   (the exact factorisation of the nodal triple sum
//   of functionsImpl.F90:1494-1538), B_R = B_F * Re[H_m(w1) H_n(w2) conj H_o(w1+w2)].
// part_mf / part_mr receive one nm^3 partial per point group (n_groups of them);
// bf_out / br_out (optional) receive B_F / B_R per point, (nm^3, npts).
cudaError_t launch_bfm_fp64(cudaStream_t st, const double *A, const double *Q, int K, int nm,
                            const PointSrc &ps, long long npts, FrfPar frf, int n_groups,
                            double *part_mf, double *part_mr, double *bf_out, double *br_out);
int bfm_fp64_groups(long long npts, int nm);

// out[x] = sum_g part[g * len + x] (fixed order); optional second array.
cudaError_t launch_reduce_groups(cudaStream_t st, int n_groups, long long len, const double *part,
                                 double *out, const double *part2, double *out2);

}  // namespace bsa
