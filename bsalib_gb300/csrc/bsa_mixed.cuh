// bsa_mixed.cuh -- operand preparation of the split-precision Classic contraction, shared by
// the single-analysis path (bsa_mixed.cu) and the batched sweep (bsa_batch.cu).
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "bsa_common.cuh"

namespace bsa {
namespace mixed {

// U[(r*Mp + a*nm + b)][k] = Q[k][a] A(f_r)[k][b], r < nf, row stride Kp (k >= K zero)
cudaError_t prep_u(cudaStream_t st, int nf, int nm, int K, int Kp, int Mp, const float *A, const double *Q,
                   __nv_bfloat16 *Uh, __nv_bfloat16 *Ul);
// T[(t*NMT + j)][k] = A(row of t)[k][j0 + j] for `rows` row blocks (is_sum: the f1 + f2 table),
// NMT <= 32
cudaError_t prep_b(cudaStream_t st, int rows, int nm, int NMT, int j0, int K, int Kp, int nf, int n_pad, int trunc,
                   int sum_base, int is_sum, const float *A, __nv_bfloat16 *Th, __nv_bfloat16 *Tl);
// FRF tables Hg[c][j] = H_j(w_c), Hs[s][j] = H_j(w_r + w_c), s = r + c < 2 nf - 1; pairs:
// each 16 bytes hold modes 2i, 2i + 1 as {Re, Re, Im, Im} (the E form's layout, even NMT)
cudaError_t prep_h(cudaStream_t st, int nf, int nm, int NMT, const double *f, FrfPar frf, float2 *Hg, float2 *Hs,
                   bool pairs = false);

}  // namespace mixed
}  // namespace bsa
