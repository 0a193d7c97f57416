// bsa_epi.cuh -- epilogue of the split-precision Classic contraction (k_bfm_mixed and its
// batched form k_bfm_batch): FRF products x integration weight x the two TMEM accumulators of
// one N tile, reduced into per-thread FP32 moment partials.
//
// The FRF values one N tile reads are the same for every TMEM lane (row): H_j(w_c) and
// H_j(w_r + w_c) for the tile's columns c and all j, and H_j(w_r).  Each epilogue warp
// stages them in its own shared-memory buffer one tile ahead with cp.async (double
// buffered), so the tile's arithmetic reads shared memory only; no barrier spans warps.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "bsa_common.cuh"
#include "bsa_tc.cuh"

namespace bsa {
namespace epi {

using namespace tc;

// The staged values of one N tile: hs[c*NMT + j] = H_j(w_r + w_c0+c), hg[c*NMT + j] =
// H_j(w_c0+c), hr[j] = H_j(w_r).
struct HTile {
    float2 hs[128];
    float2 hg[128];
    float2 hr[32];
};

__device__ __forceinline__ void cp_async16(void *dst, const void *src, bool valid) {
    // src-size 0 fills the 16 bytes with zeros and reads nothing
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(su32(dst)), "l"(src), "r"(valid ? 16 : 0)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// One warp stages the tile (r, columns c0 .. c0 + NC - 1) of a grid with nf columns; Hg has nf
// rows and Hs 2 nf - 1 rows of NMT entries.  Entries past the tables are zero.
template <int NMT>
__device__ __forceinline__ void stage(HTile *dst, const float2 *Hg, const float2 *Hs, int nf, int r, int c0,
                                      int lane) {
    constexpr int NC = kBN / NMT;
    constexpr int NCH = NC * NMT / 2;  // 16-byte chunks of hs (and of hg)
    constexpr int NCR = NMT / 2;
    for (int x = lane; x < 2 * NCH + NCR; x += 32) {
        if (x < NCH) {
            const int row = r + c0 + (2 * x) / NMT;
            const bool v = row < 2 * nf - 1;
            cp_async16(dst->hs + 2 * x, v ? (const void *)(Hs + (size_t)(r + c0) * NMT + 2 * x) : (const void *)Hs, v);
        } else if (x < 2 * NCH) {
            const int y = x - NCH;
            const bool v = c0 + (2 * y) / NMT < nf;
            cp_async16(dst->hg + 2 * y, v ? (const void *)(Hg + (size_t)c0 * NMT + 2 * y) : (const void *)Hg, v);
        } else {
            const int y = x - 2 * NCH;
            cp_async16(dst->hr + 2 * y, Hg + (size_t)r * NMT + 2 * y, true);
        }
    }
    cp_async_commit();
}

// The tile's contribution to the partial moments of TMEM lane (a, b).  taddr: TMEM address of
// the lane's D1 accumulator (D3 follows 128 columns later).  Weight of point (r, c): wv_r times
// the classic edge factor when vect (b1: r is an edge row), else wv_r.
template <int NMT>
__device__ __forceinline__ void tile(const HTile &hb, uint32_t taddr, int a, int b, int c0, int nf, bool vect,
                                     bool b1, float wv_r, float (&acc)[5][NMT]) {
    constexpr int NC = kBN / NMT;
    const float2 hra = hb.hr[a];
#pragma unroll
    for (int q = 0; q < kBN / 32; ++q) {
#pragma unroll
        for (int pass = 0; pass < 2; ++pass) {
            uint32_t v[32];
            tmem_ld32(taddr + pass * 128 + q * 32, v);
            tmem_wait_ld();
            float2 PA = make_float2(0.f, 0.f), PB = PA;
            float wc = 0.f;
            bool cval = false;
            int c = 0;
#pragma unroll
            for (int e = 0; e < 32; ++e) {
                const int col = q * 32 + e;
                const int cc = col / NMT, j = col % NMT;
                if (cc >= NC) continue;
                if (j == 0 || e == 0) {
                    c = cc;
                    const int cg = c0 + cc;
                    cval = cg < nf;  // warp-uniform
                    if (cval) {
                        const bool b2 = (cg == 0 || cg == nf - 1);
                        wc = vect ? wv_r * ((b1 && b2) ? -0.5f : ((b1 || b2) ? 0.5f : 1.f)) : wv_r;
                        const float2 hcb = hb.hg[cc * NMT + b];
                        if (pass == 0) {
                            const float2 t1 = cmul(hra, hcb);  // term 1 at (r, c)
                            PA = make_float2(wc * t1.x, wc * t1.y);
                        } else {
                            const float2 hsa = hb.hs[cc * NMT + a];
                            const float2 hsb = hb.hs[cc * NMT + b];
                            const float2 t3 = cmul(hcb, conjf2(hsa));  // term 3 at (r, c)
                            PA = make_float2(wc * t3.x, wc * t3.y);
                            const float2 t2 = cmul(hra, conjf2(hsb));  // term 2 at (c, r)
                            PB = make_float2(wc * t2.x, wc * t2.y);
                        }
                    }
                }
                // columns j >= nm multiply zero B rows and zero FRF entries: they add zeros
                if (cval) {
                    const float x = __uint_as_float(v[e]);
                    if (pass == 0) {
                        const float2 hs = hb.hs[c * NMT + j];
                        const float F1 = PA.x * hs.x + PA.y * hs.y;  // Re[P1 conj(H_j(s))]
                        acc[0][j] = fmaf(F1, x, acc[0][j]);
                        acc[3][j] = fmaf(wc, x, acc[3][j]);
                    } else {
                        const float2 hr = hb.hr[j];
                        const float2 hc = hb.hg[c * NMT + j];
                        const float F3 = hr.x * PA.x - hr.y * PA.y;  // Re[H_j(w_r) P3]
                        const float F2 = hc.x * PB.x - hc.y * PB.y;  // Re[H_j(w_c) P2]
                        acc[1][j] = fmaf(F3, x, acc[1][j]);
                        acc[2][j] = fmaf(F2, x, acc[2][j]);
                        acc[4][j] = fmaf(wc, x, acc[4][j]);
                    }
                }
            }
        }
    }
}

}  // namespace epi
}  // namespace bsa
