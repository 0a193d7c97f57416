// bsa_epi.cuh -- epilogue of the split-precision Classic contraction (k_bfm_mixed and its
// batched form k_bfm_batch): FRF products x integration weight x the two TMEM accumulators of
// one N tile, reduced into per-thread FP32 moment partials.
//
// An N tile holds NC = 128 / NMT grid columns x NMT modes j.  With more than 32 kept modes the
// modes are split into JH = 2 halves of NMT = 32 (the B tables hold one half per block of rows)
// and every grid row is swept once per half, so a thread keeps 5 x 32 FP32 partials whatever
// the mode count.  The FRF values one N tile reads are the same for every TMEM lane (row):
// H_j(w_c) and H_j(w_r + w_c) for the tile's columns c and all W = NMT x JH modes, and H_j(w_r).
// They are staged in shared memory one tile ahead with cp.async (double buffered), so the
// tile's arithmetic reads shared memory only.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "bsa_common.cuh"
#include "bsa_tc.cuh"

namespace bsa {
namespace epi {

using namespace tc;

// The staged values of one N tile: hs[c*W + j] = H_j(w_r + w_c0+c), hg[c*W + j] = H_j(w_c0+c),
// hr[j] = H_j(w_r), j < W = NMT x JH.
template <int NMT, int JH>
struct HTile {
    static constexpr int NC = kBN / NMT, W = NMT * JH;
    float2 hs[NC * W];
    float2 hg[NC * W];
    float2 hr[W];
};

__device__ __forceinline__ void cp_async16(void *dst, const void *src, bool valid) {
    // src-size 0 fills the 16 bytes with zeros and reads nothing
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(su32(dst)), "l"(src), "r"(valid ? 16 : 0)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Named barrier of the four epilogue warps (barrier 0 is __syncthreads).
__device__ __forceinline__ void epi_sync() { asm volatile("bar.sync 1, 128;" ::: "memory"); }

// Threads t = 0 .. nt - 1 stage the tile (r, columns c0 .. c0 + NC - 1) of a grid with nf
// columns; Hg has nf rows and Hs 2 nf - 1 rows of W entries.  Entries past the tables are zero.
template <int NMT, int JH>
__device__ __forceinline__ void stage(HTile<NMT, JH> *dst, const float2 *Hg, const float2 *Hs, int nf, int r,
                                      int c0, int t, int nt) {
    constexpr int NC = kBN / NMT, W = NMT * JH;
    constexpr int NCH = NC * W / 2;  // 16-byte chunks of hs (and of hg)
    constexpr int NCR = W / 2;
    for (int x = t; x < 2 * NCH + NCR; x += nt) {
        if (x < NCH) {
            const bool v = r + c0 + (2 * x) / W < 2 * nf - 1;
            cp_async16(dst->hs + 2 * x, v ? (const void *)(Hs + (size_t)(r + c0) * W + 2 * x) : (const void *)Hs, v);
        } else if (x < 2 * NCH) {
            const int y = x - NCH;
            const bool v = c0 + (2 * y) / W < nf;
            cp_async16(dst->hg + 2 * y, v ? (const void *)(Hg + (size_t)c0 * W + 2 * y) : (const void *)Hg, v);
        } else {
            const int y = x - 2 * NCH;
            cp_async16(dst->hr + 2 * y, Hg + (size_t)r * W + 2 * y, true);
        }
    }
    cp_async_commit();
}

// The tile's contribution to the partial moments of TMEM lane (a, b), modes j = jh NMT + j' of
// half jh.  taddr: TMEM address of the lane's D1 accumulator (D3 follows 128 columns later).
// Weight of point (r, c): wv_r times the classic edge factor when vect (b1: r is an edge row),
// else wv_r.
//
// SYM (symmetric D1): D1(r, c)[(a, b), j] = D1(c, r)[(a, j), b], so D1 is formed for columns
// c >= r only (d1 false: not formed for this tile) and each value also stands for term 1 at
// (c, r) with (m, n, o) = (a, j, b): weight w(c, r) = w(r, c), FRF Re[H_a(w_c) H_j(w_r)
// conj H_b(w_r + w_c)]; those go to acc[5] (response) and acc[6] (force), c > r only.
//
// d3off: TMEM column offset of the D3 accumulator from taddr (128; 0 when the tile's D3 sits
// where a D1 would, the first half of an N = 256 pair).
template <int NMT, int JH, bool SYM = false, int KINDS = 5>
__device__ __forceinline__ void tile(const HTile<NMT, JH> &hb, uint32_t taddr, int a, int b, int c0, int nf,
                                     bool vect, bool b1, float wv_r, int jh, float (&acc)[KINDS][NMT], int r = 0,
                                     bool d1 = true, uint32_t d3off = 128) {
    constexpr int NC = kBN / NMT, W = NMT * JH;
    const int jo = jh * NMT;
    const float2 hra = hb.hr[a];
#pragma unroll
    for (int q = 0; q < kBN / 32; ++q) {
#pragma unroll
        for (int pass = 0; pass < 2; ++pass) {
            if (SYM && pass == 0 && !d1) continue;  // warp-uniform: no D1 in this tile
            uint32_t v[32];
            tmem_ld32(taddr + (pass ? d3off : 0u) + q * 32, v);
            tmem_wait_ld();
            float2 PA = make_float2(0.f, 0.f), PB = PA;
            float wc = 0.f, wn = 0.f, wt = 0.f;
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
                        const float2 hcb = hb.hg[cc * W + b];
                        if (pass == 0) {
                            // SYM: term 1 at (r, c) for c >= r, its mirror at (c, r) for c > r
                            wn = SYM ? (cg >= 0 && cg >= r ? wc : 0.f) : wc;
                            const float2 t1 = cmul(hra, hcb);  // term 1 at (r, c)
                            PA = make_float2(wn * t1.x, wn * t1.y);
                            if (SYM) {
                                wt = cg > r ? wc : 0.f;
                                const float2 tt = cmul(hb.hg[cc * W + a], conjf2(hb.hs[cc * W + b]));
                                PB = make_float2(wt * tt.x, wt * tt.y);
                            }
                        } else {
                            const float2 hsa = hb.hs[cc * W + a];
                            const float2 hsb = hb.hs[cc * W + b];
                            const float2 t3 = cmul(hcb, conjf2(hsa));  // term 3 at (r, c)
                            PA = make_float2(wc * t3.x, wc * t3.y);
                            const float2 t2 = cmul(hra, conjf2(hsb));  // term 2 at (c, r)
                            PB = make_float2(wc * t2.x, wc * t2.y);
                        }
                    }
                }
                // modes j >= nm multiply zero B rows and zero FRF entries: they add zeros
                if (cval) {
                    const float x = __uint_as_float(v[e]);
                    if (pass == 0) {
                        const float2 hs = hb.hs[c * W + jo + j];
                        const float F1 = PA.x * hs.x + PA.y * hs.y;  // Re[P1 conj(H_j(s))]
                        acc[0][j] = fmaf(F1, x, acc[0][j]);
                        acc[3][j] = fmaf(wn, x, acc[3][j]);
                        if constexpr (SYM) {
                            const float2 hr = hb.hr[jo + j];
                            const float FT = PB.x * hr.x - PB.y * hr.y;  // Re[P1T H_j(w_r)]
                            acc[5][j] = fmaf(FT, x, acc[5][j]);
                            acc[6][j] = fmaf(wt, x, acc[6][j]);
                        }
                    } else {
                        const float2 hr = hb.hr[jo + j];
                        const float2 hc = hb.hg[c * W + jo + j];
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
