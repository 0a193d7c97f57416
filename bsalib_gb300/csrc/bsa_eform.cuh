// bsa_eform.cuh -- pieces of the E form of the Classic split contraction shared by the
// single-analysis kernel (bsa_classic_e.cu, k_bfm_e) and the batched sweep (bsa_batch.cu,
// k_bfm_e_batch): the pipeline constants, the FRF staging of one unit (grid row p, two N
// tiles of grid columns) and the epilogue of one N tile for the three warpgroups.
//
// E(f_p, f_q)[(a, b), j] = sum_k Q[k][a] A(f_p)[k][b] A(f_q)[k][j] for q >= p feeds the six
// contributions (i) T1 at (p, q), (iv) T1 at (q, p), (iii) T3 at (p, c), (v) T2 at (c, p),
// (ii) T2 at (d, q), (vi) T3 at (q, d), with f_c = f_q - f_p and f_d = f_p - f_q on the grid
// (q - p <= h); the derivation heads bsa_classic_e.cu.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "bsa_common.cuh"
#include "bsa_epi.cuh"
#include "bsa_tc.cuh"

namespace bsa {
namespace ecls {

using namespace tc;

constexpr int kStages = 2;
constexpr int kStageBytes = 6 * kTileBytes;  // U hi, U lo, B0 hi, B1 hi, B0 lo, B1 lo
constexpr int kKindsWG = 3;  // per epilogue warpgroup: two response kinds and one force kind
constexpr int kKinds = 3 * kKindsWG;  // 0 K_i, 1 K_iv, 2 F14, 3 K_iii, 4 K_v, 5 F35, 6 K_ii, 7 K_vi, 8 F26
constexpr int kFlushTiles = 64;
constexpr int kBarBytes = 256;
constexpr int kEpi = 384;  // three epilogue warpgroups

// Warp layouts of the E-form kernels.  Plain: 14 warps, the TMA warp 0, the MMA warp 1, the
// epilogue warps 2-13, at most 128 registers a thread.  Register split: 16 warps, the epilogue
// warpgroups first (warps 0-11), then a producer warpgroup of the TMA warp 12, the MMA warp 13
// and two idle warps; launched at 128 registers a thread, the producer warpgroup keeps 40 and
// the epilogue warpgroups take 152 (setmaxnreg): 384 x 152 + 128 x 40 = 63 488 of the launch's
// 65 536.  Measured 17 % faster for the 48-mode width (two passes of 24 modes) of the
// single-analysis kernel and slower below it, so the 48-mode kernels (single analysis and
// batched) use it and the others keep the plain layout.
template <bool RS>
struct ELayout {
    static constexpr int threads = RS ? 512 : 448;
    static constexpr int warp_tma = RS ? 12 : 0, warp_mma = RS ? 13 : 1, epi_warp0 = RS ? 0 : 2;
};
constexpr int kRegsEpi = 152, kRegsProd = 40;
static_assert(kEpi * kRegsEpi + (ELayout<true>::threads - kEpi) * kRegsProd <= ELayout<true>::threads * 128,
              "register split above the registers the block is launched with");
constexpr bool use_regsplit(int NMT, int JH) { return JH == 2 && NMT == 24; }

__device__ __forceinline__ void regs_producer() { asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;" ::"n"(kRegsProd)); }
__device__ __forceinline__ void regs_epilogue() { asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;" ::"n"(kRegsEpi)); }

// A register-split kernel needs its 128 registers a thread at launch: a setmaxnreg.inc the
// block cannot satisfy would wait for ever, so the host checks before every launch.
template <class K>
inline cudaError_t regsplit_check(K kern) {
    cudaFuncAttributes fa;
    cudaError_t e = cudaFuncGetAttributes(&fa, kern);
    if (e != cudaSuccess) return e;
    return fa.numRegs * ELayout<true>::threads >= kEpi * kRegsEpi + (ELayout<true>::threads - kEpi) * kRegsProd
               ? cudaSuccess
               : cudaErrorInvalidConfiguration;
}

// FRF values of one unit (row p, columns q0 .. q0 + 2 NC - 1): H_j at the row, and per
// column H_j(v), H_j(u + v), H_j(v - u), H_j(u - v), all W = NMT x JH modes (above 24 kept
// modes the G rows hold one half of NMT modes at a time, JH = 2, and every unit is swept
// once per half; the row modes a, b of a TMEM lane range over all W).
// Two of these sit back to back in shared memory and both take 16-byte copies and loads, so the
// size is a multiple of 16 bytes (the weights alone are not, for 24 modes a pass).
template <int NMT, int JH = 1>
struct alignas(16) UTile {
    static constexpr int NC2 = 2 * (kBN / NMT), W = NMT * JH;
    float2 hr[W];
    float2 hg[NC2 * W];
    float2 hs[NC2 * W];
    float2 hdp[NC2 * W];
    float2 hdm[NC2 * W];
    float wk[3][NC2];  // per warpgroup the integration weight of each column's target point
};
static_assert(sizeof(UTile<24, 2>) % 16 == 0 && sizeof(UTile<24, 1>) % 16 == 0 && sizeof(UTile<12, 2>) % 16 == 0,
              "staging tiles 16-byte multiples");

struct EParams {
    int nf, h, nm, Mp, MT, nk, ks_last, n_ntiles;
    int wmode;
    double wval;
    const float2 *Hg;  // [nf][W]
    const float2 *Hs;  // [2 nf - 1][W]
    double *part;      // [grid][kKinds][W][128]
    int *err;
    // Sampled form only (k_bfm_e with SAMPLE): slot[i1 + nf i2] = row of grid point (i1, i2)
    // in sF / sR ([slot][nm^3], m fastest), or -1 where the point is not sampled.
    const int *slot;
    double *sF, *sR;
    // Diagnostics (bsa_gpu_setWaitTest): t + 1 makes CTA 0's MMA warp omit the accumulator-ready
    // signal of its tile t, so the epilogue's bounded wait runs out; 0 = off.
    int test_skip_tile1;
    // Shard of the product rows (bsa_gpu_setClassicShard): rows p = p0 + (pstep_m1 + 1) l, l = 0, 1, ...
    // (zero-initialised: every row).
    int p0, pstep_m1;
};

// Shared-memory float2 load the compiler does not hoist (keeps the per-mode FRF values out
// of the registers the accumulators need).
__device__ __forceinline__ float2 lds2(const float2 *p) {
    float2 r;
    asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(r.x), "=f"(r.y) : "r"(su32(p)));
    return r;
}

// The FRF rows of the E form are in the mode-pair layout (prep_h with pairs): the 16 bytes of
// modes 2i, 2i + 1 hold {Re H_2i, Re H_2i+1, Im H_2i, Im H_2i+1}.  ldc: mode m as a complex
// value; lds_pair: modes m, m + 1 (m even) as the lane pairs {Re, Re} and {Im, Im}, one 16-byte
// shared load the compiler does not hoist.
__device__ __forceinline__ float2 ldc(const float2 *row, int m) {
    const float *r = reinterpret_cast<const float *>(row) + 4 * (m >> 1) + (m & 1);
    return make_float2(r[0], r[2]);
}
__device__ __forceinline__ ulonglong2 lds_pair(const float2 *row, int m) {
    ulonglong2 r;
    asm volatile("ld.shared.v2.u64 {%0, %1}, [%2];" : "=l"(r.x), "=l"(r.y) : "r"(su32(row + m)));
    return r;
}

__device__ __forceinline__ void epi_sync384() { asm volatile("bar.sync 1, 384;" ::: "memory"); }

// Units of grid row p: pairs of N tiles from the one holding column p (columns q < p masked).
__device__ __forceinline__ int n_units(int p, int ntl, int NC) { return (ntl - p / NC + 1) / 2; }

// Integration weight of grid point (r, c) (intgSpectraVect_, BsaClassicImpl.F90:596-632, with
// the reference's vertex weight -d^2 / 2).
__device__ __forceinline__ float wpt(int r, int c, int nf, bool vect, float wv) {
    if (!vect) return wv;
    const bool b1 = r == 0 || r == nf - 1, b2 = c == 0 || c == nf - 1;
    return wv * ((b1 && b2) ? -0.5f : ((b1 || b2) ? 0.5f : 1.f));
}

// Stage unit (p, N tiles nt, nt + 1) with threads t < nt_ (cp.async, zero where out of range).
template <int NMT, int JH = 1>
__device__ __forceinline__ void stage_unit(UTile<NMT, JH> *dst, const EParams &P, int p, int nt, int t, int nt_) {
    constexpr int NC = kBN / NMT, NC2 = 2 * NC, W = NMT * JH, CH = W / 2;  // 16-byte chunks per column row
    const int q0 = nt * NC;
    const int nch = CH + 4 * NC2 * CH;
    for (int x = t; x < nch; x += nt_) {
        if (x < CH) {
            epi::cp_async16(dst->hr + 2 * x, P.Hg + (size_t)p * W + 2 * x, true);
            continue;
        }
        const int y = x - CH, which = y / (NC2 * CH), z = y - which * NC2 * CH, cc = z / CH, k = z - cc * CH;
        const int q = q0 + cc;
        int row;
        bool v;
        float2 *d;
        const float2 *tab = P.Hg;
        if (which == 0) {
            row = q;
            v = q < P.nf;
            d = dst->hg;
        } else if (which == 1) {
            row = p + q;
            v = row <= 2 * P.nf - 2;
            tab = P.Hs;
            d = dst->hs;
        } else if (which == 2) {
            row = q - p + P.h;
            v = row >= 0 && row < P.nf;
            d = dst->hdp;
        } else {
            row = p - q + P.h;
            v = row >= 0 && row < P.nf;
            d = dst->hdm;
        }
        epi::cp_async16(d + cc * W + 2 * k, v ? (const void *)(tab + (size_t)row * W + 2 * k) : (const void *)tab,
                        v);
    }
    // the weights (zero where a contribution does not exist), the same for every TMEM lane:
    //   wg 0: w(p, q);  wg 1: w(p, c), f_c = f_q - f_p;  wg 2: w(d, q), f_d = f_p - f_q;  half on q = p
    if (t < 3 * NC2) {
        const int wg = t / NC2, cc = t - wg * NC2, q = q0 + cc;
        const bool vect = P.wmode == kWeightClassicVect, valid = q >= p && q < P.nf, vd = valid && q - p <= P.h;
        const float wv = (float)P.wval, dl = q == p ? 0.5f : 1.f;
        float w;
        if (wg == 0)
            w = valid ? dl * wpt(p, q, P.nf, vect, wv) : 0.f;
        else if (wg == 1)
            w = vd ? dl * wpt(p, q - p + P.h, P.nf, vect, wv) : 0.f;
        else
            w = vd ? dl * wpt(p - q + P.h, q, P.nf, vect, wv) : 0.f;
        dst->wk[wg][cc] = w;
    }
    epi::cp_async_commit();
}

// One N tile of a unit (TMEM columns taddr .. taddr + 127): the unit's grid columns staged at
// column slots slot0 + ci, with their weights (stage_unit).  Warpgroup wg accumulates kinds
// 3 wg .. 3 wg + 2:
//   wg 0: (i)   Re[w_pq H_a(u) H_b(v) conj H_j(u+v)],   (iv) Re[w_pq H_a(v) conj H_b(u+v) H_j(u)],   w_pq
//   wg 1: (iii) Re[w_pc H_b(v-u) conj H_a(v) H_j(u)],   (v)  Re[w_pc H_a(u) conj H_b(v) H_j(v-u)],   w_pc
//   wg 2: (ii)  Re[w_dq H_b(u-v) H_a(v) conj H_j(u)],   (vi) Re[w_dq H_b(v) conj H_a(u) H_j(u-v)],   w_dq
// each times x.  One code path for the three (the per-column setup picks the factors and the
// staged rows; a conj on H_j is folded into the factor), so the three warpgroups share one
// instruction stream.
template <int NMT, int JH = 1>
__device__ __forceinline__ void unit_half(const UTile<NMT, JH> &hb, uint32_t taddr, int wg, int a, int b,
                                          int slot0, f2x (&acc)[kKindsWG][NMT / 2], int jo = 0) {
    static_assert(NMT % 2 == 0, "modes in lane pairs");
    constexpr int NC = kBN / NMT, W = NMT * JH;
    const float2 hra = ldc(hb.hr, a);
    // the current column's factors as lane pairs: {Re P, Re P}, {-Im P, -Im P}, {w, w}; a
    // column that runs on into the next 16-column TMEM load keeps them (the loops unroll)
    f2x p1r = 0ull, p1i = 0ull, p2r = 0ull, p2i = 0ull, wk2 = 0ull;
    const float2 *X = hb.hr, *Y = hb.hr;  // per-mode factors of the two response kinds
#pragma unroll
    for (int qc = 0; qc < kBN / 16; ++qc) {
        uint32_t v[16];
        tmem_ld16(taddr + qc * 16, v);
        tmem_wait_ld();
#pragma unroll
        for (int e = 0; e < 16; e += 2) {  // two modes j, j + 1 of one column (NMT and 16 even)
            const int col = qc * 16 + e;
            const int ci = col / NMT, j = col % NMT;
            if (ci >= NC) continue;
            if (j == 0) {
                const int sl = (slot0 + ci) * W;
                const float wk = hb.wk[wg][slot0 + ci];
                const float2 Hbv = ldc(hb.hg + sl, b), Hav = ldc(hb.hg + sl, a);
                float2 t1, t2;
                if (wg == 0) {
                    t1 = conjf2(cmul(hra, Hbv));               // conj: pairs with conj H_j(u+v)
                    t2 = cmul(Hav, conjf2(ldc(hb.hs + sl, b)));
                    X = hb.hs + sl;
                    Y = hb.hr;
                } else if (wg == 1) {
                    t1 = cmul(ldc(hb.hdp + sl, b), conjf2(Hav));
                    t2 = cmul(hra, conjf2(Hbv));
                    X = hb.hr;
                    Y = hb.hdp + sl;
                } else {
                    t1 = conjf2(cmul(ldc(hb.hdm + sl, b), Hav));    // conj: pairs with conj H_j(u)
                    t2 = cmul(Hbv, conjf2(hra));
                    X = hb.hr;
                    Y = hb.hdm + sl;
                }
                X += jo;  // this pass's half of the modes j (jo even)
                Y += jo;
                p1r = pk2(wk * t1.x, wk * t1.x);
                p1i = pk2(-wk * t1.y, -wk * t1.y);
                p2r = pk2(wk * t2.x, wk * t2.x);
                p2i = pk2(-wk * t2.y, -wk * t2.y);
                wk2 = pk2(wk, wk);
            }
            const f2x x2 = pk2(__uint_as_float(v[e]), __uint_as_float(v[e + 1]));
            const ulonglong2 xq = lds_pair(X, j), yq = lds_pair(Y, j);
            // Re[P1 X_j] x and Re[P2 Y_j] x for modes j, j + 1
            acc[0][j >> 1] = fma2(fma2(p1i, xq.y, mul2(p1r, xq.x)), x2, acc[0][j >> 1]);
            acc[1][j >> 1] = fma2(fma2(p2i, yq.y, mul2(p2r, yq.x)), x2, acc[1][j >> 1]);
            acc[2][j >> 1] = fma2(wk2, x2, acc[2][j >> 1]);
        }
    }
}

// Sampled form of unit_half (the diagnostic instantiation of k_bfm_e): each contribution of
// the tile to a grid point listed in P.slot is added, unweighted, to that point's force and
// response bispectra (B = 2 (T1 + T2 + T3), FP64 atomics), with the same FRF factors as the
// moment epilogue (FP32 from the staged rows).  Targets per warpgroup as in unit_half:
//   wg 0: (i) T1 at (p, q), m n o = a b j;   (iv) T1 at (q, p), a j b
//   wg 1: (iii) T3 at (p, c), j b a;          (v) T2 at (c, p), j a b        (f_c = f_q - f_p)
//   wg 2: (ii) T2 at (d, q), b a j;           (vi) T3 at (q, d), b j a       (f_d = f_p - f_q)
// A diagonal product (q = p) feeds them at half weight, as in the moment form.
template <int NMT, int JH = 1>
__device__ __forceinline__ void unit_half_sample(const UTile<NMT, JH> &hb, uint32_t taddr, int wg, int a, int b,
                                                 int p, int q0, int slot0, const EParams &P, int jo, bool vrow) {
    constexpr int NC = kBN / NMT, W = NMT * JH;
    const int nm = P.nm, nm2 = nm * nm;
    const size_t nm3 = (size_t)nm2 * nm;
    const float2 hra = ldc(hb.hr, a);
#pragma unroll 1
    for (int qc = 0; qc < kBN / 16; ++qc) {
        uint32_t v[16];
        tmem_ld16(taddr + qc * 16, v);  // warp-collective: every lane loads
        tmem_wait_ld();
        if (!vrow) continue;
#pragma unroll 1
        for (int e = 0; e < 16; ++e) {
            const int col = qc * 16 + e;
            const int ci = col / NMT, j = col % NMT, jg = jo + j;
            if (ci >= NC || jg >= nm) continue;
            const int q = q0 + slot0 + ci;
            const bool valid = q >= p && q < P.nf;
            if (!(wg == 0 ? valid : (valid && q - p <= P.h))) continue;
            const int sl = (slot0 + ci) * W;
            const float2 Hbv = ldc(hb.hg + sl, b), Hav = ldc(hb.hg + sl, a);
            int i1a, i2a, i1b, i2b, ia, ib;
            float2 t1, t2, xj, yj;
            if (wg == 0) {
                i1a = p, i2a = q, ia = a + nm * b + nm2 * jg;
                i1b = q, i2b = p, ib = a + nm * jg + nm2 * b;
                t1 = conjf2(cmul(hra, Hbv));
                t2 = cmul(Hav, conjf2(ldc(hb.hs + sl, b)));
                xj = ldc(hb.hs + sl, jg);
                yj = ldc(hb.hr, jg);
            } else if (wg == 1) {
                const int c = q - p + P.h;
                i1a = p, i2a = c, ia = jg + nm * b + nm2 * a;
                i1b = c, i2b = p, ib = jg + nm * a + nm2 * b;
                t1 = cmul(ldc(hb.hdp + sl, b), conjf2(Hav));
                t2 = cmul(hra, conjf2(Hbv));
                xj = ldc(hb.hr, jg);
                yj = ldc(hb.hdp + sl, jg);
            } else {
                const int d = p - q + P.h;
                i1a = d, i2a = q, ia = b + nm * a + nm2 * jg;
                i1b = q, i2b = d, ib = b + nm * jg + nm2 * a;
                t1 = conjf2(cmul(ldc(hb.hdm + sl, b), Hav));
                t2 = cmul(Hbv, conjf2(hra));
                xj = ldc(hb.hr, jg);
                yj = ldc(hb.hdm + sl, jg);
            }
            const float x = __uint_as_float(v[e]);
            const double f = (q == p ? 1.0 : 2.0) * (double)x;  // 2 x, half weight on the diagonal
            const int sa = P.slot[i1a + P.nf * i2a], sb = P.slot[i1b + P.nf * i2b];
            if (sa >= 0) {
                atomicAdd(P.sF + (size_t)sa * nm3 + ia, f);
                atomicAdd(P.sR + (size_t)sa * nm3 + ia, f * (double)(t1.x * xj.x - t1.y * xj.y));
            }
            if (sb >= 0) {
                atomicAdd(P.sF + (size_t)sb * nm3 + ib, f);
                atomicAdd(P.sR + (size_t)sb * nm3 + ib, f * (double)(t2.x * yj.x - t2.y * yj.y));
            }
        }
    }
}

}  // namespace ecls
}  // namespace bsa
