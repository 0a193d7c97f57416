// bsa_mixed.cu -- split-precision (BF16x3) tensor-core contraction of the Classic grid,
// written for sm_103a with tcgen05 MMA, TMEM accumulators and TMA-fed shared memory.
//
// Exact restructuring of the BFM contraction (functionsImpl.F90:1494-1538, three terms):
// with U(f)[(a,b), k] = Q[k][a] A(f)[k][b] and, for a grid row r and column c,
//   D1(r,c)[(a,b), j] = sum_k U(f_r)[(a,b),k] A(f_c)[k][j]
//   D3(r,c)[(a,b), j] = sum_k U(f_r)[(a,b),k] Z(r+c)[k][j],   Z(s) = A(f1+f2)
// term 1 at (f1,f2) = (r,c) is D1 with (m,n,o) = (a,b,j), term 3 at (r,c) is D3 with
// (m,n,o) = (j,b,a), and term 2 at (c,r) is the same D3 with (m,n,o) = (j,a,b).  So the
// whole grid is two GEMM families sharing their A operand (the rows of U(f_r)); the FRF
// product (getRM_full_vect_cls_, :1598-1738) and the integration weights
// (intgSpectraVect_, BsaClassicImpl.F90:567-633) are applied in the epilogue, which reduces
// straight to third moments: no bispectrum is ever stored.
//
// Precision: every operand is split into bf16 hi + lo; D = Ahi Bhi + Ahi Blo + Alo Bhi with
// FP32 accumulation in TMEM.  The FRF is evaluated in FP64 (the K - w^2 M cancellation near
// resonance) and rounded once; per-thread moment partials are FP32 over at most a few
// hundred points and are accumulated in FP64 in global memory.
//
// Kernel roles (192 threads, one CTA per SM): warp 0 issues TMA loads, warp 1 owns TMEM
// and issues tcgen05.mma from one thread, warps 2-5 drain TMEM (one thread per TMEM lane).
// Every wait on an mbarrier is bounded by a global-timer budget; on expiry the kernel sets
// an error flag, stops issuing work, lets in-flight copies and MMAs land, frees TMEM and
// returns, so the host gets BSA_ERR_TIMEOUT and the context stays usable.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/bsa_gpu.h"
#include "bsa_engine.cuh"
#include "bsa_epi.cuh"
#include "bsa_tc.cuh"

namespace bsa {
namespace mixed {

using namespace tc;

constexpr int kStages = 2;
constexpr int kStageBytes = 6 * kTileBytes;      // U hi/lo, Bg hi/lo, Bs hi/lo
constexpr int kKinds = 5;                        // mr1, mr3, mr2, mf1, mf23 (+ mr1T, mf1T with SYM)
constexpr int kFlushTiles = 64;                  // FP32 -> FP64 flush period (N tiles)
constexpr int kBarBytes = 256;                   // mbarriers + TMEM slot
constexpr int kHBytes = 4 * (int)sizeof(epi::HTile<32, 2>);  // FRF staging, 2 x 2 tiles (largest form)

struct Params {
    int nf;          // grid size
    int rb, re;      // grid rows r in [rb, re) evaluated by this launch
    int sym_rows;    // central symmetry: rows r < sym_rows weigh twice (0: off)
    int nm;          // kept modes
    int Mp;          // rows per frequency in U (nm^2 rounded up to 128)
    int MT;          // Mp / 128
    int nk;          // K chunks (Kp / 64)
    int ks_last;     // 16-wide K steps of the last chunk that hold data (the rest is zero padding)
    int n_ntiles;    // ceil(nf / NC)
    int g_half;      // B rows of one mode half in the grid table (nf NMT)
    int s_half;      // B rows of one mode half in the sum table ((2 nf - 1) NMT)
    int wmode;       // kWeightClassicVect or kWeightUniform
    double wval;
    const float2 *Hg;  // [nf][W]  H_j(w_c), W = NMT JH
    const float2 *Hs;  // [2nf-1][W]  H_j(w_r + w_c), s = r + c
    double *part;      // [grid][kKinds][W][128]
    int *err;
};

// Work units of one (grid row r, mode half): the N tiles of the row as
//   kind 1: two N tiles nt, nt + 1 without D1, their D3 in one N = 256 MMA (B = S(nt) | S(nt + 1));
//   kind 2: one N tile without D1 (D3 alone, N = 128);
//   kind 0: an N tile with D1 and D3 in one N = 256 MMA (B = G(nt) | S(nt)).
// Without SYM every tile is kind 0.  With SYM the tiles nt < ntr = r / NC hold only columns
// c < r (no D1): they come first, in pairs, an odd one alone.  Pairing them keeps 24 MMAs per
// 96 KB stage, where a lone D3 tile has 12 per 64 KB and waits on its operands.
struct Units {
    int ntr, npair, single, n;
    __device__ __forceinline__ Units(int r, int ntl, bool sym, int NC) {
        ntr = sym ? min(ntl, r / NC) : 0;
        npair = ntr >> 1;
        single = ntr & 1;
        n = npair + single + (ntl - ntr);
    }
    __device__ __forceinline__ void at(int u, int &kind, int &nt) const {
        if (u < npair) {
            kind = 1;
            nt = 2 * u;
        } else if (u < npair + single) {
            kind = 2;
            nt = ntr - 1;
        } else {
            kind = 0;
            nt = ntr + (u - npair - single);
        }
    }
};

// Grid rows r of CTA g: r = rb + g / MT, then every (grid / MT)-th row; row tile g % MT.  Per row
// the mode halves jh < JH, per half the work units: the sequence of all three roles.
// Stage layout: U hi, U lo, B0 hi, B1 hi, B0 lo, B1 lo (B0 | B1 the 256 B rows of a unit).
template <int NMT, int JH, bool SYM>
__global__ void __launch_bounds__(192, 1)
    k_bfm_mixed(const __grid_constant__ CUtensorMap tmUh, const __grid_constant__ CUtensorMap tmUl,
                const __grid_constant__ CUtensorMap tmGh, const __grid_constant__ CUtensorMap tmGl,
                const __grid_constant__ CUtensorMap tmSh, const __grid_constant__ CUtensorMap tmSl, const Params p) {
    constexpr int NC = kBN / NMT;         // grid columns per N tile
    constexpr int BROWS = NC * NMT;       // B rows loaded by TMA per tile
    constexpr int W = NMT * JH;           // FRF table width
    constexpr int KINDS = SYM ? kKinds + 2 : kKinds;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t *bars = (uint64_t *)(smem + kStages * kStageBytes);
    uint64_t *full = bars, *empty = bars + kStages, *tfull = bars + 2 * kStages, *tempty = bars + 2 * kStages + 2;
    uint64_t *done = bars + 2 * kStages + 4;
    uint32_t *tmem_slot = (uint32_t *)(bars + 2 * kStages + 5);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int *err = p.err;

    // Rows of the B tiles that TMA never writes (BROWS..127) are zero for the whole run.
    for (int s = 0; s < kStages; ++s)
        for (int t = 2; t < 6; ++t) {
            uint8_t *tile = smem + s * kStageBytes + t * kTileBytes;
            for (int x = threadIdx.x; x < (128 - BROWS) * 128 / 16; x += blockDim.x)
                ((uint4 *)(tile + BROWS * 128))[x] = make_uint4(0, 0, 0, 0);
        }
    if (threadIdx.x == 0) {
        for (int s = 0; s < kStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&tfull[b], 1);
            mbar_init(&tempty[b], 128);
        }
        mbar_init(done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(su32(tmem_slot)) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tmem_slot;

    const int mt = blockIdx.x % p.MT;
    const int rstep = gridDim.x / p.MT;
    const int r0 = blockIdx.x / p.MT;
    const uint32_t tx_bytes = 2u * kTileBytes + 4u * (uint32_t)(BROWS * 128);  // kind 0, 1; kind 2 has 2 B tiles

    if (warp == 0) {
        // ---------------- TMA producer ----------------
        if (lane == 0) {
            uint32_t it = 0;
            bool ok = true;
            for (int r = p.rb + r0; r < p.re && ok; r += rstep)
                for (int jh = 0; jh < JH && ok; ++jh) {
                    const Units un(r, p.n_ntiles, SYM, NC);
                    for (int u = 0; u < un.n && ok; ++u) {
                        int kind, nt;
                        un.at(u, kind, nt);
                        for (int kc = 0; kc < p.nk && ok; ++kc, ++it) {
                            const int s = it % kStages;
                            const uint32_t ph = (it / kStages) & 1u;
                            if (!mbar_wait(&empty[s], ph ^ 1u, err, 1)) { ok = false; break; }
                            uint8_t *st = smem + s * kStageBytes;
                            mbar_expect_tx(&full[s], kind == 2 ? tx_bytes - 2u * (uint32_t)(BROWS * 128) : tx_bytes);
                            const int x = kc * kBK;
                            const int yu = r * p.Mp + mt * kBM;
                            tma_2d(st + 0 * kTileBytes, &tmUh, &full[s], x, yu);
                            tma_2d(st + 1 * kTileBytes, &tmUl, &full[s], x, yu);
                            const int ys = jh * p.s_half + (r + nt * NC) * NMT;  // S(nt)
                            if (kind == 0) {
                                const int yg = jh * p.g_half + nt * BROWS;
                                tma_2d(st + 2 * kTileBytes, &tmGh, &full[s], x, yg);
                                tma_2d(st + 4 * kTileBytes, &tmGl, &full[s], x, yg);
                                tma_2d(st + 3 * kTileBytes, &tmSh, &full[s], x, ys);
                                tma_2d(st + 5 * kTileBytes, &tmSl, &full[s], x, ys);
                            } else if (kind == 1) {
                                tma_2d(st + 2 * kTileBytes, &tmSh, &full[s], x, ys);
                                tma_2d(st + 4 * kTileBytes, &tmSl, &full[s], x, ys);
                                tma_2d(st + 3 * kTileBytes, &tmSh, &full[s], x, ys + BROWS);  // S(nt + 1)
                                tma_2d(st + 5 * kTileBytes, &tmSl, &full[s], x, ys + BROWS);
                            } else {
                                tma_2d(st + 3 * kTileBytes, &tmSh, &full[s], x, ys);
                                tma_2d(st + 5 * kTileBytes, &tmSl, &full[s], x, ys);
                            }
                        }
                    }
                }
            // Let the copies already issued land before the CTA can leave (bounded).
            const uint32_t last = it;
            for (uint32_t q = (last > (uint32_t)kStages ? last - kStages : 0); q < last; ++q) {
                const int s = q % kStages;
                const uint32_t ph = (q / kStages) & 1u;
                const uint64_t t0 = gtime();
                while (!mbar_try(&full[s], ph) && gtime() - t0 < kWaitNs) {
                }
            }
        }
        __syncwarp();
    } else if (warp == 1) {
        // ---------------- MMA issuer ----------------
        if (lane == 0) {
            uint32_t it = 0, tile = 0;
            bool ok = true;
            for (int r = p.rb + r0; r < p.re && ok; r += rstep)
                for (int jh = 0; jh < JH && ok; ++jh) {
                    const Units un(r, p.n_ntiles, SYM, NC);
                    for (int u = 0; u < un.n && ok; ++u, ++tile) {
                        int kind, nt;
                        un.at(u, kind, nt);
                        const int buf = tile & 1;
                        const uint32_t tph = (tile >> 1) & 1u;
                        if (!mbar_wait(&tempty[buf], tph ^ 1u, err, 2)) { ok = false; break; }
                        fence_after();
                        const uint32_t d1 = tmem + buf * 256, d3 = d1 + 128;
                        for (int kc = 0; kc < p.nk; ++kc, ++it) {
                            const int s = it % kStages;
                            const uint32_t ph = (it / kStages) & 1u;
                            if (!mbar_wait(&full[s], ph, err, 3)) { ok = false; break; }
                            fence_after();
                            const uint32_t base = su32(smem + s * kStageBytes);
                            // K steps past the data in the last chunk multiply zero padding: skip them
                            const int nks = kc == p.nk - 1 ? p.ks_last : kBK / 16;
#pragma unroll
                            for (int ks = 0; ks < kBK / 16; ++ks) {
                                if (ks >= nks) break;
                                const uint32_t off = ks * 32;
                                const uint64_t uh = sdesc(base + 0 * kTileBytes + off), ul = sdesc(base + 1 * kTileBytes + off);
                                const uint32_t acc = (kc > 0 || ks > 0) ? 1u : 0u;
                                if (kind != 2) {  // [D1 | D3] or [D3(nt) | D3(nt + 1)]: B0 | B1, N = 256
                                    const uint64_t bh = sdesc(base + 2 * kTileBytes + off), bl = sdesc(base + 4 * kTileBytes + off);
                                    mma256(d1, uh, bh, acc);
                                    mma256(d1, uh, bl, 1u);
                                    mma256(d1, ul, bh, 1u);
                                } else {  // D3 alone: B1, N = 128
                                    const uint64_t bh = sdesc(base + 3 * kTileBytes + off), bl = sdesc(base + 5 * kTileBytes + off);
                                    mma(d3, uh, bh, acc);
                                    mma(d3, uh, bl, 1u);
                                    mma(d3, ul, bh, 1u);
                                }
                            }
                            mma_commit(&empty[s]);  // stage free once these MMAs have read it
                        }
                        if (!ok) break;
                        mma_commit(&tfull[buf]);  // accumulators ready for the epilogue
                    }
                }
            // Every MMA issued so far completes before TMEM is released.
            mma_commit(done);
            const uint64_t t0 = gtime();
            while (!mbar_try(done, 0) && gtime() - t0 < kWaitNs) {
            }
        }
        __syncwarp();
    } else {
        // ---------------- epilogue: FRF x weight, reduce to moments ----------------
        // The four warps share one double-buffered FRF staging slot (epi_sync orders it).  After
        // a failed wait a warp keeps walking the tile sequence without work, so every warp
        // reaches every epi_sync.
        const int quarter = warp & 3;
        const int et = threadIdx.x - 64;               // 0 .. 127
        const int row = quarter * 32 + lane;          // TMEM lane = row of the M tile
        const int grow = mt * kBM + row;               // row of U(f_r): a * nm + b
        const bool vrow = grow < p.nm * p.nm;
        const int a = vrow ? grow / p.nm : 0, b = vrow ? grow % p.nm : 0;
        const uint32_t lane_base = tmem + ((uint32_t)(quarter * 32) << 16);
        const float wvf = (float)p.wval;
        const bool vect = p.wmode == kWeightClassicVect;
        using HT = epi::HTile<NMT, JH>;
        HT *hbs = (HT *)(smem + kStages * kStageBytes + kBarBytes);
        double *part = p.part + (size_t)blockIdx.x * KINDS * W * 128 + row;
        for (int k = 0; k < KINDS * W; ++k) part[(size_t)k * 128] = 0.0;
        float acc[KINDS][NMT];
        auto zero = [&]() {
#pragma unroll
            for (int k = 0; k < KINDS; ++k)
#pragma unroll
                for (int j = 0; j < NMT; ++j) acc[k][j] = 0.f;
        };
        // Only this thread adds into its partials; a reduction (fire and forget) keeps the
        // 5 x NMT old values out of the registers, and one thread's adds to one address apply
        // in program order, so the sums stay deterministic.
        auto flush = [&](int jh) {
#pragma unroll
            for (int k = 0; k < KINDS; ++k)
#pragma unroll
                for (int j = 0; j < NMT; ++j) {
                    atomicAdd(part + (size_t)(k * W + jh * NMT + j) * 128, (double)acc[k][j]);
                    acc[k][j] = 0.f;
                }
        };
        uint32_t tile = 0;
        bool ok = true;
        // FRF staging of unit (r, jh, u) into slot pair hb[0..1] (the tiles the unit covers)
        auto stage_unit = [&](HT *hb, int r, int u) {
            const Units un(r, p.n_ntiles, SYM, NC);
            int kind, nt;
            un.at(u, kind, nt);
            epi::stage<NMT, JH>(hb, p.Hg, p.Hs, p.nf, r, nt * NC, et, 128);
            if (kind == 1) epi::stage<NMT, JH>(hb + 1, p.Hg, p.Hs, p.nf, r, (nt + 1) * NC, et, 128);
        };
        if (p.rb + r0 < p.re) stage_unit(hbs, p.rb + r0, 0);
        int since = 0;  // tiles accumulated since the last flush
        for (int r = p.rb + r0; r < p.re; r += rstep) {
            const bool b1 = (r == 0 || r == p.nf - 1);
            const float wv_r = r < p.sym_rows ? 2.f * wvf : wvf;  // central symmetry: the mirror row
            const Units un(r, p.n_ntiles, SYM, NC);
            for (int jh = 0; jh < JH; ++jh) {
                zero();
                since = 0;
                for (int u = 0; u < un.n; ++u, ++tile) {
                    int kind, nt;
                    un.at(u, kind, nt);
                    const int buf = tile & 1;
                    const uint32_t tph = (tile >> 1) & 1u;
                    epi::cp_async_wait_all();
                    epi::epi_sync();  // this unit's values are in; the other slot pair is no longer read
                    // stage the next unit's FRF values (they depend on the row and columns only)
                    if (u + 1 < un.n)
                        stage_unit(hbs + 2 * (buf ^ 1), r, u + 1);
                    else if (jh + 1 < JH)
                        stage_unit(hbs + 2 * (buf ^ 1), r, 0);
                    else if (r + rstep < p.re)
                        stage_unit(hbs + 2 * (buf ^ 1), r + rstep, 0);
                    if (ok) {
                        // warp-uniform outcome: tcgen05.ld below is .sync.aligned
                        ok = __all_sync(0xffffffffu, mbar_wait(&tfull[buf], tph, err, 4));
                        if (ok) {
                            fence_after();
                            const uint32_t ta = lane_base + buf * 256;
                            const HT *hb = hbs + 2 * buf;
                            if (kind == 1) {
                                epi::tile<NMT, JH, SYM, KINDS>(hb[0], ta, a, b, nt * NC, p.nf, vect, b1, wv_r, jh, acc, r,
                                                               false, 0u);
                                epi::tile<NMT, JH, SYM, KINDS>(hb[1], ta, a, b, (nt + 1) * NC, p.nf, vect, b1, wv_r, jh,
                                                               acc, r, false);
                            } else {
                                epi::tile<NMT, JH, SYM, KINDS>(hb[0], ta, a, b, nt * NC, p.nf, vect, b1, wv_r, jh, acc, r,
                                                               kind == 0);
                            }
                            fence_before();
                            mbar_arrive(&tempty[buf]);
                            since += kind == 1 ? 2 : 1;
                            // one flush site: a second inlined copy of the flush made the
                            // compiler spill the accumulators
                            if (since >= kFlushTiles || u + 1 == un.n) {
                                flush(jh);
                                since = 0;
                            }
                        }
                    }
                }
            }
        }
        epi::cp_async_wait_all();
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
}

// ------------------------------------------------------------------------------------
// Operand preparation (FP32 -> bf16 hi/lo; the U products Q A formed in FP32).
// ------------------------------------------------------------------------------------

// U[(r*Mp + a*nm + b)][k] = Q[k][a] * A(f_r)[k][b]   (rows >= nm^2 and k >= K are zero).
// Each thread writes 8 consecutive k of one row as one 16-byte store per hi / lo table.
__global__ void k_prep_u(int nm, int K, int Kp, int Mp, const float *__restrict__ A, const double *__restrict__ Q,
                         __nv_bfloat16 *__restrict__ Uh, __nv_bfloat16 *__restrict__ Ul) {
    const int r = blockIdx.x, k0 = blockIdx.y * 64;
    __shared__ float As[64][65], Qs[64][65];  // nm <= 64
    const float *Ar = A + (size_t)r * K * nm;
    for (int e = threadIdx.x; e < 64 * nm; e += blockDim.x) {
        const int kk = e / nm, m = e % nm, k = k0 + kk;
        As[kk][m] = k < K ? Ar[(size_t)k * nm + m] : 0.f;
        Qs[kk][m] = k < K ? (float)Q[(size_t)k * nm + m] : 0.f;
    }
    __syncthreads();
    const int nm2 = nm * nm;
    for (int e = threadIdx.x; e < Mp * 8; e += blockDim.x) {
        const int row = e >> 3, kv = (e & 7) * 8;
        __align__(16) __nv_bfloat16 hi[8], lo[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const float u = row < nm2 ? Qs[kv + q][row / nm] * As[kv + q][row % nm] : 0.f;
            split_bf16f(u, hi[q], lo[q]);
        }
        const size_t o = ((size_t)r * Mp + row) * Kp + k0 + kv;
        *(uint4 *)(Uh + o) = *(const uint4 *)hi;
        *(uint4 *)(Ul + o) = *(const uint4 *)lo;
    }
}

// T[(t*NMT + j)][k] = A(src(t))[k][j0 + j], j < NMT <= 32; src(t) < 0 gives a zero row (j0 + j >= nm
// too).
__global__ void k_prep_b(int nm, int NMT, int j0, int K, int Kp, int nf, int n_pad, int trunc, int sum_base,
                         int is_sum, const float *__restrict__ A, __nv_bfloat16 *__restrict__ Th,
                         __nv_bfloat16 *__restrict__ Tl) {
    const int t = blockIdx.x, k0 = blockIdx.y * 64;
    int src = t;
    if (is_sum) {
        if (trunc) {
            const int c = t - n_pad;
            src = (c >= 0 && c < nf) ? c : -1;
        } else {
            src = sum_base + t;
        }
    }
    __shared__ float As[64][33];
    for (int e = threadIdx.x; e < 64 * NMT; e += blockDim.x) {
        const int kk = e / NMT, jj = e % NMT, m = j0 + jj, k = k0 + kk;
        As[kk][jj] = (src >= 0 && k < K && m < nm) ? A[((size_t)src * K + k) * nm + m] : 0.f;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < NMT * 8; e += blockDim.x) {
        const int j = e >> 3, kv = (e & 7) * 8;
        __align__(16) __nv_bfloat16 hi[8], lo[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) split_bf16f(As[kv + q][j], hi[q], lo[q]);
        const size_t o = ((size_t)t * NMT + j) * Kp + k0 + kv;
        *(uint4 *)(Th + o) = *(const uint4 *)hi;
        *(uint4 *)(Tl + o) = *(const uint4 *)lo;
    }
}

// FRF tables in FP64, rounded once to FP32: Hg[c][j] = H_j(w_c), Hs[s][j] = H_j(w_r + w_c).
// Complex values in mode order, or with pairs (even NMT) in mode pairs: the 16 bytes of modes
// 2i, 2i + 1 hold {Re H_2i, Re H_2i+1, Im H_2i, Im H_2i+1}, so one 16-byte load gives two
// modes' real parts and imaginary parts as FP32 lane pairs.
__global__ void k_prep_h(int nf, int nm, int NMT, const double *__restrict__ f, FrfPar frf, float2 *__restrict__ Hg,
                         float2 *__restrict__ Hs, int pairs) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int ng = nf * NMT, ns = (2 * nf - 1) * NMT;
    if (t >= ng + ns) return;
    const bool g = t < ng;
    const int u = g ? t : t - ng, row = u / NMT, j = u % NMT;
    double hr = 0, hi = 0;
    if (j < nm) {
        const int r = row / 2, c = row - r;
        const double w = g ? f[row] * kPi2 : f[r] * kPi2 + f[c] * kPi2;
        frf_eval(frf.M[j], frf.K[j], frf.C[j], w, hr, hi);
    }
    float2 *tab = g ? Hg : Hs;
    if (pairs) {
        float *rf = reinterpret_cast<float *>(tab + (size_t)row * NMT) + 4 * (j >> 1) + (j & 1);
        rf[0] = (float)hr;
        rf[2] = (float)hi;
    } else {
        tab[u] = make_float2((float)hr, (float)hi);
    }
}

// m3[m + nm n + nm^2 o] from the per-CTA FP64 partials: three term contributions each, and
// with the symmetric D1 (kinds 7) term 1's mirror, kept at (m, o, n).
__global__ void k_mixed_reduce(int nm, int NMT, int MT, int grid, int kinds, const double *__restrict__ part,
                               double *__restrict__ m3mf, double *__restrict__ m3mr) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int nm3 = nm * nm * nm;
    if (x >= nm3) return;
    const int m = x % nm, n = (x / nm) % nm, o = x / (nm * nm);
    auto sum = [&](int kind, int a, int b, int j) {
        const int R = a * nm + b, mtile = R / 128, lane = R % 128;
        double s = 0.0;
        for (int g = mtile; g < grid; g += MT) s += part[(((size_t)g * kinds + kind) * NMT + j) * 128 + lane];
        return s;
    };
    double mr = sum(0, m, n, o) + sum(1, o, n, m) + sum(2, n, o, m);
    double mf = sum(3, m, n, o) + sum(4, o, n, m) + sum(4, n, o, m);
    if (kinds > kKinds) {
        mr += sum(5, m, o, n);
        mf += sum(6, m, o, n);
    }
    m3mr[x] = 2.0 * mr;  // B_F = 2 * (term1 + term2 + term3)
    m3mf[x] = 2.0 * mf;
}

cudaError_t prep_u(cudaStream_t st, int nf, int nm, int K, int Kp, int Mp, const float *A, const double *Q,
                   __nv_bfloat16 *Uh, __nv_bfloat16 *Ul) {
    k_prep_u<<<dim3(nf, Kp / 64), 256, 0, st>>>(nm, K, Kp, Mp, A, Q, Uh, Ul);
    return cudaGetLastError();
}

cudaError_t prep_b(cudaStream_t st, int rows, int nm, int NMT, int j0, int K, int Kp, int nf, int n_pad, int trunc,
                   int sum_base, int is_sum, const float *A, __nv_bfloat16 *Th, __nv_bfloat16 *Tl) {
    k_prep_b<<<dim3(rows, Kp / 64), 256, 0, st>>>(nm, NMT, j0, K, Kp, nf, n_pad, trunc, sum_base, is_sum, A, Th, Tl);
    return cudaGetLastError();
}

cudaError_t prep_h(cudaStream_t st, int nf, int nm, int NMT, const double *f, FrfPar frf, float2 *Hg, float2 *Hs,
                   bool pairs) {
    const int nh = (nf + 2 * nf - 1) * NMT;
    k_prep_h<<<(nh + 255) / 256, 256, 0, st>>>(nf, nm, NMT, f, frf, Hg, Hs, pairs ? 1 : 0);
    return cudaGetLastError();
}

template <int NMT, int JH, bool SYM>
static cudaError_t launch_gemm(cudaStream_t st, const CUtensorMap *maps, const Params &p, int grid) {
    const size_t smem = (size_t)kStages * kStageBytes + 1024 + kBarBytes + kHBytes;
    cudaError_t e =
        cudaFuncSetAttribute(k_bfm_mixed<NMT, JH, SYM>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    k_bfm_mixed<NMT, JH, SYM><<<grid, 192, smem, st>>>(maps[0], maps[1], maps[2], maps[3], maps[4], maps[5], p);
    return cudaGetLastError();
}

}  // namespace mixed

int Engine::contract_mixed(const PointSrc &ps, long long npts, double *m3mf, double *m3mr) {
    using namespace mixed;
    (void)npts;
    const int nf = ps.nf, nm = nme;
    if (nm > 64) return fail(BSA_ERR_UNSUPPORTED, "BF16x3 contraction supports at most 64 kept modes");
    // the E form (bsa_classic_e.cu): one GEMM family over half the grid pairs; whole odd grid,
    // truncated S(f1 + f2), at most 48 kept modes, no central symmetry
    if (nm <= kEFormMaxModes && ps.mode == kPointsGrid && ps.r0 == 0 && ps.nr == nf && ps.sym_rows == 0 && ps.trunc == 1 &&
        (nf & 1) && use_e_form && plan_prefer_e(nm, K, nf))
        return contract_e(ps, m3mf, m3mr);
    // FRF-table width per mode half (tile plan; default the narrowest that holds the modes);
    // 64 = two halves of 32 (JH = 2)
    const int Wd = plan_d_width(nm, K, nf);
    const int JH = Wd > 32 ? 2 : 1;
    const int NMT = Wd / JH;
    const int W = NMT * JH;
    const int NC = kBN / NMT;
    const int Kp = ((K + kBK - 1) / kBK) * kBK;
    const int Mp = ((nm * nm + kBM - 1) / kBM) * kBM;
    const int MT = Mp / kBM;
    const int ns = 2 * nf - 1;
    int dev = 0, nsm = 0;
    cudaError_t e;
    if ((e = cudaGetDevice(&dev)) || (e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev)))
        return cuda_fail(e, "device query");
    int grid = (nsm / MT) * MT;
    if (grid < MT) grid = MT;
    const size_t uel = (size_t)nf * Mp * Kp, gel = (size_t)JH * nf * NMT * Kp, sel = (size_t)JH * ns * NMT * Kp;
    const size_t bytesA = 2 * uel * 2, bytesB = 2 * (gel + sel) * 2;
    const size_t bytesH = sizeof(float2) * (size_t)(nf + ns) * W;
    // symmetric D1 (term 1 from the columns c >= r only): one launch over the whole grid, up to
    // 24 kept modes (two more partial kinds per lane fit the registers there)
    const bool symd1 = JH == 1 && NMT <= 24 && ps.r0 == 0 && ps.nr == nf && ps.sym_rows == 0;
    const int kinds = symd1 ? kKinds + 2 : kKinds;
    const size_t bytesP = sizeof(double) * (size_t)grid * kinds * W * 128;
    if ((e = dMixA.reserve(bytesA)) || (e = dMixB.reserve(bytesB)) || (e = dMixH.reserve(bytesH + 256)) ||
        (e = dMixPart.reserve(bytesP + 256)))
        return cuda_fail(e, "allocating BF16x3 operands");
    __nv_bfloat16 *Uh = dMixA.as<__nv_bfloat16>(), *Ul = Uh + uel;
    __nv_bfloat16 *Gh = dMixB.as<__nv_bfloat16>(), *Gl = Gh + gel, *Sh = Gl + gel, *Sl = Sh + sel;
    float2 *Hg = dMixH.as<float2>(), *Hs = Hg + (size_t)nf * W;
    int *derr = (int *)((char *)dMixPart.p + bytesP);
    if ((e = cudaEventRecord(ev2, stream))) return cuda_fail(e, "event");
    if ((e = cudaMemsetAsync(derr, 0, sizeof(int), stream))) return cuda_fail(e, "memset");
    {
        const float *A = dA32.as<float>();
        dim3 gu(nf, Kp / 64);
        k_prep_u<<<gu, 256, 0, stream>>>(nm, K, Kp, Mp, A, dQ.as<double>(), Uh, Ul);
        dim3 gg(nf, Kp / 64), gs(ns, Kp / 64);
        // B tables: one block of rows per mode half, modes jh NMT .. jh NMT + NMT - 1
        for (int jh = 0; jh < JH; ++jh) {
            const size_t og = (size_t)jh * nf * NMT * Kp, os = (size_t)jh * ns * NMT * Kp;
            k_prep_b<<<gg, 256, 0, stream>>>(nm, NMT, jh * NMT, K, Kp, nf, ps.n_pad, ps.trunc, ps.sum_base, 0, A,
                                             Gh + og, Gl + og);
            k_prep_b<<<gs, 256, 0, stream>>>(nm, NMT, jh * NMT, K, Kp, nf, ps.n_pad, ps.trunc, ps.sum_base, 1, A,
                                             Sh + os, Sl + os);
        }
        const int nh = (nf + ns) * W;
        k_prep_h<<<(nh + 255) / 256, 256, 0, stream>>>(nf, nm, W, ps.fgrid, frf(), Hg, Hs, 0);
        if ((e = cudaGetLastError())) return cuda_fail(e, "BF16x3 operand preparation");
        kernels += 2 + 2 * JH;
    }
    CUtensorMap maps[6];
    const uint64_t grows = (uint64_t)JH * nf * NMT, srows = (uint64_t)JH * ns * NMT;
    if (!make_map(&maps[0], Uh, Kp, (uint64_t)nf * Mp, kBM) || !make_map(&maps[1], Ul, Kp, (uint64_t)nf * Mp, kBM) ||
        !make_map(&maps[2], Gh, Kp, grows, NC * NMT) || !make_map(&maps[3], Gl, Kp, grows, NC * NMT) ||
        !make_map(&maps[4], Sh, Kp, srows, NC * NMT) || !make_map(&maps[5], Sl, Kp, srows, NC * NMT))
        return fail(BSA_ERR_CUDA, "cuTensorMapEncodeTiled failed");
    Params prm{};
    prm.nf = nf;
    prm.rb = ps.r0;
    prm.re = ps.r0 + ps.nr;
    prm.sym_rows = ps.sym_rows;
    prm.nm = nm;
    prm.Mp = Mp;
    prm.MT = MT;
    prm.nk = Kp / kBK;
    prm.ks_last = (K - (prm.nk - 1) * kBK + 15) / 16;
    prm.n_ntiles = (nf + NC - 1) / NC;
    prm.g_half = nf * NMT;
    prm.s_half = ns * NMT;
    prm.wmode = ps.wmode;
    prm.wval = ps.wval;
    prm.Hg = Hg;
    prm.Hs = Hs;
    prm.part = dMixPart.as<double>();
    prm.err = derr;
    if ((e = cudaEventRecord(evg0, stream))) return cuda_fail(e, "event");
    switch (NMT * JH) {
    case 8: e = symd1 ? launch_gemm<8, 1, true>(stream, maps, prm, grid) : launch_gemm<8, 1, false>(stream, maps, prm, grid); break;
    case 16: e = symd1 ? launch_gemm<16, 1, true>(stream, maps, prm, grid) : launch_gemm<16, 1, false>(stream, maps, prm, grid); break;
    case 24: e = symd1 ? launch_gemm<24, 1, true>(stream, maps, prm, grid) : launch_gemm<24, 1, false>(stream, maps, prm, grid); break;
    case 32: e = launch_gemm<32, 1, false>(stream, maps, prm, grid); break;
    default: e = launch_gemm<32, 2, false>(stream, maps, prm, grid); break;
    }
    if (e) return cuda_fail(e, "BF16x3 tcgen05 contraction kernel");
    if ((e = cudaEventRecord(evg1, stream))) return cuda_fail(e, "event");
    const long long nm3 = (long long)nm * nm * nm;
    if ((e = dOut.reserve(sizeof(double) * (3 * (size_t)nm * nm + 2 * (size_t)nm3)))) return cuda_fail(e, "out");
    double *o = dOut.as<double>() + 3 * (size_t)nm * nm;
    k_mixed_reduce<<<(unsigned)((nm3 + 127) / 128), 128, 0, stream>>>(nm, W, MT, grid, kinds, prm.part, o, o + nm3);
    if ((e = cudaGetLastError())) return cuda_fail(e, "BF16x3 reduction");
    kernels += 2;
    std::vector<double> h(2 * (size_t)nm3);
    int herr = 0;
    if ((e = cudaMemcpyAsync(h.data(), o, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, stream)) ||
        (e = cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, stream)) ||
        (e = cudaEventRecord(ev1, stream)) || (e = cudaStreamSynchronize(stream)))
        return cuda_fail(e, "BF16x3 contraction");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ev2, ev1);
    last_ms_contraction = ms;
    cudaEventElapsedTime(&ms, evg0, evg1);
    last_ms_gemm = ms;
    d2h += (double)sizeof(double) * h.size() + sizeof(int);
    if (herr) return fail(BSA_ERR_TIMEOUT, "BF16x3 kernel: a pipeline wait ran out of its budget (role %d)", herr);
    if (m3mf) std::memcpy(m3mf, h.data(), sizeof(double) * nm3);
    if (m3mr) std::memcpy(m3mr, h.data() + nm3, sizeof(double) * nm3);
    return BSA_OK;
}

}  // namespace bsa
