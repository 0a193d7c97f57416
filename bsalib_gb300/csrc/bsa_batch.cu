// bsa_batch.cu -- many Classic analyses (structures x wind cases) in one persistent
// split-precision launch per group of cases.
//
// Each case is snapshotted when it is added (bsa_gpu_batchAdd: its validated inputs, the
// derived tables and its grid), so the caller can set up the next case at once.  At
// bsa_gpu_batchRun the cases are grouped by their FRF-table width (8, 16, 24, 32 kept modes,
// or 64: two halves of 32) and by device memory; for each group the operands of every case are prepared into
// shared tables (one U, G, S table each, rows of all cases stacked with a common K stride), and
// one launch of k_bfm_batch walks a work list of (case, grid row, row tile) items with the
// k_bfm_mixed pipeline (TMA warp, MMA warp, four TMEM-draining warps).  The epilogue adds its
// FP32 partial moments into per-case FP64 accumulators (atomics: the summation order varies
// from run to run in the last bits) and the last epilogue warp to finish a case stamps its
// completion time, which gives per-case latencies within the launch.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/bsa_gpu.h"
#include "bsa_eform.cuh"
#include "bsa_engine.cuh"
#include "bsa_epi.cuh"
#include "bsa_kernels.cuh"
#include "bsa_mixed.cuh"
#include "bsa_tc.cuh"

namespace bsa {
namespace batch {

using namespace tc;

constexpr int kStages = 2;
constexpr int kStageBytes = 6 * kTileBytes;
constexpr int kKinds = 5;  // mr1, mr3, mr2, mf1, mf23 (+ mr1T, mf1T with SYM)
constexpr int kFlushTiles = 64;
constexpr int kBarBytes = 256;                              // mbarriers + TMEM slot
constexpr int kHBytes = 4 * (int)sizeof(epi::HTile<32, 2>);  // FRF staging, 2 x 2 tiles (largest form)
constexpr size_t kSmem = (size_t)kStages * kStageBytes + 1024 + kBarBytes + kHBytes;

struct CaseP {
    int nf, nm, Mp, MT, nk, ks_last, n_ntiles, wmode;
    double wval;
    int u_row0;       // first U-table row of the case
    int g_row0;       // first G-table row
    int s_row0;       // first S-table row
    int hg0, hs0;     // first FRF-table entries (float2)
    long long part0;  // first accumulator (double) of the case: [KINDS][NMT][Mp]
    unsigned nitems;  // work items of the case
};

struct BItem {
    int c, r, mt, pad;
};

struct BParams {
    const BItem *items;
    int nitems;
    const CaseP *cases;
    const float2 *Hg, *Hs;
    double *part;
    unsigned *done_cnt;           // per case: epilogue warps that finished an item
    unsigned long long *t_done;   // per case: completion time (global timer, ns)
    unsigned long long *t_start;  // launch start (global timer, ns)
    int *err;
};

// Work units of one (grid row r, mode half), as in the single-analysis kernel (bsa_mixed.cu):
// kind 0 one N tile with [D1 | D3] (N = 256), kind 1 two N tiles without D1 (symmetric D1) with
// [D3(nt) | D3(nt + 1)], kind 2 one N tile without D1 (D3 alone, N = 128).
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

// Items w = blockIdx.x, blockIdx.x + gridDim.x, ...; per item the mode halves jh < JH, per half
// the row's work units: the sequence of all three roles.  Stage layout: U hi, U lo, B0 hi, B1
// hi, B0 lo, B1 lo.  SYM (every case a whole grid, at most 24 kept modes): symmetric D1.
template <int NMT, int JH, bool SYM>
__global__ void __launch_bounds__(192, 1)
    k_bfm_batch(const __grid_constant__ CUtensorMap tmUh, const __grid_constant__ CUtensorMap tmUl,
                const __grid_constant__ CUtensorMap tmGh, const __grid_constant__ CUtensorMap tmGl,
                const __grid_constant__ CUtensorMap tmSh, const __grid_constant__ CUtensorMap tmSl, const BParams p) {
    constexpr int NC = kBN / NMT;
    constexpr int BROWS = NC * NMT;
    constexpr int W = NMT * JH;
    constexpr int KINDS = SYM ? kKinds + 2 : kKinds;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t *bars = (uint64_t *)(smem + kStages * kStageBytes);
    uint64_t *full = bars, *empty = bars + kStages, *tfull = bars + 2 * kStages, *tempty = bars + 2 * kStages + 2;
    uint64_t *done = bars + 2 * kStages + 4;
    uint32_t *tmem_slot = (uint32_t *)(bars + 2 * kStages + 5);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int *err = p.err;
    if (blockIdx.x == 0 && threadIdx.x == 0) *p.t_start = gtime();

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
    const uint32_t tx_bytes = 2u * kTileBytes + 4u * (uint32_t)(BROWS * 128);

    if (warp == 0) {
        // ---------------- TMA producer ----------------
        if (lane == 0) {
            uint32_t it = 0;
            bool ok = true;
            for (int w = blockIdx.x; w < p.nitems && ok; w += gridDim.x) {
                const BItem im = p.items[w];
                const CaseP cs = p.cases[im.c];
                const Units un(im.r, cs.n_ntiles, SYM, NC);
                for (int jh = 0; jh < JH && ok; ++jh)
                    for (int u = 0; u < un.n && ok; ++u) {
                        int kind, nt;
                        un.at(u, kind, nt);
                        for (int kc = 0; kc < cs.nk && ok; ++kc, ++it) {
                            const int s = it % kStages;
                            const uint32_t ph = (it / kStages) & 1u;
                            if (!mbar_wait(&empty[s], ph ^ 1u, err, 1)) { ok = false; break; }
                            uint8_t *st = smem + s * kStageBytes;
                            mbar_expect_tx(&full[s], kind == 2 ? tx_bytes - 2u * (uint32_t)(BROWS * 128) : tx_bytes);
                            const int x = kc * kBK;
                            const int yu = cs.u_row0 + im.r * cs.Mp + im.mt * kBM;
                            tma_2d(st + 0 * kTileBytes, &tmUh, &full[s], x, yu);
                            tma_2d(st + 1 * kTileBytes, &tmUl, &full[s], x, yu);
                            const int ys = cs.s_row0 + jh * (2 * cs.nf - 1) * NMT + (im.r + nt * NC) * NMT;
                            if (kind == 0) {
                                const int yg = cs.g_row0 + jh * cs.nf * NMT + nt * BROWS;
                                tma_2d(st + 2 * kTileBytes, &tmGh, &full[s], x, yg);
                                tma_2d(st + 4 * kTileBytes, &tmGl, &full[s], x, yg);
                                tma_2d(st + 3 * kTileBytes, &tmSh, &full[s], x, ys);
                                tma_2d(st + 5 * kTileBytes, &tmSl, &full[s], x, ys);
                            } else if (kind == 1) {
                                tma_2d(st + 2 * kTileBytes, &tmSh, &full[s], x, ys);
                                tma_2d(st + 4 * kTileBytes, &tmSl, &full[s], x, ys);
                                tma_2d(st + 3 * kTileBytes, &tmSh, &full[s], x, ys + BROWS);
                                tma_2d(st + 5 * kTileBytes, &tmSl, &full[s], x, ys + BROWS);
                            } else {
                                tma_2d(st + 3 * kTileBytes, &tmSh, &full[s], x, ys);
                                tma_2d(st + 5 * kTileBytes, &tmSl, &full[s], x, ys);
                            }
                        }
                    }
            }
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
            for (int w = blockIdx.x; w < p.nitems && ok; w += gridDim.x) {
                const BItem im = p.items[w];
                const CaseP cs = p.cases[im.c];
                const Units un(im.r, cs.n_ntiles, SYM, NC);
                for (int jh = 0; jh < JH && ok; ++jh)
                    for (int u = 0; u < un.n && ok; ++u, ++tile) {
                        int kind, nt;
                        un.at(u, kind, nt);
                        const int buf = tile & 1;
                        const uint32_t tph = (tile >> 1) & 1u;
                        if (!mbar_wait(&tempty[buf], tph ^ 1u, err, 2)) { ok = false; break; }
                        fence_after();
                        const uint32_t d1 = tmem + buf * 256, d3 = d1 + 128;
                        for (int kc = 0; kc < cs.nk; ++kc, ++it) {
                            const int s = it % kStages;
                            const uint32_t ph = (it / kStages) & 1u;
                            if (!mbar_wait(&full[s], ph, err, 3)) { ok = false; break; }
                            fence_after();
                            const uint32_t base = su32(smem + s * kStageBytes);
                            const int nks = kc == cs.nk - 1 ? cs.ks_last : kBK / 16;
                            for (int ks = 0; ks < nks; ++ks) {
                                const uint32_t off = ks * 32;
                                const uint64_t uh = sdesc(base + 0 * kTileBytes + off), ul = sdesc(base + 1 * kTileBytes + off);
                                const uint32_t acc = (kc > 0 || ks > 0) ? 1u : 0u;
                                if (kind != 2) {  // B0 | B1, N = 256
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
                            mma_commit(&empty[s]);
                        }
                        if (!ok) break;
                        mma_commit(&tfull[buf]);
                    }
            }
            mma_commit(done);
            const uint64_t t0 = gtime();
            while (!mbar_try(done, 0) && gtime() - t0 < kWaitNs) {
            }
        }
        __syncwarp();
    } else {
        // ---------------- epilogue: FRF x weight, partial moments per case ----------------
        // One double-buffered FRF staging slot shared by the four warps (epi_sync orders it);
        // after a failed wait a warp walks the tile sequence without work, so every warp
        // reaches every epi_sync.
        const int quarter = warp & 3;
        const int et = threadIdx.x - 64;
        const int row = quarter * 32 + lane;
        const uint32_t lane_base = tmem + ((uint32_t)(quarter * 32) << 16);
        using HT = epi::HTile<NMT, JH>;
        HT *hbs = (HT *)(smem + kStages * kStageBytes + kBarBytes);
        float acc[KINDS][NMT];
        uint32_t tile = 0;
        bool ok = true;
        // FRF staging of unit u of row r of a case into the slot pair hb[0..1]
        auto stage_unit = [&](HT *hb, const CaseP &c, int r, int u) {
            const Units un(r, c.n_ntiles, SYM, NC);
            int kind, nt;
            un.at(u, kind, nt);
            epi::stage<NMT, JH>(hb, p.Hg + c.hg0, p.Hs + c.hs0, c.nf, r, nt * NC, et, 128);
            if (kind == 1) epi::stage<NMT, JH>(hb + 1, p.Hg + c.hg0, p.Hs + c.hs0, c.nf, r, (nt + 1) * NC, et, 128);
        };
        if (blockIdx.x < p.nitems) {
            const BItem i0 = p.items[blockIdx.x];
            stage_unit(hbs, p.cases[i0.c], i0.r, 0);
        }
        for (int w = blockIdx.x; w < p.nitems; w += gridDim.x) {
            const BItem im = p.items[w];
            const CaseP cs = p.cases[im.c];
            const int r = im.r;
            const int grow = im.mt * kBM + row;
            const bool vrow = grow < cs.nm * cs.nm;
            const int a = vrow ? grow / cs.nm : 0, b = vrow ? grow % cs.nm : 0;
            const float wvf = (float)cs.wval;
            const bool vect = cs.wmode == kWeightClassicVect, b1 = (r == 0 || r == cs.nf - 1);
            double *part = p.part + cs.part0 + grow;
            const Units un(r, cs.n_ntiles, SYM, NC);
            for (int jh = 0; jh < JH; ++jh) {
#pragma unroll
                for (int k = 0; k < KINDS; ++k)
#pragma unroll
                    for (int j = 0; j < NMT; ++j) acc[k][j] = 0.f;
                int since = 0;  // tiles accumulated since the last flush
                for (int u = 0; u < un.n; ++u, ++tile) {
                    int kind, nt;
                    un.at(u, kind, nt);
                    const int buf = tile & 1;
                    const uint32_t tph = (tile >> 1) & 1u;
                    epi::cp_async_wait_all();
                    epi::epi_sync();  // this unit's values are in; the other slot pair is no longer read
                    // stage the next unit: this half's next one, this item's next half, or the
                    // first unit of the CTA's next item
                    if (u + 1 < un.n) {
                        stage_unit(hbs + 2 * (buf ^ 1), cs, r, u + 1);
                    } else if (jh + 1 < JH) {
                        stage_unit(hbs + 2 * (buf ^ 1), cs, r, 0);
                    } else if (w + (int)gridDim.x < p.nitems) {
                        const BItem in = p.items[w + gridDim.x];
                        stage_unit(hbs + 2 * (buf ^ 1), p.cases[in.c], in.r, 0);
                    }
                    if (!ok) continue;
                    ok = __all_sync(0xffffffffu, mbar_wait(&tfull[buf], tph, err, 4));
                    if (!ok) continue;
                    fence_after();
                    const uint32_t ta = lane_base + buf * 256;
                    const HT *hb = hbs + 2 * buf;
                    if (kind == 1) {
                        epi::tile<NMT, JH, SYM, KINDS>(hb[0], ta, a, b, nt * NC, cs.nf, vect, b1, wvf, jh, acc, r, false,
                                                       0u);
                        epi::tile<NMT, JH, SYM, KINDS>(hb[1], ta, a, b, (nt + 1) * NC, cs.nf, vect, b1, wvf, jh, acc, r,
                                                       false);
                    } else {
                        epi::tile<NMT, JH, SYM, KINDS>(hb[0], ta, a, b, nt * NC, cs.nf, vect, b1, wvf, jh, acc, r,
                                                       kind == 0);
                    }
                    fence_before();
                    mbar_arrive(&tempty[buf]);
                    since += kind == 1 ? 2 : 1;
                    if ((since >= kFlushTiles || u + 1 == un.n) && vrow) {
#pragma unroll
                        for (int k = 0; k < KINDS; ++k)
#pragma unroll
                            for (int j = 0; j < NMT; ++j) {
                                if (acc[k][j] != 0.f)
                                    atomicAdd(part + (size_t)(k * W + jh * NMT + j) * cs.Mp, (double)acc[k][j]);
                                acc[k][j] = 0.f;
                            }
                        since = 0;
                    }
                }
            }
            if (!ok) continue;
            // this warp's share of the item is in the accumulators: count it, stamp the case
            __syncwarp();
            if (lane == 0) {
                __threadfence();
                const unsigned old = atomicAdd(p.done_cnt + im.c, 1u);
                if (old + 1 == 4u * cs.nitems) p.t_done[im.c] = gtime();
            }
        }
        epi::cp_async_wait_all();
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
}

// m3 of case c at out + out_off[c]: [m + nm n + nm^2 o] = 2 (T1 at (m,n,o) + T3 at (o,n,m) + T2 at (n,o,m))
template <int NMT, int KINDS>
__global__ void k_batch_reduce(const CaseP *__restrict__ cases, const long long *__restrict__ out_off,
                               const double *__restrict__ part, double *__restrict__ m3mf, double *__restrict__ m3mr) {
    const CaseP cs = cases[blockIdx.y];
    const int nm = cs.nm, nm3 = nm * nm * nm;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= nm3) return;
    const int m = x % nm, n = (x / nm) % nm, o = x / (nm * nm);
    const double *pc = part + cs.part0;
    auto s = [&](int kind, int aa, int bb, int j) { return pc[(size_t)(kind * NMT + j) * cs.Mp + aa * nm + bb]; };
    double mr = s(0, m, n, o) + s(1, o, n, m) + s(2, n, o, m);
    double mf = s(3, m, n, o) + s(4, o, n, m) + s(4, n, o, m);
    if (KINDS > kKinds) {  // symmetric D1: term 1 of the mirrored points
        mr += s(5, m, o, n);
        mf += s(6, m, o, n);
    }
    m3mr[out_off[blockIdx.y] + x] = 2.0 * mr;
    m3mf[out_off[blockIdx.y] + x] = 2.0 * mf;
}


// E form over a work list (cases of at most 48 kept modes on odd whole grids with the
// truncated sum): per (case, grid row p, row tile) item the row's units (pairs of N tiles of
// columns q >= p, once per mode half) of bsa_classic_e.cu's pipeline, whose three epilogue
// warpgroups add the six contributions of each E(f_p, f_q) element into the case's
// accumulators [9 kinds][W][Mp].  Only the U and G tables are read (no S table).
template <int NMT, int JH, bool RS = ecls::use_regsplit(NMT, JH)>
__global__ void __launch_bounds__(ecls::ELayout<RS>::threads, 1)  // 128 registers a thread at launch
    k_bfm_e_batch(const __grid_constant__ CUtensorMap tmUh, const __grid_constant__ CUtensorMap tmUl,
                  const __grid_constant__ CUtensorMap tmGh, const __grid_constant__ CUtensorMap tmGl, const BParams p) {
    using namespace ecls;
    constexpr int NC = kBN / NMT;
    constexpr int BROWS = NC * NMT;
    constexpr int W = NMT * JH;
    using L = ELayout<RS>;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t *bars = (uint64_t *)(smem + ecls::kStages * ecls::kStageBytes);
    uint64_t *full = bars, *empty = bars + ecls::kStages, *tfull = bars + 2 * ecls::kStages,
             *tempty = bars + 2 * ecls::kStages + 2;
    uint64_t *done = bars + 2 * ecls::kStages + 4;
    uint32_t *tmem_slot = (uint32_t *)(bars + 2 * ecls::kStages + 5);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int *err = p.err;
    if (blockIdx.x == 0 && threadIdx.x == 0) *p.t_start = gtime();

    for (int s = 0; s < ecls::kStages; ++s)
        for (int t = 2; t < 6; ++t) {
            uint8_t *tile = smem + s * ecls::kStageBytes + t * kTileBytes;
            for (int x = threadIdx.x; x < (128 - BROWS) * 128 / 16; x += blockDim.x)
                ((uint4 *)(tile + BROWS * 128))[x] = make_uint4(0, 0, 0, 0);
        }
    if (threadIdx.x == 0) {
        for (int s = 0; s < ecls::kStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&tfull[b], 1);
            mbar_init(&tempty[b], kEpi);
        }
        mbar_init(done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (warp == L::warp_mma) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(su32(tmem_slot)) : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tmem_slot;
    const uint32_t tx_bytes = 2u * kTileBytes + 4u * (uint32_t)(BROWS * 128);

    if (RS ? warp >= L::warp_tma : warp < L::epi_warp0) {
      if constexpr (RS) regs_producer();  // the whole producer warpgroup, before its warps part
      if (warp == L::warp_tma) {
        // ---------------- TMA producer ----------------
        if (lane == 0) {
            uint32_t it = 0;
            bool ok = true;
            for (int w = blockIdx.x; w < p.nitems && ok; w += gridDim.x) {
                const BItem im = p.items[w];
                const CaseP cs = p.cases[im.c];
                const int nu = n_units(im.r, cs.n_ntiles, NC), nt0 = im.r / NC;
                const int yu = cs.u_row0 + im.r * cs.Mp + im.mt * kBM;
                for (int jh = 0; jh < JH && ok; ++jh)
                for (int u = 0; u < nu && ok; ++u)
                    for (int kc = 0; kc < cs.nk && ok; ++kc, ++it) {
                        const int s = it % ecls::kStages;
                        const uint32_t ph = (it / ecls::kStages) & 1u;
                        if (!mbar_wait(&empty[s], ph ^ 1u, err, 1)) { ok = false; break; }
                        uint8_t *st = smem + s * ecls::kStageBytes;
                        mbar_expect_tx(&full[s], tx_bytes);
                        const int x = kc * kBK;
                        // rows past the case's columns read the next case's rows (masked)
                        const int yg = cs.g_row0 + jh * cs.nf * NMT + (nt0 + 2 * u) * BROWS;
                        tma_2d(st + 0 * kTileBytes, &tmUh, &full[s], x, yu);
                        tma_2d(st + 1 * kTileBytes, &tmUl, &full[s], x, yu);
                        tma_2d(st + 2 * kTileBytes, &tmGh, &full[s], x, yg);
                        tma_2d(st + 4 * kTileBytes, &tmGl, &full[s], x, yg);
                        tma_2d(st + 3 * kTileBytes, &tmGh, &full[s], x, yg + BROWS);
                        tma_2d(st + 5 * kTileBytes, &tmGl, &full[s], x, yg + BROWS);
                    }
            }
            const uint32_t last = it;
            for (uint32_t q = (last > (uint32_t)ecls::kStages ? last - ecls::kStages : 0); q < last; ++q) {
                const int s = q % ecls::kStages;
                const uint32_t ph = (q / ecls::kStages) & 1u;
                const uint64_t t0 = gtime();
                while (!mbar_try(&full[s], ph) && gtime() - t0 < kWaitNs) {
                }
            }
        }
        __syncwarp();
      } else if (warp == L::warp_mma) {
        // ---------------- MMA issuer ----------------
        if (lane == 0) {
            uint32_t it = 0, tile = 0;
            bool ok = true;
            for (int w = blockIdx.x; w < p.nitems && ok; w += gridDim.x) {
                const BItem im = p.items[w];
                const CaseP cs = p.cases[im.c];
                const int nu = n_units(im.r, cs.n_ntiles, NC) * JH;  // units of every mode half
                for (int u = 0; u < nu && ok; ++u, ++tile) {
                    const int buf = tile & 1;
                    const uint32_t tph = (tile >> 1) & 1u;
                    if (!mbar_wait(&tempty[buf], tph ^ 1u, err, 2)) { ok = false; break; }
                    fence_after();
                    const uint32_t d = tmem + buf * 256;
                    for (int kc = 0; kc < cs.nk; ++kc, ++it) {
                        const int s = it % ecls::kStages;
                        const uint32_t ph = (it / ecls::kStages) & 1u;
                        if (!mbar_wait(&full[s], ph, err, 3)) { ok = false; break; }
                        fence_after();
                        const uint32_t base = su32(smem + s * ecls::kStageBytes);
                        const int nks = kc == cs.nk - 1 ? cs.ks_last : kBK / 16;
                        for (int ks = 0; ks < nks; ++ks) {
                            const uint32_t off = ks * 32;
                            const uint64_t uh = sdesc(base + 0 * kTileBytes + off), ul = sdesc(base + 1 * kTileBytes + off);
                            const uint64_t bh = sdesc(base + 2 * kTileBytes + off), bl = sdesc(base + 4 * kTileBytes + off);
                            const uint32_t acc = (kc > 0 || ks > 0) ? 1u : 0u;
                            mma256(d, uh, bh, acc);
                            mma256(d, uh, bl, 1u);
                            mma256(d, ul, bh, 1u);
                        }
                        mma_commit(&empty[s]);
                    }
                    if (!ok) break;
                    mma_commit(&tfull[buf]);
                }
            }
            mma_commit(done);
            const uint64_t t0 = gtime();
            while (!mbar_try(done, 0) && gtime() - t0 < kWaitNs) {
            }
        }
        __syncwarp();
      }
    } else {
        if constexpr (RS) regs_epilogue();
        // ---------------- three epilogue warpgroups ----------------
        // After a failed wait a warp walks the unit sequence without work, so every warp
        // reaches every epi_sync384.
        const int wg = (warp - L::epi_warp0) >> 2;
        const int quarter = warp & 3;
        const int et = threadIdx.x - 32 * L::epi_warp0;
        const int row = quarter * 32 + lane;
        const uint32_t lane_base = tmem + ((uint32_t)(quarter * 32) << 16);
        using UT = UTile<NMT, JH>;
        UT *hbs = (UT *)(smem + ecls::kStages * ecls::kStageBytes + ecls::kBarBytes);
        const int k0 = wg * kKindsWG;
        f2x acc[kKindsWG][NMT / 2];  // modes j, j + 1 as FP32 lane pairs
#pragma unroll
        for (int k = 0; k < kKindsWG; ++k)
#pragma unroll
            for (int j = 0; j < NMT / 2; ++j) acc[k][j] = 0ull;
        // FRF staging of unit u of item im
        auto stage = [&](UT *dst, const BItem &im, int u) {
            const CaseP c = p.cases[im.c];
            EParams ep{};
            ep.nf = c.nf;
            ep.h = (c.nf - 1) / 2;
            ep.Hg = p.Hg + c.hg0;
            ep.Hs = p.Hs + c.hs0;
            ep.wmode = c.wmode;
            ep.wval = c.wval;
            stage_unit<NMT, JH>(dst, ep, im.r, im.r / NC + 2 * u, et, kEpi);
        };
        uint32_t tile = 0;
        bool ok = true;
        if (blockIdx.x < p.nitems) stage(hbs, p.items[blockIdx.x], 0);
        for (int w = blockIdx.x; w < p.nitems; w += gridDim.x) {
            const BItem im = p.items[w];
            const CaseP *csp = p.cases + im.c;  // fields read where used (register pressure)
            const int r = im.r;
            const int grow = im.mt * kBM + row;
            const int nm = csp->nm;
            const bool vrow = grow < nm * nm;
            const int a = vrow ? grow / nm : 0, b = vrow ? grow % nm : 0;
            const int nu = n_units(r, csp->n_ntiles, NC);
            int since = 0;
            for (int jh = 0; jh < JH; ++jh)
            for (int u = 0; u < nu; ++u, ++tile) {
                const int buf = tile & 1;
                const uint32_t tph = (tile >> 1) & 1u;
                epi::cp_async_wait_all();
                epi_sync384();  // this unit's values are in; the other slot is free
                if (u + 1 < nu)
                    stage(hbs + (buf ^ 1), im, u + 1);
                else if (jh + 1 < JH)
                    stage(hbs + (buf ^ 1), im, 0);
                else if (w + (int)gridDim.x < p.nitems)
                    stage(hbs + (buf ^ 1), p.items[w + gridDim.x], 0);
                if (!ok) continue;
                ok = __all_sync(0xffffffffu, mbar_wait(&tfull[buf], tph, err, 4));
                if (!ok) continue;
                fence_after();
                const UT &hb = hbs[buf];
                for (int h2 = 0; h2 < 2; ++h2)
                    unit_half<NMT, JH>(hb, lane_base + buf * 256 + h2 * 128, wg, a, b, h2 * NC, acc, jh * NMT);
                fence_before();
                mbar_arrive(&tempty[buf]);
                since += 2;
                // flush at the end of every mode half of every item (the next item may be
                // another case's, or leave this lane without a row)
                if (since >= kFlushTiles || u + 1 == nu) {
                    const int Mp = csp->Mp;
                    double *part = p.part + csp->part0 + grow;
#pragma unroll
                    for (int k = 0; k < kKindsWG; ++k)
#pragma unroll
                        for (int j = 0; j < NMT / 2; ++j) {
                            const float2 s2 = up2(acc[k][j]);
                            double *pk = part + (size_t)((k0 + k) * W + jh * NMT + 2 * j) * Mp;
                            if (vrow && s2.x != 0.f) atomicAdd(pk, (double)s2.x);
                            if (vrow && s2.y != 0.f) atomicAdd(pk + Mp, (double)s2.y);
                            acc[k][j] = 0ull;
                        }
                    since = 0;
                }
            }
            if (!ok) continue;
            // this warp's share of the item is in the accumulators: count it, stamp the case
            __syncwarp();
            if (lane == 0) {
                __threadfence();
                const unsigned old = atomicAdd(p.done_cnt + im.c, 1u);
                if (old + 1 == 12u * csp->nitems) p.t_done[im.c] = gtime();
            }
        }
        epi::cp_async_wait_all();
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == L::warp_mma) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
}

// m3 of case c from the E-form accumulators (kinds: 0 K_i, 1 K_iv, 2 F14, 3 K_iii, 4 K_v,
// 5 F35, 6 K_ii, 7 K_vi, 8 F26, each at the lane's (a, b) and j).
template <int W>
__global__ void k_batch_reduce_e(const CaseP *__restrict__ cases, const long long *__restrict__ out_off,
                                 const double *__restrict__ part, double *__restrict__ m3mf, double *__restrict__ m3mr) {
    const CaseP cs = cases[blockIdx.y];
    const int nm = cs.nm, nm3 = nm * nm * nm;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= nm3) return;
    const int m = x % nm, n = (x / nm) % nm, o = x / (nm * nm);
    const double *pc = part + cs.part0;
    auto s = [&](int kind, int aa, int bb, int j) { return pc[(size_t)(kind * W + j) * cs.Mp + aa * nm + bb]; };
    const double mr = s(0, m, n, o) + s(1, m, o, n) + s(3, o, n, m) + s(4, n, o, m) + s(6, n, m, o) + s(7, o, m, n);
    const double mf = s(2, m, n, o) + s(2, m, o, n) + s(5, o, n, m) + s(5, n, o, m) + s(8, n, m, o) + s(8, o, m, n);
    m3mr[out_off[blockIdx.y] + x] = 2.0 * mr;  // B_F = 2 (T1 + T2 + T3)
    m3mf[out_off[blockIdx.y] + x] = 2.0 * mf;
}

}  // namespace batch

// ------------------------------------------------------------------------------------
// Host side
// ------------------------------------------------------------------------------------
struct BatchCase {
    Settings set;
    int nnl = 0, psd_type = 0, nme = 0, K = 0;
    bool trunc = true;
    std::vector<int> modes;
    std::vector<double> hL, hQ, hCoh, hM, hK, hC, hWd3, hWd2;
    std::vector<float> hL32;
    std::vector<PsdNode> hPsd;
    std::vector<double> f;  // Classic grid
};

static std::vector<BatchCase> g_batch;

// Snapshot of the validated current inputs.
int Engine::batch_add(int *id) {
    int rc = validate();
    if (rc) return rc;
    if (set.onlyd) return fail(BSA_ERR_UNSUPPORTED, "the batched sweep runs the full-tensor Classic analysis");
    if (nme > 64) return fail(BSA_ERR_UNSUPPORTED, "the batched sweep supports at most 64 kept modes");
    BatchCase c;
    if ((rc = classic_grid(c.f))) return rc;
    if (c.f.size() < 2) return fail(BSA_ERR_ARG, "classic grid needs at least 2 frequencies");
    c.set = set;
    c.nnl = in.nnl;
    c.psd_type = in.psd_type;
    c.nme = nme;
    c.K = K;
    c.trunc = classic_trunc;
    c.modes = modes;
    c.hL = hL; c.hQ = hQ; c.hCoh = hCoh; c.hM = hM; c.hK = hK; c.hC = hC; c.hWd3 = hWd3; c.hWd2 = hWd2;
    c.hL32 = hL32; c.hPsd = hPsd;
    g_batch.push_back(std::move(c));
    if (id) *id = (int)g_batch.size() - 1;
    return BSA_OK;
}

// Makes case c the engine's problem (derived tables only; no caller arrays are read).
void Engine::batch_install(const BatchCase &c) {
    in = Inputs();
    in.nnl = c.nnl;
    in.psd_type = c.psd_type;
    set = c.set;
    classic_trunc = c.trunc;
    nme = c.nme;
    K = c.K;
    modes = c.modes;
    hL = c.hL; hQ = c.hQ; hCoh = c.hCoh; hM = c.hM; hK = c.hK; hC = c.hC; hWd3 = c.hWd3; hWd2 = c.hWd2;
    hL32 = c.hL32; hPsd = c.hPsd;
    derived_ok = true;
    dev_uploaded = false;
}

int Engine::batch_run(double *m3mf, double *m3mr, double *m2mr, double *case_ms, double *total_ms) {
    using namespace batch;
    const int nc = (int)g_batch.size();
    if (nc == 0) return fail(BSA_ERR_STATE, "empty batch");
    kernels = 0;
    graph_launches = 0;
    h2d = d2h = 0;
    std::vector<long long> off3(nc), off2(nc);
    long long t3 = 0, t2 = 0;
    for (int c = 0; c < nc; ++c) {
        off3[c] = t3;
        off2[c] = t2;
        t3 += (long long)g_batch[c].nme * g_batch[c].nme * g_batch[c].nme;
        t2 += (long long)g_batch[c].nme * g_batch[c].nme;
    }
    int rc = ensure_stream();
    if (rc) return rc;
    cudaError_t e;
    int dev = 0, nsm = 0;
    if ((e = cudaGetDevice(&dev)) || (e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev)))
        return cuda_fail(e, "device query");
    // groups: same NMT, cases in K order, device bytes bounded
    // FRF-table width of a case; above 32 modes two halves of 32 (JH = 2)
    std::vector<int> order(nc);
    for (int c = 0; c < nc; ++c) order[c] = c;
    // E form (bsa_classic_e.cu) for cases of at most 48 kept modes on odd grids with the
    // truncated sum; those form groups of their own
    auto e_ok = [&](int c) {
        const BatchCase &b = g_batch[c];
        return use_e_form && b.nme <= kEFormMaxModes && b.trunc && (b.f.size() & 1) != 0 &&
               plan_prefer_e(b.nme, b.K, (int)b.f.size());
    };
    // group width: the FRF-table width of the D1 / D3 form, or of the E form (8, 16, 24; 32 and
    // 48 as two mode halves of 16 and 24)
    auto width = [&](int c) {
        const BatchCase &b = g_batch[c];
        return e_ok(c) ? plan_e_width(b.nme, b.K, (int)b.f.size()) : plan_d_width(b.nme, b.K, (int)b.f.size());
    };
    std::sort(order.begin(), order.end(), [&](int x, int y) {
        const int a = width(x), b = width(y);
        if (a != b) return a < b;
        if (e_ok(x) != e_ok(y)) return e_ok(x);
        return g_batch[x].K < g_batch[y].K;
    });
    // the caller's problem is put back once the sweep is done
    BatchCase saved;
    saved.set = set;
    saved.nnl = in.nnl;
    saved.psd_type = in.psd_type;
    saved.nme = nme;
    saved.K = K;
    saved.trunc = classic_trunc;
    saved.modes = modes;
    saved.hL = hL; saved.hQ = hQ; saved.hCoh = hCoh; saved.hM = hM; saved.hK = hK; saved.hC = hC;
    saved.hWd3 = hWd3; saved.hWd2 = hWd2; saved.hL32 = hL32; saved.hPsd = hPsd;
    const Inputs saved_in = in;
    const bool saved_ok = derived_ok;
    struct Restore {
        Engine &E;
        const BatchCase &c;
        const Inputs &in;
        bool ok;
        ~Restore() {
            E.batch_install(c);
            E.in = in;
            E.derived_ok = ok;
        }
    } restore{*this, saved, saved_in, saved_ok};
    std::vector<double> h3f(t3), h3r(t3), h2(t2 * 3);
    std::vector<double> lat(nc, 0.0);
    double total = 0.0, gemm = 0.0, points = 0.0;
    const double budget = 24e9;
    size_t g0 = 0;
    while (g0 < order.size()) {
        const int Wd = width(order[g0]);
        const bool eform = e_ok(order[g0]);
        int NMT;
        if (eform) {
            const BatchCase &c0 = g_batch[order[g0]];
            NMT = Wd / plan_e_split(Wd, c0.nme, c0.K, (int)c0.f.size());
        } else {
            NMT = Wd > 32 ? 32 : Wd;
        }
        const int JH = Wd / NMT;
        size_t g1 = g0;
        double rows = 0.0;
        while (g1 < order.size() && width(order[g1]) == Wd && e_ok(order[g1]) == eform) {
            // U, G and S rows of the case; hi + lo bf16 at the group's K stride, which is
            // this case's (the group is in K order)
            const BatchCase &c = g_batch[order[g1]];
            const double Kp = (double)(((c.K + kBK - 1) / kBK) * kBK);
            const double Mp = (double)(((c.nme * c.nme + kBM - 1) / kBM) * kBM);
            const double nf = (double)c.f.size();
            const double add = nf * Mp + (double)JH * (eform ? nf : 3 * nf - 1) * NMT;
            if (g1 > g0 && 4.0 * Kp * (rows + add) > budget) break;
            rows += add;
            ++g1;
        }
        // common K stride: the largest case of the group (the group is in K order)
        const int Kmax = g_batch[order[g1 - 1]].K;
        const int Kp = ((Kmax + kBK - 1) / kBK) * kBK;
        std::vector<CaseP> cp(g1 - g0);
        std::vector<BItem> items;
        long long urows = 0, grows = 0, srows = 0, hg = 0, hs = 0, parts = 0;
        for (size_t k = g0; k < g1; ++k) {
            const BatchCase &c = g_batch[order[k]];
            CaseP &q = cp[k - g0];
            const int nf = (int)c.f.size();
            q.nf = nf;
            q.nm = c.nme;
            q.Mp = ((c.nme * c.nme + kBM - 1) / kBM) * kBM;
            q.MT = q.Mp / kBM;
            q.nk = ((c.K + kBK - 1) / kBK);
            q.ks_last = (c.K - (q.nk - 1) * kBK + 15) / 16;
            q.n_ntiles = (nf + (kBN / NMT) - 1) / (kBN / NMT);
            const bool scalar = c.set.scalar != 0 ||
                                (c.set.test == 0 && c.set.ibisp && (long long)nf * nf * c.nme * c.nme * c.nme > 1000000000LL);
            q.wmode = scalar ? kWeightUniform : kWeightClassicVect;
            double delta = c.f[1] - c.f[0];
            if (c.set.defsc == 1) delta *= kPi2;
            q.wval = delta * delta;
            q.u_row0 = (int)urows;
            q.g_row0 = (int)grows;
            q.s_row0 = (int)srows;
            q.hg0 = (int)hg;
            q.hs0 = (int)hs;
            q.part0 = parts;
            q.nitems = (unsigned)(nf * q.MT);
            urows += (long long)nf * q.Mp;
            grows += (long long)JH * nf * NMT;
            if (!eform) srows += (long long)JH * (2 * nf - 1) * NMT;
            hg += (long long)nf * Wd;
            hs += (long long)(2 * nf - 1) * Wd;
            parts += (long long)(eform ? ecls::kKinds : Wd <= 24 ? kKinds + 2 : kKinds) * Wd * q.Mp;
            for (int r = 0; r < nf; ++r)
                for (int mt = 0; mt < q.MT; ++mt) items.push_back(BItem{(int)(k - g0), r, mt, 0});
        }
        if (urows > 0x7fffffffLL || srows > 0x7fffffffLL) return fail(BSA_ERR_ARG, "batch group too large");
        const size_t uel = (size_t)urows * Kp, gel = (size_t)grows * Kp, sel = (size_t)srows * Kp;
        if ((e = dMixA.reserve(2 * uel * 2)) || (e = dMixB.reserve(2 * (gel + sel) * 2)) ||
            (e = dMixH.reserve(sizeof(float2) * (size_t)(hg + hs) + 256)) ||
            (e = dMixPart.reserve(sizeof(double) * (size_t)parts + 4096)) ||
            (e = dMshIdx.reserve(sizeof(CaseP) * cp.size() + sizeof(BItem) * items.size() +
                                 (sizeof(unsigned) + 2 * sizeof(unsigned long long) + sizeof(long long)) * cp.size() + 1024)) ||
            (e = dMshT.reserve(sizeof(double) * 3 * (size_t)t2 + 64)))
            return cuda_fail(e, "allocating batch operands");
        __nv_bfloat16 *Uh = dMixA.as<__nv_bfloat16>(), *Ul = Uh + uel;
        __nv_bfloat16 *Gh = dMixB.as<__nv_bfloat16>(), *Gl = Gh + gel, *Sh = Gl + gel, *Sl = Sh + sel;
        float2 *Hg = dMixH.as<float2>(), *Hs = Hg + hg;
        double *part = dMixPart.as<double>();
        int *derr = (int *)(part + parts);
        char *ib = (char *)dMshIdx.p;
        CaseP *d_cases = (CaseP *)ib;
        BItem *d_items = (BItem *)(((uintptr_t)(d_cases + cp.size()) + 15) & ~(uintptr_t)15);
        unsigned *d_cnt = (unsigned *)(d_items + items.size());
        unsigned long long *d_tdone = (unsigned long long *)(((uintptr_t)(d_cnt + cp.size()) + 15) & ~(uintptr_t)15);
        unsigned long long *d_tstart = d_tdone + cp.size();
        long long *d_off = (long long *)(d_tstart + 1);
        double *d_m2 = dMshT.as<double>();
        if ((e = cudaEventRecord(ev2, stream))) return cuda_fail(e, "event");
        if ((e = cudaMemsetAsync(part, 0, sizeof(double) * (size_t)parts + sizeof(int), stream)) ||
            (e = cudaMemsetAsync(d_cnt, 0, sizeof(unsigned) * cp.size(), stream)) ||
            (e = cudaMemsetAsync(d_tdone, 0, sizeof(unsigned long long) * (cp.size() + 1), stream)))
            return cuda_fail(e, "batch memset");
        // per case: its tables, A(f) in FP32, operands into the group tables, m2
        for (size_t k = g0; k < g1; ++k) {
            const BatchCase &c = g_batch[order[k]];
            const CaseP &q = cp[k - g0];
            batch_install(c);
            if ((rc = upload_problem())) return rc;
            const int nf = q.nf;
            std::vector<double> ftab = c.f;
            if (!c.trunc)
                for (int s = 0; s < 2 * nf - 1; ++s) ftab.push_back(2.0 * c.f[0] + s * (c.f[1] - c.f[0]));
            if ((rc = build_atable(ftab, true))) return rc;
            const float *A = dA32.as<float>();
            if ((e = mixed::prep_u(stream, nf, c.nme, c.K, Kp, q.Mp, A, dQ.as<double>(), Uh + (size_t)q.u_row0 * Kp,
                                   Ul + (size_t)q.u_row0 * Kp)) ||
                (e = mixed::prep_h(stream, nf, c.nme, Wd, dFreq.as<double>(), frf(), Hg + q.hg0, Hs + q.hs0, eform)))
                return cuda_fail(e, "batch operand preparation");
            for (int jh = 0; jh < JH; ++jh) {
                const size_t og = ((size_t)q.g_row0 + (size_t)jh * nf * NMT) * Kp;
                const size_t os = ((size_t)q.s_row0 + (size_t)jh * (2 * nf - 1) * NMT) * Kp;
                if ((e = mixed::prep_b(stream, nf, c.nme, NMT, jh * NMT, c.K, Kp, nf, (nf - 1) / 2, c.trunc ? 1 : 0, nf,
                                       0, A, Gh + og, Gl + og)) ||
                    (!eform && (e = mixed::prep_b(stream, 2 * nf - 1, c.nme, NMT, jh * NMT, c.K, Kp, nf, (nf - 1) / 2,
                                       c.trunc ? 1 : 0, nf, 1, A, Sh + os, Sl + os))))
                    return cuda_fail(e, "batch operand preparation");
            }
            // second-order moments (FP64 over the FP32 A table), rectangle or trapezoid weights
            double delta = c.f[1] - c.f[0];
            if (c.set.defsc == 1) delta *= kPi2;
            std::vector<double> wf(nf, delta);
            if (q.wmode == kWeightClassicVect) { wf[0] = delta / 2; wf[nf - 1] = delta / 2; }
            const int nm2 = c.nme * c.nme;
            if ((e = upload(dWf, wf, stream)) || (e = dPsdF.reserve(sizeof(double) * (size_t)nf * nm2)))
                return cuda_fail(e, "batch m2");
            double *m2o = d_m2 + 3 * off2[order[k]];
            if ((e = launch_force_psd32(stream, nf, (int)c.set.tc.size(), c.nnl, c.nme, dL32.as<float>(), A,
                                        dPsdF.as<double>())) ||
                (e = launch_m2(stream, 0, nf, c.nme, 0, dFreq.as<double>(), dWf.as<double>(), dPsdF.as<double>(), frf(),
                               m2o, m2o + nm2, m2o + 2 * nm2)))
                return cuda_fail(e, "batch m2");
            kernels += 4 + (eform ? 1 : 2) * JH;
        }
        std::vector<long long> offs(cp.size());
        for (size_t k = g0; k < g1; ++k) offs[k - g0] = off3[order[k]];
        if ((e = cudaMemcpyAsync(d_cases, cp.data(), sizeof(CaseP) * cp.size(), cudaMemcpyHostToDevice, stream)) ||
            (e = cudaMemcpyAsync(d_items, items.data(), sizeof(BItem) * items.size(), cudaMemcpyHostToDevice, stream)) ||
            (e = cudaMemcpyAsync(d_off, offs.data(), sizeof(long long) * offs.size(), cudaMemcpyHostToDevice, stream)))
            return cuda_fail(e, "batch tables");
        CUtensorMap maps[6];
        const int BROWS = (kBN / NMT) * NMT;
        if (!make_map(&maps[0], Uh, Kp, (uint64_t)urows, kBM) || !make_map(&maps[1], Ul, Kp, (uint64_t)urows, kBM) ||
            !make_map(&maps[2], Gh, Kp, (uint64_t)grows, BROWS) || !make_map(&maps[3], Gl, Kp, (uint64_t)grows, BROWS) ||
            (!eform && (!make_map(&maps[4], Sh, Kp, (uint64_t)srows, BROWS) ||
                        !make_map(&maps[5], Sl, Kp, (uint64_t)srows, BROWS))))
            return fail(BSA_ERR_CUDA, "cuTensorMapEncodeTiled failed");
        BParams prm{d_items, (int)items.size(), d_cases, Hg, Hs, part, d_cnt, d_tdone, d_tstart, derr};
        const size_t smem = kSmem;
        const int grid = (int)std::min<long long>((long long)items.size(), nsm);
        if ((e = cudaEventRecord(evg0, stream))) return cuda_fail(e, "event");
        auto launch = [&](auto kern) {
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            kern<<<grid, 192, smem, stream>>>(maps[0], maps[1], maps[2], maps[3], maps[4], maps[5], prm);
        };
        // the warp layout of each instantiation (register split for the 48-mode width) is its
        // template default; a split kernel is launched only at its full launch registers
        auto launch_e = [&](auto kern, size_t ut, bool rs) -> bool {  // UTile bytes ut: fits with the stages (static_assert in bsa_classic_e.cu)
            const size_t sm = (size_t)ecls::kStages * ecls::kStageBytes + 1024 + ecls::kBarBytes + 2 * ut;
            cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
            if (rs && ecls::regsplit_check(kern) != cudaSuccess) return false;
            kern<<<grid, rs ? ecls::ELayout<true>::threads : ecls::ELayout<false>::threads, sm, stream>>>(
                maps[0], maps[1], maps[2], maps[3], prm);
            return true;
        };
        bool launched = true;
        if (eform) {
            switch (NMT * 10 + JH) {
            case 81: launched = launch_e(k_bfm_e_batch<8, 1>, sizeof(ecls::UTile<8, 1>), ecls::use_regsplit(8, 1)); break;
            case 82: launched = launch_e(k_bfm_e_batch<8, 2>, sizeof(ecls::UTile<8, 2>), ecls::use_regsplit(8, 2)); break;
            case 122: launched = launch_e(k_bfm_e_batch<12, 2>, sizeof(ecls::UTile<12, 2>), ecls::use_regsplit(12, 2)); break;
            case 161: launched = launch_e(k_bfm_e_batch<16, 1>, sizeof(ecls::UTile<16, 1>), ecls::use_regsplit(16, 1)); break;
            case 162: launched = launch_e(k_bfm_e_batch<16, 2>, sizeof(ecls::UTile<16, 2>), ecls::use_regsplit(16, 2)); break;
            case 241: launched = launch_e(k_bfm_e_batch<24, 1>, sizeof(ecls::UTile<24, 1>), ecls::use_regsplit(24, 1)); break;
            default: launched = launch_e(k_bfm_e_batch<24, 2>, sizeof(ecls::UTile<24, 2>), ecls::use_regsplit(24, 2)); break;
            }
            if (!launched) return fail(BSA_ERR_STATE, "batched E-form kernel: launch registers below its register split");
        } else {
            switch (Wd) {
            case 8: launch(k_bfm_batch<8, 1, true>); break;
            case 16: launch(k_bfm_batch<16, 1, true>); break;
            case 24: launch(k_bfm_batch<24, 1, true>); break;
            case 32: launch(k_bfm_batch<32, 1, false>); break;
            default: launch(k_bfm_batch<32, 2, false>); break;
            }
        }
        if ((e = cudaGetLastError())) return cuda_fail(e, "batched tcgen05 contraction kernel");
        if ((e = cudaEventRecord(evg1, stream))) return cuda_fail(e, "event");
        // reduce into the case-ordered output (device copy of the whole output, rows of this group)
        if ((e = dOut.reserve(sizeof(double) * 2 * (size_t)t3))) return cuda_fail(e, "out");
        double *o = dOut.as<double>();
        int maxnm3 = 1;
        for (const CaseP &q : cp) maxnm3 = std::max(maxnm3, q.nm * q.nm * q.nm);
        dim3 rg((maxnm3 + 127) / 128, (unsigned)cp.size());
        if (eform) switch (Wd) {
        case 8: k_batch_reduce_e<8><<<rg, 128, 0, stream>>>(d_cases, d_off, part, o, o + t3); break;
        case 16: k_batch_reduce_e<16><<<rg, 128, 0, stream>>>(d_cases, d_off, part, o, o + t3); break;
        case 24: k_batch_reduce_e<24><<<rg, 128, 0, stream>>>(d_cases, d_off, part, o, o + t3); break;
        case 32: k_batch_reduce_e<32><<<rg, 128, 0, stream>>>(d_cases, d_off, part, o, o + t3); break;
        default: k_batch_reduce_e<48><<<rg, 128, 0, stream>>>(d_cases, d_off, part, o, o + t3); break;
        }
        else switch (Wd) {
        case 8: k_batch_reduce<8, kKinds + 2><<<rg, 128, 0, stream>>>(d_cases, d_off, part, o, o + t3); break;
        case 16: k_batch_reduce<16, kKinds + 2><<<rg, 128, 0, stream>>>(d_cases, d_off, part, o, o + t3); break;
        case 24: k_batch_reduce<24, kKinds + 2><<<rg, 128, 0, stream>>>(d_cases, d_off, part, o, o + t3); break;
        case 32: k_batch_reduce<32, kKinds><<<rg, 128, 0, stream>>>(d_cases, d_off, part, o, o + t3); break;
        default: k_batch_reduce<64, kKinds><<<rg, 128, 0, stream>>>(d_cases, d_off, part, o, o + t3); break;
        }
        if ((e = cudaGetLastError())) return cuda_fail(e, "batch reduction");
        kernels += 2;
        std::vector<unsigned long long> td(cp.size() + 1);
        int herr = 0;
        if ((e = cudaMemcpyAsync(td.data(), d_tdone, sizeof(unsigned long long) * (cp.size() + 1), cudaMemcpyDeviceToHost,
                                 stream)) ||
            (e = cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, stream)) ||
            (e = cudaEventRecord(ev1, stream)) || (e = cudaStreamSynchronize(stream)))
            return cuda_fail(e, "batch run");
        if (herr) return fail(BSA_ERR_TIMEOUT, "batched kernel: a pipeline wait ran out of its budget (role %d)", herr);
        // results of this group: moments and m2 of its cases
        for (size_t k = g0; k < g1; ++k) {
            const int c = order[k];
            const long long n3 = (long long)g_batch[c].nme * g_batch[c].nme * g_batch[c].nme;
            const long long n2 = (long long)g_batch[c].nme * g_batch[c].nme;
            if ((e = cudaMemcpy(h3f.data() + off3[c], o + off3[c], sizeof(double) * n3, cudaMemcpyDeviceToHost)) ||
                (e = cudaMemcpy(h3r.data() + off3[c], o + t3 + off3[c], sizeof(double) * n3, cudaMemcpyDeviceToHost)) ||
                (e = cudaMemcpy(h2.data() + 3 * off2[c], d_m2 + 3 * off2[c], sizeof(double) * 3 * n2,
                                cudaMemcpyDeviceToHost)))
                return cuda_fail(e, "batch results");
            lat[c] = (double)(td[k - g0] - td[cp.size()]) * 1e-6;  // ms from the launch start
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, ev2, ev1);
        total += ms;
        cudaEventElapsedTime(&ms, evg0, evg1);
        gemm += ms;
        for (const CaseP &q : cp) points += (double)q.nf * q.nf;
        g0 = g1;
    }
    for (int c = 0; c < nc; ++c) {
        const long long n3 = (long long)g_batch[c].nme * g_batch[c].nme * g_batch[c].nme;
        const long long n2 = (long long)g_batch[c].nme * g_batch[c].nme;
        if (m3mf) std::memcpy(m3mf + off3[c], h3f.data() + off3[c], sizeof(double) * n3);
        if (m3mr) std::memcpy(m3mr + off3[c], h3r.data() + off3[c], sizeof(double) * n3);
        if (m2mr) std::memcpy(m2mr + off2[c], h2.data() + 3 * off2[c] + n2, sizeof(double) * n2);
        if (case_ms) case_ms[c] = lat[c];
    }
    if (total_ms) *total_ms = total;
    last_ms = total;
    last_ms_contraction = total;
    last_ms_gemm = gemm;
    last_points = points;
    return BSA_OK;
}

}  // namespace bsa

using bsa::eng;

extern "C" {

int bsa_gpu_batchAdd(int *case_id) {
    bsa::Engine &E = eng();
    if (E.halted) return BSA_ERR_STATE;
    return E.batch_add(case_id);
}

int bsa_gpu_batchCase(int c, int *nm, int *nf) {
    if (c < 0 || c >= (int)bsa::g_batch.size()) return BSA_ERR_ARG;
    if (nm) *nm = bsa::g_batch[c].nme;
    if (nf) *nf = (int)bsa::g_batch[c].f.size();
    return BSA_OK;
}

int bsa_gpu_batchRun(double *m3mf, double *m3mr, double *m2mr, double *case_ms, double *total_ms) {
    bsa::Engine &E = eng();
    if (E.halted) return BSA_ERR_STATE;
    return E.batch_run(m3mf, m3mr, m2mr, case_ms, total_ms);
}

int bsa_gpu_batchClear(void) {
    bsa::g_batch.clear();
    return BSA_OK;
}

}  // extern "C"
