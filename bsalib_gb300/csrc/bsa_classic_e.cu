// bsa_classic_e.cu -- the Classic split-precision contraction in its E form.
//
// With A(f) = S(f) L and E(x, y)[(a, b), j] = sum_k Q[k][a] A(x)[k][b] A(y)[k][j], the three
// terms of the BFM at a grid point (f1, f2) (functionsImpl.F90:1494-1538) are
//   T1(f1, f2)[m, n, o] = E(f1, f2)[(m, n), o]
//   T2(f1, f2)[m, n, o] = E(f1 + f2, f2)[(n, m), o]
//   T3(f1, f2)[m, n, o] = E(f1, f1 + f2)[(o, n), m]
// and E is symmetric: E(x, y)[(a, b), j] = E(y, x)[(a, j), b].  On the Classic grid
// (f_i = (i - h) df, h = (nf - 1) / 2) with S(f1 + f2) read as zero beyond the grid (the
// reference's truncation, BsaClassicImpl.F90:103-119), every E that T2 and T3 need is an E of
// two grid frequencies.  So the whole grid needs E(f_p, f_q) for q >= p only: one GEMM family
// over half the grid pairs instead of D1 on half and D3 on all of them (a third of the MMAs of
// bsa_mixed.cu's form).  Each element x = E(f_p, f_q)[(a, b), j] (u = f_p, v = f_q) then feeds
//   (i)   T1 at (p, q):              m n o = a b j   Re[H_a(u) H_b(v) conj H_j(u + v)]
//   (iv)  T1 at (q, p), q > p:       a j b           Re[H_a(v) H_j(u) conj H_b(u + v)]
//   (iii) T3 at (p, c), f_c = v - u: j b a           Re[H_j(u) H_b(v - u) conj H_a(v)]
//   (v)   T2 at (c, p):              j a b           Re[H_j(v - u) H_a(u) conj H_b(v)]
//   (ii)  T2 at (d, q), f_d = u - v: b a j           Re[H_b(u - v) H_a(v) conj H_j(u)]
//   (vi)  T3 at (q, d):              b j a           Re[H_b(v) H_j(u - v) conj H_a(u)]
// each with its point's integration weight; (iii)-(vi) exist where q - p <= h.  A diagonal
// element (q = p) feeds all six at half weight (its transpose is in the same tile).
//
// The kernel is bsa_mixed.cu's pipeline (a TMA warp, a tcgen05 MMA warp, BF16x3, FP32 TMEM
// accumulators, 2 stages of 96 KB, N = 256 MMAs over two N tiles of grid columns) with three
// epilogue warpgroups on the same TMEM buffer, one per weight: the first accumulates (i), (iv)
// and their force moment, the second (iii), (v) and theirs, the third (ii), (vi) and theirs
// (warp layouts, plain or register split: ELayout in bsa_eform.cuh).  The FRF values a unit
// reads (H at the row, at the unit's columns, at the row + column sums and at the column - row
// and row - column differences) are staged in shared memory one unit ahead.  Used for whole-grid launches with the truncated sum, up to
// 48 kept modes (above 24 the G rows hold one half of the modes, JH = 2, and each unit is
// swept once per half; a width of 16 or 24 may also run as two halves of 8 or 12, which halves
// the epilogue's accumulators at the same MMA work, the tile plan's choice) and no central
// symmetry; bsa_mixed.cu's form otherwise.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "../../include/bsa_gpu.h"
#include "bsa_engine.cuh"
#include "bsa_eform.cuh"
#include "bsa_epi.cuh"
#include "bsa_mixed.cuh"
#include "bsa_tc.cuh"

namespace bsa {
namespace ecls {

using namespace tc;

// SAMPLE = true is the diagnostic instantiation: the same products, with the epilogue writing
// the unweighted per-point bispectra of the grid points P.slot lists (unit_half_sample) instead
// of the weighted moment partials.
template <int NMT, int JH, bool SAMPLE, bool RS = use_regsplit(NMT, JH)>
__global__ void __launch_bounds__(ELayout<RS>::threads, 1)  // 128 registers a thread at launch
    k_bfm_e(const __grid_constant__ CUtensorMap tmUh, const __grid_constant__ CUtensorMap tmUl,
            const __grid_constant__ CUtensorMap tmGh, const __grid_constant__ CUtensorMap tmGl, const EParams P) {
    constexpr int NC = kBN / NMT;
    constexpr int BROWS = NC * NMT;
    constexpr int W = NMT * JH;
    using L = ELayout<RS>;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t *bars = (uint64_t *)(smem + kStages * kStageBytes);
    uint64_t *full = bars, *empty = bars + kStages, *tfull = bars + 2 * kStages, *tempty = bars + 2 * kStages + 2;
    uint64_t *done = bars + 2 * kStages + 4;
    uint32_t *tmem_slot = (uint32_t *)(bars + 2 * kStages + 5);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int *err = P.err;

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

    const int mt = blockIdx.x % P.MT;
    // grid rows p of this CTA: every (grid / MT)-th row of the shard's rows p0 + pstep l
    const int pstep = P.pstep_m1 + 1;
    const int rstep = (gridDim.x / P.MT) * pstep;
    const int r0 = P.p0 + (blockIdx.x / P.MT) * pstep;
    const uint32_t tx_bytes = 2u * kTileBytes + 4u * (uint32_t)(BROWS * 128);

    if (RS ? warp >= L::warp_tma : warp < L::epi_warp0) {
      if constexpr (RS) regs_producer();  // the whole producer warpgroup, before its warps part
      if (warp == L::warp_tma) {
        // ---------------- TMA producer ----------------
        if (lane == 0) {
            uint32_t it = 0;
            bool ok = true;
            for (int p = r0; p < P.nf && ok; p += rstep) {
                const int nu = n_units(p, P.n_ntiles, NC), nt0 = p / NC;
                for (int jh = 0; jh < JH && ok; ++jh)
                for (int u = 0; u < nu && ok; ++u)
                    for (int kc = 0; kc < P.nk && ok; ++kc, ++it) {
                        const int s = it % kStages;
                        const uint32_t ph = (it / kStages) & 1u;
                        if (!mbar_wait(&empty[s], ph ^ 1u, err, 1)) { ok = false; break; }
                        uint8_t *st = smem + s * kStageBytes;
                        mbar_expect_tx(&full[s], tx_bytes);
                        const int x = kc * kBK;
                        const int yu = p * P.Mp + mt * kBM;
                        // G rows of mode half jh; rows past a half's columns read the next
                        // half's rows or zeros (masked in the epilogue)
                        const int yg = jh * P.nf * NMT + (nt0 + 2 * u) * BROWS;
                        tma_2d(st + 0 * kTileBytes, &tmUh, &full[s], x, yu);
                        tma_2d(st + 1 * kTileBytes, &tmUl, &full[s], x, yu);
                        tma_2d(st + 2 * kTileBytes, &tmGh, &full[s], x, yg);
                        tma_2d(st + 4 * kTileBytes, &tmGl, &full[s], x, yg);
                        tma_2d(st + 3 * kTileBytes, &tmGh, &full[s], x, yg + BROWS);
                        tma_2d(st + 5 * kTileBytes, &tmGl, &full[s], x, yg + BROWS);
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
      } else if (warp == L::warp_mma) {
        // ---------------- MMA issuer ----------------
        if (lane == 0) {
            uint32_t it = 0, tile = 0;
            bool ok = true;
            for (int p = r0; p < P.nf && ok; p += rstep) {
                const int nu = n_units(p, P.n_ntiles, NC) * JH;  // units of every mode half
                for (int u = 0; u < nu && ok; ++u, ++tile) {
                    const int buf = tile & 1;
                    const uint32_t tph = (tile >> 1) & 1u;
                    if (!mbar_wait(&tempty[buf], tph ^ 1u, err, 2)) { ok = false; break; }
                    fence_after();
                    const uint32_t d = tmem + buf * 256;
                    for (int kc = 0; kc < P.nk; ++kc, ++it) {
                        const int s = it % kStages;
                        const uint32_t ph = (it / kStages) & 1u;
                        if (!mbar_wait(&full[s], ph, err, 3)) { ok = false; break; }
                        fence_after();
                        const uint32_t base = su32(smem + s * kStageBytes);
                        const int nks = kc == P.nk - 1 ? P.ks_last : kBK / 16;
#pragma unroll
                        for (int ks = 0; ks < kBK / 16; ++ks) {
                            if (ks >= nks) break;
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
                    if (!(P.test_skip_tile1 == (int)tile + 1 && blockIdx.x == 0)) mma_commit(&tfull[buf]);
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
        const int wg = (warp - L::epi_warp0) >> 2;
        const int quarter = warp & 3;               // TMEM lane quarter of this warp
        const int et = threadIdx.x - 32 * L::epi_warp0;  // 0 .. 383
        const int row = quarter * 32 + lane;
        const int grow = mt * kBM + row;
        const bool vrow = grow < P.nm * P.nm;
        const int a = vrow ? grow / P.nm : 0, b = vrow ? grow % P.nm : 0;
        const uint32_t lane_base = tmem + ((uint32_t)(quarter * 32) << 16);
        using UT = UTile<NMT, JH>;
        UT *hbs = (UT *)(smem + kStages * kStageBytes + kBarBytes);
        double *part = P.part + (size_t)blockIdx.x * kKinds * W * 128 + row;
        const int k0 = wg * kKindsWG;
        for (int k = 0; k < kKindsWG * W; ++k) part[(size_t)(k0 * W + k) * 128] = 0.0;
        f2x acc[kKindsWG][NMT / 2];  // modes j, j + 1 as FP32 lane pairs
#pragma unroll
        for (int k = 0; k < kKindsWG; ++k)
#pragma unroll
            for (int j = 0; j < NMT / 2; ++j) acc[k][j] = 0ull;
        uint32_t tile = 0;
        bool ok = true;
        int since = 0;
        if (r0 < P.nf) stage_unit<NMT, JH>(hbs, P, r0, r0 / NC, et, kEpi);
        for (int p = r0; p < P.nf; p += rstep) {
            const int nu = n_units(p, P.n_ntiles, NC), nt0 = p / NC;
            for (int jh = 0; jh < JH; ++jh)
            for (int u = 0; u < nu; ++u, ++tile) {
                const int buf = tile & 1;
                const uint32_t tph = (tile >> 1) & 1u;
                epi::cp_async_wait_all();
                epi_sync384();  // this unit's values are in; the other slot is free
                if (u + 1 < nu)
                    stage_unit<NMT, JH>(hbs + (buf ^ 1), P, p, nt0 + 2 * (u + 1), et, kEpi);
                else if (jh + 1 < JH)
                    stage_unit<NMT, JH>(hbs + (buf ^ 1), P, p, nt0, et, kEpi);
                else if (p + rstep < P.nf)
                    stage_unit<NMT, JH>(hbs + (buf ^ 1), P, p + rstep, (p + rstep) / NC, et, kEpi);
                if (ok) {
                    ok = __all_sync(0xffffffffu, mbar_wait(&tfull[buf], tph, err, 4));
                    if (ok) {
                        fence_after();
                        const UT &hb = hbs[buf];
                        const int q0 = (nt0 + 2 * u) * NC;
                        // two N tiles: TMEM columns 0-127 hold columns q0 .., 128-255 q0 + NC ..
                        for (int h2 = 0; h2 < 2; ++h2) {
                            if constexpr (SAMPLE)
                                unit_half_sample<NMT, JH>(hb, lane_base + buf * 256 + h2 * 128, wg, a, b, p, q0,
                                                          h2 * NC, P, jh * NMT, vrow);
                            else
                                unit_half<NMT, JH>(hb, lane_base + buf * 256 + h2 * 128, wg, a, b, h2 * NC, acc,
                                                   jh * NMT);
                        }
                        fence_before();
                        mbar_arrive(&tempty[buf]);
                        since += 2;
                        // flush every kFlushTiles tiles, at the end of each mode half (JH > 1) and
                        // at the end of the CTA's rows
                        const bool last = u + 1 == nu && ((JH > 1) || p + rstep >= P.nf);
                        if (!SAMPLE && (since >= kFlushTiles || last) && vrow) {
#pragma unroll
                            for (int k = 0; k < kKindsWG; ++k)
#pragma unroll
                                for (int j = 0; j < NMT / 2; ++j) {
                                    const float2 s2 = up2(acc[k][j]);
                                    double *pk = part + (size_t)((k0 + k) * W + jh * NMT + 2 * j) * 128;
                                    if (s2.x != 0.f) atomicAdd(pk, (double)s2.x);
                                    if (s2.y != 0.f) atomicAdd(pk + 128, (double)s2.y);
                                    acc[k][j] = 0ull;
                                }
                            since = 0;
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
    if (warp == L::warp_mma) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
}

}  // namespace ecls
}  // namespace bsa

namespace bsa {
namespace ecls {

// m3[m + nm n + nm^2 o] from the per-CTA FP64 partials of the E form (kinds: 0 K_i, 1 K_iv,
// 2 F14, 3 K_iii, 4 K_v, 5 F35, 6 K_ii, 7 K_vi, 8 F26, each kept at the lane's (a, b) and j).
__global__ void k_e_reduce(int nm, int W, int MT, int grid, const double *__restrict__ part,
                           double *__restrict__ m3mf, double *__restrict__ m3mr) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int nm3 = nm * nm * nm;
    if (x >= nm3) return;
    const int m = x % nm, n = (x / nm) % nm, o = x / (nm * nm);
    auto sum = [&](int kind, int a, int b, int j) {
        const int R = a * nm + b, mtile = R / 128, lane = R % 128;
        double s = 0.0;
        for (int g = mtile; g < grid; g += MT) s += part[(((size_t)g * kKinds + kind) * W + j) * 128 + lane];
        return s;
    };
    const double mr = sum(0, m, n, o) + sum(1, m, o, n) + sum(3, o, n, m) + sum(4, n, o, m) + sum(6, n, m, o) +
                      sum(7, o, m, n);
    const double mf = sum(2, m, n, o) + sum(2, m, o, n) + sum(5, o, n, m) + sum(5, n, o, m) + sum(8, n, m, o) +
                      sum(8, o, m, n);
    m3mr[x] = 2.0 * mr;  // B_F = 2 (T1 + T2 + T3)
    m3mf[x] = 2.0 * mf;
}

template <int NMT, int JH, bool SAMPLE = false>
static cudaError_t launch_k(cudaStream_t st, const CUtensorMap *maps, const EParams &p, int grid) {
    const size_t smem = (size_t)kStages * kStageBytes + 1024 + kBarBytes + 2 * sizeof(UTile<NMT, JH>);
    static_assert((size_t)kStages * kStageBytes + 1024 + kBarBytes + 2 * sizeof(UTile<NMT, JH>) <= 232448,
                  "shared memory of one CTA");
    cudaError_t e =
        cudaFuncSetAttribute(k_bfm_e<NMT, JH, SAMPLE>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    constexpr bool RS = use_regsplit(NMT, JH);
    if (RS && (e = regsplit_check(k_bfm_e<NMT, JH, SAMPLE>)) != cudaSuccess) return e;
    k_bfm_e<NMT, JH, SAMPLE><<<grid, ELayout<RS>::threads, smem, st>>>(maps[0], maps[1], maps[2], maps[3], p);
    return cudaGetLastError();
}

}  // namespace ecls

// The E form of the Classic contraction (see the top of this file): whole grid, truncated
// S(f1 + f2), at most 48 kept modes (above 24 in two mode halves of 16 or 24).  Called by
// contract_mixed; with smp, the sampled instantiation writes the per-point bispectra of the
// grid points smp->slot lists into smp->sF / smp->sR (zeroed here) and no moments.
int Engine::contract_e(const PointSrc &ps, double *m3mf, double *m3mr, const ESample *smp) {
    using namespace ecls;
    const int nf = ps.nf, nm = nme;
    const int W = plan_e_width(nm, K, nf);  // 8, 16, 24; 32 and 48 as two mode halves
    const int JH = plan_e_split(W, nm, K, nf), NMT = W / JH;  // 16 and 24 in one or two passes
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
    const size_t uel = (size_t)nf * Mp * Kp, gel = (size_t)JH * nf * NMT * Kp;
    const size_t bytesA = 2 * uel * 2, bytesB = 2 * gel * 2;
    const size_t bytesH = sizeof(float2) * (size_t)(nf + ns) * W;
    const size_t bytesP = sizeof(double) * (size_t)grid * kKinds * W * 128;
    if ((e = dMixA.reserve(bytesA)) || (e = dMixB.reserve(bytesB)) || (e = dMixH.reserve(bytesH + 256)) ||
        (e = dMixPart.reserve(bytesP + 256)))
        return cuda_fail(e, "allocating BF16x3 operands");
    __nv_bfloat16 *Uh = dMixA.as<__nv_bfloat16>(), *Ul = Uh + uel;
    __nv_bfloat16 *Gh = dMixB.as<__nv_bfloat16>(), *Gl = Gh + gel;
    float2 *Hg = dMixH.as<float2>(), *Hs = Hg + (size_t)nf * W;
    int *derr = (int *)((char *)dMixPart.p + bytesP);
    if ((e = cudaEventRecord(ev2, stream))) return cuda_fail(e, "event");
    if ((e = cudaMemsetAsync(derr, 0, sizeof(int), stream))) return cuda_fail(e, "memset");
    {
        const float *A = dA32.as<float>();
        if ((e = mixed::prep_u(stream, nf, nm, K, Kp, Mp, A, dQ.as<double>(), Uh, Ul)) ||
            (e = mixed::prep_h(stream, nf, nm, W, ps.fgrid, frf(), Hg, Hs, true)))
            return cuda_fail(e, "BF16x3 operand preparation");
        for (int jh = 0; jh < JH; ++jh) {  // G rows of mode half jh at jh nf NMT
            const size_t og = (size_t)jh * nf * NMT * Kp;
            if ((e = mixed::prep_b(stream, nf, nm, NMT, jh * NMT, K, Kp, nf, ps.n_pad, ps.trunc, ps.sum_base, 0, A,
                                   Gh + og, Gl + og)))
                return cuda_fail(e, "BF16x3 operand preparation");
        }
        kernels += 2 + JH;
    }
    CUtensorMap maps[4];
    if (!make_map(&maps[0], Uh, Kp, (uint64_t)nf * Mp, kBM) || !make_map(&maps[1], Ul, Kp, (uint64_t)nf * Mp, kBM) ||
        !make_map(&maps[2], Gh, Kp, (uint64_t)JH * nf * NMT, NC * NMT) ||
        !make_map(&maps[3], Gl, Kp, (uint64_t)JH * nf * NMT, NC * NMT))
        return fail(BSA_ERR_CUDA, "cuTensorMapEncodeTiled failed");
    EParams prm{};
    prm.nf = nf;
    prm.h = (nf - 1) / 2;
    prm.nm = nm;
    prm.Mp = Mp;
    prm.MT = MT;
    prm.nk = Kp / kBK;
    prm.ks_last = (K - (prm.nk - 1) * kBK + 15) / 16;
    prm.n_ntiles = (nf + NC - 1) / NC;
    prm.wmode = ps.wmode;
    prm.wval = ps.wval;
    prm.Hg = Hg;
    prm.Hs = Hs;
    prm.part = dMixPart.as<double>();
    prm.err = derr;
    prm.test_skip_tile1 = wait_test_tile1;
    wait_test_tile1 = 0;  // one analysis only
    if (cls_shards > 1 && !smp) {  // product rows p = rank + shards l (bsa_gpu_setClassicShard)
        prm.p0 = cls_shard;
        prm.pstep_m1 = cls_shards - 1;
    }
    const long long nm3 = (long long)nm * nm * nm;
    if (smp) {
        prm.slot = smp->slot;
        prm.sF = smp->sF;
        prm.sR = smp->sR;
        if ((e = cudaMemsetAsync(smp->sF, 0, sizeof(double) * (size_t)smp->nslot * nm3, stream)) ||
            (e = cudaMemsetAsync(smp->sR, 0, sizeof(double) * (size_t)smp->nslot * nm3, stream)))
            return cuda_fail(e, "memset");
    }
    if ((e = cudaEventRecord(evg0, stream))) return cuda_fail(e, "event");
    switch ((smp ? 1000 : 0) + NMT * 10 + JH) {
    case 81: e = launch_k<8, 1>(stream, maps, prm, grid); break;
    case 82: e = launch_k<8, 2>(stream, maps, prm, grid); break;
    case 122: e = launch_k<12, 2>(stream, maps, prm, grid); break;
    case 161: e = launch_k<16, 1>(stream, maps, prm, grid); break;
    case 162: e = launch_k<16, 2>(stream, maps, prm, grid); break;
    case 241: e = launch_k<24, 1>(stream, maps, prm, grid); break;
    case 242: e = launch_k<24, 2>(stream, maps, prm, grid); break;
    case 1081: e = launch_k<8, 1, true>(stream, maps, prm, grid); break;
    case 1082: e = launch_k<8, 2, true>(stream, maps, prm, grid); break;
    case 1122: e = launch_k<12, 2, true>(stream, maps, prm, grid); break;
    case 1161: e = launch_k<16, 1, true>(stream, maps, prm, grid); break;
    case 1162: e = launch_k<16, 2, true>(stream, maps, prm, grid); break;
    case 1241: e = launch_k<24, 1, true>(stream, maps, prm, grid); break;
    case 1242: e = launch_k<24, 2, true>(stream, maps, prm, grid); break;
    default: return fail(BSA_ERR_STATE, "no E-form kernel for %d modes in %d passes", NMT, JH);
    }
    if (e) return cuda_fail(e, "BF16x3 tcgen05 contraction kernel (E form)");
    if ((e = cudaEventRecord(evg1, stream))) return cuda_fail(e, "event");
    if (smp) {
        int herr = 0;
        if ((e = cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, stream)) ||
            (e = cudaEventRecord(ev1, stream)) || (e = cudaStreamSynchronize(stream)))
            return cuda_fail(e, "BF16x3 contraction (sampled)");
        kernels += 1;
        float ms = 0.f;
        cudaEventElapsedTime(&ms, evg0, evg1);
        last_ms_gemm = ms;
        if (herr) return fail(BSA_ERR_TIMEOUT, "BF16x3 kernel: a pipeline wait ran out of its budget (role %d)", herr);
        return BSA_OK;
    }
    if ((e = dOut.reserve(sizeof(double) * (3 * (size_t)nm * nm + 2 * (size_t)nm3)))) return cuda_fail(e, "out");
    double *o = dOut.as<double>() + 3 * (size_t)nm * nm;
    k_e_reduce<<<(unsigned)((nm3 + 127) / 128), 128, 0, stream>>>(nm, W, MT, grid, prm.part, o, o + nm3);
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
