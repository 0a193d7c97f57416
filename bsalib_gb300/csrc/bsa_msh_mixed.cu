// bsa_msh_mixed.cu -- split-precision (BF16x3) tensor-core evaluation of Mesher zones.
//
// A rectangular zone whose lattice is aligned with the frequency axes has its BFM points at
// (f1, f2) = (r_i, c_j): every point of lattice line i shares f1 = r_i, every point of
// column j shares f2 = c_j.  With U(f)[(a,b), k] = Q_ka A_kb(f) and Z = A(f1+f2) per point,
// the three terms of the factored BFM (functionsImpl.F90:247-465, direct form) at (i, j) are
//   T1 = U(r_i) A(c_j)      (m,n,o) = (a, b, j')     one GEMM per line i, B = the zone's columns
//   T3 = U(r_i) Z(i,j)      (m,n,o) = (j', b, a)     same line, B = the line's sum rows
//   T2 = U(c_j) Z(i,j)      (m,n,o) = (j', a, b)     one GEMM per column j, B = the column's sums
// and B_F = 2 (T1 + T2 + T3).  Unlike the Classic grid, (c_j, r_i) is not a point of the zone,
// so T2 needs its own GEMM family (tasks of kind 1).
//
// k_msh_mixed runs those GEMMs as tcgen05 MMAs fed by TMA, with the k_bfm_mixed pipeline
// (one TMA warp, one MMA-issuing warp, four TMEM-draining warps, double-buffered TMEM,
// bounded mbarrier waits) and stores the three term tensors in FP32.  k_msh_moments then
// integrates them: the BFM lattice trapezoid for m3mf, and for m3mr the bilinear
// interpolation onto the BRM lattice refined by (Fi, Fj) times the FRF product
// Re[H_m(w1) H_n(w2) conj H_o(w1+w2)] (getRM_full_scalar_msh_, :1031-1115) with the
// trapezoid weights of the refined lattice (_shared_poly2d.fi:470-2166), the FRF evaluated
// in FP64 and rounded once.  Zones whose lattice is rotated against the axes go to the FP64
// point kernel.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <vector>

#include "../../include/bsa_gpu.h"
#include "bsa_engine.cuh"
#include "bsa_kernels.cuh"
#include "bsa_tc.cuh"

namespace bsa {
namespace mshmix {

using namespace tc;

constexpr int kStages = 2;
constexpr int kStageBytes = 6 * kTileBytes;  // U hi/lo, G hi/lo, S hi/lo

// One task: a lattice line of a zone, i.e. one U(f) row block against the points of the line.
struct Task {
    int u_row;    // first U-table row of the line's U(f) (a multiple of Mp)
    int g_row;    // first column-table row of the zone (D1 operand), -1 for kind 1
    int s_row;    // first sum-table row of the line's points (NMT rows per point)
    int ncols;    // points on the line
    int p0;       // output index of the line's first point
    int pstride;  // output index step between consecutive points of the line
    int kind;     // 0: D1 -> T1 and D3 -> T3;  1: D3 -> T2
};

struct MParams {
    int nm, NMT, NC, BROWS, Mp, MT, nk, ks_last;
    int nitems;
    const Task *tasks;
    const int4 *items;  // (task, row tile, first N tile, end N tile)
    float *T1, *T3, *T2;  // [point][j'][a*nm + b], points nm3p (nm^3 rounded up to 4) apart
    int nm3p;
    int *err;
    int *head;  // device work queue: the next unclaimed item (zero at launch)
};

constexpr int kQueue = 4;  // item slots between the producer and the two consumer roles

// Work item w = (task, row tile, N tiles [nt0, nt1)).  The items sit in a device queue (the
// zone list expanded into lines and columns, row tiles and N tiles); a CTA's TMA thread claims
// the next one with an atomic on the queue head and publishes its index through a ring of
// kQueue shared-memory slots (mbarriers qfull / qempty: the MMA thread and the four epilogue
// warps read each slot once), so all three roles walk the same (item, K chunk) sequence, one
// TMEM buffer per item, and a CTA whose items are short (small zones, lone N tiles) simply
// claims more of them.  Each CTA ends on the first index past the queue.  The items of one
// task are consecutive (row tile major), so the CTAs running at the same time share its U row
// blocks and its B tiles through L2 instead of each streaming them from HBM.  Stage layout:
// U hi, U lo, B0 hi, B1 hi, B0 lo, B1 lo, the unit's 256 B rows B0 | B1 in one N = 256 MMA:
//   kind 0 items (one N tile): B0 = G(nt), B1 = S(nt) -> [D1 | D3];
//   kind 1 items of two N tiles: B0 = S(nt), B1 = S(nt + 1) -> [D3(nt) | D3(nt + 1)];
//   kind 1 items of one N tile: B1 = S(nt), N = 128 into the D3 half.
// A lone D3 tile has 12 MMAs per 64 KB stage and waits on its operands; paired it has 24 per
// 96 KB, as a line tile.
__global__ void __launch_bounds__(192, 1)
    k_msh_mixed(const __grid_constant__ CUtensorMap tmUh, const __grid_constant__ CUtensorMap tmUl,
                const __grid_constant__ CUtensorMap tmGh, const __grid_constant__ CUtensorMap tmGl,
                const __grid_constant__ CUtensorMap tmSh, const __grid_constant__ CUtensorMap tmSl, const MParams p) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t *bars = (uint64_t *)(smem + kStages * kStageBytes);
    uint64_t *full = bars, *empty = bars + kStages, *tfull = bars + 2 * kStages, *tempty = bars + 2 * kStages + 2;
    uint64_t *done = bars + 2 * kStages + 4;
    uint64_t *qfull = bars + 2 * kStages + 5, *qempty = qfull + kQueue;
    uint32_t *tmem_slot = (uint32_t *)(qempty + kQueue);
    volatile int *ring = (volatile int *)(qempty + kQueue + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    int *err = p.err;
    const int nwork = p.nitems;

    // B-tile rows that TMA never writes (BROWS..127) stay zero for the whole run.
    for (int s = 0; s < kStages; ++s)
        for (int t = 2; t < 6; ++t) {
            uint8_t *tile = smem + s * kStageBytes + t * kTileBytes;
            for (int x = threadIdx.x; x < (128 - p.BROWS) * 128 / 16; x += blockDim.x)
                ((uint4 *)(tile + p.BROWS * 128))[x] = make_uint4(0, 0, 0, 0);
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
        for (int q = 0; q < kQueue; ++q) {
            mbar_init(&qfull[q], 1);
            mbar_init(&qempty[q], 1 + 4);  // the MMA thread and the four epilogue warps
        }
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

    if (warp == 0) {
        // ---------------- TMA producer ----------------
        if (lane == 0) {
            uint32_t it = 0;
            bool ok = true;
            for (int qi = 0; ok; ++qi) {
                // claim the next item of the queue and publish it to the MMA and epilogue roles
                const int slot = qi % kQueue;
                if (!mbar_wait(&qempty[slot], ((qi / kQueue) & 1u) ^ 1u, err, 5)) { ok = false; break; }
                const int w = atomicAdd(p.head, 1);
                ring[slot] = w;
                mbar_arrive(&qfull[slot]);
                if (w >= nwork) break;
                const int4 wi = p.items[w];
                const Task tk = p.tasks[wi.x];
                const int mt = wi.y;
                const int nt = wi.z, cnt = wi.w - wi.z;
                const bool wide = tk.kind == 0 || cnt == 2;  // two B tiles, N = 256
                const uint32_t tx = 2u * kTileBytes + (wide ? 4u : 2u) * (uint32_t)(p.BROWS * 128);
                for (int kc = 0; kc < p.nk && ok; ++kc, ++it) {
                    const int s = it % kStages;
                    const uint32_t ph = (it / kStages) & 1u;
                    if (!mbar_wait(&empty[s], ph ^ 1u, err, 1)) { ok = false; break; }
                    uint8_t *st = smem + s * kStageBytes;
                    mbar_expect_tx(&full[s], tx);
                    const int x = kc * kBK;
                    const int yu = tk.u_row + mt * kBM;
                    tma_2d(st + 0 * kTileBytes, &tmUh, &full[s], x, yu);
                    tma_2d(st + 1 * kTileBytes, &tmUl, &full[s], x, yu);
                    const int ys = tk.s_row + nt * p.BROWS;
                    if (tk.kind == 0) {
                        const int yg = tk.g_row + nt * p.BROWS;
                        tma_2d(st + 2 * kTileBytes, &tmGh, &full[s], x, yg);
                        tma_2d(st + 4 * kTileBytes, &tmGl, &full[s], x, yg);
                        tma_2d(st + 3 * kTileBytes, &tmSh, &full[s], x, ys);
                        tma_2d(st + 5 * kTileBytes, &tmSl, &full[s], x, ys);
                    } else if (cnt == 2) {
                        tma_2d(st + 2 * kTileBytes, &tmSh, &full[s], x, ys);
                        tma_2d(st + 4 * kTileBytes, &tmSl, &full[s], x, ys);
                        tma_2d(st + 3 * kTileBytes, &tmSh, &full[s], x, ys + p.BROWS);
                        tma_2d(st + 5 * kTileBytes, &tmSl, &full[s], x, ys + p.BROWS);
                    } else {
                        tma_2d(st + 3 * kTileBytes, &tmSh, &full[s], x, ys);
                        tma_2d(st + 5 * kTileBytes, &tmSl, &full[s], x, ys);
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
            for (int qi = 0; ok; ++qi) {
                const int slot = qi % kQueue;
                if (!mbar_wait(&qfull[slot], (qi / kQueue) & 1u, err, 6)) { ok = false; break; }
                const int w = ring[slot];
                mbar_arrive(&qempty[slot]);
                if (w >= nwork) break;
                const int4 wi = p.items[w];
                const Task tk = p.tasks[wi.x];
                const bool wide = tk.kind == 0 || wi.w - wi.z == 2;
                {
                    const int buf = tile & 1;
                    const uint32_t tph = (tile >> 1) & 1u;
                    ++tile;
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
                        for (int ks = 0; ks < nks; ++ks) {
                            const uint32_t off = ks * 32;
                            const uint64_t uh = sdesc(base + 0 * kTileBytes + off), ul = sdesc(base + 1 * kTileBytes + off);
                            const uint32_t acc = (kc > 0 || ks > 0) ? 1u : 0u;
                            if (wide) {  // B0 | B1, N = 256
                                const uint64_t bh = sdesc(base + 2 * kTileBytes + off), bl = sdesc(base + 4 * kTileBytes + off);
                                mma256(d1, uh, bh, acc);
                                mma256(d1, uh, bl, 1u);
                                mma256(d1, ul, bh, 1u);
                            } else {  // B1 alone into the D3 half
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
        // ---------------- epilogue: TMEM -> FP32 term tensors ----------------
        const int quarter = warp & 3;
        const int row = quarter * 32 + lane;  // TMEM lane = row of the M tile
        const uint32_t lane_base = tmem + ((uint32_t)(quarter * 32) << 16);
        const int nm = p.nm, nm2 = nm * nm;
        uint32_t tile = 0;
        bool ok = true;
        for (int qi = 0; ok; ++qi) {
            const int slot = qi % kQueue;
            // warp-uniform: every lane waits, reads the slot, then one arrive per warp
            if (!__all_sync(0xffffffffu, mbar_wait(&qfull[slot], (qi / kQueue) & 1u, err, 7))) { ok = false; break; }
            const int w = ring[slot];
            __syncwarp();
            if (lane == 0) mbar_arrive(&qempty[slot]);
            if (w >= nwork) break;
            const int4 wi = p.items[w];
            const Task tk = p.tasks[wi.x];
            const int mt = wi.y;
            const int grow = mt * kBM + row;  // row of U: a * nm + b
            const bool vrow = grow < nm2;
            const int cnt = wi.w - wi.z;
            // the two accumulator halves: [T1 | T3] of one N tile (kind 0), [T2 | T2] of two
            // N tiles, or the second half alone
            float *const outA = tk.kind == 0 ? p.T1 : p.T2;
            float *const outB = tk.kind == 0 ? p.T3 : p.T2;
            {
                const int buf = tile & 1;
                const uint32_t tph = (tile >> 1) & 1u;
                ++tile;
                // warp-uniform outcome: tcgen05.ld below is .sync.aligned
                const bool got = __all_sync(0xffffffffu, mbar_wait(&tfull[buf], tph, err, 4));
                if (!got) { ok = false; break; }
                fence_after();
                for (int acc = (tk.kind == 0 || cnt == 2 ? 0 : 1); acc < 2; ++acc) {
                    float *const out = acc == 0 ? outA : outB;
                    const int c0 = (wi.z + (tk.kind == 1 && cnt == 2 ? acc : 0)) * p.NC;
                    for (int q = 0; q < kBN / 32; ++q) {
                        uint32_t v[32];
                        tmem_ld32(lane_base + buf * 256 + acc * 128 + q * 32, v);
                        tmem_wait_ld();
#pragma unroll
                        for (int e = 0; e < 32; ++e) {
                            const int col = q * 32 + e;
                            const int c = col / p.NMT, j = col - c * p.NMT;
                            if (!vrow || c >= p.NC || j >= nm || c0 + c >= tk.ncols) continue;
                            const size_t pt = (size_t)tk.p0 + (size_t)(c0 + c) * tk.pstride;
                            out[pt * p.nm3p + (size_t)j * nm2 + grow] = __uint_as_float(v[e]);
                        }
                    }
                }
                fence_before();
                mbar_arrive(&tempty[buf]);
            }
        }
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
}

// ------------------------------------------------------------------------------------
// Operand preparation from the FP32 A(f) table (rows named by an index list).
// ------------------------------------------------------------------------------------
// U[(r*Mp + a*nm + b)][k] = Q[k][a] A(src[r])[k][b]   (rows >= nm^2 and k >= K are zero)
// One block per (row block r, 32 k); nm <= 64.
__global__ void k_prep_u_rows(int nm, int K, int Kp, int Mp, const int *__restrict__ src, const float *__restrict__ A,
                              const double *__restrict__ Q, __nv_bfloat16 *__restrict__ Uh,
                              __nv_bfloat16 *__restrict__ Ul) {
    const int r = blockIdx.x, k0 = blockIdx.y * 32;
    __shared__ float As[32][65], Qs[32][65];
    const float *Ar = A + (size_t)src[r] * K * nm;
    for (int e = threadIdx.x; e < 32 * nm; e += blockDim.x) {
        const int kk = e / nm, m = e % nm, k = k0 + kk;
        As[kk][m] = k < K ? Ar[(size_t)k * nm + m] : 0.f;
        Qs[kk][m] = k < K ? (float)Q[(size_t)k * nm + m] : 0.f;
    }
    __syncthreads();
    const int nm2 = nm * nm;
    for (int e = threadIdx.x; e < Mp * 4; e += blockDim.x) {
        const int row = e >> 2, kv = (e & 3) * 8;
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

// T[(t*NMT + j)][k] = A(src[t])[k][j]   (j >= nm and k >= K are zero)
__global__ void k_prep_b_rows(int nm, int NMT, int K, int Kp, const int *__restrict__ src, const float *__restrict__ A,
                              __nv_bfloat16 *__restrict__ Th, __nv_bfloat16 *__restrict__ Tl) {
    const int t = blockIdx.x, k0 = blockIdx.y * 64;
    __shared__ float As[64][65];
    const float *Ar = A + (size_t)src[t] * K * nm;
    for (int e = threadIdx.x; e < 64 * nm; e += blockDim.x) {
        const int kk = e / nm, m = e % nm, k = k0 + kk;
        As[kk][m] = k < K ? Ar[(size_t)k * nm + m] : 0.f;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < NMT * 8; e += blockDim.x) {
        const int j = e >> 3, kv = (e & 7) * 8;
        __align__(16) __nv_bfloat16 hi[8], lo[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) split_bf16f(j < nm ? As[kv + q][j] : 0.f, hi[q], lo[q]);
        const size_t o = ((size_t)t * NMT + j) * Kp + k0 + kv;
        *(uint4 *)(Th + o) = *(const uint4 *)hi;
        *(uint4 *)(Tl + o) = *(const uint4 *)lo;
    }
}

// ------------------------------------------------------------------------------------
// Zone integration of the term tensors.
// ------------------------------------------------------------------------------------
// An axis-aligned zone of the batch: BFM point (i, j) at (fi0 + i dI, fj0 + j dJ), term
// tensors at point pbase + i*nj + j, cells (i0, j0), 0 <= i0 < ni-1, 0 <= j0 < nj-1,
// numbered from cbase; BRM point (qi, qj), 0 <= qi <= (ni-1) Fi, 0 <= qj <= (nj-1) Fj, at
// qbase + qi * ((nj-1) Fj + 1) + qj in the FRF table.
struct ZoneM {
    double fi0, fj0, dI, dJ, wI, wJ, sym;
    int ni, nj, Fi, Fj;
    int pbase, cbase, qbase;
    float wb;  // sym wI wJ rounded once: the BFM-lattice trapezoid weight of an interior point
};

__device__ __forceinline__ int zone_of(const ZoneM *__restrict__ zones, int nz, int idx, int which) {
    int lo = 0, hi = nz - 1;  // last zone whose base (cells: which 0, BRM points: which 1) <= idx
    while (lo < hi) {
        const int mid = (lo + hi + 1) / 2;
        const int base = which == 0 ? zones[mid].cbase : zones[mid].qbase;
        if (base <= idx) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// FRF row of a BRM point: H_m(w1), H_m(w2), H_m(w1 + w2) (3 nm values), the point's weight
// as (w, 0), and a zero pad to an even count, so rows start on 16-byte boundaries.
__host__ __device__ __forceinline__ int frf_row(int nm) { return (3 * nm + 2) & ~1; }

// Per BRM point q: H_m(w1), H_m(w2), H_m(w1 + w2) evaluated in FP64 and rounded once
// (Hq[q][frf_row], the weight at 3 nm), and its integration weight sym (wI/Fi)(wJ/Fj) t_i t_j
// (also Wq[q]).
__global__ void k_msh_frf(int nm, int nz, const ZoneM *__restrict__ zones, int nq, FrfPar frf,
                          float2 *__restrict__ Hq, float *__restrict__ Wq) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)nq * 3 * nm) return;
    const int q = (int)(t / (3 * nm)), r = (int)(t % (3 * nm)), which = r / nm, m = r % nm;
    const ZoneM z = zones[zone_of(zones, nz, q, 1)];
    const int NI = (z.ni - 1) * z.Fi, NJ = (z.nj - 1) * z.Fj;
    const int loc = q - z.qbase, qi = loc / (NJ + 1), qj = loc % (NJ + 1);
    const double v1 = (z.fi0 + ((double)qi / z.Fi) * z.dI) * kPi2;
    const double v2 = (z.fj0 + ((double)qj / z.Fj) * z.dJ) * kPi2;
    const double w = which == 0 ? v1 : which == 1 ? v2 : v1 + v2;
    double hr, hi;
    frf_eval(frf.M[m], frf.K[m], frf.C[m], w, hr, hi);
    const int hs = frf_row(nm);
    float2 *row = Hq + (size_t)q * hs;
    row[r] = make_float2((float)hr, (float)hi);
    if (r == 0) {
        const double ti = (qi == 0 || qi == NI) ? 0.5 : 1.0, tj = (qj == 0 || qj == NJ) ? 0.5 : 1.0;
        const float wq = (float)(z.sym * (z.wI / z.Fi) * (z.wJ / z.Fj) * ti * tj);
        Wq[q] = wq;
        row[3 * nm] = make_float2(wq, 0.f);
        if (hs > 3 * nm + 1) row[3 * nm + 1] = make_float2(0.f, 0.f);
    }
}

constexpr int kQB = 16;      // BRM points per work item
constexpr int kMomEPT = 3;   // term-tensor elements per thread (same j', b; consecutive a)
constexpr int kVY = 64;      // staged (j', mode) pairs per point
constexpr int kWin = 776;    // corner window (floats): 3 x 256 elements + alignment slack
constexpr int kHrow = 194;   // FRF row capacity (float2): frf_row(64)

// Bulk copy global -> shared (16-byte aligned, size a multiple of 16), completing on bar.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     su32(dst)),
                 "l"(src), "r"(bytes), "r"(su32(bar))
                 : "memory");
}

// Element layout of the moment pass.  A thread holds the EPT elements (j', a = arow EPT + u, b),
// u < EPT, of the term tensors (e = j' nm^2 + a nm + b), AR = ceil(nm / EPT) a-rows per j'.
//   JB = 1 (nm > ~19): a block covers RB = 256 / nm whole a-rows of one j' (thread t: a-row
//     t / nm of the chunk, b = t % nm), nchj blocks per j';
//   JB > 1: a block covers JB consecutive modes j' whole (thread t: jl = t / (AR nm)).
// Either way the block's elements are one contiguous range of each point's term tensor, which
// one bulk copy per (term, corner) brings in.
struct MomLayout {
    int JB, AR, RB, nchj;
    static MomLayout make(int nm) {
        MomLayout L;
        L.AR = (nm + kMomEPT - 1) / kMomEPT;
        const int per_j = L.AR * nm;
        L.JB = std::max(1, std::min(256 / per_j, kVY / nm));
        L.RB = L.JB > 1 ? L.AR : 256 / nm;
        L.nchj = L.JB > 1 ? 1 : (L.AR + L.RB - 1) / L.RB;
        return L;
    }
    int groups(int nm) const { return (nm + JB - 1) / JB; }
    // dynamic shared memory of k_msh_moments
    static size_t smem() {
        return (size_t)kQB * kVY * 16 + (size_t)kQB * 64 * 16 + (size_t)kQB * kHrow * 8 + (size_t)12 * kWin * 4 + 16;
    }
};

// One unit of a block's work: the BRM points q0 .. q0 + nb - 1 (in the cell's row-major order)
// of cell loc of zone z, with the cell geometry they need.  Built by one thread and read by all
// from shared memory.
struct MomItem {
    int z, loc, q0, nb, nq, nqj, qi0, qj0, rowq, nj;  // rowq: BRM points per zone lattice row
    int valid, zend;                                  // zend: the zone's last item of this block
    // corner staging: the cell's left corner column (i0, j0), (i0 + 1, j0) is in slot cl of
    // the corner windows, its right column in slot 1 - cl; reuse: the left column is the
    // previous cell's right column, still staged (the next cell of a zone row)
    int cl, reuse;
    long long qbase, P00;
    float wp[4];  // BFM lattice trapezoid weights of the corners the cell owns
    float rFi, rFj;
};

// The item (z, loc, q0) of a cell that exists.
__device__ __forceinline__ void mom_fill(const ZoneM *__restrict__ zones, int z, int loc, int q0, MomItem &it) {
    const ZoneM &Z = zones[z];
    const int ni = Z.ni, nj = Z.nj, Fi = Z.Fi, Fj = Z.Fj;
    const int i0 = loc / (nj - 1), j0 = loc - i0 * (nj - 1);
    const int NJ = (nj - 1) * Fj, NI = (ni - 1) * Fi;
    const int qi0 = i0 * Fi, qi1 = (i0 == ni - 2) ? NI : (i0 + 1) * Fi - 1;
    const int qj0 = j0 * Fj, qj1 = (j0 == nj - 2) ? NJ : (j0 + 1) * Fj - 1;
    it.z = z;
    it.loc = loc;
    it.q0 = q0;
    it.nqj = qj1 - qj0 + 1;
    it.nq = (qi1 - qi0 + 1) * it.nqj;
    it.nb = min(kQB, it.nq - q0);
    it.qi0 = qi0;
    it.qj0 = qj0;
    it.rowq = NJ + 1;
    it.nj = nj;
    it.valid = 1;
    it.zend = 0;
    it.cl = 0;
    it.reuse = 0;
    it.qbase = Z.qbase;
    it.P00 = (long long)Z.pbase + (long long)i0 * nj + j0;
    const int ci[4] = {i0, i0, i0 + 1, i0 + 1}, cj[4] = {j0, j0 + 1, j0, j0 + 1};
    for (int k = 0; k < 4; ++k) {
        const bool own = (ci[k] == i0 || i0 == ni - 2) && (cj[k] == j0 || j0 == nj - 2);
        const float ti = (ci[k] == 0 || ci[k] == ni - 1) ? 0.5f : 1.f;
        const float tj = (cj[k] == 0 || cj[k] == nj - 1) ? 0.5f : 1.f;
        it.wp[k] = own ? Z.wb * ti * tj : 0.f;
    }
    it.rFi = 1.f / (float)Fi;
    it.rFj = 1.f / (float)Fj;
}

// Block column g of G owns the cells loc = r, r + G, ... of each zone, r = (g + s_z) mod G with
// s_z a hash of the zone's frequency origin (so every block column gets its share of the
// zones' first cells, and the split of a zone depends on the zone alone).
__device__ __forceinline__ int mom_first(const ZoneM &Z, int G, int g) {
    const unsigned long long h = (unsigned long long)__double_as_longlong(Z.fi0) * 0x9E3779B97F4A7C15ull ^
                                 (unsigned long long)__double_as_longlong(Z.fj0) * 0xC2B2AE3D27D4EB4Full;
    const int sz = (int)((h >> 33) % (unsigned long long)G);
    return (g + sz) % G;
}

// First cell at or after (z, loc) that block column g owns, as an item at q0 = 0; valid = 0
// past the last zone.  newz: loc is to be taken from zone z's own start.
__device__ __forceinline__ void mom_seek(const ZoneM *__restrict__ zones, int nz, int G, int g, int z, int loc,
                                         bool newz, MomItem &it) {
    while (z < nz) {
        if (newz) loc = mom_first(zones[z], G, g);
        if (loc < (zones[z].ni - 1) * (zones[z].nj - 1)) break;
        ++z;
        newz = true;
    }
    if (z < nz) {
        mom_fill(zones, z, loc, 0, it);
    } else {
        it.valid = 0;
        it.z = nz;
    }
}

// Block (g, y), y = group * nchj + chunk: the cells of every zone that block column g owns
// (mom_first).  Each BRM point belongs to the cell (min(qi/Fi, ni-2), min(qj/Fj, nj-2)) and
// each BFM point to the cell (min(i, ni-2), min(j, nj-2)), so every lattice point is counted
// once.  part[g][6][nm^3]: m3mf of T1, T3, T2, then m3mr of T1, T3, T2.  A zone's cells are
// summed in FP32 registers and each zone sum added in FP64 to the thread's own elements of
// part (a read-modify-write in global memory once per zone, no atomics), so each zone's share
// depends on that zone alone and the result is the same, to ~1e-13, for any zone order.
//
// The FRF products factor through per-point vectors staged in shared memory: with w the
// point's weight, V_j'(a) = w H1(a) conj H3(j'), Y_j'(b) = w H1(j') H2(b),
//   T1: Re[H1(a) H2(b) conj H3(j')] w = Re[H2(b) V_j'(a)]
//   T3: Re[H1(j') H2(b) conj H3(a)] w = Re[Y_j'(b) conj H3(a)]
//   T2: Re[H1(j') H2(a) conj H3(b)] w = Re[Y_j'(a) conj H3(b)]
// and the bilinear interpolation of each term over the cell is c0 + ti (c2 - c0) + tj (c1 - c0)
// + ti tj (c0 - c1 - c2 + c3), its coefficients formed once per cell.  The b-indexed values are
// read once per point for the thread's EPT elements.  The arithmetic runs on FP32 pairs: T1
// and T2 of one element share every step (V, Y staged as {Vr, Yr, Vi, Yi}, H2, H3 as {H2r,
// H3r, -H2i, H3i}, so {T1, T2} = {H2r, H3r} (.) {Vr, Yr} + {-H2i, H3i} (.) {Vi, Yi}), and T3
// runs on pairs of elements; 32 instead of 54 FP32 instructions per point for 3 elements.
//
// Pipeline: thread 32 builds each work item two items ahead and warp 0 issues its bulk copies
// one item ahead (one mbarrier phase per item, the copies spread over the warp's lanes): the
// FRF rows of the item's points (one copy per lattice-row segment) and, at a cell's first
// item, the block's element window of the corners x 3 terms.  Both run after the item's
// second block barrier, beside the other warps' arithmetic.  The
// windows sit in two column slots: the next cell of a zone row finds its left corner column
// staged as the previous cell's right one and copies only its right column, so each BFM
// point's window is copied about twice (once per cell row it bounds) instead of four times.
// The copies land while the current item computes.  The waits are bounded (err code 5 on
// timeout).
__global__ __launch_bounds__(256, 2) void k_msh_moments(int nm, int nm3p, MomLayout L, const ZoneM *__restrict__ zones,
                                                        int nz, const float *__restrict__ T1,
                                                        const float *__restrict__ T3, const float *__restrict__ T2,
                                                        const float2 *__restrict__ Hq, double *__restrict__ part,
                                                        int *__restrict__ err) {
    constexpr int EPT = kMomEPT;
    extern __shared__ __align__(16) unsigned char msm[];
    float4(*VY)[kVY] = reinterpret_cast<float4(*)[kVY]>(msm);                            // {Vr, Yr, Vi, Yi}
    float4(*H23)[64] = reinterpret_cast<float4(*)[64]>(msm + kQB * kVY * 16);            // {H2r, H3r, -H2i, H3i}
    float2 *Hraw = reinterpret_cast<float2 *>(msm + kQB * kVY * 16 + kQB * 64 * 16);     // [kQB][hs]
    float *Cs = reinterpret_cast<float *>(Hraw + kQB * kHrow);                           // [2][2][3][kWin]
    uint64_t *bar = reinterpret_cast<uint64_t *>(Cs + 12 * kWin);
    const ulonglong2(*VYp)[kVY] = reinterpret_cast<const ulonglong2(*)[kVY]>(msm);      // the same, as pairs
    const ulonglong2(*H23p)[64] = reinterpret_cast<const ulonglong2(*)[64]>(msm + kQB * kVY * 16);
    __shared__ ulonglong2 tq[kQB];  // {ti, ti}, {tj, tj}
    __shared__ f2x tq2[kQB];        // {ti tj, ti tj}
    __shared__ MomItem sit[3];      // the current item and the two after it
    const int nm2 = nm * nm, nm3 = nm2 * nm, tid = threadIdx.x, hs = frf_row(nm);
    const int grp = blockIdx.y / L.nchj, chunk = blockIdx.y % L.nchj;
    const int jg0 = grp * L.JB, njb = min(L.JB, nm - jg0), per_j = L.AR * nm;
    // this thread's elements and the block's window [win0, win0 + wlen) of a point's tensor
    int jl, arow, b;
    bool tval;
    int win0, wlen;
    if (L.JB > 1) {
        jl = tid / per_j;
        const int rem = tid - jl * per_j;
        arow = rem / nm;
        b = rem - arow * nm;
        tval = jl < njb;
        win0 = (jg0 * nm2) & ~3;
        wlen = (((jg0 + njb) * nm2 + 3) & ~3) - win0;
    } else {
        jl = 0;
        arow = chunk * L.RB + tid / nm;
        b = tid % nm;
        tval = tid < L.RB * nm && arow < L.AR;
        const int a0 = chunk * L.RB * EPT, a1 = min(nm, (chunk + 1) * L.RB * EPT);
        win0 = (jg0 * nm2 + a0 * nm) & ~3;
        wlen = ((jg0 * nm2 + a1 * nm + 3) & ~3) - win0;
    }
    const int nval = tval ? min(EPT, nm - arow * EPT) : 0;  // valid elements
    const int ev0 = tval ? (jg0 + jl) * nm2 + arow * EPT * nm + b : 0;  // element u: ev0 + u nm
    const int wofs = tval ? ev0 - win0 : 0;                           // in the window
    // elements past a = nm - 1 (u >= nval) read the next staged V, Y, H entries, which lie inside
    // the dynamic shared memory (VY is followed by H23, H23 by Hraw); their sums are never stored
    const int ia0 = tval ? jl * nm + arow * EPT : 0, ih0 = tval ? arow * EPT : 0;
    const int yb = tval ? jl * nm + b : 0, bb = tval ? b : 0;
    // conversion roles: (jl, m) pairs of VY, modes of H23
    const int st = tid & (kVY - 1), sq0 = tid / kVY;
    const int sjl = st / nm, sm = st - sjl * nm;
    const bool svy = sjl < njb;
    const float *Ts[3] = {T1, T3, T2};

    // corner window of slot s (column), row r (0: i0, 1: i0 + 1), term t
    auto cwin = [&](int s, int r, int t) { return Cs + ((s * 2 + r) * 3 + t) * kWin; };
    // warp 0: the copies of item it (one mbarrier phase) spread over its lanes: lane l < 16 the
    // FRF rows of the item's points on BRM lattice row r0 + l of the cell (at most 16 rows),
    // lanes 20-31 at a cell's first item the corner window (column, row, term) = lane - 20;
    // corner (r, c) of the cell is BFM point P00 + r nj + c
    auto issue = [&](const MomItem &it, int lane) {
        if (lane == 0) {
            uint32_t bytes = (uint32_t)it.nb * hs * 8;
            if (it.q0 == 0) bytes += (it.reuse ? 6u : 12u) * (uint32_t)wlen * 4;
            mbar_expect_tx(bar, bytes);
        }
        __syncwarp();
        if (lane < kQB) {
            const int r0 = it.q0 / it.nqj, qr = r0 + lane;
            const int qs = max(it.q0, qr * it.nqj), qn = min((qr + 1) * it.nqj, it.q0 + it.nb);
            if (qs < qn) {
                const size_t gq = (size_t)it.qbase + (size_t)(it.qi0 + qr) * it.rowq + (it.qj0 + qs - qr * it.nqj);
                bulk_g2s(Hraw + (qs - it.q0) * hs, Hq + gq * hs, (uint32_t)(qn - qs) * hs * 8, bar);
            }
        } else if (lane >= 20 && it.q0 == 0) {
            const int w = lane - 20, t = w >> 2, col = (w >> 1) & 1, r = w & 1;
            if (col >= it.reuse)
                bulk_g2s(cwin(col == 0 ? it.cl : 1 - it.cl, r, t),
                         Ts[t] + (size_t)(it.P00 + (long long)r * it.nj + col) * nm3p + win0, (uint32_t)wlen * 4, bar);
        }
    };
    // thread 32: nx = the item after p; p's zone ends with p when nx is in another zone
    auto build = [&](MomItem &p, MomItem &nx) {
        if (!p.valid) {
            nx.valid = 0;
            nx.z = nz;
            return;
        }
        if (p.q0 + kQB < p.nq) {
            mom_fill(zones, p.z, p.loc, p.q0 + kQB, nx);
            nx.cl = p.cl;
        } else {
            mom_seek(zones, nz, gridDim.x, blockIdx.x, p.z, p.loc + gridDim.x, false, nx);
            // the next cell of the zone row keeps this cell's right corner column
            nx.reuse = nx.valid && nx.z == p.z && nx.loc == p.loc + 1 && nx.loc % (p.nj - 1) != 0;
            nx.cl = nx.reuse ? 1 - p.cl : 0;
        }
        p.zend = nx.z != p.z;
    };

    static_assert(EPT == 2 || EPT == 3, "T3 runs on the element pair (0, 1), element 2 alone");
    float zf[EPT][3];  // the zone's FP32 m3mf sums
    // the cell's bilinear coefficients {A, B, C, D} and the zone's m3mr sums: {T1, T2} of each
    // element as pairs, T3 of elements 0 and 1 as a pair, T3 of element 2 alone
    f2x c12[EPT][4], z12[EPT], c3p[4], z3p;
    float c3s[4], z3s;
#pragma unroll
    for (int u = 0; u < EPT; ++u) {
        z12[u] = 0ull;
#pragma unroll
        for (int t = 0; t < 3; ++t) zf[u][t] = 0.f;
    }
    z3p = 0ull;
    z3s = 0.f;
    // the sums over zones: this thread's elements of the block column's partial
    double *pg = part + (size_t)blockIdx.x * 6 * nm3 + ev0;
#pragma unroll
    for (int u = 0; u < EPT; ++u)
        if (u < nval)
#pragma unroll
            for (int t = 0; t < 6; ++t) pg[(size_t)t * nm3 + u * nm] = 0.0;

    if (tid == 0) {
        mbar_init(bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (tid == 32) {
        mom_seek(zones, nz, gridDim.x, blockIdx.x, 0, 0, true, sit[0]);
        build(sit[0], sit[1]);
    }
    __syncthreads();
    if (tid < 32 && sit[0].valid) issue(sit[0], tid);
    bool ok = true;
    // Item k sits in slot k % 3: built by thread 32 during item k - 2, its copies issued by
    // warp 0 during item k - 1, its zone-end flag set when item k + 1 is built.
    for (int k = 0; sit[k % 3].valid; ++k) {
        const MomItem &cur = sit[k % 3];
        if (!mbar_wait(bar, (uint32_t)(k & 1), err, 5)) ok = false;
        __syncthreads();  // every thread done with the previous item's VY, H23 and tq
        const int nb = cur.nb;
        const bool zend = cur.zend;
        if (cur.q0 == 0) {
            // corner values c0..c3 of element u, term t -> {c0, c2 - c0, c1 - c0, c0 - c1 - c2 + c3}
            const float *csl = cwin(cur.cl, 0, 0), *csr = cwin(1 - cur.cl, 0, 0);
            auto coef = [&](int u, int t, float (&c)[4]) {
                const int o = t * kWin + (u < nval ? wofs + u * nm : wofs);
                const float c0 = csl[o], c1 = csr[o], c2 = csl[o + 3 * kWin], c3 = csr[o + 3 * kWin];
                zf[u][t] += fmaf(cur.wp[3], c3, fmaf(cur.wp[2], c2, fmaf(cur.wp[1], c1, cur.wp[0] * c0)));
                c[0] = c0;
                c[1] = c2 - c0;
                c[2] = c1 - c0;
                c[3] = (c0 - c1) - (c2 - c3);
            };
#pragma unroll
            for (int u = 0; u < EPT; ++u) {
                float a[4], b[4];
                coef(u, 0, a);
                coef(u, 2, b);
#pragma unroll
                for (int c = 0; c < 4; ++c) c12[u][c] = pk2(a[c], b[c]);
            }
            {
                float a[4], b[4];
                coef(0, 1, a);
                coef(1, 1, b);
                if constexpr (EPT == 3) coef(2, 1, c3s);
#pragma unroll
                for (int c = 0; c < 4; ++c) c3p[c] = pk2(a[c], b[c]);
            }
        }
        // FRF rows -> V, Y, H2, H3 of the item's points; (ti, tj)
        for (int ql = sq0; ql < nb; ql += 256 / kVY) {
            const float2 *h = Hraw + ql * hs;
            if (svy) {
                const float w = h[3 * nm].x;
                const int jg = jg0 + sjl;
                const float2 h1 = h[sm], h2 = h[nm + sm];
                const float2 h1j = h[jg], h3j = h[2 * nm + jg];
                // V = w H1(m) conj H3(j'),  Y = w H1(j') H2(m)
                VY[ql][st] = make_float4(w * (h1.x * h3j.x + h1.y * h3j.y), w * (h1j.x * h2.x - h1j.y * h2.y),
                                         w * (h1.y * h3j.x - h1.x * h3j.y), w * (h1j.x * h2.y + h1j.y * h2.x));
            }
            if (st < nm) {
                const float2 h2 = h[nm + st], h3 = h[2 * nm + st];
                H23[ql][st] = make_float4(h2.x, h3.x, -h2.y, h3.y);
            }
        }
        if (tid < nb) {
            const int qq = cur.q0 + tid, qr = qq / cur.nqj, qc = qq - qr * cur.nqj;
            const float ti = (float)qr * cur.rFi, tj = (float)qc * cur.rFj;
            tq[tid] = make_ulonglong2(pk2(ti, ti), pk2(tj, tj));
            tq2[tid] = pk2(ti * tj, ti * tj);
        }
        // VY, H23 and tq ready; FRF rows and corners consumed, the item's fields read
        if (__syncthreads_or(!ok)) break;  // a copy did not arrive: leave with the error code set
        // the next item's copies and the item after it run under this item's arithmetic
        MomItem &nxt = sit[(k + 1) % 3];
        if (tid < 32 && nxt.valid) issue(nxt, tid);
        if (tid == 32) build(nxt, sit[(k + 2) % 3]);
        for (int ql = 0; ql < nb; ++ql) {
            const ulonglong2 tt = tq[ql];
            const f2x ti2 = tt.x, tj2 = tt.y, tij2 = tq2[ql];
            const ulonglong2 hb = H23p[ql][bb];  // {H2r(b), H3r(b)}, {-H2i(b), H3i(b)}
            const float4 ybv = VY[ql][yb];       // .y, .w: Y_j'(b)
            float f3[EPT];
#pragma unroll
            for (int u = 0; u < EPT; ++u) {
                const ulonglong2 va = VYp[ql][ia0 + u];  // {Vr(a), Yr(a)}, {Vi(a), Yi(a)}
                const float4 h3a = H23[ql][ih0 + u];     // .y, .w: H3(a)
                // {T1, T2} = {Re[H2(b) V_j'(a)], Re[Y_j'(a) conj H3(b)]}
                const f2x f12 = fma2(hb.y, va.y, mul2(hb.x, va.x));
                f3[u] = fmaf(ybv.w, h3a.w, ybv.y * h3a.y);  // T3 = Re[Y_j'(b) conj H3(a)]
                const f2x v = fma2(tij2, c12[u][3], fma2(tj2, c12[u][2], fma2(ti2, c12[u][1], c12[u][0])));
                z12[u] = fma2(f12, v, z12[u]);
            }
            {
                const f2x v = fma2(tij2, c3p[3], fma2(tj2, c3p[2], fma2(ti2, c3p[1], c3p[0])));
                z3p = fma2(pk2(f3[0], f3[1]), v, z3p);
                if constexpr (EPT == 3) {
                    const float ti = up2(ti2).x, tj = up2(tj2).x, tij = up2(tij2).x;
                    const float vs = fmaf(tij, c3s[3], fmaf(tj, c3s[2], fmaf(ti, c3s[1], c3s[0])));
                    z3s = fmaf(f3[EPT - 1], vs, z3s);
                }
            }
        }
        if (zend) {
            const float2 p3 = up2(z3p);
#pragma unroll
            for (int u = 0; u < EPT; ++u) {
                const float2 p12 = up2(z12[u]);
                const float zr[3] = {p12.x, u == 0 ? p3.x : u == 1 ? p3.y : z3s, p12.y};
#pragma unroll
                for (int t = 0; t < 3; ++t) {
                    if (u < nval) {
                        pg[(size_t)t * nm3 + u * nm] += (double)zf[u][t];
                        pg[(size_t)(3 + t) * nm3 + u * nm] += (double)zr[t];
                    }
                    zf[u][t] = 0.f;
                }
                z12[u] = 0ull;
            }
            z3p = 0ull;
            z3s = 0.f;
        }
    }
}

// Per-zone mode-diagonal response moments m3mr(m, m, m) of the zone alone (the refinement
// criterion's quantity): one block per zone, threads over its BRM points, the three terms
// summed at element (m, m, m) before the FRF (the same FRF for all three there).
__global__ void k_msh_zone_diag(int nm, size_t nm3p, const ZoneM *__restrict__ zones, const float *__restrict__ T1,
                                const float *__restrict__ T3, const float *__restrict__ T2,
                                const float2 *__restrict__ Hq, const float *__restrict__ Wq,
                                double *__restrict__ zdiag) {
    const ZoneM z = zones[blockIdx.x];
    const int nm2 = nm * nm;
    const int NI = (z.ni - 1) * z.Fi, NJ = (z.nj - 1) * z.Fj, nq = (NI + 1) * (NJ + 1);
    __shared__ double red[256];
    for (int m = 0; m < nm; ++m) {
        const size_t em = (size_t)m * nm2 + (size_t)m * nm + m;
        double s = 0.0;
        for (int q = threadIdx.x; q < nq; q += blockDim.x) {
            const int qi = q / (NJ + 1), qj = q % (NJ + 1);
            const int i0 = min(qi / z.Fi, z.ni - 2), j0 = min(qj / z.Fj, z.nj - 2);
            const float ti = (float)(qi - i0 * z.Fi) / (float)z.Fi, tj = (float)(qj - j0 * z.Fj) / (float)z.Fj;
            const size_t P00 = (size_t)z.pbase + (size_t)i0 * z.nj + j0, P01 = P00 + 1, P10 = P00 + z.nj,
                         P11 = P10 + 1;
            float c[4];
            const size_t P[4] = {P00, P01, P10, P11};
#pragma unroll
            for (int k = 0; k < 4; ++k)
                c[k] = T1[P[k] * nm3p + em] + T3[P[k] * nm3p + em] + T2[P[k] * nm3p + em];
            const float v = (c[0] * (1.f - tj) + c[1] * tj) * (1.f - ti) + (c[2] * (1.f - tj) + c[3] * tj) * ti;
            const size_t gq = (size_t)z.qbase + q;
            const float2 *hrow = Hq + gq * frf_row(nm);
            const float2 h1 = hrow[m], h2 = hrow[nm + m], h3 = hrow[2 * nm + m];
            const float F = (h1.x * h2.x - h1.y * h2.y) * h3.x + (h1.x * h2.y + h1.y * h2.x) * h3.y;
            s += (double)(Wq[gq] * F * v);
        }
        red[threadIdx.x] = s;
        __syncthreads();
        for (int h = blockDim.x / 2; h > 0; h >>= 1) {
            if ((int)threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
            __syncthreads();
        }
        if (threadIdx.x == 0) zdiag[(size_t)blockIdx.x * nm + m] = 2.0 * red[0];
        __syncthreads();
    }
}

// m3[m + nm n + nm^2 o] = 2 sum_g (T1 at (a,b,j') = (m,n,o) + T3 at (o,n,m) + T2 at (n,o,m)).
__global__ void k_msh_reduce(int nm, int G, const double *__restrict__ part, double *__restrict__ m3mf,
                             double *__restrict__ m3mr) {
    const int nm2 = nm * nm, nm3 = nm2 * nm;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= nm3) return;
    const int m = x % nm, n = (x / nm) % nm, o = x / nm2;
    const int e1 = o * nm2 + m * nm + n, e3 = m * nm2 + o * nm + n, e2 = m * nm2 + n * nm + o;
    double sf = 0.0, sr = 0.0;
    for (int g = 0; g < G; ++g) {
        const double *pg = part + (size_t)g * 6 * nm3;
        sf += pg[e1] + pg[(size_t)nm3 + e3] + pg[(size_t)2 * nm3 + e2];
        sr += pg[(size_t)3 * nm3 + e1] + pg[(size_t)4 * nm3 + e3] + pg[(size_t)5 * nm3 + e2];
    }
    m3mf[x] = 2.0 * sf;
    m3mr[x] = 2.0 * sr;
}

// ------------------------------------------------------------------------------------
// Device-side expansion of a zone pass: the zone list (one ZoneX per axis-aligned zone, with
// its offsets) becomes, on the device, the distinct frequencies (A-table rows), the distinct
// line / column frequencies (U blocks), the point and column index tables, the tasks and the
// work queue.  Frequencies meet in open-addressing hash tables keyed by round(f 2^40) (values
// equal to ~1e-12 Hz share a row); the occupied slots are then numbered in slot order.
// ------------------------------------------------------------------------------------
struct ZoneX {
    double fi0, fj0, dI, dJ;  // f1 = fi0 + i dI (lines), f2 = fj0 + j dJ (columns)
    int ni, nj;
    long long pbase;  // first BFM point of the zone
    int gbase;        // first column (G row block)
    int tbase;        // first task: ni line tasks, then nj column tasks
    long long ibase;  // first work item
};

constexpr unsigned long long kEmptyKey = 0x8080808080808080ull;  // memset pattern 0x80

__device__ __forceinline__ long long fkey(double f) { return __double2ll_rn(f * 1099511627776.0); }  // 2^40

__device__ __forceinline__ unsigned long long fhash(long long q, int bits) {
    return ((unsigned long long)q * 0x9E3779B97F4A7C15ull) >> (64 - bits);
}

// Insert f's key; the table is at most half full.  A row's frequency is its key q 2^-40 (within
// 4.6e-13 Hz of every frequency it serves), so the rows' values do not depend on which thread
// inserted first.
__device__ __forceinline__ void ht_insert(unsigned long long *keys, int bits, double f) {
    const long long q = fkey(f);
    const unsigned long long mask = (1ull << bits) - 1;
    unsigned long long h = fhash(q, bits);
    for (unsigned long long probe = 0; probe <= mask; ++probe, h = (h + 1) & mask) {
        const unsigned long long prev = atomicCAS(&keys[h], kEmptyKey, (unsigned long long)q);
        if (prev == kEmptyKey || prev == (unsigned long long)q) return;
    }
}

// Row of f (its slot's number); -1 if absent (never for an inserted f).
__device__ __forceinline__ int ht_find(const unsigned long long *keys, const int *ids, int bits, double f) {
    const long long q = fkey(f);
    const unsigned long long mask = (1ull << bits) - 1;
    unsigned long long h = fhash(q, bits);
    for (unsigned long long probe = 0; probe <= mask; ++probe, h = (h + 1) & mask) {
        const unsigned long long k = keys[h];
        if (k == (unsigned long long)q) return ids[h];
        if (k == kEmptyKey) return -1;
    }
    return -1;
}

// Line, column and point frequencies of a zone, rounded as written (no contraction).
__device__ __forceinline__ double zx_line(const ZoneX &z, int i) { return __dadd_rn(z.fi0, __dmul_rn((double)i, z.dI)); }
__device__ __forceinline__ double zx_col(const ZoneX &z, int j) { return __dadd_rn(z.fj0, __dmul_rn((double)j, z.dJ)); }

__global__ void k_fx_insert(int nz, const ZoneX *__restrict__ zx, unsigned long long *keysF, int bitsF,
                            unsigned long long *keysU, int bitsU) {
    const ZoneX z = zx[blockIdx.x];
    const long long n = (long long)z.ni + z.nj + (long long)z.ni * z.nj;
    for (long long x = threadIdx.x; x < n; x += blockDim.x) {
        double f;
        bool lc = true;
        if (x < z.ni) {
            f = zx_line(z, (int)x);
        } else if (x < z.ni + z.nj) {
            f = zx_col(z, (int)(x - z.ni));
        } else {
            const long long y = x - z.ni - z.nj;
            const int i = (int)(y / z.nj), j = (int)(y - (long long)i * z.nj);
            f = __dadd_rn(zx_line(z, i), zx_col(z, j));
            lc = false;
        }
        ht_insert(keysF, bitsF, f);
        if (lc) ht_insert(keysU, bitsU, f);
    }
}

constexpr int kScanBlock = 1024;

// Occupied slots per block of kScanBlock slots.
__global__ void k_fx_count(int cap, const unsigned long long *__restrict__ keys, int *__restrict__ cnt) {
    const int s = blockIdx.x * kScanBlock + threadIdx.x;
    const int occ = s < cap && keys[s] != kEmptyKey;
    const int c = __syncthreads_count(occ);
    if (threadIdx.x == 0) cnt[blockIdx.x] = c;
}

// Exclusive scan of the block counts in place (one block); cnt[nb] receives the total.
__global__ void k_fx_scan(int nb, int *__restrict__ cnt) {
    __shared__ int carry;
    __shared__ int ws[32];
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int b0 = 0; b0 < nb; b0 += blockDim.x) {
        const int b = b0 + threadIdx.x;
        const int v = b < nb ? cnt[b] : 0;
        int x = v;  // inclusive warp scan
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, o);
            if ((threadIdx.x & 31) >= o) x += y;
        }
        if ((threadIdx.x & 31) == 31) ws[threadIdx.x >> 5] = x;
        __syncthreads();
        if (threadIdx.x < 32) {
            int w = threadIdx.x < (int)(blockDim.x >> 5) ? ws[threadIdx.x] : 0;
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, w, o);
                if (threadIdx.x >= o) w += y;
            }
            ws[threadIdx.x] = w;  // inclusive over warps
        }
        __syncthreads();
        const int excl = carry + x - v + ((threadIdx.x >> 5) ? ws[(threadIdx.x >> 5) - 1] : 0);
        if (b < nb) cnt[b] = excl;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = excl + v;
        __syncthreads();
    }
    if (threadIdx.x == 0) cnt[nb] = carry;
}

// Number the occupied slots in slot order; the row's frequency is its key q 2^-40.
__global__ void k_fx_ids(int cap, const unsigned long long *__restrict__ keys, const int *__restrict__ off,
                         int *__restrict__ ids, double *__restrict__ freq) {
    __shared__ int ws[kScanBlock / 32];
    const int s = blockIdx.x * kScanBlock + threadIdx.x;
    const int occ = s < cap && keys[s] != kEmptyKey;
    const unsigned bal = __ballot_sync(0xffffffffu, occ);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) ws[warp] = __popc(bal);
    __syncthreads();
    int before = 0;
    for (int w = 0; w < warp; ++w) before += ws[w];
    if (occ) {
        const int id = off[blockIdx.x] + before + __popc(bal & ((1u << lane) - 1u));
        ids[s] = id;
        freq[id] = __ll2double_rn((long long)keys[s]) * 9.094947017729282379150390625e-13;  // 2^-40
    }
}

// The zone's tables: U block and A row of its lines and columns, its point (sum) rows in line
// and in column order, its tasks and its work items, in the order the host would list them.
__global__ void k_fx_expand(int nz, const ZoneX *__restrict__ zx, const unsigned long long *__restrict__ keysF,
                            const int *__restrict__ idsF, int bitsF, const unsigned long long *__restrict__ keysU,
                            const int *__restrict__ idsU, int bitsU, long long npts, int Mp, int NMT, int NC, int MT,
                            int *__restrict__ usrc, int *__restrict__ gsrc, int *__restrict__ ssrc,
                            Task *__restrict__ tasks, int4 *__restrict__ items, int *__restrict__ err) {
    const ZoneX z = zx[blockIdx.x];
    const int ntl_l = (z.nj + NC - 1) / NC, ntl_c = (z.ni + NC - 1) / NC, nic = (ntl_c + 1) / 2;
    const long long line_items = (long long)z.ni * MT * ntl_l;
    for (int x = threadIdx.x; x < z.ni + z.nj; x += blockDim.x) {
        const bool line = x < z.ni;
        const int i = line ? x : x - z.ni;
        const double f = line ? zx_line(z, i) : zx_col(z, i);
        int fid = ht_find(keysF, idsF, bitsF, f), uid = ht_find(keysU, idsU, bitsU, f);
        if (fid < 0 || uid < 0) {  // never for an inserted frequency; row 0 keeps every index valid
            atomicCAS(err, 0, 8);
            fid = max(fid, 0);
            uid = max(uid, 0);
        }
        usrc[uid] = fid;  // zones sharing the frequency write the same value
        if (line) {
            tasks[z.tbase + i] = Task{uid * Mp, z.gbase * NMT, (int)((z.pbase + (long long)i * z.nj) * NMT), z.nj,
                                      (int)(z.pbase + (long long)i * z.nj), 1, 0};
        } else {
            gsrc[z.gbase + i] = fid;
            tasks[z.tbase + z.ni + i] = Task{uid * Mp, -1, (int)((npts + z.pbase + (long long)i * z.ni) * NMT), z.ni,
                                             (int)(z.pbase + i), z.nj, 1};
        }
    }
    for (long long y = threadIdx.x; y < (long long)z.ni * z.nj; y += blockDim.x) {
        const int i = (int)(y / z.nj), j = (int)(y - (long long)i * z.nj);
        int fid = ht_find(keysF, idsF, bitsF, __dadd_rn(zx_line(z, i), zx_col(z, j)));
        if (fid < 0) {
            atomicCAS(err, 0, 8);
            fid = 0;
        }
        ssrc[z.pbase + y] = fid;                                    // line order (line tasks)
        ssrc[npts + z.pbase + (long long)j * z.ni + i] = fid;       // column order (column tasks)
    }
    const long long nit = line_items + (long long)z.nj * MT * nic;
    for (long long y = threadIdx.x; y < nit; y += blockDim.x) {
        int4 it;
        if (y < line_items) {
            const int i = (int)(y / ((long long)MT * ntl_l));
            const int r = (int)(y - (long long)i * MT * ntl_l), mt = r / ntl_l, nt = r - mt * ntl_l;
            it = make_int4(z.tbase + i, mt, nt, nt + 1);
        } else {
            const long long yc = y - line_items;
            const int j = (int)(yc / ((long long)MT * nic));
            const int r = (int)(yc - (long long)j * MT * nic), mt = r / nic, k = r - mt * nic;
            it = make_int4(z.tbase + z.ni + j, mt, 2 * k, min(2 * k + 2, ntl_c));
        }
        items[z.ibase + y] = it;
    }
}

}  // namespace mshmix

// ------------------------------------------------------------------------------------
// Host side: zone batches -> operand tables -> tasks -> contraction -> zone integration.
// ------------------------------------------------------------------------------------
namespace {

// The lattice of z aligned with the axes, as (f1 index axis, f2 index axis); false if rotated.
bool axis_aligned(const ZoneDev &z, ZoneDev &out) {
    if (z.dIj == 0.0 && z.dJi == 0.0) {
        out = z;
        return true;
    }
    if (z.dIi == 0.0 && z.dJj == 0.0) {  // f1 runs along J, f2 along I: relabel the axes
        out = z;
        out.dIi = z.dJi; out.dIj = 0.0; out.dJi = 0.0; out.dJj = z.dIj;
        out.wI = z.wJ; out.wJ = z.wI;
        out.ni = z.nj; out.nj = z.ni;
        out.Fi = z.Fj; out.Fj = z.Fi;
        return true;
    }
    return false;
}

// Distinct frequencies of a zone batch.  Values closer than kFreqTol (1 + |f|) are one entry:
// the sums r_i + c_j of lattices with equal steps on both axes repeat up to the last bits of
// their rounding, and one A(f) row serves them all (A(f) moves on the scale of the spectra's
// bandwidths, ~1e-3 Hz, not 1e-12 Hz).  A run of sorted values within the tolerance of its
// first element keeps that first element; at() returns the nearest kept value.
constexpr double kFreqTol = 1e-12;

struct FreqIndex {
    std::vector<double> v;
    void add(double f) { v.push_back(f); }
    void seal() {
        std::sort(v.begin(), v.end());
        size_t w = 0;
        for (size_t r = 0; r < v.size(); ++r)
            if (w == 0 || v[r] - v[w - 1] > kFreqTol * (1.0 + std::fabs(v[w - 1]))) v[w++] = v[r];
        v.resize(w);
    }
    int at(double f) const {
        const size_t i = (size_t)(std::lower_bound(v.begin(), v.end(), f) - v.begin());
        if (i == v.size()) return (int)i - 1;
        if (i > 0 && f - v[i - 1] <= v[i] - f) return (int)i - 1;
        return (int)i;
    }
};

}  // namespace

int Engine::msh_mixed_batch(const std::vector<ZoneDev> &zs, std::vector<double> &accF, std::vector<double> &accR,
                            float &ms_gemm, float &ms_all, double *zdiag) {
    using namespace mshmix;
    const int nm = nme, nm2 = nm * nm, nm3 = nm2 * nm;
    const int NMT = plan_msh_width(nm, K), NC = kBN / NMT, BROWS = NC * NMT;
    const int Kp = ((K + kBK - 1) / kBK) * kBK, Mp = ((nm2 + kBM - 1) / kBM) * kBM, MT = Mp / kBM;
    // Per-zone records and offsets (O(zones) on the host): ZoneM for the zone integration, ZoneX
    // for the expansion -- the first BFM point, column, task and work item of every zone.
    long long npts = 0, ncells = 0, ncol = 0, nbrm = 0, ntasks = 0, nitems = 0;
    std::vector<ZoneM> zm;
    std::vector<ZoneX> zx;
    zm.reserve(zs.size());
    zx.reserve(zs.size());
    for (const ZoneDev &z : zs) {
        zm.push_back(ZoneM{z.fi0, z.fj0, z.dIi, z.dJj, z.wI, z.wJ, z.sym, z.ni, z.nj, z.Fi, z.Fj, (int)npts, (int)ncells,
                           (int)nbrm, (float)(z.sym * z.wI * z.wJ)});
        zx.push_back(ZoneX{z.fi0, z.fj0, z.dIi, z.dJj, z.ni, z.nj, npts, (int)ncol, (int)ntasks, nitems});
        const long long ntl_l = (z.nj + NC - 1) / NC, ntl_c = (z.ni + NC - 1) / NC;
        nitems += (long long)z.ni * MT * ntl_l + (long long)z.nj * MT * ((ntl_c + 1) / 2);
        npts += (long long)z.ni * z.nj;
        ncells += (long long)(z.ni - 1) * (z.nj - 1);
        ncol += z.nj;
        ntasks += z.ni + z.nj;
        nbrm += (long long)((z.ni - 1) * z.Fi + 1) * ((z.nj - 1) * z.Fj + 1);
    }
    if (2 * npts * NMT > 0x7fffffffLL || nitems > 0x7fffffffLL || nbrm > 0x7fffffffLL)
        return fail(BSA_ERR_ARG, "Mesher zone pass too large");
    cudaError_t e;
    int rc;
    if ((e = cudaEventRecord(ev2, stream))) return cuda_fail(e, "event");
    // index tables, tasks, zone records and the work queue (U blocks: at most one per line /
    // column frequency)
    const size_t nlc = (size_t)ntasks;
    const size_t nidx = nlc + ncol + 2 * (size_t)npts;
    auto al16 = [](const void *q) { return (((uintptr_t)q) + 15) & ~(uintptr_t)15; };
    if ((e = dMshIdx.reserve(nidx * sizeof(int) + ntasks * sizeof(Task) + zm.size() * sizeof(ZoneM) +
                             nitems * sizeof(int4) + zx.size() * sizeof(ZoneX) + 128)))
        return cuda_fail(e, "allocating Mesher tables");
    char *ib = (char *)dMshIdx.p;
    int *d_usrc = (int *)ib, *d_gsrc = d_usrc + nlc, *d_ssrc = d_gsrc + ncol;
    Task *d_tasks = (Task *)al16(d_ssrc + 2 * npts);
    ZoneM *d_zones = (ZoneM *)al16(d_tasks + ntasks);
    int4 *d_items = (int4 *)al16(d_zones + zm.size());
    ZoneX *d_zx = (ZoneX *)al16(d_items + nitems);
    int nU = 0, *d_xerr = nullptr;
    if ((e = cudaMemcpyAsync(d_zones, zm.data(), zm.size() * sizeof(ZoneM), cudaMemcpyHostToDevice, stream)))
        return cuda_fail(e, "Mesher zone upload");
    h2d += (double)(zm.size() * sizeof(ZoneM));
    if (msh_dev_expand && !pod_truncates()) {
        // The pass expanded on the device: distinct frequencies through hash tables, numbered in
        // slot order (A rows into dFreq, U blocks), then every zone's tables and work items.
        const long long nF_max = (long long)nlc + npts;
        int bitsF = 4, bitsU = 4;
        while ((1LL << bitsF) < 2 * nF_max) ++bitsF;
        while ((1LL << bitsU) < 2 * (long long)nlc) ++bitsU;
        const long long capF = 1LL << bitsF, capU = 1LL << bitsU;
        if (capF > (1LL << 30)) return fail(BSA_ERR_ARG, "Mesher zone pass too large");
        const int nbF = (int)((capF + kScanBlock - 1) / kScanBlock), nbU = (int)((capU + kScanBlock - 1) / kScanBlock);
        const size_t hbytes = (size_t)(capF + capU) * (8 + 4) + (size_t)(nbF + nbU + 2) * 4 + 16 * 8 +
                              (size_t)capU * 8;
        if ((e = dHash.reserve(hbytes)) || (e = dFreq.reserve(sizeof(double) * (size_t)nF_max)))
            return cuda_fail(e, "allocating Mesher frequency tables");
        unsigned long long *keysF = dHash.as<unsigned long long>(), *keysU = keysF + capF;
        double *ufreq = (double *)(keysU + capU);
        int *idsF = (int *)(ufreq + capU), *idsU = idsF + capF, *cntF = idsU + capU, *cntU = cntF + nbF + 1;
        d_xerr = cntU + nbU + 1;
        if ((e = cudaMemsetAsync(keysF, 0x80, (size_t)(capF + capU) * 8, stream)) ||
            (e = cudaMemsetAsync(d_xerr, 0, sizeof(int), stream)) ||
            (e = cudaMemcpyAsync(d_zx, zx.data(), zx.size() * sizeof(ZoneX), cudaMemcpyHostToDevice, stream)))
            return cuda_fail(e, "Mesher expansion set-up");
        h2d += (double)(zx.size() * sizeof(ZoneX));
        const int nz = (int)zx.size();
        k_fx_insert<<<nz, 256, 0, stream>>>(nz, d_zx, keysF, bitsF, keysU, bitsU);
        k_fx_count<<<nbF, kScanBlock, 0, stream>>>((int)capF, keysF, cntF);
        k_fx_scan<<<1, 1024, 0, stream>>>(nbF, cntF);
        k_fx_ids<<<nbF, kScanBlock, 0, stream>>>((int)capF, keysF, cntF, idsF, dFreq.as<double>());
        k_fx_count<<<nbU, kScanBlock, 0, stream>>>((int)capU, keysU, cntU);
        k_fx_scan<<<1, 1024, 0, stream>>>(nbU, cntU);
        k_fx_ids<<<nbU, kScanBlock, 0, stream>>>((int)capU, keysU, cntU, idsU, ufreq);
        int counts[2] = {0, 0};
        if ((e = cudaGetLastError()) ||
            (e = cudaMemcpyAsync(&counts[0], cntF + nbF, sizeof(int), cudaMemcpyDeviceToHost, stream)) ||
            (e = cudaMemcpyAsync(&counts[1], cntU + nbU, sizeof(int), cudaMemcpyDeviceToHost, stream)) ||
            (e = cudaStreamSynchronize(stream)))
            return cuda_fail(e, "Mesher frequency tables");
        nU = counts[1];
        k_fx_expand<<<nz, 256, 0, stream>>>(nz, d_zx, keysF, idsF, bitsF, keysU, idsU, bitsU, npts, Mp, NMT, NC, MT,
                                            d_usrc, d_gsrc, d_ssrc, d_tasks, d_items, d_xerr);
        if ((e = cudaGetLastError())) return cuda_fail(e, "Mesher zone expansion");
        kernels += 8;
        if ((rc = build_atable_dev(counts[0], true))) return rc;
    } else {
        // The same tables built on the host (and the frequencies of the truncated POD form,
        // whose A table is formed from host frequencies).
        FreqIndex F, UF;
        for (const ZoneDev &z : zs) {
            for (int i = 0; i < z.ni; ++i) {
                const double r = z.fi0 + i * z.dIi;
                F.add(r);
                UF.add(r);
                for (int j = 0; j < z.nj; ++j) F.add(r + (z.fj0 + j * z.dJj));
            }
            for (int j = 0; j < z.nj; ++j) {
                F.add(z.fj0 + j * z.dJj);
                UF.add(z.fj0 + j * z.dJj);
            }
        }
        F.seal();
        UF.seal();
        nU = (int)UF.v.size();
        std::vector<int> usrc(nU), gsrc((size_t)ncol), ssrc(2 * (size_t)npts);
        for (int u = 0; u < nU; ++u) usrc[u] = F.at(UF.v[u]);
        std::vector<Task> tasks;
        tasks.reserve(ntasks);
        for (size_t k = 0; k < zs.size(); ++k) {
            const ZoneDev &z = zs[k];
            const long long pb = zx[k].pbase, gb = zx[k].gbase;
            for (int j = 0; j < z.nj; ++j) gsrc[gb + j] = F.at(z.fj0 + j * z.dJj);
            for (int i = 0; i < z.ni; ++i) {
                const double r = z.fi0 + i * z.dIi;
                for (int j = 0; j < z.nj; ++j) {
                    const int row = F.at(r + (z.fj0 + j * z.dJj));
                    ssrc[pb + (size_t)i * z.nj + j] = row;         // line order (kind 0)
                    ssrc[npts + pb + (size_t)j * z.ni + i] = row;  // column order (kind 1)
                }
                tasks.push_back(Task{UF.at(r) * Mp, (int)gb * NMT, (int)(pb + (long long)i * z.nj) * NMT, z.nj,
                                     (int)(pb + (long long)i * z.nj), 1, 0});
            }
            for (int j = 0; j < z.nj; ++j)
                tasks.push_back(Task{UF.at(z.fj0 + j * z.dJj) * Mp, -1, (int)(npts + pb + (long long)j * z.ni) * NMT,
                                     z.ni, (int)(pb + j), z.nj, 1});
        }
        // work items: per task, its row tiles x N tiles (one, or two for column tasks), consecutive
        std::vector<int4> witems;
        witems.reserve(nitems);
        for (size_t t = 0; t < tasks.size(); ++t) {
            const int ntl = (tasks[t].ncols + NC - 1) / NC;
            const int step = tasks[t].kind == 1 ? 2 : 1;  // column tasks: two N tiles per item
            for (int mt = 0; mt < MT; ++mt)
                for (int nt = 0; nt < ntl; nt += step)
                    witems.push_back(make_int4((int)t, mt, nt, std::min(nt + step, ntl)));
        }
        if ((long long)witems.size() != nitems) return fail(BSA_ERR_STATE, "Mesher work-item count");
        if ((e = cudaMemcpyAsync(d_usrc, usrc.data(), nU * sizeof(int), cudaMemcpyHostToDevice, stream)) ||
            (e = cudaMemcpyAsync(d_gsrc, gsrc.data(), ncol * sizeof(int), cudaMemcpyHostToDevice, stream)) ||
            (e = cudaMemcpyAsync(d_ssrc, ssrc.data(), 2 * npts * sizeof(int), cudaMemcpyHostToDevice, stream)) ||
            (e = cudaMemcpyAsync(d_tasks, tasks.data(), tasks.size() * sizeof(Task), cudaMemcpyHostToDevice, stream)) ||
            (e = cudaMemcpyAsync(d_items, witems.data(), witems.size() * sizeof(int4), cudaMemcpyHostToDevice,
                                 stream)))
            return cuda_fail(e, "Mesher task upload");
        h2d += (double)((nU + ncol + 2 * npts) * sizeof(int) + tasks.size() * sizeof(Task) +
                        witems.size() * sizeof(int4));
        if ((rc = build_atable(F.v, true, true))) return rc;
    }
    const size_t uel = (size_t)nU * Mp * Kp, gel = (size_t)ncol * NMT * Kp, sel = 2 * (size_t)npts * NMT * Kp;
    const int nm3p = (nm3 + 3) & ~3, hs = frf_row(nm);
    const size_t tel = (size_t)npts * nm3p;
    int dev = 0, nsm = 0;
    if ((e = cudaGetDevice(&dev)) || (e = cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev)))
        return cuda_fail(e, "device query");
    const MomLayout ML = MomLayout::make(nm);
    const int nchunks = ML.groups(nm) * ML.nchj;
    // one wave of two resident blocks per SM where the element chunks allow it
    const int G = (int)std::max(1LL, std::min((long long)(2 * nsm) / nchunks, ncells));
    auto reserve_pass = [&]() -> cudaError_t {
        cudaError_t r;
        if ((r = dMixA.reserve(2 * uel * 2)) || (r = dMixB.reserve(2 * (gel + sel) * 2)) ||
            (r = dMshT.reserve(3 * tel * sizeof(float))) ||
            (r = dMixPart.reserve((size_t)G * 6 * nm3 * sizeof(double) + 2 * (size_t)nm3 * sizeof(double) + 256)) ||
            (r = dMixH.reserve((size_t)nbrm * hs * sizeof(float2) + (size_t)nbrm * sizeof(float) + 256 +
                               (zdiag ? zm.size() * nm * sizeof(double) : 0))))
            return r;
        return cudaSuccess;
    };
    if ((e = reserve_pass()) == cudaErrorMemoryAllocation) {
        // each buffer keeps the largest size an earlier pass asked for, and passes that peak in
        // different operands can hold more together than one pass needs: start over from empty
        cudaGetLastError();
        dMixA.release(); dMixB.release(); dMshT.release(); dMixPart.release(); dMixH.release();
        release_device_cache();
        e = reserve_pass();
    }
    if (e) return cuda_fail(e, "allocating Mesher BF16x3 operands");
    __nv_bfloat16 *Uh = dMixA.as<__nv_bfloat16>(), *Ul = Uh + uel;
    __nv_bfloat16 *Gh = dMixB.as<__nv_bfloat16>(), *Gl = Gh + gel, *Sh = Gl + gel, *Sl = Sh + sel;
    float *T1 = dMshT.as<float>(), *T3 = T1 + tel, *T2 = T3 + tel;
    double *part = dMixPart.as<double>(), *red = part + (size_t)G * 6 * nm3;
    int *derr = (int *)(red + 2 * (size_t)nm3), *dhead = derr + 1;
    if ((e = cudaMemsetAsync(derr, 0, 2 * sizeof(int), stream)))  // error flag and queue head
        return cuda_fail(e, "Mesher task upload");
    CUtensorMap maps[6];
    if (!make_map(&maps[0], Uh, Kp, (uint64_t)nU * Mp, kBM) || !make_map(&maps[1], Ul, Kp, (uint64_t)nU * Mp, kBM) ||
        !make_map(&maps[2], Gh, Kp, (uint64_t)ncol * NMT, BROWS) || !make_map(&maps[3], Gl, Kp, (uint64_t)ncol * NMT, BROWS) ||
        !make_map(&maps[4], Sh, Kp, 2 * (uint64_t)npts * NMT, BROWS) ||
        !make_map(&maps[5], Sl, Kp, 2 * (uint64_t)npts * NMT, BROWS))
        return fail(BSA_ERR_CUDA, "cuTensorMapEncodeTiled failed");
    MParams prm{};
    prm.nm = nm; prm.NMT = NMT; prm.NC = NC; prm.BROWS = BROWS; prm.Mp = Mp; prm.MT = MT;
    prm.nk = Kp / kBK;
    prm.ks_last = (K - (prm.nk - 1) * kBK + 15) / 16;
    prm.nitems = (int)nitems;
    prm.tasks = d_tasks;
    prm.items = d_items;
    prm.T1 = T1; prm.T3 = T3; prm.T2 = T2;
    prm.nm3p = nm3p;
    prm.err = derr;
    prm.head = dhead;
    const long long nwork = nitems;
    const int grid = (int)std::min<long long>(nwork, nsm);
    const size_t smem = (size_t)kStages * kStageBytes + 1024 + 256;
    if ((e = cudaFuncSetAttribute(k_msh_mixed, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)) ||
        (e = cudaFuncSetAttribute(k_msh_moments, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)MomLayout::smem())))
        return cuda_fail(e, "kernel attribute");
    float2 *Hq = dMixH.as<float2>();
    float *Wq = (float *)(Hq + (size_t)nbrm * hs);
    double *d_zdiag = zdiag ? (double *)(((uintptr_t)(Wq + nbrm) + 255) & ~(uintptr_t)255) : nullptr;
    // The pass's device work: operand rows, the tcgen05 contraction (bracketed by the timing
    // events), the FRF rows, the zone integration and its reductions.
    auto launch_all = [&](bool captured) -> cudaError_t {
        auto mark = [&](cudaEvent_t ev) {
            return captured ? cudaEventRecordWithFlags(ev, stream, cudaEventRecordExternal) : cudaEventRecord(ev, stream);
        };
        k_prep_u_rows<<<dim3(nU, Kp / 32), 256, 0, stream>>>(nm, K, Kp, Mp, d_usrc, dA32.as<float>(), dQ.as<double>(),
                                                             Uh, Ul);
        k_prep_b_rows<<<dim3((unsigned)ncol, Kp / 64), 256, 0, stream>>>(nm, NMT, K, Kp, d_gsrc, dA32.as<float>(), Gh,
                                                                         Gl);
        k_prep_b_rows<<<dim3((unsigned)(2 * npts), Kp / 64), 256, 0, stream>>>(nm, NMT, K, Kp, d_ssrc, dA32.as<float>(),
                                                                               Sh, Sl);
        cudaError_t r = mark(evg0);
        if (r) return r;
        k_msh_mixed<<<grid, 192, smem, stream>>>(maps[0], maps[1], maps[2], maps[3], maps[4], maps[5], prm);
        if ((r = mark(evg1))) return r;
        const long long nt = nbrm * 3 * nm;
        k_msh_frf<<<(unsigned)((nt + 255) / 256), 256, 0, stream>>>(nm, (int)zm.size(), d_zones, (int)nbrm, frf(), Hq,
                                                                     Wq);
        k_msh_moments<<<dim3(G, nchunks), 256, MomLayout::smem(), stream>>>(nm, nm3p, ML, d_zones, (int)zm.size(), T1,
                                                                           T3, T2, Hq, part, derr);
        k_msh_reduce<<<(nm3 + 127) / 128, 128, 0, stream>>>(nm, G, part, red, red + nm3);
        if (zdiag)
            k_msh_zone_diag<<<(unsigned)zm.size(), 256, 0, stream>>>(nm, (size_t)nm3p, d_zones, T1, T3, T2, Hq, Wq,
                                                                      d_zdiag);
        return cudaGetLastError();
    };
    // ... launched as one CUDA graph (one graph per zone pass: per refinement level of the
    // adaptive Mesher), captured from the stream; where capture or instantiation is not
    // available the same sequence is launched directly.
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    bool graphed = false;
    if (msh_graphs && cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
        const cudaError_t le = launch_all(true);
        const cudaError_t ce = cudaStreamEndCapture(stream, &graph);
        graphed = le == cudaSuccess && ce == cudaSuccess && graph &&
                  cudaGraphInstantiate(&gexec, graph, 0) == cudaSuccess && cudaGraphLaunch(gexec, stream) == cudaSuccess;
        if (!graphed) {
            cudaGetLastError();
            if (gexec) cudaGraphExecDestroy(gexec);
            if (graph) cudaGraphDestroy(graph);
            gexec = nullptr;
            graph = nullptr;
        }
    }
    if (!graphed && (e = launch_all(false))) return cuda_fail(e, "Mesher BF16x3 pass");
    kernels += 7 + (zdiag ? 1 : 0);
    graph_launches += graphed ? 1 : 0;
    std::vector<double> h(2 * (size_t)nm3);
    int herr = 0, xerr = 0;
    if ((d_xerr && (e = cudaMemcpyAsync(&xerr, d_xerr, sizeof(int), cudaMemcpyDeviceToHost, stream))) ||
        (e = cudaMemcpyAsync(h.data(), red, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, stream)) ||
        (e = cudaMemcpyAsync(&herr, derr, sizeof(int), cudaMemcpyDeviceToHost, stream)) ||
        (zdiag && (e = cudaMemcpyAsync(zdiag, d_zdiag, sizeof(double) * zm.size() * nm, cudaMemcpyDeviceToHost,
                                       stream))) ||
        (e = cudaEventRecord(ev1, stream)) || (e = cudaStreamSynchronize(stream)))
        return cuda_fail(e, "Mesher BF16x3 evaluation");
    if (gexec) cudaGraphExecDestroy(gexec);
    if (graph) cudaGraphDestroy(graph);
    d2h += (double)sizeof(double) * h.size() + sizeof(int);
    if (xerr) return fail(BSA_ERR_STATE, "Mesher zone expansion: a frequency missing from its table");
    if (herr) return fail(BSA_ERR_TIMEOUT, "Mesher BF16x3 kernel: a pipeline wait ran out of its budget (role %d)", herr);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, evg0, evg1);
    ms_gemm += ms;
    cudaEventElapsedTime(&ms, ev2, ev1);
    ms_all += ms;
    for (int x = 0; x < nm3; ++x) {
        accF[x] += h[x];
        accR[x] += h[nm3 + x];
    }
    return BSA_OK;
}

// Zones in the split precision: axis-aligned zones in batches through the tensor cores,
// rotated ones through the FP64 point kernel.
int Engine::run_zones_mixed(const std::vector<ZoneDev> &zones, double *m3mf, double *m3mr, double *npts,
                            double *zdiag) {
    int rc = upload_problem();
    if (rc) return rc;
    const int nm = nme;
    const long long nm3 = (long long)nm * nm * nm;
    if (nm > 64) return fail(BSA_ERR_UNSUPPORTED, "at most 64 kept modes");
    std::vector<ZoneDev> axis, rot;
    double nbfm = 0.0, nbrm = 0.0;
    for (const ZoneDev &z : zones) {
        if (z.ni < 2 || z.nj < 2 || z.Fi < 1 || z.Fj < 1)
            return fail(BSA_ERR_ARG, "zone lattice needs ni, nj >= 2 and Fi, Fj >= 1");
        ZoneDev a;
        if (axis_aligned(z, a)) axis.push_back(a); else rot.push_back(z);
        nbfm += (double)z.ni * z.nj;
        nbrm += (double)((z.ni - 1) * z.Fi + 1) * ((z.nj - 1) * z.Fj + 1);
    }
    if (zdiag && !rot.empty()) return fail(BSA_ERR_UNSUPPORTED, "per-zone moments need axis-aligned zones");
    std::vector<double> accF(nm3, 0.0), accR(nm3, 0.0);
    float ms_gemm = 0.f, ms_all = 0.f;
    int nk = 0;
    double hb = 0.0, db = 0.0;
    if (!rot.empty()) {
        std::vector<double> f(nm3), r(nm3);
        int rc = run_zones_fp64(rot, f.data(), r.data(), nullptr);
        if (rc) return rc;
        ms_gemm += (float)last_ms_gemm;
        ms_all += (float)last_ms;
        nk = kernels;
        hb = h2d;
        db = d2h;
        for (long long x = 0; x < nm3; ++x) { accF[x] += f[x]; accR[x] += r[x]; }
    }
    kernels = 0;
    graph_launches = 0;
    h2d = d2h = 0;
    if (!axis.empty()) {
        // batches by device bytes: U blocks of the distinct line / column frequencies, column
        // and sum tables, term tensors and BRM-point FRF tables, and the FP32 A row and nodal
        // spectra of each distinct frequency (a point may bring a sum frequency of its own)
        const int NMT = plan_msh_width(nm, K);
        const double Kp = (double)(((K + 63) / 64) * 64), Mp = (double)(((nm * nm + 127) / 128) * 128);
        const double per_f = (double)K * nm * 4.0 + (double)K * 8.0;
        const double per_u = Mp * Kp * 4.0 + per_f, per_col = NMT * Kp * 4.0 + per_f;
        const double per_pt = 2.0 * NMT * Kp * 4.0 + 3.0 * nm3 * 4.0 + per_f, per_q = 3.0 * nm * 8.0 + 4.0;
        // as much of the zone list per pass as 40 % of the device memory holds (one pass for the
        // reference layouts of the bench's structures on a GB300: the 60-mode bridge needs about
        // 88 GB), at least 4 GB; from the total, not the free memory, so the batching of a zone
        // list does not depend on what earlier analyses left allocated
        size_t fr = 0, tot = 0;
        if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) tot = 0;
        const double budget = msh_pass_bytes > 0.0 ? msh_pass_bytes : std::max(4e9, 0.4 * (double)tot);
        // A zone too large for a quarter of a pass is split into strips of consecutive lattice
        // lines that share their boundary lines (the trapezoid's half weights of a shared BFM /
        // BRM line from both strips add up to the unsplit zone's interior weight, and every cell
        // is interpolated within one strip): the same integrals in passes that fit.  A zone with
        // so many columns that their U blocks alone crowd a pass is first cut the same way into
        // blocks of columns that share their boundary columns.
        std::vector<int> parent;
        {
            std::vector<ZoneDev> split;
            auto by_lines = [&](const ZoneDev &z, int k) {
                const double NJ = (double)((z.nj - 1) * z.Fj + 1);
                const double line = per_u + per_pt * z.nj + per_q * z.Fi * NJ;  // bytes one more line adds
                const double fixed = per_u * z.nj + per_col * z.nj + per_q * NJ;
                const double whole = fixed + line * z.ni;
                if (whole <= 0.25 * budget && (long long)z.ni * z.nj <= 1000000) {
                    split.push_back(z);
                    parent.push_back(k);
                    return;
                }
                const int L = (int)std::max(2.0, std::min(std::floor((0.25 * budget - fixed) / line),
                                                          std::floor(1000000.0 / z.nj)));
                for (int i0 = 0; i0 < z.ni - 1;) {
                    const int i1 = std::min(i0 + L - 1, z.ni - 1);
                    ZoneDev st = z;
                    st.fi0 = z.fi0 + i0 * z.dIi;
                    st.ni = i1 - i0 + 1;
                    split.push_back(st);
                    parent.push_back(k);
                    i0 = i1;
                }
            };
            for (size_t k = 0; k < axis.size(); ++k) {
                const ZoneDev &z = axis[k];
                // bytes a column adds to a two-line strip: its U block, column row, two points and
                // their BRM cells
                const double col = per_u + per_col + 2.0 * per_pt + per_q * z.Fj * (2.0 * z.Fi + 1.0);
                const int Jc = (int)std::max(2.0, std::floor(0.125 * budget / col));
                if (z.nj <= Jc) {
                    by_lines(z, (int)k);
                    continue;
                }
                for (int j0 = 0; j0 < z.nj - 1;) {
                    const int j1 = std::min(j0 + Jc - 1, z.nj - 1);
                    ZoneDev cb = z;
                    cb.fj0 = z.fj0 + j0 * z.dJj;
                    cb.nj = j1 - j0 + 1;
                    by_lines(cb, (int)k);
                    j0 = j1;
                }
            }
            axis.swap(split);
        }
        std::vector<double> zsplit(zdiag ? axis.size() * (size_t)nm : 0, 0.0);
        size_t b0 = 0;
        while (b0 < axis.size()) {
            std::vector<double> uf;
            double bytes = 0.0;
            size_t b1 = b0;
            long long pts = 0;
            while (b1 < axis.size()) {
                const ZoneDev &z = axis[b1];
                size_t nu_new = 0;
                std::vector<double> cand;
                for (int i = 0; i < z.ni; ++i) cand.push_back(z.fi0 + i * z.dIi);
                for (int j = 0; j < z.nj; ++j) cand.push_back(z.fj0 + j * z.dJj);
                for (double f : cand)
                    if (!std::binary_search(uf.begin(), uf.end(), f)) ++nu_new;
                const double nq = (double)((z.ni - 1) * z.Fi + 1) * ((z.nj - 1) * z.Fj + 1);
                const double add = per_u * nu_new + per_col * z.nj + per_pt * z.ni * z.nj + per_q * nq;
                if (b1 > b0 && (bytes + add > budget || pts + (long long)z.ni * z.nj > 4000000)) break;
                bytes += add;
                pts += (long long)z.ni * z.nj;
                uf.insert(uf.end(), cand.begin(), cand.end());
                std::sort(uf.begin(), uf.end());
                uf.erase(std::unique(uf.begin(), uf.end()), uf.end());
                ++b1;
            }
            std::vector<ZoneDev> batch(axis.begin() + b0, axis.begin() + b1);
            if ((rc = msh_mixed_batch(batch, accF, accR, ms_gemm, ms_all, zdiag ? zsplit.data() + b0 * nm : nullptr)))
                return rc;
            b0 = b1;
        }
        if (zdiag) {  // per-zone moments of the caller's zones: the sum over each zone's strips
            for (size_t k = 0; k < zones.size() * (size_t)nm; ++k) zdiag[k] = 0.0;
            for (size_t k = 0; k < axis.size(); ++k)
                for (int m = 0; m < nm; ++m) zdiag[(size_t)parent[k] * nm + m] += zsplit[k * nm + m];
        }
    }
    if (m3mf) std::memcpy(m3mf, accF.data(), sizeof(double) * nm3);
    if (m3mr) std::memcpy(m3mr, accR.data(), sizeof(double) * nm3);
    kernels += nk;
    h2d += hb;
    d2h += db;
    last_ms_gemm = ms_gemm;
    last_ms_contraction = ms_all;
    last_ms = ms_all;
    last_points = nbrm;
    if (npts) {
        npts[0] = nbfm;
        npts[1] = nbrm;
    }
    return BSA_OK;
}

}  // namespace bsa

using bsa::eng;

extern "C" int bsa_gpu_mshZonesDiag(const bsa_zone *zones, int nz, double *m3mf, double *m3mr, double *zdiag) {
    bsa::Engine &E = eng();
    if (E.halted) return BSA_ERR_STATE;
    if (!zones || nz <= 0 || !zdiag) return E.fail(BSA_ERR_ARG, "empty zone list or no per-zone output");
    if (E.precision != BSA_PREC_BF16X3 || E.set.onlyd)
        return E.fail(BSA_ERR_UNSUPPORTED, "per-zone moments are produced by the split-precision zone path");
    std::vector<bsa::ZoneDev> zd(nz);
    for (int k = 0; k < nz; ++k) zd[k] = bsa::zone_from_abi(zones[k]);
    return E.run_zones_mixed(zd, m3mf, m3mr, nullptr, zdiag);
}
