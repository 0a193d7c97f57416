// bsa_atable_tc.cu -- the FP32 A(f) table on the tensor cores (tcgen05, kind::tf32, split).
//
// A(f)[(comp, i)][m] = s_i sum_j c_ij^|f| s_j L[(comp, j)][m], s = sqrt(S(f)) (the coherent
// cross-PSD times the projected coefficients, functionsImpl.F90:1450-1477): per frequency and
// component a GEMM of the generated n x n matrix C(f) = [c_ij^|f|] with B = diag(s) L.  One CTA
// per (frequency, component, 128 rows i): its 256 threads generate the tile c_ij^|f| s_j of each
// 32-wide j chunk straight into shared memory (128-byte swizzled, K-major, the layout the MMA
// descriptors name) split as tf32 hi + lo (hi = the value rounded to tf32, lo = the rounded
// remainder), the B tile (L, split the same way once per call, f-independent) arrives by
// cp.async one chunk ahead, and one thread issues per K step hi x [B hi | B lo] (one MMA of
// twice the mode width) and lo x B hi into FP32 TMEM accumulators (two stages, mbarrier-
// ordered); the epilogue adds the hi x lo columns and scales row i by s_i.  The split keeps
// ~21 bits of each product; c^|f| comes from ex2.approx (relative error ~2^-22).  Every
// mbarrier wait is bounded (error flag).
#include <cuda_runtime.h>

#include <cstdint>

#include "bsa_kernels.cuh"
#include "bsa_tc.cuh"

namespace bsa {
namespace atc {

using namespace tc;

constexpr int kRows = 128;            // i rows per CTA (TMEM lanes)
constexpr int kKc = 32;               // j per chunk: one 128-byte swizzle row of fp32
constexpr int kATile = kRows * 128;   // bytes of one A tile (hi or lo)

template <int N>
struct Layout {
    static constexpr int kBTile = N * 128;
    static constexpr int kStage = 2 * kATile + 2 * kBTile;
    static constexpr int kBars = 2 * kStage;  // offset of the barrier block
};

// x rounded to tf32 (10 explicit mantissa bits), to nearest with ties away from zero, for
// finite x: half the weight of the last kept bit is added to the sign-magnitude bit pattern
// and the 13 dropped bits are cleared (a carry into the exponent is the correct rounding up).
// Two integer ALU instructions in place of a conversion instruction, beside the ex2 of the
// same element on the special-function pipe.
__device__ __forceinline__ uint32_t tf32_rna(float x) { return (__float_as_uint(x) + 0x1000u) & 0xFFFFE000u; }

// 128-byte swizzle: 16-byte chunk c of row r sits at chunk c ^ (r mod 8) of its 128-byte row.
__device__ __forceinline__ uint32_t swz(int r, int c) { return (uint32_t)(r * 128 + ((c ^ (r & 7)) << 4)); }

template <int N>
__device__ __forceinline__ void mma_tf32(uint32_t d, uint64_t a, uint64_t b, uint32_t acc) {
    // kind::tf32, D f32 (bit 4), A = B = tf32 (format 2 at bits 7 and 10), K-major, M = 128, N
    constexpr uint32_t idesc = (1u << 4) | (2u << 7) | (2u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
        "l"(a), "l"(b), "r"(idesc), "r"(acc)
        : "memory");
}

constexpr int kThreads = 256;

// B tables of the A(f) GEMM, f-independent: Bt[(comp, chunk)][m][32] = L[(comp, chunk*32 + q)][m]
// as tf32 hi and lo (zero for m >= nm or j >= n), rows of 128 bytes in plain order.
__global__ void k_atable_btab(int ntc, int n, int nm, int N, int nk, const float *__restrict__ L,
                              uint32_t *__restrict__ Bh, uint32_t *__restrict__ Bl) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long tot = (long long)ntc * nk * N * kKc;
    if (t >= tot) return;
    const int q = (int)(t % kKc), m = (int)((t / kKc) % N);
    const long long cc = t / ((long long)kKc * N);
    const int kc = (int)(cc % nk), itc = (int)(cc / nk), j = kc * kKc + q;
    const float v = (m < nm && j < n) ? L[((size_t)itc * n + j) * nm + m] : 0.f;
    const uint32_t h = tf32_rna(v);
    Bh[t] = h;
    Bl[t] = tf32_rna(v - __uint_as_float(h));
}

__device__ __forceinline__ float ex2_approx(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ void cp_async16(uint32_t dst, const void *src) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}

// One CTA per (frequency, component, 128 rows i).  A tile of chunk kc: c_ij^|f| s_j, generated;
// B tile: copied from the B tables (cp.async, one chunk ahead).  256 threads generate and copy,
// thread 0 issues the MMAs, all eight warps drain TMEM.
template <int N>
__global__ void __launch_bounds__(kThreads, 2) k_atable_tc(int ntc, int n, int nm, int MT, const double *__restrict__ f,
                                                        const float *__restrict__ logc, const double *__restrict__ S,
                                                        const uint32_t *__restrict__ Bth,
                                                        const uint32_t *__restrict__ Btl, float *__restrict__ A,
                                                        int *err) {
    using LY = Layout<N>;
    constexpr float LOG2E = 1.4426950408889634f;
    extern __shared__ uint8_t smem_raw[];
    uint8_t *smem = (uint8_t *)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    uint64_t *freeb = (uint64_t *)(smem + LY::kBars), *done = freeb + 2;
    uint32_t *tmem_slot = (uint32_t *)(done + 1);
    float *ss = (float *)(smem + LY::kBars + 64);  // s_j = sqrt(S_j(f)), zero for j >= n
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int mt = blockIdx.x % MT, t0 = blockIdx.x / MT, itc = t0 % ntc, fi = t0 / ntc;
    const int i0 = mt * kRows;
    const int nk = (n + kKc - 1) / kKc;
    const float af = (float)fabs(f[fi]);
    const float sc = af * LOG2E;  // c^|f| = 2^(|f| log2(e) ln c)
    const double *Sf = S + ((size_t)fi * ntc + itc) * n;
    const float *lc = logc + (size_t)itc * n * n;
    const uint32_t *bth = Bth + (size_t)itc * nk * N * kKc, *btl = Btl + (size_t)itc * nk * N * kKc;

    for (int j = tid; j < nk * kKc; j += kThreads) ss[j] = j < n ? sqrtf((float)Sf[j]) : 0.f;
    if (tid == 0) {
        mbar_init(&freeb[0], 1);
        mbar_init(&freeb[1], 1);
        mbar_init(done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(tmem_slot)), "r"(2 * N)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = *tmem_slot;

    // A tasks of a thread: (row r, 4-wide chunk c) = (t >> 3, t & 7), t = tid + 256 u, u < 4
    constexpr int NU = kRows * 8 / kThreads;
    const float *rowp[NU];
    bool rval[NU];
    const int cofs = (tid & 7) * 4;  // the same for every u (256 is a multiple of 8)
#pragma unroll
    for (int u = 0; u < NU; ++u) {
        const int tt = tid + kThreads * u, gi = i0 + (tt >> 3);
        rowp[u] = lc + (size_t)min(gi, n - 1) * n;
        rval[u] = gi < n;
    }
    // n a multiple of 4: one 16-byte load per task (rows of log c 16-byte aligned); columns past
    // n read the row's last four values (s_j = 0 there)
    const bool vec = (n & 3) == 0;
    float pre[NU][4];
    auto load_chunk = [&](int j0) {  // log c of the chunk, columns clamped (s_j = 0 there)
        if (vec) {
#pragma unroll
            for (int u = 0; u < NU; ++u) {
                const float4 x = __ldg((const float4 *)(rowp[u] + min(j0 + cofs, n - 4)));
                pre[u][0] = x.x;
                pre[u][1] = x.y;
                pre[u][2] = x.z;
                pre[u][3] = x.w;
            }
        } else {
#pragma unroll
            for (int u = 0; u < NU; ++u)
#pragma unroll
                for (int q = 0; q < 4; ++q) pre[u][q] = rowp[u][min(j0 + cofs + q, n - 1)];
        }
    };
    auto copy_b = [&](int kc, int s) {  // B tile of chunk kc into stage s (swizzled 16-byte pieces)
        uint8_t *Bh = smem + s * LY::kStage + 2 * kATile, *Bl = Bh + LY::kBTile;
        const uint32_t *gh = bth + (size_t)kc * N * kKc, *gl = btl + (size_t)kc * N * kKc;
        for (int x = tid; x < N * 8; x += kThreads) {
            const int m = x >> 3, c = x & 7;
            cp_async16(su32(Bh + swz(m, c)), gh + m * kKc + c * 4);
            cp_async16(su32(Bl + swz(m, c)), gl + m * kKc + c * 4);
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
    load_chunk(0);
    copy_b(0, 0);
    bool ok = true;
    // Chunk kc: its A tile is generated into stage s = kc & 1 (whose chunk kc - 2 MMAs were
    // waited for one chunk ago) while the MMAs of chunk kc - 1 run; then, those MMAs done, the
    // B tile of chunk kc + 1 is copied into stage s ^ 1 and chunk kc's MMAs are issued.
    for (int kc = 0; kc < nk; ++kc) {
        const int s = kc & 1;
        uint8_t *Ah = smem + s * LY::kStage, *Al = Ah + kATile;
        const int j0 = kc * kKc;
#pragma unroll
        for (int u = 0; u < NU; ++u) {
            const int tt = tid + kThreads * u, r = tt >> 3, c = tt & 7;
            const float4 sj = *(const float4 *)&ss[j0 + c * 4];
            const float s4[4] = {sj.x, sj.y, sj.z, sj.w};
            uint32_t h[4], l[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const float g = af == 0.f ? 1.f : ex2_approx(sc * pre[u][q]);  // c^0 = 1
                const float v = rval[u] ? g * s4[q] : 0.f;
                h[q] = tf32_rna(v);
                // the remainder is exact in FP32; the MMA reads its top 19 bits (truncation
                // costs at most 2^-10 of the remainder, ~2^-21 of v)
                l[q] = __float_as_uint(v - __uint_as_float(h[q]));
            }
            *(uint4 *)(Ah + swz(r, c)) = make_uint4(h[0], h[1], h[2], h[3]);
            *(uint4 *)(Al + swz(r, c)) = make_uint4(l[0], l[1], l[2], l[3]);
        }
        if (kc + 1 < nk) load_chunk(j0 + kKc);
        // stage s ^ 1 was read by the MMAs of chunk kc - 1: free before the next chunk's B copy
        if (kc >= 1 && ok) ok = mbar_wait(&freeb[s ^ 1], (uint32_t)((kc - 1) >> 1) & 1u, err, 11);
        if (kc + 1 < nk && ok) copy_b(kc + 1, s ^ 1);
        // this chunk's B copy (issued one chunk ago, or before the loop for chunk 0) has landed
        if (kc + 1 < nk && ok)
            asm volatile("cp.async.wait_group 1;" ::: "memory");
        else
            asm volatile("cp.async.wait_group 0;" ::: "memory");
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // generic and cp.async writes -> MMA reads
        ok = __syncthreads_and(ok);
        if (!ok) break;
        if (tid == 0) {
            fence_after();
            const uint32_t ah = su32(Ah), al = su32(Al), bh = su32(Al + kATile);
            // hi x [B hi | B lo] (the lo tile follows the hi tile: one B operand of 2N rows) into
            // columns [0, 2N), then lo x B hi into [0, N): A hi is read once per K step
#pragma unroll
            for (int ks = 0; ks < kKc / 8; ++ks) {  // K = 8 per tf32 MMA: 32 bytes of each row
                const uint32_t off = ks * 32;
                const uint32_t acc = (kc > 0 || ks > 0) ? 1u : 0u;
                mma_tf32<2 * N>(tmem, sdesc(ah + off), sdesc(bh + off), acc);
                mma_tf32<N>(tmem, sdesc(al + off), sdesc(bh + off), 1u);
            }
            mma_commit(&freeb[s]);
        }
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    if (tid == 0) mma_commit(done);  // every MMA issued completes before this arrives
    const bool got = __all_sync(0xffffffffu, mbar_wait(done, 0, err, 12));
    fence_after();
    if (got && ok && (warp >> 2) < N / 32) {
        // warps w and w + 4 read TMEM lanes 32 (w mod 4) .., columns 32 (w div 4) ..
        const int r = (warp & 3) * 32 + lane, gi = i0 + r, q = warp >> 2;
        const uint32_t taddr = tmem + ((uint32_t)((warp & 3) * 32) << 16) + q * 32;
        uint32_t v[32], w[32];
        tmem_ld32(taddr, v);      // hi x hi + lo x hi
        tmem_ld32(taddr + N, w);  // hi x lo
        tmem_wait_ld();
        if (gi < n) {
            float *out = A + (((size_t)fi * ntc + itc) * n + gi) * nm;
            const float si = ss[gi];
#pragma unroll
            for (int e = 0; e < 32; ++e) {
                const int m = q * 32 + e;
                if (m < nm) out[m] = si * (__uint_as_float(v[e]) + __uint_as_float(w[e]));
            }
        }
    }
    fence_before();
    __syncthreads();
    fence_after();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * N) : "memory");
}

template <int N>
cudaError_t launch(cudaStream_t st, int nf, const double *f, int ntc, int nnl, int nm, const float *logc,
                   const double *S, const float *L, float *A, uint32_t *btab, int *err) {
    const int MT = (nnl + kRows - 1) / kRows, nk = (nnl + kKc - 1) / kKc;
    const long long nb = (long long)ntc * nk * N * kKc;
    uint32_t *Bh = btab, *Bl = btab + nb;
    k_atable_btab<<<(unsigned)((nb + 255) / 256), 256, 0, st>>>(ntc, nnl, nm, N, nk, L, Bh, Bl);
    const size_t smem = (size_t)Layout<N>::kBars + 64 + sizeof(float) * (size_t)nk * kKc + 1024;
    cudaError_t e = cudaFuncSetAttribute(k_atable_tc<N>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const long long nblk = (long long)nf * ntc * MT;
    if (nblk > 0x7fffffffLL) return cudaErrorInvalidValue;
    k_atable_tc<N><<<(unsigned)nblk, kThreads, smem, st>>>(ntc, nnl, nm, MT, f, logc, S, Bh, Bl, A, err);
    return cudaGetLastError();
}

}  // namespace atc

size_t atable_tc_scratch(int ntc, int nnl, int nm) {
    const int N = nm <= 32 ? 32 : 64, nk = (nnl + atc::kKc - 1) / atc::kKc;
    return 2 * sizeof(uint32_t) * (size_t)ntc * nk * N * atc::kKc;
}

cudaError_t launch_atable_tc(cudaStream_t st, int nf, const double *f, int ntc, int nnl, int nm, const float *logc,
                             const double *S, const float *L, float *A, void *scratch, int *err) {
    if (nf == 0) return cudaSuccess;
    if (nm > 64) return cudaErrorInvalidValue;
    if ((size_t)nnl * sizeof(float) > 96 * 1024) return cudaErrorInvalidValue;  // s table in shared memory
    uint32_t *bt = (uint32_t *)scratch;
    return nm <= 32 ? atc::launch<32>(st, nf, f, ntc, nnl, nm, logc, S, L, A, bt, err)
                    : atc::launch<64>(st, nf, f, ntc, nnl, nm, logc, S, L, A, bt, err);
}

}  // namespace bsa
