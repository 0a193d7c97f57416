// bsa_noalloc.cu -- the point-set third-moment reduction for callers that cannot allocate
// device memory.
//
// Some callers cannot call cudaMalloc: a host that hands the library device buffers from
// its own pool or arena allocator (and forbids allocation behind its back), or code running
// where allocation is not allowed at that moment.  bsa_gpu_pointMomentsNoAlloc takes every
// input and output as a caller-owned device pointer and keeps its only scratch -- the
// per-group partial moment sums of the FP64 contraction -- in a fixed file-scope device
// array, so it never calls cudaMalloc, cudaFree or any allocating routine.
//
// The scratch array holds kScratchDoubles doubles (4 MiB) on every GPU that loads the
// library, for the life of the process.  It bounds the number of point groups the FP64
// contraction runs in parallel: G = min(the allocating path's group count, 2^18 / nm^3).
// Up to about 20 kept modes that is the allocating path's count; above it the launch has
// fewer CTAs (nm = 32: 8 groups, 128 CTAs instead of about 1200; nm = 64: one group of 64
// CTAs striding over every point), so for large mode counts and many points the allocating
// entry point bsa_gpu_mshMoments is the faster choice.  Every call shares it and overwrites it completely
// before reading it (each group writes all of its nm^3 partials), so nothing needs
// clearing between calls; calls that overlap on the GPU (different streams, or other host
// threads) race on it and must be serialised by the caller.
#include <cuda_runtime.h>

#include <atomic>
#include <cstdio>

#include "../../include/bsa_gpu.h"
#include "bsa_engine.cuh"
#include "bsa_kernels.cuh"

namespace {

constexpr long long kScratchDoubles = 1ll << 19;  // 4 MiB: 2 * 64^3 doubles, one group at 64 modes
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_noalloc_scratch[kScratchDoubles];

// Device address of the scratch array, resolved once per device.  In host code the name
// g_noalloc_scratch is only a host-side stand-in, not a device address.  Atomic so that two
// host threads making the first call on one device both store the same resolved address
// without a data race.
std::atomic<double *> g_scratch_ptr[kMaxDevices] = {};

int set_error(int code, const char *msg) {
    bsa::eng().last_error = msg;
    return code;
}

}  // namespace

extern "C" int bsa_gpu_pointMomentsNoAlloc(const double *A, int K, int nm, const double *Q, const int *ix,
                                           const int *iy, const int *iz, const double *f1, const double *f2,
                                           const double *w, int npts, const double *Mm, const double *Km,
                                           const double *Cm, double *m3mf, double *m3mr, void *stream) {
    if (!A || !Q || !ix || !iy || !iz || !f1 || !f2 || !w || !Mm || !Km || !Cm || !m3mf || !m3mr)
        return set_error(BSA_ERR_ARG, "bsa_gpu_pointMomentsNoAlloc: null pointer argument");
    if (K < 1 || npts < 1) return set_error(BSA_ERR_ARG, "bsa_gpu_pointMomentsNoAlloc: K and npts must be >= 1");
    if (nm < 1 || nm > 64)
        return set_error(BSA_ERR_ARG, "bsa_gpu_pointMomentsNoAlloc: nm must be in 1..64 (the 4 MiB scratch holds 2*nm^3 doubles)");
    const long long nm3 = (long long)nm * nm * nm;
    if (2 * nm3 > kScratchDoubles)
        return set_error(BSA_ERR_ARG, "bsa_gpu_pointMomentsNoAlloc: 2*nm^3 partial sums exceed the 4 MiB scratch");

    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_error(BSA_ERR_CUDA, "bsa_gpu_pointMomentsNoAlloc: cudaGetDevice failed");
    if (dev < 0 || dev >= kMaxDevices) return set_error(BSA_ERR_UNSUPPORTED, "bsa_gpu_pointMomentsNoAlloc: device ordinal too large");
    double *scratch = g_scratch_ptr[dev].load(std::memory_order_acquire);
    if (!scratch) {
        // Set-up, once per device, with that device current.
        double *ptr = nullptr;
        e = cudaGetSymbolAddress((void **)&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || !ptr) {
            static char buf[256];
            snprintf(buf, sizeof buf, "bsa_gpu_pointMomentsNoAlloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
            return set_error(BSA_ERR_CUDA, buf);
        }
        g_scratch_ptr[dev].store(ptr, std::memory_order_release);
        scratch = ptr;
    }

    long long g = bsa::bfm_fp64_groups(npts, nm);
    const long long gmax = kScratchDoubles / (2 * nm3);
    if (g > gmax) g = gmax;
    const int G = (int)g;

    bsa::PointSrc ps{};
    ps.mode = bsa::kPointsList;
    ps.wmode = bsa::kWeightList;
    ps.ix = ix;
    ps.iy = iy;
    ps.iz = iz;
    ps.f1 = f1;
    ps.f2 = f2;
    ps.w = w;
    bsa::FrfPar frf{Mm, Km, Cm};
    cudaStream_t st = (cudaStream_t)stream;
    double *part_mf = scratch, *part_mr = scratch + (size_t)G * nm3;
    e = bsa::launch_bfm_fp64(st, A, Q, K, nm, ps, npts, frf, G, part_mf, part_mr, nullptr, nullptr);
    if (e != cudaSuccess) return set_error(BSA_ERR_CUDA, "bsa_gpu_pointMomentsNoAlloc: contraction launch failed");
    e = bsa::launch_reduce_groups(st, G, nm3, part_mf, m3mf, part_mr, m3mr);
    if (e != cudaSuccess) return set_error(BSA_ERR_CUDA, "bsa_gpu_pointMomentsNoAlloc: reduction launch failed");
    return BSA_OK;
}
