// bsa_host.cu -- host side of libbsagpu: the BsaLib API state (borrowed inputs, settings),
// validation and projection, the Classic / point-set drivers, and the BsaCL-compatible
// entry points.  All exported symbols are declared in include/bsa_gpu.h.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/bsa_gpu.h"
#include "bsa_common.cuh"
#include "bsa_engine.cuh"
#include "bsa_kernels.cuh"

namespace bsa {

Engine &eng() {
    static Engine e;
    return e;
}

int Engine::fail(int code, const char *fmt, ...) {
    if (!halted) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        last_error = buf;
        halted = true;
    }
    return code;
}

int Engine::cuda_fail(cudaError_t e, const char *what) {
    return fail(e == cudaErrorMemoryAllocation ? BSA_ERR_NOMEM : BSA_ERR_CUDA, "%s: %s", what,
                cudaGetErrorString(e));
}

// Device blocks released by the engine are kept for the next request of a similar size
// (bsa_Init ... bsa_Finalise cycles would otherwise pay cudaMalloc / cudaFree of the operand
// tables every analysis).  Blocks are 2 MB multiples; a request takes the smallest cached block
// that holds it and is at most twice its size.  At most a quarter of the device memory stays
// cached; a failed cudaMalloc frees the cache and retries; bsa_gpu_releaseDeviceCache frees it.
// The engine's work is ordered on its one stream, and released blocks are handed out again only
// to later work of that stream (bsa_Finalise synchronises it before releasing).
namespace {
struct BlockCache {
    std::mutex m;
    std::multimap<size_t, void *> blocks;
    size_t cached = 0, limit = 0;
    void flush() {
        for (auto &b : blocks) cudaFree(b.second);
        blocks.clear();
        cached = 0;
    }
};
BlockCache &cache() {
    static BlockCache c;
    return c;
}
}  // namespace

void DevBuf::release() {
    if (p) {
        BlockCache &c = cache();
        std::lock_guard<std::mutex> lk(c.m);
        if (c.limit == 0) {
            size_t fr = 0, tot = 0;
            c.limit = cudaMemGetInfo(&fr, &tot) == cudaSuccess ? tot / 4 : (size_t)1 << 30;
        }
        if (c.cached + bytes <= c.limit) {
            c.blocks.emplace(bytes, p);
            c.cached += bytes;
        } else {
            cudaFree(p);
        }
    }
    p = nullptr;
    bytes = 0;
}

cudaError_t DevBuf::reserve(size_t nbytes) {
    if (nbytes <= bytes && p) return cudaSuccess;
    release();
    if (nbytes == 0) return cudaSuccess;
    const size_t want = (nbytes + ((size_t)2 << 20) - 1) & ~(((size_t)2 << 20) - 1);
    BlockCache &c = cache();
    {
        std::lock_guard<std::mutex> lk(c.m);
        auto it = c.blocks.lower_bound(want);
        if (it != c.blocks.end() && it->first <= 2 * want) {
            p = it->second;
            bytes = it->first;
            c.cached -= bytes;
            c.blocks.erase(it);
            return cudaSuccess;
        }
    }
    cudaError_t e = cudaMalloc(&p, want);
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();
        {
            std::lock_guard<std::mutex> lk(c.m);
            c.flush();
        }
        e = cudaMalloc(&p, want);
    }
    if (e == cudaSuccess) bytes = want;
    else p = nullptr;
    return e;
}

void release_device_cache() {
    BlockCache &c = cache();
    std::lock_guard<std::mutex> lk(c.m);
    c.flush();
}

void Engine::reset_inputs() {
    in = Inputs();
    own_i.clear();
    own_d.clear();
    set = Settings();
    derived_ok = false;
    // controls of the GPU path return to their defaults with the inputs
    precision = BSA_PREC_FP64;
    classic_trunc = true;
    shard_r0 = 0;
    shard_r1 = -1;
    cls_shard = 0;
    cls_shards = 1;
    pod_trunc_lim = 0.0;
    pod_nmodes = 0;
    export_fn = nullptr;
    export_user = nullptr;
    brm_file_close(-1);
    visual = false;
    visual_modal = true;
    visual_idx[0] = visual_idx[1] = visual_idx[2] = 1;
    brm_export_mode = 0;
    classic_sym = false;
    use_e_form = true;
    validate_deltas = true;
    bfm_mlr = true;
    bkg_restrict = false;
    premesh_diag_crest = false;
    premesh_mode_base = false;
}

void Engine::free_device() {
    if (stream) cudaStreamSynchronize(stream);  // the blocks go back to the cache for reuse
    for (DevBuf *b : {&dL, &dQ, &dLogc, &dPsdPar, &dFrfM, &dFrfK, &dFrfC, &dFreq, &dS, &dA, &dPartF, &dPartR,
                      &dOut, &dPsdF, &dWf, &dPts, &dPtsD, &dBF, &dBR, &dMixA, &dMixB, &dMixH, &dMixPart, &dA32,
                      &dZones, &dZidx, &dWd3, &dWd2, &dMshT, &dMshIdx, &dLogc32, &dL32, &dPod, &dFlag, &dSlot, &dHash})
        b->release();
    if (stream) cudaStreamDestroy(stream);
    stream = nullptr;
    if (ev0) cudaEventDestroy(ev0);
    if (ev1) cudaEventDestroy(ev1);
    if (ev2) cudaEventDestroy(ev2);
    if (evg0) cudaEventDestroy(evg0);
    if (evg1) cudaEventDestroy(evg1);
    ev0 = ev1 = ev2 = evg0 = evg1 = nullptr;
    dev_uploaded = false;
}

int Engine::ensure_stream() {
    if (stream) return BSA_OK;
    cudaError_t e = cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamCreate");
    if ((e = cudaEventCreate(&ev0)) != cudaSuccess) return cuda_fail(e, "cudaEventCreate");
    if ((e = cudaEventCreate(&ev1)) != cudaSuccess) return cuda_fail(e, "cudaEventCreate");
    if ((e = cudaEventCreate(&ev2)) != cudaSuccess) return cuda_fail(e, "cudaEventCreate");
    if ((e = cudaEventCreate(&evg0)) != cudaSuccess) return cuda_fail(e, "cudaEventCreate");
    if ((e = cudaEventCreate(&evg1)) != cudaSuccess) return cuda_fail(e, "cudaEventCreate");
    return BSA_OK;
}

static long corr_index(int ni, int nj, int tot) {
    // util_getCorrVectIndex, src/utils/utility.F90:60-71 (1-based)
    if (nj >= ni) return (long)(ni - 1) * tot + nj - ((long)ni * ni - ni) / 2;
    return (long)(nj - 1) * tot + ni - ((long)nj * nj - nj) / 2;
}

// validateAll_ (src/bsa/BsaLibImpl.F90:469-535) restricted to what the BFM path reads:
// sizes, mode validation (validateModalInfo_, :545-599), the projection PHItimesC
// (setPhitimesCLocalInstance_, :611-671) and the device-side parameter tables.
int Engine::validate() {
    if (halted) return BSA_ERR_STATE;
    if (derived_ok) return BSA_OK;
    const Inputs &I = in;
    const bool ext = I.ext_phitc != nullptr;
    if (I.nn <= 0) return fail(BSA_ERR_STATE, "total number of nodes not set");
    if (!I.n_load || I.nnl <= 0) return fail(BSA_ERR_STATE, "loaded nodes not set");
    if (!I.Mg || !I.Kg || !I.Cg) return fail(BSA_ERR_STATE, "modal matrices not set");
    if (!I.corr) return fail(BSA_ERR_STATE, "nodal coherence not set");
    if (!I.unod || !I.wz || !I.sigma || !I.L) return fail(BSA_ERR_STATE, "wind field data not set");
    if (I.psd_type == 3 && !I.ubref) return fail(BSA_ERR_STATE, "zone mean wind speeds not set");
    if (I.ncorr != ((long)I.nn * I.nn + I.nn) / 2)
        return fail(BSA_ERR_ARG, "nodal coherence has %lld rows, expected (nn^2+nn)/2", (long long)I.ncorr);
    if (set.tc.empty() || set.tc.size() > 3) return fail(BSA_ERR_ARG, "1 to 3 turbulent components");
    for (int tc : set.tc)
        if (tc < 1 || tc > 3) return fail(BSA_ERR_ARG, "turbulent component id out of range");
    if (!(I.psd_type == 1 || I.psd_type == 2 || I.psd_type == 3 || I.psd_type == 5))
        return fail(BSA_ERR_UNSUPPORTED, "PSD type %d has no model function", I.psd_type);
    for (int i = 0; i < I.nnl; ++i)
        if (I.n_load[i] < 1 || I.n_load[i] > I.nn) return fail(BSA_ERR_ARG, "loaded node id out of range");
    const int tcmax = *std::max_element(set.tc.begin(), set.tc.end());
    const int nnl = I.nnl;
    int nd = 0;
    if (ext) {
        if (I.ext_nnl != nnl) return fail(BSA_ERR_ARG, "N. of loaded nodes does not match");
        if (I.ext_nd < 3 + tcmax) return fail(BSA_ERR_ARG, "projected coefficients have too few columns");
        if (!I.ext_modes || I.ext_nme <= 0) return fail(BSA_ERR_STATE, "kept-mode list not set");
        modes.assign(I.ext_modes, I.ext_modes + I.ext_nme);
        for (int m : modes)
            if (m < 1 || m > I.nm) return fail(BSA_ERR_ARG, "kept mode id out of range");
        nme = I.ext_nme;
        nd = I.ext_nd;
        phitc.assign(I.ext_phitc, I.ext_phitc + (size_t)nme * nnl * nd);
    } else {
        if (I.nlibs <= 0) return fail(BSA_ERR_STATE, "number of nodal DOFs not set");
        if (!I.libs_load || I.nlibsl <= 0) return fail(BSA_ERR_STATE, "loaded nodal DOFs not set");
        if (!I.phi || I.nm <= 0) return fail(BSA_ERR_STATE, "modal matrix not set");
        if (!I.wfc) return fail(BSA_ERR_STATE, "wind force coefficients were not acquired");
        const int ndofs = I.ndofs ? I.ndofs : I.nn * I.nlibs;
        if (I.phi_ndofs != ndofs) return fail(BSA_ERR_ARG, "NDOFs does not match modal matrix size");
        if (ndofs != I.nn * I.nlibs) return fail(BSA_ERR_ARG, "incorrect value for ndofs");
        if (I.wfc_nn != I.nnl) return fail(BSA_ERR_ARG, "N. of loaded nodes does not match");
        if (I.wfc_nl != I.nlibsl) return fail(BSA_ERR_ARG, "N. of loaded libs does not match");
        if (I.wfc_nd < 3 + tcmax) return fail(BSA_ERR_ARG, "wind force coefficients have too few columns");
        for (int l = 0; l < I.nlibsl; ++l)
            if (I.libs_load[l] < 1 || I.libs_load[l] > I.nlibs) return fail(BSA_ERR_ARG, "loaded DOF id out of range");
        // validateModalInfo_: keep modes with max|Phi| == 1 exactly.
        modes.clear();
        for (int m = 0; m < I.nm; ++m) {
            double mx = 0.0;
            for (int d = 0; d < ndofs; ++d) mx = std::max(mx, std::fabs(I.phi[(size_t)d + (size_t)ndofs * m]));
            if (mx == 1.0) modes.push_back(m + 1);
        }
        nme = (int)modes.size();
        if (nme == 0) return fail(BSA_ERR_ARG, "effective number of modes to be kept is 0");
        if (nme > 64) return fail(BSA_ERR_UNSUPPORTED, "more than 64 kept modes");
        // PHItimesC(im, in, id) = sum_l wfc(l, id, in) Phi((n-1)*nlibs + libs_load(l), modes(im))
        nd = I.wfc_nd;
        const int nl = I.nlibsl;
        phitc.assign((size_t)nme * nnl * nd, 0.0);
        for (int i = 0; i < nnl; ++i) {
            const int skip = (I.n_load[i] - 1) * I.nlibs;
            for (int id = 0; id < nd; ++id)
                for (int im = 0; im < nme; ++im) {
                    double s = 0.0;
                    for (int l = 0; l < nl; ++l)
                        s += I.wfc[(size_t)l + (size_t)nl * ((size_t)id + (size_t)nd * i)] *
                             I.phi[(size_t)(skip + I.libs_load[l] - 1) + (size_t)ndofs * (modes[im] - 1)];
                    phitc[(size_t)im + (size_t)nme * ((size_t)i + (size_t)nnl * id)] += s;
                }
        }
    }
    if (nme > 64) return fail(BSA_ERR_UNSUPPORTED, "more than 64 kept modes");
    // Device layouts: k = itc * nnl + i.
    const int ntc = (int)set.tc.size();
    K = ntc * nnl;
    hL.assign((size_t)K * nme, 0.0);
    hQ.assign((size_t)K * nme, 0.0);
    for (int itc = 0; itc < ntc; ++itc) {
        const int tc = set.tc[itc];
        for (int i = 0; i < nnl; ++i)
            for (int m = 0; m < nme; ++m) {
                hL[((size_t)itc * nnl + i) * nme + m] = phitc[(size_t)m + (size_t)nme * ((size_t)i + (size_t)nnl * (tc - 1))];
                hQ[((size_t)itc * nnl + i) * nme + m] = phitc[(size_t)m + (size_t)nme * ((size_t)i + (size_t)nnl * (tc + 2))];
            }
    }
    // Diagonal-only spectra: the three per-node projected sums of one mode multiply.
    hWd3.assign((size_t)K * nme, 0.0);
    hWd2.assign((size_t)K * nme, 0.0);
    for (size_t x = 0; x < hWd3.size(); ++x) {
        hWd3[x] = hQ[x] * hL[x] * hL[x];
        hWd2[x] = hL[x] * hL[x];
    }
    const long ncorr = (long)I.ncorr;
    hCoh.assign((size_t)ntc * nnl * nnl, 0.0);
    for (int itc = 0; itc < ntc; ++itc)
        for (int i = 0; i < nnl; ++i)
            for (int j = 0; j < nnl; ++j) {
                const long id = corr_index(I.n_load[i], I.n_load[j], I.nn);
                const double c = I.corr[(size_t)(id - 1) + (size_t)ncorr * (set.tc[itc] - 1)];
                hCoh[((size_t)itc * nnl + i) * nnl + j] = c;
            }
    hL32.assign(hL.begin(), hL.end());
    const int idir = set.dirs.empty() ? 1 : set.dirs[0];
    hPsd.assign((size_t)ntc * nnl, PsdNode{});
    for (int itc = 0; itc < ntc; ++itc) {
        const int tc = set.tc[itc];
        for (int i = 0; i < nnl; ++i) {
            const int n = I.n_load[i];
            const int wz = I.wz[n - 1];
            if (wz < 1 || wz > I.nz) return fail(BSA_ERR_ARG, "wind zone of node %d out of range", n);
            PsdNode p;
            p.U = I.unod[n - 1];
            p.sigma = I.sigma[(size_t)(tc - 1) + 3 * (size_t)(wz - 1)];
            const int lrow = (I.psd_type == 1 && tc == 1) ? 1 : tc;  // vonKarmanPSD_ u form reads L(1, idir, wz)
            p.Ls = I.L[(size_t)(lrow - 1) + 3 * ((size_t)(idir - 1) + 3 * (size_t)(wz - 1))];
            p.Uref = I.ubref ? I.ubref[wz - 1] : 0.0;
            hPsd[(size_t)itc * nnl + i] = p;
        }
    }
    hM.resize(nme); hK.resize(nme); hC.resize(nme);
    for (int im = 0; im < nme; ++im) {
        const int m = modes[im] - 1;
        hM[im] = I.Mg[m];
        hK[im] = I.Kg[m];
        hC[im] = I.Cg[(size_t)m + (size_t)I.nm * m];
    }
    derived_ok = true;
    dev_uploaded = false;
    return BSA_OK;
}


int Engine::upload_problem() {
    int rc = validate();
    if (rc) return rc;
    if ((rc = ensure_stream())) return rc;
    if (dev_uploaded) return BSA_OK;
    cudaError_t e;
    if ((e = upload(dL, hL, stream)) || (e = upload(dQ, hQ, stream)) || (e = upload(dLogc, hCoh, stream)) ||
        (e = upload(dPsdPar, hPsd, stream)) || (e = upload(dFrfM, hM, stream)) || (e = upload(dFrfK, hK, stream)) ||
        (e = upload(dFrfC, hC, stream)) || (e = upload(dWd3, hWd3, stream)) || (e = upload(dWd2, hWd2, stream)) ||
        (e = upload(dL32, hL32, stream)) || (e = dLogc32.reserve(sizeof(float) * hCoh.size())))
        return cuda_fail(e, "uploading problem data");
    // log c in place (FP64) and its FP32 copy
    if ((e = launch_log_coh(stream, hCoh.size(), dLogc.as<double>(), dLogc32.as<float>())))
        return cuda_fail(e, "coherence table");
    kernels += 1;
    dev_uploaded = true;
    return BSA_OK;
}

FrfPar Engine::frf() const { return FrfPar{dFrfM.as<double>(), dFrfK.as<double>(), dFrfC.as<double>()}; }

// Nodal PSD table S[f][k] for a host list of frequencies (into dFreq, dS).
int Engine::build_psd(const std::vector<double> &freqs) {
    cudaError_t e;
    if ((e = upload(dFreq, freqs, stream))) return cuda_fail(e, "uploading frequencies");
    return build_psd_dev((int)freqs.size());
}

// Nodal PSD table S[f][k] for the nf frequencies already in dFreq (fp32: the formulas
// evaluated in FP32, for the split-precision A tables).
int Engine::build_psd_dev(int nf, bool fp32) {
    const int ntc = (int)set.tc.size();
    cudaError_t e;
    if ((e = dS.reserve(sizeof(double) * (size_t)nf * ntc * in.nnl))) return cuda_fail(e, "allocating S");
    if ((e = launch_nodal_psd(stream, nf, dFreq.as<double>(), ntc, set.tc.data(), in.nnl, dPsdPar.as<PsdNode>(),
                              in.psd_type, set.defsc, dS.as<double>(), fp32)))
        return cuda_fail(e, "nodal PSD kernel");
    kernels += 1;
    return BSA_OK;
}

// Nodal PSD + A(f) for a host list of frequencies, into dA (FP64) or dA32 (FP32) rows.
int Engine::build_atable(const std::vector<double> &freqs, bool fp32, bool msh) {
    if (msh && pod_truncates()) return pod_atable(freqs, fp32);  // bsa_pod.cu
    cudaError_t e;
    if ((e = upload(dFreq, freqs, stream))) return cuda_fail(e, "uploading frequencies");
    return build_atable_dev((int)freqs.size(), fp32);
}

// Nodal PSD + A(f) for the nf frequencies already in dFreq (not the truncated POD form).
int Engine::build_atable_dev(int nf, bool fp32) {
    const int ntc = (int)set.tc.size();
    cudaError_t e;
    int rc = build_psd_dev(nf, fp32);
    if (rc) return rc;
    if (fp32) {
        // FP32 table on the tensor cores (tf32 hi/lo split, FP32-level accuracy)
        if ((e = dA32.reserve(sizeof(float) * (size_t)nf * K * nme)) ||
            (e = dFlag.reserve(256 + atable_tc_scratch(ntc, in.nnl, nme))))
            return cuda_fail(e, "allocating A");
        int *flag = dFlag.as<int>();
        if ((e = cudaMemsetAsync(flag, 0, sizeof(int), stream))) return cuda_fail(e, "memset");
        e = launch_atable_tc(stream, nf, dFreq.as<double>(), ntc, in.nnl, nme, dLogc32.as<float>(), dS.as<double>(),
                             dL32.as<float>(), dA32.as<float>(), (char *)dFlag.p + 256, flag);
        if (e) return cuda_fail(e, "A-table kernel");
        kernels += 2;
        int hflag = 0;
        if ((e = cudaMemcpyAsync(&hflag, flag, sizeof(int), cudaMemcpyDeviceToHost, stream)) ||
            (e = cudaStreamSynchronize(stream)))
            return cuda_fail(e, "A-table kernel");
        if (hflag) return fail(BSA_ERR_TIMEOUT, "A-table kernel: a pipeline wait ran out of its budget (role %d)", hflag);
        return BSA_OK;
    } else {
        if ((e = dA.reserve(sizeof(double) * (size_t)nf * K * nme))) return cuda_fail(e, "allocating A");
        e = launch_atable(stream, nf, dFreq.as<double>(), ntc, in.nnl, nme, dLogc.as<double>(), dS.as<double>(),
                          dL.as<double>(), dA.as<double>());
    }
    if (e) return cuda_fail(e, "A-table kernel");
    kernels += 1;
    return BSA_OK;
}

// computeFreqsVect_ (BsaClassicImpl.F90:443-560).
int Engine::classic_grid(std::vector<double> &f) {
    if (set.nfreqs == 0 || set.df == 0.0) return fail(BSA_ERR_ARG, "either NFREQs or DF are == 0");
    if (!in.natf) return fail(BSA_ERR_STATE, "natural frequencies not set");
    double df = set.df;
    double df_ref = INFINITY, max_ref = -INFINITY;
    for (int m = 0; m < in.nm; ++m) {
        if (!in.xsi) return fail(BSA_ERR_STATE, "damping (bsa_setTotDamping) not set");
        df_ref = std::min(df_ref, in.xsi[m] * in.natf[m]);
        max_ref = std::max(max_ref, in.natf[m]);
    }
    df_ref /= 5.0;
    const bool big = df > df_ref;
    int nf1 = set.nfreqs - 1;
    if (set.test == 0) {
        double mxf = df * nf1;
        if (mxf < max_ref) {
            if (big) {
                mxf = df_ref * nf1;
                if (mxf < max_ref) nf1 = (int)std::ceil(max_ref / df_ref);
                df = df_ref;
            } else {
                nf1 = (int)std::ceil(max_ref / df);
            }
        }
    }
    int nf, n0;
    if (set.defsc == 1) {
        nf = nf1 * 2 + 1;
        n0 = -nf1;
    } else {
        if (nf1 % 2 != 0) nf1 += 1;
        nf = nf1 + 1;
        n0 = 0;
    }
    f.resize(nf);
    for (int i = n0; i <= nf1; ++i) f[i - n0] = (double)i * df;
    return BSA_OK;
}

// Classic analysis on the GPU (mainClassic_, BsaClassicImpl.F90:39-376): every grid point,
// moments reduced in the kernel epilogue.  Optional materialised bispectra (nf, nf, nm^3).
int Engine::run_classic(double *m2mf, double *m2mr, double *m2o2mr, double *m3mf, double *m3mr, double *bf_host,
                        double *br_host, std::vector<double> *grid_out) {
    kernels = 0;
    graph_launches = 0;
    h2d = d2h = 0;
    last_ms_gemm = 0;
    int rc = upload_problem();
    if (rc) return rc;
    std::vector<double> f;
    if ((rc = classic_grid(f))) return rc;
    if (grid_out) *grid_out = f;
    const int nf = (int)f.size();
    if (nf < 2) return fail(BSA_ERR_ARG, "classic grid needs at least 2 frequencies");
    // Row shard (f1 index): the moments of all shards sum to the full grid's.  With
    // bsa_gpu_setClassicShard the rows are the shard's contiguous block (the second-order
    // moments, and the bispectrum outside the E form); the E form shards its products instead.
    int r0 = std::min(std::max(shard_r0, 0), nf);
    int r1 = shard_r1 < 0 ? nf : std::min(shard_r1, nf);
    if (cls_shards > 1) {
        if (cls_shards > nf) return fail(BSA_ERR_ARG, "%d shards of a %d-row grid", cls_shards, nf);
        const int base = nf / cls_shards, extra = nf % cls_shards;
        r0 = cls_shard * base + std::min(cls_shard, extra);
        r1 = r0 + base + (cls_shard < extra ? 1 : 0);
    }
    if (r1 <= r0) return fail(BSA_ERR_ARG, "empty classic row shard [%d, %d)", r0, r1);
    if ((bf_host || br_host) && (r0 != 0 || r1 != nf))
        return fail(BSA_ERR_ARG, "materialised bispectra need the full grid");
    // Vectorised / scalar branch (checkMaxAllocation_, BsaClassicImpl.F90:384-434): only the
    // integration weights differ here, the spectra are never stored.
    bool scalar = set.scalar != 0;
    if (set.test == 0 && !scalar && set.ibisp && (long long)nf * nf * dim_bisp() > 1000000000LL) scalar = true;
    double delta = f[1] - f[0];
    if (set.defsc == 1) delta *= kPi2;
    const bool analytic = !classic_trunc;
    std::vector<double> ftab = f;
    if (analytic) {
        // s-table: f1 + f2 = 2 f[0] + s df, s = i1 + i2.
        const double d = f[1] - f[0];
        for (int s = 0; s < 2 * nf - 1; ++s) ftab.push_back(2.0 * f[0] + s * d);
    }
    // Diagonal-only spectra read the nodal PSD table alone and stay FP64 (O(K nm) per point).
    const bool diagonal = set.onlyd != 0;
    // The split-precision contraction reduces to moments only; it reads an FP32 A table.
    const bool mixed = !diagonal && precision == BSA_PREC_BF16X3 && !bf_host && !br_host;
    if (mixed && nme > 64) return fail(BSA_ERR_UNSUPPORTED, "BF16x3 contraction supports at most 64 kept modes");
    cudaError_t e;
    if ((e = cudaEventRecord(ev0, stream))) return cuda_fail(e, "event");
    if ((rc = diagonal ? build_psd(ftab) : build_atable(ftab, mixed))) return rc;
    const long long nm2 = dim_psd();
    if (set.ipsd && (m2mf || m2mr || m2o2mr)) {
        std::vector<double> wf(nf, scalar ? delta : delta);
        if (!scalar) { wf[0] = delta / 2; wf[nf - 1] = delta / 2; }
        if ((e = upload(dWf, wf, stream))) return cuda_fail(e, "weights");
        if ((e = dPsdF.reserve(sizeof(double) * (size_t)nf * nm2))) return cuda_fail(e, "psd");
        if ((e = dOut.reserve(sizeof(double) * (3 * (size_t)nm2 + 2 * (size_t)dim_bisp()))))
            return cuda_fail(e, "out");
        e = diagonal ? launch_force_psd_diag(stream, nf, K, nme, dS.as<double>(), dWd2.as<double>(), dPsdF.as<double>())
            : mixed  ? launch_force_psd32(stream, nf, (int)set.tc.size(), in.nnl, nme, dL32.as<float>(),
                                          dA32.as<float>(), dPsdF.as<double>())
                     : launch_force_psd(stream, nf, (int)set.tc.size(), in.nnl, nme, dL.as<double>(), dA.as<double>(),
                                        dPsdF.as<double>());
        if (e) return cuda_fail(e, "force PSD kernel");
        double *o = dOut.as<double>();
        if ((e = launch_m2(stream, r0, r1, nme, diagonal ? 1 : 0, dFreq.as<double>(), dWf.as<double>(),
                           dPsdF.as<double>(), frf(), o, o + nm2, o + 2 * nm2)))
            return cuda_fail(e, "m2 kernel");
        kernels += 2;
        std::vector<double> h(3 * (size_t)nm2);
        if ((e = cudaMemcpyAsync(h.data(), o, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, stream)) ||
            (e = cudaStreamSynchronize(stream)))
            return cuda_fail(e, "m2 copy");
        d2h += (double)sizeof(double) * h.size();
        if (m2mf) std::memcpy(m2mf, h.data(), sizeof(double) * nm2);
        if (m2mr) std::memcpy(m2mr, h.data() + nm2, sizeof(double) * nm2);
        if (m2o2mr) std::memcpy(m2o2mr, h.data() + 2 * nm2, sizeof(double) * nm2);
    }
    last_points = 0;
    if (set.ibisp && (m3mf || m3mr || bf_host || br_host)) {
        PointSrc ps{};
        ps.mode = kPointsGrid;
        ps.nf = nf;
        ps.n_pad = (nf - 1) / 2;
        ps.trunc = analytic ? 0 : 1;
        ps.sum_base = nf;
        ps.wmode = scalar ? kWeightUniform : kWeightClassicVect;
        ps.wval = delta * delta;
        ps.fgrid = dFreq.as<double>();
        ps.r0 = r0;
        ps.nr = r1 - r0;
        long long npts = (long long)(r1 - r0) * nf;
        // Central symmetry (bsa_gpu_setClassicSymmetry): on the grid f = -N..N every quantity
        // of the path is even in f (S and c^|f| depend on |f|, H(-w) = conj H(w), the sum
        // truncation and the integration weights are symmetric), so B(f_r, f_c) equals
        // B(f_nf-1-r, f_nf-1-c).  Rows r < n_pad then stand for their mirrors with twice the
        // weight, the centre row (its own mirror) once; rows above it are not evaluated.
        // The split path's E form (bsa_classic_e.cu) already forms each distinct product of the
        // whole grid once, which half the rows would not improve on: there the symmetry is not
        // applied.
        bool e_form = mixed && use_e_form && nme <= kEFormMaxModes && !analytic && (nf & 1) &&
                      plan_prefer_e(nme, K, nf) && ((r0 == 0 && r1 == nf) || cls_shards > 1);
        if (e_form && cls_shards > 1) {
            // the E form of a shard: every output point, the products of rows p = shard + shards l
            ps.r0 = 0;
            ps.nr = nf;
        }
        const bool file_export = brm_file_wanted(true);
        const bool sym =
            classic_sym && set.defsc == 1 && !bf_host && !br_host && !export_fn && !file_export && !e_form;
        if (sym) {
            ps.sym_rows = ps.n_pad;
            ps.nr = std::max(0, std::min(r1, ps.n_pad + 1) - r0);
            npts = (long long)ps.nr * nf;
        }
        if (sym && ps.nr == 0) {
            const long long nb = dim_bisp();
            if (m3mf) std::memset(m3mf, 0, sizeof(double) * nb);
            if (m3mr) std::memset(m3mr, 0, sizeof(double) * nb);
            rc = BSA_OK;
        } else if ((export_fn || file_export) && !bf_host && !br_host) {
            if (r0 != 0 || r1 != nf) return fail(BSA_ERR_ARG, "the bispectrum export needs the full grid");
            rc = classic_export(ps, f, m3mf, m3mr);
        } else {
            rc = diagonal ? contract_diag(ps, npts, 0, m3mf, m3mr, bf_host, br_host)
                 : mixed  ? contract_mixed(ps, npts, m3mf, m3mr)
                          : contract(ps, npts, m3mf, m3mr, bf_host, br_host);
        }
        if (rc) return rc;
        last_points = (double)npts;
    }
    if ((e = cudaEventRecord(ev1, stream)) || (e = cudaEventSynchronize(ev1))) return cuda_fail(e, "event");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ev0, ev1);
    last_ms = ms;
    return BSA_OK;
}

// The Classic grid in column blocks with materialised response bispectra, each block handed
// to the export callback (BsaClassicImpl.F90:175-191); third moments summed over the blocks.
// FP64 tables: the A table is rebuilt in FP64 when the analysis prepared the FP32 one.
int Engine::classic_export(PointSrc ps, const std::vector<double> &f, double *m3mf, double *m3mr) {
    const int nf = ps.nf;
    const long long nb = dim_bisp();
    int rc;
    if (precision == BSA_PREC_BF16X3 && !set.onlyd) {
        std::vector<double> ftab = f;
        if (!ps.trunc)
            for (int s = 0; s < 2 * nf - 1; ++s) ftab.push_back(2.0 * f[0] + s * (f[1] - f[0]));
        if ((rc = build_atable(ftab, false))) return rc;
        ps.fgrid = dFreq.as<double>();
    }
    const long long budget = 1LL << 30;  // bytes of one block's host bispectra
    const int cols = (int)std::max(1LL, std::min((long long)nf, budget / (16LL * nf * nb)));
    // the export file, if this analysis writes one: the grid as one rectangular zone
    if ((rc = brm_file_open(true, 1)) || (rc = brm_file_zone(1, nf, nf))) return rc;
    std::vector<double> br((size_t)cols * nf * nb), f1((size_t)cols * nf), f2((size_t)cols * nf);
    std::vector<double> accF(nb, 0.0), accR(nb, 0.0), mf(nb), mr(nb);
    for (int c0 = 0; c0 < nf; c0 += cols) {
        const int nc = std::min(cols, nf - c0);
        const long long npts = (long long)nc * nf;
        ps.pbase = (long long)c0 * nf;
        rc = set.onlyd ? contract_diag(ps, npts, 0, mf.data(), mr.data(), nullptr, br.data())
                       : contract(ps, npts, mf.data(), mr.data(), nullptr, br.data());
        if (rc) return rc;
        for (long long p = 0; p < npts; ++p) {
            f1[p] = f[p % nf];
            f2[p] = f[c0 + p / nf];
        }
        if ((rc = emit_brm((int)npts, f1.data(), f2.data(), br.data()))) return rc;
        for (long long x = 0; x < nb; ++x) {
            accF[x] += mf[x];
            accR[x] += mr[x];
        }
    }
    if ((rc = brm_file_close((long long)nf * nf))) return rc;
    if (m3mf) std::memcpy(m3mf, accF.data(), sizeof(double) * nb);
    if (m3mr) std::memcpy(m3mr, accR.data(), sizeof(double) * nb);
    return BSA_OK;
}

// Contraction + FRF + reduction over a point source; dA must hold every row it names.
int Engine::contract(const PointSrc &ps, long long npts, double *m3mf, double *m3mr, double *bf_host,
                     double *br_host) {
    const long long nm3 = (long long)nme * nme * nme;
    cudaError_t e;
    const int G = bfm_fp64_groups(npts, nme);
    if ((e = dPartF.reserve(sizeof(double) * (size_t)G * nm3)) || (e = dPartR.reserve(sizeof(double) * (size_t)G * nm3)))
        return cuda_fail(e, "allocating partial sums");
    if ((e = dOut.reserve(sizeof(double) * (3 * (size_t)nme * nme + 2 * (size_t)nm3)))) return cuda_fail(e, "out");
    double *bfd = nullptr, *brd = nullptr;
    if (bf_host || br_host) {
        if ((e = dBF.reserve(sizeof(double) * (size_t)npts * nm3)) || (e = dBR.reserve(sizeof(double) * (size_t)npts * nm3)))
            return cuda_fail(e, "allocating bispectra");
        bfd = dBF.as<double>();
        brd = dBR.as<double>();
    }
    if ((e = cudaEventRecord(ev2, stream))) return cuda_fail(e, "event");
    if ((e = cudaEventRecord(evg0, stream))) return cuda_fail(e, "event");
    if ((e = launch_bfm_fp64(stream, dA.as<double>(), dQ.as<double>(), K, nme, ps, npts, frf(), G, dPartF.as<double>(),
                             dPartR.as<double>(), bfd, brd)))
        return cuda_fail(e, "FP64 contraction kernel");
    if ((e = cudaEventRecord(evg1, stream))) return cuda_fail(e, "event");
    double *o = dOut.as<double>() + 3 * (size_t)nme * nme;
    if ((e = launch_reduce_groups(stream, G, nm3, dPartF.as<double>(), o, dPartR.as<double>(), o + nm3)))
        return cuda_fail(e, "reduction kernel");
    kernels += 2;
    std::vector<double> h(2 * (size_t)nm3);
    if ((e = cudaMemcpyAsync(h.data(), o, sizeof(double) * h.size(), cudaMemcpyDeviceToHost, stream)))
        return cuda_fail(e, "moment copy");
    if (bf_host && (e = cudaMemcpyAsync(bf_host, bfd, sizeof(double) * (size_t)npts * nm3, cudaMemcpyDeviceToHost, stream)))
        return cuda_fail(e, "bispectrum copy");
    if (br_host && (e = cudaMemcpyAsync(br_host, brd, sizeof(double) * (size_t)npts * nm3, cudaMemcpyDeviceToHost, stream)))
        return cuda_fail(e, "bispectrum copy");
    if ((e = cudaEventRecord(ev1, stream)) || (e = cudaStreamSynchronize(stream))) return cuda_fail(e, "sync");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ev2, ev1);
    last_ms_contraction = ms;
    cudaEventElapsedTime(&ms, evg0, evg1);
    last_ms_gemm = ms;
    d2h += (double)sizeof(double) * h.size() + (bf_host ? 8.0 * npts * nm3 : 0.0) + (br_host ? 8.0 * npts * nm3 : 0.0);
    if (m3mf) std::memcpy(m3mf, h.data(), sizeof(double) * nm3);
    if (m3mr) std::memcpy(m3mr, h.data() + nm3, sizeof(double) * nm3);
    return BSA_OK;
}

// Point-set evaluation with analytic f1+f2 (Mesher functions and BsaCL semantics).
int Engine::run_points(const double *fi, const double *fj, const double *w, double wuniform, long long npts,
                       double *m3mf, double *m3mr, double *bfm, double *brm, const std::vector<ZoneDev> *zones,
                       const int *zid, const int *zi, const int *zj, const long long *cptr, const double *cq) {
    kernels = 0;
    graph_launches = 0;
    h2d = d2h = 0;
    last_ms_gemm = 0;
    int rc = upload_problem();
    if (rc) return rc;
    if (npts <= 0) return fail(BSA_ERR_ARG, "empty point set");
    // Distinct frequencies: f1, f2 and f1+f2 of every point share one A table.
    std::vector<double> ftab;
    ftab.reserve(3 * (size_t)npts);
    std::vector<int> ix(npts), iy(npts), iz(npts);
    {
        std::vector<std::pair<double, int>> key;
        key.reserve(3 * (size_t)npts);
        for (long long p = 0; p < npts; ++p) {
            key.push_back({fi[p], (int)(3 * p)});
            key.push_back({fj[p], (int)(3 * p + 1)});
            key.push_back({fi[p] + fj[p], (int)(3 * p + 2)});
        }
        std::sort(key.begin(), key.end());
        int row = -1;
        double last = NAN;
        for (auto &kv : key) {
            if (!(kv.first == last)) {
                ftab.push_back(kv.first);
                last = kv.first;
                ++row;
            }
            const int p = kv.second / 3, which = kv.second % 3;
            (which == 0 ? ix : which == 1 ? iy : iz)[p] = row;
        }
    }
    cudaError_t e;
    if ((e = cudaEventRecord(ev0, stream))) return cuda_fail(e, "event");
    if ((rc = set.onlyd ? build_psd(ftab) : build_atable(ftab, false, true))) return rc;
    std::vector<double> f1(fi, fi + npts), f2(fj, fj + npts);
    h2d += (double)npts * (3 * sizeof(int) + (w ? 3 : 2) * sizeof(double));
    const size_t n = (size_t)npts;
    if ((e = dPts.reserve(n * 3 * sizeof(int))) || (e = dPtsD.reserve(n * 3 * sizeof(double))))
        return cuda_fail(e, "points");
    int *dix = dPts.as<int>(), *diy = dix + n, *diz = diy + n;
    double *df1 = dPtsD.as<double>(), *df2 = df1 + n, *dw = df2 + n;
    if ((e = cudaMemcpyAsync(dix, ix.data(), n * sizeof(int), cudaMemcpyHostToDevice, stream)) ||
        (e = cudaMemcpyAsync(diy, iy.data(), n * sizeof(int), cudaMemcpyHostToDevice, stream)) ||
        (e = cudaMemcpyAsync(diz, iz.data(), n * sizeof(int), cudaMemcpyHostToDevice, stream)) ||
        (e = cudaMemcpyAsync(df1, f1.data(), n * sizeof(double), cudaMemcpyHostToDevice, stream)) ||
        (e = cudaMemcpyAsync(df2, f2.data(), n * sizeof(double), cudaMemcpyHostToDevice, stream)) ||
        (w && (e = cudaMemcpyAsync(dw, w, n * sizeof(double), cudaMemcpyHostToDevice, stream))))
        return cuda_fail(e, "point upload");
    PointSrc ps{};
    ps.mode = kPointsList;
    ps.wmode = w ? kWeightList : kWeightUniform;
    ps.wval = wuniform;
    ps.ix = dix; ps.iy = diy; ps.iz = diz;
    ps.f1 = df1; ps.f2 = df2; ps.w = w ? dw : nullptr;
    if (zones) {
        if ((e = upload(dZones, *zones, stream)) || (e = dZidx.reserve(n * 3 * sizeof(int))))
            return cuda_fail(e, "zone upload");
        int *dzid = dZidx.as<int>(), *dzi = dzid + n, *dzj = dzi + n;
        if ((e = cudaMemcpyAsync(dzid, zid, n * sizeof(int), cudaMemcpyHostToDevice, stream)) ||
            (e = cudaMemcpyAsync(dzi, zi, n * sizeof(int), cudaMemcpyHostToDevice, stream)) ||
            (e = cudaMemcpyAsync(dzj, zj, n * sizeof(int), cudaMemcpyHostToDevice, stream)))
            return cuda_fail(e, "zone upload");
        h2d += (double)n * 3 * sizeof(int);
        ps.zones = dZones.as<ZoneDev>();
        ps.zid = dzid;
        ps.zi = dzi;
        ps.zj = dzj;
    }
    if (cptr) {
        const size_t ne = (size_t)cptr[n];
        if ((e = dCptr.reserve((n + 1) * sizeof(long long))) || (e = dCq.reserve((3 * ne + 1) * sizeof(double))))
            return cuda_fail(e, "BRM point lists");
        if ((e = cudaMemcpyAsync(dCptr.p, cptr, (n + 1) * sizeof(long long), cudaMemcpyHostToDevice, stream)) ||
            (ne && (e = cudaMemcpyAsync(dCq.p, cq, 3 * ne * sizeof(double), cudaMemcpyHostToDevice, stream))))
            return cuda_fail(e, "BRM point lists");
        h2d += (double)(n + 1) * sizeof(long long) + 3.0 * ne * sizeof(double);
        ps.cptr = dCptr.as<long long>();
        ps.cq = dCq.as<double>();
    }
    // Mesher functions: the diagonal-only form is getFM_diag_tnm_scalar_msh_'s.
    rc = set.onlyd ? contract_diag(ps, npts, 1, m3mf, m3mr, bfm, brm) : contract(ps, npts, m3mf, m3mr, bfm, brm);
    if (rc) return rc;
    last_points = (double)npts;
    if ((e = cudaEventRecord(ev1, stream)) || (e = cudaEventSynchronize(ev1))) return cuda_fail(e, "event");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ev0, ev1);
    last_ms = ms;
    return BSA_OK;
}

// Classic bispectra at listed grid points (bsa_gpu_clsBispectraAt): FP64 through the point
// form of the FP64 kernel on the grid's A table (S(f1 + f2) truncated or analytic as the
// analysis reads it); BF16x3 through the sampled instantiation of the E-form contraction, the
// analysis's own products (whole odd grid, truncated sum, at most 48 kept modes).
int Engine::classic_points(const int *i1, const int *i2, long long npts, double *bf, double *br) {
    kernels = 0;
    graph_launches = 0;
    h2d = d2h = 0;
    last_ms_gemm = 0;
    int rc = upload_problem();
    if (rc) return rc;
    if (set.onlyd) return fail(BSA_ERR_UNSUPPORTED, "per-point Classic bispectra need the full-tensor spectra");
    std::vector<double> f;
    if ((rc = classic_grid(f))) return rc;
    const int nf = (int)f.size(), h = (nf - 1) / 2;
    for (long long p = 0; p < npts; ++p)
        if (i1[p] < 0 || i1[p] >= nf || i2[p] < 0 || i2[p] >= nf)
            return fail(BSA_ERR_ARG, "grid point %lld = (%d, %d) outside the %d-point grid", p, i1[p], i2[p], nf);
    const long long nm3 = dim_bisp();
    const bool analytic = !classic_trunc;
    cudaError_t e;
    if ((e = cudaEventRecord(ev0, stream))) return cuda_fail(e, "event");
    if (precision == BSA_PREC_BF16X3) {
        if (analytic || !(nf & 1) || nme > kEFormMaxModes)
            return fail(BSA_ERR_UNSUPPORTED,
                        "split-precision point bispectra come from the E-form contraction: truncated S(f1+f2), odd "
                        "grid, at most %d kept modes", kEFormMaxModes);
        if ((rc = build_atable(f, true))) return rc;
        // slot of every grid point (first occurrence of a repeated point)
        std::vector<int> slot((size_t)nf * nf, -1), first((size_t)npts);
        int nslot = 0;
        for (long long p = 0; p < npts; ++p) {
            int &s = slot[(size_t)i1[p] + (size_t)nf * i2[p]];
            if (s < 0) s = nslot++;
            first[p] = s;
        }
        if ((e = upload(dSlot, slot, stream)) || (e = dBF.reserve(sizeof(double) * (size_t)nslot * nm3)) ||
            (e = dBR.reserve(sizeof(double) * (size_t)nslot * nm3)))
            return cuda_fail(e, "allocating sampled bispectra");
        PointSrc ps{};
        ps.mode = kPointsGrid;
        ps.nf = nf;
        ps.n_pad = h;
        ps.trunc = 1;
        ps.sum_base = nf;
        ps.wmode = kWeightUniform;
        ps.wval = 1.0;
        ps.fgrid = dFreq.as<double>();
        ps.r0 = 0;
        ps.nr = nf;
        ESample smp{dSlot.as<int>(), dBF.as<double>(), dBR.as<double>(), nslot};
        if ((rc = contract_e(ps, nullptr, nullptr, &smp))) return rc;
        std::vector<double> hf((size_t)nslot * nm3), hr((size_t)nslot * nm3);
        if ((e = cudaMemcpyAsync(hf.data(), smp.sF, sizeof(double) * hf.size(), cudaMemcpyDeviceToHost, stream)) ||
            (e = cudaMemcpyAsync(hr.data(), smp.sR, sizeof(double) * hr.size(), cudaMemcpyDeviceToHost, stream)) ||
            (e = cudaStreamSynchronize(stream)))
            return cuda_fail(e, "sampled bispectra copy");
        d2h += 16.0 * nslot * nm3;
        for (long long p = 0; p < npts; ++p) {
            if (bf) std::memcpy(bf + p * nm3, hf.data() + (size_t)first[p] * nm3, sizeof(double) * nm3);
            if (br) std::memcpy(br + p * nm3, hr.data() + (size_t)first[p] * nm3, sizeof(double) * nm3);
        }
    } else {
        std::vector<double> ftab = f;
        if (analytic)
            for (int s2 = 0; s2 < 2 * nf - 1; ++s2) ftab.push_back(2.0 * f[0] + s2 * (f[1] - f[0]));
        if ((rc = build_atable(ftab, false))) return rc;
        const size_t n = (size_t)npts;
        std::vector<int> iz(n);
        std::vector<double> f1(n), f2(n);
        for (size_t p = 0; p < n; ++p) {
            const int s2 = i1[p] + i2[p];
            iz[p] = analytic ? nf + s2 : ((s2 - h >= 0 && s2 - h < nf) ? s2 - h : -1);
            f1[p] = f[i1[p]];
            f2[p] = f[i2[p]];
        }
        if ((e = dPts.reserve(n * 3 * sizeof(int))) || (e = dPtsD.reserve(n * 3 * sizeof(double))))
            return cuda_fail(e, "points");
        int *dix = dPts.as<int>(), *diy = dix + n, *diz = diy + n;
        double *df1 = dPtsD.as<double>(), *df2 = df1 + n;
        if ((e = cudaMemcpyAsync(dix, i1, n * sizeof(int), cudaMemcpyHostToDevice, stream)) ||
            (e = cudaMemcpyAsync(diy, i2, n * sizeof(int), cudaMemcpyHostToDevice, stream)) ||
            (e = cudaMemcpyAsync(diz, iz.data(), n * sizeof(int), cudaMemcpyHostToDevice, stream)) ||
            (e = cudaMemcpyAsync(df1, f1.data(), n * sizeof(double), cudaMemcpyHostToDevice, stream)) ||
            (e = cudaMemcpyAsync(df2, f2.data(), n * sizeof(double), cudaMemcpyHostToDevice, stream)))
            return cuda_fail(e, "point upload");
        h2d += (double)n * (3 * sizeof(int) + 2 * sizeof(double));
        PointSrc ps{};
        ps.mode = kPointsList;
        ps.wmode = kWeightUniform;
        ps.wval = 1.0;
        ps.ix = dix;
        ps.iy = diy;
        ps.iz = diz;
        ps.f1 = df1;
        ps.f2 = df2;
        std::vector<double> mf(nm3), mr(nm3);
        if ((rc = contract(ps, npts, mf.data(), mr.data(), bf, br))) return rc;
    }
    last_points = (double)npts;
    if ((e = cudaEventRecord(ev1, stream)) || (e = cudaEventSynchronize(ev1))) return cuda_fail(e, "event");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, ev0, ev1);
    last_ms = ms;
    return BSA_OK;
}

}  // namespace bsa

using bsa::eng;

#define GUARD()                                                        \
    do {                                                               \
        if (eng().halted) return BSA_ERR_STATE;                        \
    } while (0)
#define SETTER_BODY(stmt) \
    GUARD();              \
    stmt;                 \
    eng().derived_ok = false; \
    return BSA_OK

extern "C" {

int bsa_Init(void) {
    bsa::Engine &E = eng();
    E.free_device();
    E.reset_inputs();
    E.halted = false;
    E.last_error.clear();
    E.inited = true;
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0)
        return E.fail(BSA_ERR_CUDA, "no CUDA device: %s", e == cudaSuccess ? "0 devices" : cudaGetErrorString(e));
    return BSA_OK;
}

int bsa_setAnalysisType(int v) {
    GUARD();
    if (v < 0 || v > 3) return eng().fail(BSA_ERR_ARG, "invalid sub-analysis value");
    eng().set.suban = v;
    return BSA_OK;
}
int bsa_setVersion(int v) {
    GUARD();
    if (v < 0 || v > 2) return eng().fail(BSA_ERR_ARG, "invalid version value");
    eng().set.vers = v;
    return BSA_OK;
}
int bsa_setScalingConv(int v) {
    GUARD();
    if (v < 0 || v > 2) return eng().fail(BSA_ERR_ARG, "invalid scaling convention");
    if (v != 0) eng().set.defsc = v;
    eng().derived_ok = false;
    return BSA_OK;
}
int bsa_setSpectraComputation(int ipsd, int ibisp) {
    GUARD();
    eng().set.ipsd = (ipsd < 0 || ipsd > 1) ? 1 : ipsd;
    eng().set.ibisp = (ibisp < 0 || ibisp > 1) ? 1 : ibisp;
    return BSA_OK;
}
int bsa_setSpectraExtension(int v) {
    GUARD();
    if (v < 0 || v > 1) return eng().fail(BSA_ERR_ARG, "invalid only-diagonal value");
    eng().set.onlyd = v;
    return BSA_OK;
}
int bsa_setSpatialSymmetry(int v) {
    GUARD();
    eng().set.bispsym = (v == 0 || v == 4) ? v : 2;
    return BSA_OK;
}
int bsa_setSpectraSymmetries(int v) {
    GUARD();
    eng().set.spctrsym = (v == 0 || v == 1) ? v : 0;
    return BSA_OK;
}
int bsa_setTestMode(int v) {
    GUARD();
    if (v < 0 || v > 1) return eng().fail(BSA_ERR_ARG, "invalid test-mode value");
    eng().set.test = v;
    return BSA_OK;
}
int bsa_setupClassic(int nfreqs, double df) {
    GUARD();
    eng().set.nfreqs = nfreqs;
    eng().set.df = df;
    return BSA_OK;
}
int bsa_setClassicMode(int v) {
    GUARD();
    eng().set.scalar = (v == 0 || v == 1) ? v : 0;
    return BSA_OK;
}
int bsa_setupMesher(int isvd, int bkgrfmt, double bkgaext, double genpaext, double maxaext, int ifcov, int idumpmod) {
    GUARD();
    bsa::Settings &s = eng().set;
    s.svd = isvd; s.bkgrfmt = bkgrfmt; s.bkgaext = bkgaext; s.genpaext = genpaext; s.maxaext = maxaext;
    s.fcov = ifcov; s.dumpmod = idumpmod;
    return BSA_OK;
}
int bsa_setPODTruncationThreshold(double rval) {
    GUARD();
    if (rval > 0.0) eng().pod_trunc_lim = rval / 100.0;
    return BSA_OK;
}
int bsa_setPODNOfModesKept(int nmodes) {
    GUARD();
    eng().pod_nmodes = nmodes;
    return BSA_OK;
}
int bsa_doValidateZoneDeltas(int on) {
    GUARD();
    eng().validate_deltas = on != 0;
    return BSA_OK;
}
int bsa_setBfmMLR(int on) {
    GUARD();
    eng().bfm_mlr = on != 0;
    return BSA_OK;
}
int bsa_setMaxBkgPeakRestriction(int on) {
    GUARD();
    eng().bkg_restrict = on != 0;
    return BSA_OK;
}
// bsa_setPremeshScheme (BsaLibImpl.F90:796-810): 1 selects the diagonal-crest scheme; any
// other value leaves the scheme as it is.
int bsa_setPremeshScheme(int itype) {
    GUARD();
    if (itype == 1) eng().premesh_diag_crest = true;
    return BSA_OK;
}
// bsa_setPremeshMode (BsaLibImpl.F90:813-826): 0 selects the base mode, any other value
// leaves the mode as it is; the diagonal-crest scheme reads it (and refuses the base mode).
int bsa_setPremeshMode(int imode) {
    GUARD();
    if (imode == 0) eng().premesh_mode_base = true;
    return BSA_OK;
}
int bsa_setWindDirections(const int *dirs, int ndirs) {
    GUARD();
    if (!dirs || ndirs < 1 || ndirs > 3) return eng().fail(BSA_ERR_ARG, "size mismatch in setting spatial directions");
    SETTER_BODY(eng().set.dirs.assign(dirs, dirs + ndirs));
}
int bsa_setWindTurbComps(const int *tc, int ntc) {
    GUARD();
    if (!tc || ntc < 1 || ntc > 3) return eng().fail(BSA_ERR_ARG, "size mismatch in setting turbulent components");
    SETTER_BODY(eng().set.tc.assign(tc, tc + ntc));
}
int bsa_setTotalNOfNodes(int nn) { SETTER_BODY(eng().in.nn = nn); }
int bsa_setNumOfNodalDOFs(int nlibs) { SETTER_BODY(eng().in.nlibs = nlibs); }
int bsa_setTotalNumOfDOFs(int ndofs) { SETTER_BODY(eng().in.ndofs = ndofs); }
int bsa_setLoadedNodes(const int *nodes, int nnl) {
    GUARD();
    if (!nodes || nnl <= 0) return eng().fail(BSA_ERR_ARG, "empty loaded-node list");
    SETTER_BODY((eng().in.n_load = nodes, eng().in.nnl = nnl));
}
int bsa_setLoadedNodalDOFs(const int *libs, int nlibsl) {
    GUARD();
    if (!libs || nlibsl <= 0) return eng().fail(BSA_ERR_ARG, "empty loaded-DOF list");
    SETTER_BODY((eng().in.libs_load = libs, eng().in.nlibsl = nlibsl));
}
int bsa_setNodalCoords(int nn, const double *coords) {
    GUARD();
    bsa::Inputs &I = eng().in;
    if (I.nn != 0 && I.nn != nn) return eng().fail(BSA_ERR_ARG, "nodal info does not match in setting nodal coordinates");
    SETTER_BODY((I.nn = nn, I.coords = coords));
}
int bsa_setModalInfo(int ndofs, int nm, const double *phi, const double *natf) {
    GUARD();
    bsa::Inputs &I = eng().in;
    SETTER_BODY((I.ndofs = ndofs, I.phi_ndofs = ndofs, I.nm = nm, I.phi = phi, I.natf = natf));
}
int bsa_setModalMatrices(int nm, const double *M, const double *Kg, const double *Cg) {
    GUARD();
    bsa::Inputs &I = eng().in;
    if (I.nm != 0 && I.nm != nm) return eng().fail(BSA_ERR_ARG, "nm differs from previously set");
    SETTER_BODY((I.nm = nm, I.Mg = M, I.Kg = Kg, I.Cg = Cg));
}
int bsa_setTotDamping(const double *xsi, int nm) {
    GUARD();
    if (eng().in.nm == 0) return eng().fail(BSA_ERR_STATE, "NM == 0 when setting damping info");
    if (nm != eng().in.nm) return eng().fail(BSA_ERR_ARG, "damping size does not match nm");
    SETTER_BODY(eng().in.xsi = xsi);
}
int bsa_setPSDType(int ipsd) {
    GUARD();
    SETTER_BODY(eng().in.psd_type = (ipsd < 1 || ipsd > 5) ? 5 : ipsd);
}
int bsa_setWindVertProf(int v) {
    GUARD();
    if (v == 5) v = 1;
    if (v < 1 || v > 3) return eng().fail(BSA_ERR_ARG, "invalid iwprof value");
    eng().in.wprof = v;
    return BSA_OK;
}
int bsa_setWindAltDir(int v) {
    GUARD();
    if (v < 1 || v > 3) return eng().fail(BSA_ERR_ARG, "invalid ivert value");
    eng().in.vert = v;
    return BSA_OK;
}
int bsa_setAirDensity(double a) {
    GUARD();
    if (a < 0.0) return eng().fail(BSA_ERR_ARG, "air density has a negative value");
    eng().in.air_dens = a;
    return BSA_OK;
}
int bsa_setWZMeanWindVel(const double *u, int nz) { SETTER_BODY((eng().in.ubref = u, eng().in.nz = std::max(eng().in.nz, nz))); }
int bsa_setWZRefAlt(const double *z, int nz) { SETTER_BODY((eng().in.zref = z, eng().in.nz = std::max(eng().in.nz, nz))); }
int bsa_setTurbWindScales(const double *L, int nz) { SETTER_BODY((eng().in.L = L, eng().in.nz = std::max(eng().in.nz, nz))); }
int bsa_setTurbWindSDT(const double *s, int nz) { SETTER_BODY((eng().in.sigma = s, eng().in.nz = std::max(eng().in.nz, nz))); }
int bsa_setNodalVel(const double *u, int nn) { (void)nn; SETTER_BODY(eng().in.unod = u); }
int bsa_setNodalWindZones(const int *wz, int nn) { (void)nn; SETTER_BODY(eng().in.wz = wz); }
int bsa_setNodalWindAltitudes(const double *a, int nn) { (void)nn; SETTER_BODY(eng().in.walt = a); }
int bsa_setSpatialNodalCorr(const double *c, int64_t ncorr) { SETTER_BODY((eng().in.corr = c, eng().in.ncorr = ncorr)); }
int bsa_setWindFCoeffs(const double *wfc, int nl, int nd, int nn) {
    GUARD();
    bsa::Inputs &I = eng().in;
    SETTER_BODY((I.wfc = wfc, I.wfc_nl = nl, I.wfc_nd = nd, I.wfc_nn = nn));
}

int bsa_getNModesEff(int *nm_eff) {
    GUARD();
    int rc = eng().validate();
    if (rc) return rc;
    if (nm_eff) *nm_eff = eng().nme;
    return BSA_OK;
}

int bsa_Run(double *m2mf_cls, double *m2mr_cls, double *m2o2mr_cls, double *m3mf_msh, double *m3mr_msh,
            double *m3mf_cls, double *m3mr_cls) {
    GUARD();
    bsa::Engine &E = eng();
    if (!E.inited) return E.fail(BSA_ERR_STATE, "bsa_Init was not called");
    if (E.set.ipsd == 0 && E.set.ibisp == 0) return BSA_OK;  // both disabled: nothing to do
    int rc = E.validate();
    if (rc) return rc;
    const int su = E.set.suban;
    if (su == 2 || su == 3) {
        rc = E.run_mesher(m3mf_msh, m3mr_msh);
        if (rc) return rc;
    }
    if (su == 1 || su == 3 || su == 0) {
        rc = E.run_classic(m2mf_cls, m2mr_cls, m2o2mr_cls, m3mf_cls, m3mr_cls, nullptr, nullptr, nullptr);
        if (rc) return rc;
    }
    return BSA_OK;
}

int bsa_Finalise(void) {
    bsa::Engine &E = eng();
    E.free_device();
    E.reset_inputs();
    E.halted = false;
    E.inited = false;
    return BSA_OK;
}

int bsa_computeSkewness(int nm, const double *m2, const double *m3, double *sk) {
    if (nm <= 0 || !m2 || !m3 || !sk) return BSA_ERR_ARG;
    if (eng().set.onlyd) {
        // computeSkewness_ diagonal branch (BsaLibImpl.F90:1641-1644): sk = m3 / m2^(3/2).
        for (int i = 0; i < nm; ++i) sk[i] = m3[i] / std::pow(m2[i], 1.5);
        return BSA_OK;
    }
    size_t pm3 = 0;
    for (int k = 0; k < nm; ++k)
        for (int j = 0; j < nm; ++j)
            for (int i = 0; i < nm; ++i, ++pm3)
                sk[pm3] = m3[pm3] / (std::sqrt(m2[k * nm + k]) * std::sqrt(m2[j * nm + j]) * std::sqrt(m2[i * nm + i]));
    return BSA_OK;
}

const char *bsa_lastError(void) { return eng().last_error.c_str(); }

int bsa_getSpectraDims(int *dim_psd, int *dim_bisp) {
    GUARD();
    bsa::Engine &E = eng();
    int rc = E.validate();
    if (rc) return rc;
    if (dim_psd) *dim_psd = (int)E.dim_psd();
    if (dim_bisp) *dim_bisp = (int)E.dim_bisp();
    return BSA_OK;
}

int bsa_gpu_setClassicSymmetry(int on) {
    GUARD();
    eng().classic_sym = on != 0;
    return BSA_OK;
}

int bsa_setBispExportCallback(bsa_brm_export_fn fn, void *user) {
    GUARD();
    eng().export_fn = fn;
    eng().export_user = user;
    return BSA_OK;
}

int bsa_gpu_setPrecision(int prec) {
    GUARD();
    if (prec != BSA_PREC_FP64 && prec != BSA_PREC_BF16X3) return eng().fail(BSA_ERR_ARG, "unknown precision");
    eng().precision = prec;
    return BSA_OK;
}

int bsa_gpu_setClassicRows(int r_begin, int r_end) {
    GUARD();
    if (r_begin < 0 || (r_end >= 0 && r_end <= r_begin)) return eng().fail(BSA_ERR_ARG, "invalid classic row range");
    eng().shard_r0 = r_begin;
    eng().shard_r1 = r_end;
    return BSA_OK;
}

int bsa_gpu_setClassicTruncation(int on) {
    GUARD();
    eng().classic_trunc = on != 0;
    return BSA_OK;
}

int bsa_gpu_clsBispectra(double *f_out, int nf_cap, int *nf, double *bisp_f, double *bisp_r) {
    GUARD();
    bsa::Engine &E = eng();
    int rc = E.validate();
    if (rc) return rc;
    std::vector<double> grid;
    if ((rc = E.classic_grid(grid))) return rc;
    if (nf) *nf = (int)grid.size();
    if ((int)grid.size() > nf_cap) return E.fail(BSA_ERR_ARG, "grid has %zu points, capacity %d", grid.size(), nf_cap);
    const int prec = E.precision;
    E.precision = BSA_PREC_FP64;
    rc = E.run_classic(nullptr, nullptr, nullptr, nullptr, nullptr, bisp_f, bisp_r, &grid);
    E.precision = prec;
    if (rc) return rc;
    if (f_out) std::memcpy(f_out, grid.data(), sizeof(double) * grid.size());
    return BSA_OK;
}

int bsa_gpu_setClassicShard(int rank, int nshards) {
    GUARD();
    if (nshards < 1 || rank < 0 || rank >= nshards)
        return eng().fail(BSA_ERR_ARG, "shard %d of %d", rank, nshards);
    eng().cls_shard = rank;
    eng().cls_shards = nshards;
    return BSA_OK;
}

int bsa_gpu_setWaitTest(int tile) {
    GUARD();
    if (tile < -1) return eng().fail(BSA_ERR_ARG, "tile must be >= -1");
    eng().wait_test_tile1 = tile + 1;
    return BSA_OK;
}

int bsa_gpu_clsBispectraAt(const int *i1, const int *i2, int npts, double *bisp_f, double *bisp_r) {
    GUARD();
    if (!i1 || !i2 || npts <= 0) return eng().fail(BSA_ERR_ARG, "empty point list");
    return eng().classic_points(i1, i2, npts, bisp_f, bisp_r);
}

int bsa_gpu_mshBispectra(const double *fi, const double *fj, int npts, double *bfm, double *brm) {
    GUARD();
    if (!fi || !fj || npts <= 0) return eng().fail(BSA_ERR_ARG, "empty point set");
    return eng().run_points(fi, fj, nullptr, 0.0, npts, nullptr, nullptr, bfm, brm);
}

int bsa_gpu_mshMoments(const double *fi, const double *fj, const double *w, int npts, double *m3mf, double *m3mr) {
    GUARD();
    if (!fi || !fj || !w || npts <= 0) return eng().fail(BSA_ERR_ARG, "empty point set");
    return eng().run_points(fi, fj, w, 0.0, npts, m3mf, m3mr, nullptr, nullptr);
}

int bsa_gpu_getStats(bsa_gpu_stats *st) {
    if (!st) return BSA_ERR_ARG;
    st->ms_total = eng().last_ms;
    st->ms_contraction = eng().last_ms_contraction;
    st->ms_gemm = eng().last_ms_gemm;
    st->points = eng().last_points;
    st->h2d_bytes = eng().h2d;
    st->d2h_bytes = eng().d2h;
    st->kernels = eng().kernels;
    st->precision = eng().precision;
    st->graphs = eng().graph_launches;
    return BSA_OK;
}

int bsa_gpu_setMesherGraphs(int on) {
    GUARD();
    eng().msh_graphs = on != 0;
    return BSA_OK;
}

int bsa_gpu_setMesherExpansion(int on_device) {
    GUARD();
    eng().msh_dev_expand = on_device != 0;
    return BSA_OK;
}

int bsa_gpu_setMesherPassBytes(double bytes) {
    GUARD();
    eng().msh_pass_bytes = bytes > 0.0 ? bytes : 0.0;
    return BSA_OK;
}

int bsa_gpu_setClassicForm(int form) {
    if (form != 0 && form != 1) return BSA_ERR_ARG;
    eng().use_e_form = form == 1;
    return BSA_OK;
}

int bsa_gpu_releaseDeviceCache(void) {
    bsa::release_device_cache();
    return BSA_OK;
}

}  // extern "C"
