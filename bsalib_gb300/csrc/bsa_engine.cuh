// bsa_engine.cuh -- the library's single state object (BsaLib keeps the same state in
// module globals: settings, wd, struct_data; src/bsa/data/BsaLibData.F90).
#pragma once
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "../../include/bsa_gpu.h"
#include "bsa_common.cuh"

namespace bsa {

// Kept modes up to which the split contraction takes its E form (bsa_classic_e.cu; above 24
// in two mode halves).
constexpr int kEFormMaxModes = 48;

// Tile plans (bsa_plans.cu): the autotuned shape of each split-precision contraction, or the
// default rule.  Widths: E form 8 / 16 / 24 / 32 (2 x 16) / 48 (2 x 24); D1 / D3 form 8 / 16 / 24 /
// 32 / 64 (2 x 32); Mesher NMT a multiple of 8 in [nm, 64].
int plan_e_width(int nm, int K, int nf);
int plan_d_width(int nm, int K, int nf);
bool plan_prefer_e(int nm, int K, int nf);
int plan_e_split(int W, int nm, int K, int nf);  // E form passes over the modes of width W
int plan_msh_width(int nm, int K);

// Device buffer that only grows (kept across runs; freed by bsa_Finalise).
// Frees the device blocks the engine keeps for reuse after bsa_Finalise.
void release_device_cache();

struct DevBuf {
    void *p = nullptr;
    size_t bytes = 0;
    cudaError_t reserve(size_t nbytes);
    void release();
    template <class T>
    T *as() const { return (T *)p; }
};

// Borrowed caller arrays (Fortran layouts), as the reference keeps pointers to them.
struct Inputs {
    int nn = 0, nlibs = 0, ndofs = 0, phi_ndofs = 0, nnl = 0, nlibsl = 0;
    const int *n_load = nullptr, *libs_load = nullptr;
    const double *coords = nullptr;
    int nm = 0;
    const double *phi = nullptr, *natf = nullptr, *Mg = nullptr, *Kg = nullptr, *Cg = nullptr, *xsi = nullptr;
    int psd_type = 5;  // WindData_t default i_psd_type_ (src/wind/WindType.F90:76)
    int nz = 0;
    const double *ubref = nullptr, *zref = nullptr, *L = nullptr, *sigma = nullptr;
    const double *unod = nullptr, *walt = nullptr;
    const int *wz = nullptr;
    const double *corr = nullptr;
    long long ncorr = 0;
    const double *wfc = nullptr;
    int wfc_nl = 0, wfc_nd = 0, wfc_nn = 0;
    int wprof = 2, vert = 3;
    double air_dens = 1.22;
    // Projected coefficients supplied directly (BsaCL's bsaclAcquirePhiTimesCMat): then the
    // mode list and PHItimesC are taken as given instead of derived from Phi and wfc.
    const double *ext_phitc = nullptr;
    const int *ext_modes = nullptr;
    int ext_nme = 0, ext_nnl = 0, ext_nd = 0;
};

// settings_t defaults (src/settings/Settings.F90:25-116).
struct Settings {
    int suban = 2, vers = 2, defsc = 1, ipsd = 1, ibisp = 1, onlyd = 0, bispsym = 0, spctrsym = 0, test = 0;
    int nfreqs = 0, scalar = 0;
    double df = 0.0;
    int svd = 1, bkgrfmt = 20, fcov = 1, dumpmod = 0;
    double bkgaext = 2.0, genpaext = 2.0, maxaext = 2.0;
    std::vector<int> dirs{1};
    std::vector<int> tc{1};
};

struct BatchCase;  // one case of the batched Classic sweep (bsa_batch.cu)

// A dumped triangular zone (dumpTZ and DumpZone: corner C, A at the end of the J side, B,
// rotation, refinements ni = nj = n, policy) with its policy's factors resolved (BFM
// refinement levels disabled by bsa_setBfmMLR(false)) and the spatial-symmetry weight.
struct TriDump {
    double Ci, Cj, Ai, Aj, Bi, Bj, rot, sym;
    int n, pol, bfi, bfj, bri, brj, nlevs;
};

// The post-mesh lattice of one triangle (bsa_triang.cu): BFM points (evaluation coordinates,
// m3mf weights without the symmetry factor), BRM points (m3mr weights), per BRM point the BFM
// points its interpolated BFM combines (CSR qptr / qsrc / qc), and the BRM export in the
// routine's write order (written coordinates, BRM point or -1 for a slot never written).
struct TriLattice {
    std::vector<double> bf1, bf2, bw, q1, q2, qw, qc, e1, e2;
    std::vector<int> qptr, qsrc, eq;
    long long bfm_post = 0, brm_post = 0;  // the counts the reference adds to msh_*pts_post_
    int nI = 0, nJ = 0;                    // the export header's nI_, nJ_
    bool oob = false;                      // the walk used brm / work-array slots past their sizes
};
int triangle_lattice(const TriDump &t, bool visual, TriLattice &L, const char **err);
struct BrmSink;    // an open response-bispectrum export file (bsa_brmfile.cu)

// Sampled grid points of the E-form contraction: slot[i1 + nf i2] = row in sF / sR
// ([nslot][nm^3] FP64, device) of grid point (i1, i2), or -1.
struct ESample {
    const int *slot;
    double *sF, *sR;
    int nslot;
};

struct Engine {
    Inputs in;
    Settings set;
    bool inited = false, halted = false, derived_ok = false, dev_uploaded = false;
    std::string last_error;
    int precision = 0;          // BSA_PREC_FP64
    bool classic_trunc = true;  // S(f1+f2) beyond the classic grid reads zero
    int shard_r0 = 0, shard_r1 = -1;  // classic grid rows evaluated (-1: to the end)
    int cls_shard = 0, cls_shards = 1;  // bsa_gpu_setClassicShard: this shard of cls_shards
    // POD truncation requests (bsa_setPODTruncationThreshold / bsa_setPODNOfModesKept)
    std::vector<std::vector<int>> own_i;     // arrays read by bsa_loadInputFiles (owned here)
    std::vector<std::vector<double>> own_d;
    bool classic_sym = false;   // bsa_gpu_setClassicSymmetry: evaluate half the Classic grid
    bool use_e_form = true;     // bsa_gpu_setClassicForm: E form of the split contraction where it applies
    int wait_test_tile1 = 0;    // bsa_gpu_setWaitTest: tile + 1 whose ready signal CTA 0 omits (0 = off)
    bool msh_graphs = true;     // bsa_gpu_setMesherGraphs: each Mesher zone pass as one CUDA graph
    bool msh_dev_expand = true; // bsa_gpu_setMesherExpansion: zone passes expanded on the device
    double msh_pass_bytes = 0.0; // bsa_gpu_setMesherPassBytes: device bytes of one zone pass (0: default)
    // Mesher controls (BsaLibData.F90:219-233, 273): delta validation, BFM multi-level
    // refinement, background peak restricted to the first direction, diagonal-crest scheme
    bool validate_deltas = true, bfm_mlr = true, bkg_restrict = false, premesh_diag_crest = false,
         premesh_mode_base = false;
    bsa_brm_export_fn export_fn = nullptr;  // bsa_setBispExportCallback
    void *export_user = nullptr;
    // bsa_enableVisualMode / bsa_setVisualIndexes / bsa_setBRMExportDefaultMode (bsa_brmfile.cu)
    bool visual = false, visual_modal = true;
    int visual_idx[3] = {1, 1, 1};
    int brm_export_mode = 0;
    BrmSink *brm_sink = nullptr;
    double pod_trunc_lim = 0.0;
    int pod_nmodes = 0;
    // The Mesher's POD form truncates only when one of the two was set to a value that
    // drops modes (BsaLibImpl.F90:97-115, 480); the default keeps every POD mode.
    bool pod_truncates() const {
        if (set.svd != 1 || set.onlyd != 0) return false;
        return (pod_trunc_lim > 0.0 && pod_trunc_lim != 1.0) || (pod_nmodes > 0 && pod_nmodes < in.nnl);
    }

    // derived (validate)
    std::vector<int> modes;
    int nme = 0, K = 0;
    std::vector<double> phitc, hL, hQ, hM, hK, hC;
    std::vector<double> hCoh;          // coherence bases c_ij [comp][i][j]; log c formed on the device
    std::vector<double> hWd3, hWd2;  // diagonal-only weights Q L^2 and L^2, [k][m]
    std::vector<float> hL32;         // FP32 copy of L for the split-precision A(f) table
    std::vector<PsdNode> hPsd;

    // device
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr;
    DevBuf dL, dQ, dLogc, dPsdPar, dFrfM, dFrfK, dFrfC, dFreq, dS, dA, dPartF, dPartR, dOut, dPsdF, dWf, dPts,
        dPtsD, dBF, dBR, dMixA, dMixB, dMixH, dMixPart, dA32, dZones, dZidx, dWd3, dWd2, dMshT, dMshIdx, dLogc32, dL32,
        dPod, dFlag, dSlot, dHash, dCptr, dCq;

    // stats
    double last_ms = 0, last_ms_contraction = 0, last_ms_gemm = 0, last_points = 0;
    double h2d = 0, d2h = 0;
    int kernels = 0;
    int graph_launches = 0;     // CUDA graphs launched by the last run
    cudaEvent_t evg0 = nullptr, evg1 = nullptr;

    int fail(int code, const char *fmt, ...);
    int cuda_fail(cudaError_t e, const char *what);
    void reset_inputs();
    void free_device();
    int ensure_stream();
    int validate();
    int upload_problem();
    FrfPar frf() const;
    // msh: the table serves the Mesher functions, whose POD form may be truncated
    int build_atable(const std::vector<double> &freqs, bool fp32 = false, bool msh = false);
    int pod_atable(const std::vector<double> &freqs, bool fp32);
    int build_psd(const std::vector<double> &freqs);
    int build_psd_dev(int nf, bool fp32 = false);  // the nf frequencies already in dFreq
    int build_atable_dev(int nf, bool fp32);   // the same, A table (not the truncated POD form)
    // dimM_psd_ / dimM_bisp_ (src/bsa/BsaLibImpl.F90:313-355): nm / nm for the diagonal-only
    // spectra, nm^2 / nm^3 otherwise.
    long long dim_psd() const { return set.onlyd ? nme : (long long)nme * nme; }
    long long dim_bisp() const { return set.onlyd ? nme : (long long)nme * nme * nme; }
    int classic_grid(std::vector<double> &f);
    int run_classic(double *m2mf, double *m2mr, double *m2o2mr, double *m3mf, double *m3mr, double *bf_host,
                    double *br_host, std::vector<double> *grid_out);
    int classic_export(PointSrc ps, const std::vector<double> &f, double *m3mf, double *m3mr);
    int contract(const PointSrc &ps, long long npts, double *m3mf, double *m3mr, double *bf_host, double *br_host);
    int contract_mixed(const PointSrc &ps, long long npts, double *m3mf, double *m3mr);
    int contract_e(const PointSrc &ps, double *m3mf, double *m3mr, const ESample *smp = nullptr);  // bsa_classic_e.cu
    // bsa_gpu_clsBispectraAt: Classic bispectra at listed grid points in the selected precision
    int classic_points(const int *i1, const int *i2, long long npts, double *bf, double *br);
    int contract_diag(const PointSrc &ps, long long npts, int msh_form, double *m3mf, double *m3mr,
                      double *bf_host, double *br_host);
    int run_points(const double *fi, const double *fj, const double *w, double wuniform, long long npts,
                   double *m3mf, double *m3mr, double *bfm, double *brm,
                   const std::vector<ZoneDev> *zones = nullptr, const int *zid = nullptr, const int *zi = nullptr,
                   const int *zj = nullptr, const long long *cptr = nullptr, const double *cq = nullptr);
    int run_zones(const std::vector<ZoneDev> &zones, double *m3mf, double *m3mr, double *npts);
    int run_zones_fp64(const std::vector<ZoneDev> &zones, double *m3mf, double *m3mr, double *npts);
    int run_zones_mixed(const std::vector<ZoneDev> &zones, double *m3mf, double *m3mr, double *npts,
                        double *zdiag = nullptr);
    int msh_mixed_batch(const std::vector<ZoneDev> &zones, std::vector<double> &accF, std::vector<double> &accR,
                        float &ms_gemm, float &ms_all, double *zdiag);
    // the pre-mesh layout: rectangles (zones, policy, whether the walk exchanges the start
    // point's coordinates), triangles, and the dump order (k >= 0: rectangle k, k < 0:
    // triangle -k - 1)
    int mesher_zones(std::vector<ZoneDev> &zones, std::vector<int> &policy, std::vector<TriDump> *tris = nullptr,
                     std::vector<int> *order = nullptr, std::vector<unsigned char> *swapped = nullptr);
    int run_mesher(double *m3mf, double *m3mr);
    int run_triangles(const std::vector<TriDump> &tris, double *m3mf, double *m3mr, double *npts);
    int zones_export(const std::vector<ZoneDev> &zones, const std::vector<TriDump> &tris, const std::vector<int> &order,
                     const std::vector<unsigned char> &swapped);
    // response-bispectrum export files (bsa_brmfile.cu); emit_brm also feeds the callback
    bool brm_file_wanted(bool classic) const;
    int brm_file_open(bool classic, int nzones);
    int brm_file_zone(int id, int nI, int nJ);
    int emit_brm(int npts, const double *f1, const double *f2, const double *brm);
    int brm_file_close(long long total);
    int br_decomp(const double *m2mf, double *bkg, double *res);
    int modal_recomb(const double *m2mr, const double *m3mr, const double *m2o2mr, double *const *outs);
    int batch_add(int *id);
    void batch_install(const BatchCase &c);
    int batch_run(double *m3mf, double *m3mr, double *m2mr, double *case_ms, double *total_ms);
};

Engine &eng();

// A zone of the C-ABI as the device zone record (lattice steps in rad/s for the weights).
ZoneDev zone_from_abi(const bsa_zone &z);

// Host vector -> device buffer on the engine's stream (counted in the H2D statistics).
template <class T>
inline cudaError_t upload(DevBuf &b, const std::vector<T> &v, cudaStream_t st) {
    cudaError_t e = b.reserve(sizeof(T) * v.size());
    if (e != cudaSuccess || v.empty()) return e;
    eng().h2d += (double)(sizeof(T) * v.size());
    return cudaMemcpyAsync(b.p, v.data(), sizeof(T) * v.size(), cudaMemcpyHostToDevice, st);
}

}  // namespace bsa
