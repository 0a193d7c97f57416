// bsa_bsacl.cu -- BsaCL's device offload ABI (BsaCL/include/bsacl.h:28-55) on top of the
// libbsagpu engine, so that a Fortran host built for BsaCL (BsaCL/BsaCL_Fortran/bsacl_c.F90)
// links against this library unchanged.
//
// Semantics kept from BsaCL/src/bsacl.c: Acquire* borrow host pointers, no copy happens
// before bsaclInitDeviceMemory; a failure halts the runtime (sticky) and later Acquire*
// calls become no-ops; bsaclRun writes the response third moments over the outer product
// of the acquired fi x fj lists, times the uniform influence dfi * dfj * 4 pi^2
// (bsacl.c:1544-1572).  Differences, by design: the full nodal triple sum is evaluated
// through the exact factorisation, per-zone sigma / L and coherence column tc are used
// (the reference kernel reads zone 1 and column 1 only, bsacl.cl:588-589, 631), and any
// number of loaded nodes is accepted (the reference CUDA kernel sizes its shared arrays
// for at most 4, bsacl.cl:509-514).
#include <cuda_runtime.h>

#include <vector>

#include "../../include/bsa_gpu.h"
#include "bsa_engine.cuh"

namespace {

struct ClState {
    bool init = false, devmem = false, halted = false;
    unsigned n_threads = 0;
    unsigned kernel_id = 2;
    int psdid = 0;
    double *phi = nullptr, *natf = nullptr;
    uint32_t ndofs = 0, nmodes = 0;
    double *Mg = nullptr, *Cg = nullptr, *Kg = nullptr;
    int *nodes = nullptr;
    uint32_t nnl = 0, nn = 0;
    int *modes = nullptr;
    uint32_t nme = 0;
    double *wfc = nullptr;
    uint32_t wfc_nn = 0, wfc_nl = 0, wfc_nd = 0;
    int *tc = nullptr;
    uint32_t ntc = 0;
    double *phitc = nullptr;
    uint32_t pt_nme = 0, pt_nnl = 0, pt_nd = 0;
    double *corr = nullptr;
    uint32_t ncorr = 0;
    double *unod = nullptr;
    int *wz = nullptr;
    double *L = nullptr, *sigma = nullptr;
    uint32_t nwz = 0;
    std::vector<const double *> fi, fj;
    std::vector<uint32_t> nfi, nfj;
};

ClState &cl() {
    static ClState s;
    return s;
}

int cl_abort(int code) {
    cl().halted = true;
    return code;
}

}  // namespace

extern "C" {

int bsaclInit(unsigned n_threads) {
    ClState &s = cl();
    if (s.halted) return BSA_ERR_STATE;
    if (n_threads == 0) return cl_abort(BSA_ERR_ARG);
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) return cl_abort(BSA_ERR_CUDA);
    s.n_threads = n_threads;
    s.fi.assign(n_threads, nullptr);
    s.fj.assign(n_threads, nullptr);
    s.nfi.assign(n_threads, 0);
    s.nfj.assign(n_threads, 0);
    s.init = true;
    return BSA_OK;
}

// Hands the acquired arrays to the engine (the reference copies them to the device here,
// bsacl.c:1099-1297).
int bsaclInitDeviceMemory(void) {
    ClState &s = cl();
    if (s.halted) return BSA_ERR_STATE;
    if (!s.init) return cl_abort(BSA_ERR_STATE);
    if (!s.phitc || !s.modes || !s.tc || !s.corr || !s.unod || !s.wz || !s.L || !s.sigma || !s.Mg || !s.Kg ||
        !s.Cg || !s.nodes)
        return cl_abort(BSA_ERR_STATE);
    bsa::Engine &E = bsa::eng();
    E.free_device();
    E.reset_inputs();
    E.halted = false;
    E.inited = true;
    bsa::Inputs &I = E.in;
    I.nn = (int)s.nn;
    I.nnl = (int)s.nnl;
    I.n_load = s.nodes;
    I.nm = (int)s.nmodes;
    I.phi = s.phi;
    I.natf = s.natf;
    I.Mg = s.Mg;
    I.Kg = s.Kg;
    I.Cg = s.Cg;
    I.psd_type = s.psdid ? s.psdid : 5;
    I.nz = (int)s.nwz;
    I.L = s.L;
    I.sigma = s.sigma;
    I.unod = s.unod;
    I.wz = s.wz;
    I.corr = s.corr;
    I.ncorr = s.ncorr;
    I.ext_phitc = s.phitc;
    I.ext_modes = s.modes;
    I.ext_nme = (int)s.pt_nme;
    I.ext_nnl = (int)s.pt_nnl;
    I.ext_nd = (int)s.pt_nd;
    E.set.tc.assign(s.tc, s.tc + s.ntc);
    int rc = E.upload_problem();
    if (rc) return cl_abort(rc);
    s.devmem = true;
    return BSA_OK;
}

int bsaclRun(unsigned i_thread, size_t dim, double *h_res) {
    ClState &s = cl();
    if (s.halted) return BSA_ERR_STATE;
    if (!s.init) {
        int rc = bsaclInit(1);
        if (rc) return rc;
    }
    if (!s.devmem) {
        int rc = bsaclInitDeviceMemory();
        if (rc) return rc;
    }
    if (i_thread >= s.n_threads) return cl_abort(BSA_ERR_ARG);
    if (!s.fi[i_thread] || !s.fj[i_thread] || s.nfi[i_thread] < 2 || s.nfj[i_thread] < 2)
        return cl_abort(BSA_ERR_STATE);
    bsa::Engine &E = bsa::eng();
    const size_t nm3 = (size_t)E.nme * E.nme * E.nme;
    if (dim != nm3 || !h_res) return cl_abort(BSA_ERR_ARG);
    const uint32_t ni = s.nfi[i_thread], nj = s.nfj[i_thread];
    const double *fi = s.fi[i_thread], *fj = s.fj[i_thread];
    std::vector<double> p1((size_t)ni * nj), p2((size_t)ni * nj);
    for (uint32_t j = 0; j < nj; ++j)
        for (uint32_t i = 0; i < ni; ++i) {
            p1[(size_t)j * ni + i] = fi[i];
            p2[(size_t)j * ni + i] = fj[j];
        }
    const double infl = (fi[1] - fi[0]) * (fj[1] - fj[0]) * 4.0 * bsa::kPi * bsa::kPi;
    int rc = E.run_points(p1.data(), p2.data(), nullptr, infl, (long long)ni * nj, nullptr, h_res, nullptr, nullptr);
    return rc ? cl_abort(rc) : BSA_OK;
}

int bsaclSetKernelID(unsigned kid) {
    if (cl().halted) return BSA_ERR_STATE;
    if (kid != 1 && kid != 2) return cl_abort(BSA_ERR_ARG);
    cl().kernel_id = kid;
    return BSA_OK;
}

#define CL_GUARD() \
    if (cl().halted) return
void bsaclAcquirePSDId(uint32_t psdid) { CL_GUARD(); cl().psdid = (int)psdid; }
void bsaclAcquireStructModMat(double *modmat, double *natf, uint32_t ndofs, uint32_t nmodes) {
    CL_GUARD();
    ClState &s = cl();
    s.phi = modmat; s.natf = natf; s.ndofs = ndofs; s.nmodes = nmodes;
}
void bsaclAcquireModalMatrices(double *Mg, double *Cg, double *Kg) {
    CL_GUARD();
    ClState &s = cl();
    s.Mg = Mg; s.Cg = Cg; s.Kg = Kg;
}
void bsaclAcquireLoadedNodesList(int *nodes_load, uint32_t nnodes_l) {
    CL_GUARD();
    cl().nodes = nodes_load;
    cl().nnl = nnodes_l;
}
void bsaclAcquireTotalNOfNodes(uint32_t nnodes_tot) { CL_GUARD(); cl().nn = nnodes_tot; }
void bsaclAcquireUsedModesList(int *modes, uint32_t nmodes_eff) {
    CL_GUARD();
    cl().modes = modes;
    cl().nme = nmodes_eff;
}
void bsaclAcquireWindCoeffs(double *wfc, uint32_t nnodes_l, uint32_t nlibs, uint32_t ndegw) {
    CL_GUARD();
    ClState &s = cl();
    s.wfc = wfc; s.wfc_nn = nnodes_l; s.wfc_nl = nlibs; s.wfc_nd = ndegw;
}
void bsaclAcquireTurbComponentsList(int *tc, uint32_t ntc) {
    CL_GUARD();
    cl().tc = tc;
    cl().ntc = ntc;
}
void bsaclAcquirePhiTimesCMat(double *phi_T_c, uint32_t nmodes_eff, uint32_t nnodes_l, uint32_t ndegw) {
    CL_GUARD();
    ClState &s = cl();
    s.phitc = phi_T_c; s.pt_nme = nmodes_eff; s.pt_nnl = nnodes_l; s.pt_nd = ndegw;
}
void bsaclAcquireNodalCorrelation(double *nod_corr, uint32_t nnod_corr) {
    CL_GUARD();
    cl().corr = nod_corr;
    cl().ncorr = nnod_corr;
}
void bsaclAcquireWindNodalVelocities(double *nod_vel) { CL_GUARD(); cl().unod = nod_vel; }
void bsaclAcquireWindNodalWindZones(int *nod_wz) { CL_GUARD(); cl().wz = nod_wz; }
void bsaclAcquireWindTurbScales(double *wt_scl, uint32_t nwz) {
    CL_GUARD();
    cl().L = wt_scl;
    cl().nwz = nwz;
}
void bsaclAcquireWindTurbStd(double *wt_std, uint32_t nwz) {
    CL_GUARD();
    cl().sigma = wt_std;
    cl().nwz = nwz;
}
void bsaclAcquireComputationFreqs(unsigned i_thread, uint32_t nfi, double *fi, uint32_t nfj, double *fj) {
    CL_GUARD();
    ClState &s = cl();
    if (!s.init) { cl_abort(BSA_ERR_STATE); return; }
    if (i_thread >= s.n_threads) { cl_abort(BSA_ERR_ARG); return; }
    s.nfi[i_thread] = nfi; s.fi[i_thread] = fi;
    s.nfj[i_thread] = nfj; s.fj[i_thread] = fj;
}
void bsaclAcquireBaseWindTurbPSD(double *S_uvw) { (void)S_uvw; /* deprecated in the reference */ }
void bsaclSetDeviceType(uint32_t itype) { (void)itype; /* one CUDA device */ }
void bsaclVerifyMaxAllocCondition(size_t idim, unsigned int *ican) {
    CL_GUARD();
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) { if (ican) *ican = 0; return; }
    if (ican) *ican = (idim * sizeof(double) <= fr) ? 1u : 0u;
}
void bsaclAbort(int ierr) { (void)ierr; cl().halted = true; }
void bsaclFinalise(void) {
    ClState &s = cl();
    s = ClState();
    bsa::Engine &E = bsa::eng();
    E.free_device();
    E.reset_inputs();
    E.halted = false;
    E.inited = false;
}

}  // extern "C"
