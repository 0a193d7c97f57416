// bsa_mesher.cu -- the Mesher analysis: the zone layout (bsa_premesh.cu), then all zones
// evaluated in one batched device pass (the FP64 contraction over every zone's BFM lattice
// points, with the bilinear BRM neighbourhood and the trapezoid zone weights in its epilogue).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/bsa_gpu.h"
#include "bsa_engine.cuh"

namespace bsa {

// Zone integration in the precision selected by bsa_gpu_setPrecision: the split-precision
// path evaluates the axis-aligned zones on the tensor cores (bsa_msh_mixed.cu); the
// diagonal-only spectra and the FP64 setting use the FP64 point kernel.
int Engine::run_zones(const std::vector<ZoneDev> &zones, double *m3mf, double *m3mr, double *npts) {
    if (precision == BSA_PREC_BF16X3 && !set.onlyd) return run_zones_mixed(zones, m3mf, m3mr, npts);
    return run_zones_fp64(zones, m3mf, m3mr, npts);
}

// Every zone's BFM lattice points in one point list; m3mf weights are the trapezoid
// weights of the BFM lattice, the BRM lattice is handled in the kernel epilogue.
int Engine::run_zones_fp64(const std::vector<ZoneDev> &zones, double *m3mf, double *m3mr, double *npts) {
    size_t n = 0;
    double nbrm = 0.0;
    for (const ZoneDev &z : zones) {
        if (z.ni < 2 || z.nj < 2 || z.Fi < 1 || z.Fj < 1)
            return fail(BSA_ERR_ARG, "zone lattice needs ni, nj >= 2 and Fi, Fj >= 1");
        n += (size_t)z.ni * z.nj;
        nbrm += (double)((z.ni - 1) * z.Fi + 1) * ((z.nj - 1) * z.Fj + 1);
    }
    if (n == 0) return fail(BSA_ERR_ARG, "empty zone list");
    if (n > (size_t)0x7fffffff) return fail(BSA_ERR_ARG, "too many zone points");
    std::vector<double> f1(n), f2(n), w(n);
    std::vector<int> zid(n), zi(n), zj(n);
    size_t p = 0;
    for (size_t k = 0; k < zones.size(); ++k) {
        const ZoneDev &z = zones[k];
        for (int i = 0; i < z.ni; ++i)
            for (int j = 0; j < z.nj; ++j, ++p) {
                f1[p] = z.fi0 + i * z.dIi + j * z.dJi;
                f2[p] = z.fj0 + i * z.dIj + j * z.dJj;
                const double ti = (i == 0 || i == z.ni - 1) ? 0.5 : 1.0, tj = (j == 0 || j == z.nj - 1) ? 0.5 : 1.0;
                w[p] = z.sym * z.wI * z.wJ * ti * tj;
                zid[p] = (int)k;
                zi[p] = i;
                zj[p] = j;
            }
    }
    int rc = run_points(f1.data(), f2.data(), w.data(), 0.0, (long long)n, m3mf, m3mr, nullptr, nullptr, &zones,
                        zid.data(), zi.data(), zj.data());
    if (rc) return rc;
    last_points = nbrm;
    if (npts) {
        npts[0] = (double)n;
        npts[1] = nbrm;
    }
    return BSA_OK;
}

ZoneDev zone_from_abi(const bsa_zone &z) {
    ZoneDev d;
    d.fi0 = z.fi0; d.fj0 = z.fj0; d.dIi = z.dIi; d.dIj = z.dIj; d.dJi = z.dJi; d.dJj = z.dJj;
    d.ni = z.ni; d.nj = z.nj; d.Fi = z.Fi; d.Fj = z.Fj; d.sym = z.sym;
    d.wI = std::sqrt(z.dIi * z.dIi + z.dIj * z.dIj) * kPi2;
    d.wJ = std::sqrt(z.dJi * z.dJi + z.dJj * z.dJj) * kPi2;
    return d;
}

int Engine::run_mesher(double *m3mf, double *m3mr) {
    std::vector<ZoneDev> zones;
    std::vector<int> pol;
    int rc = mesher_zones(zones, pol);
    if (rc) return rc;
    if ((rc = run_zones(zones, m3mf, m3mr, nullptr)) || !(export_fn || brm_file_wanted(false))) return rc;
    const double pts = last_points;
    const float ms = last_ms;
    rc = zones_export(zones);
    last_points = pts;
    last_ms = ms;
    return rc;
}

// The Mesher's response-bispectrum export (the post-mesh interpolation hands every BRM
// lattice point of a zone to write_brm_fptr_, zones/_shared_poly2d.fi:1040-1210; the callback
// is set by bsa_setBispExportCallback, BsaLibImpl.F90:1809-1816).  Per zone: the force
// bispectra at its BFM lattice from the FP64 point path, then at every BRM lattice point the
// bilinear interpolation of the BFM values at the corners of its cell (the weights the zone
// integration uses) times Re[H_m(w1) H_n(w2) conj H_o(w1 + w2)] at the point.  One callback
// per zone, points i fastest then j, brm laid out [npts][dim_bisp].
int Engine::zones_export(const std::vector<ZoneDev> &zones) {
    const long long nb = dim_bisp();
    const int nm = nme;
    const bool diag = set.onlyd != 0;
    std::vector<double> bfm, brm, f1, f2, pi, pj, mf(nb), mr(nb), H(6 * (size_t)nm);
    int rc0 = brm_file_open(false, (int)zones.size());
    if (rc0) return rc0;
    long long total = 0;
    for (const ZoneDev &z : zones) {
        if (z.ni < 2 || z.nj < 2 || z.Fi < 1 || z.Fj < 1)
            return fail(BSA_ERR_ARG, "zone lattice needs ni, nj >= 2 and Fi, Fj >= 1");
        const int n = z.ni * z.nj;
        pi.resize(n);
        pj.resize(n);
        for (int i = 0; i < z.ni; ++i)
            for (int j = 0; j < z.nj; ++j) {
                pi[(size_t)i * z.nj + j] = z.fi0 + i * z.dIi + j * z.dJi;
                pj[(size_t)i * z.nj + j] = z.fj0 + i * z.dIj + j * z.dJj;
            }
        bfm.resize((size_t)n * nb);
        int rc = run_points(pi.data(), pj.data(), nullptr, 0.0, n, mf.data(), mr.data(), bfm.data(), nullptr, nullptr,
                            nullptr, nullptr, nullptr);
        if (rc) return rc;
        const int NI = (z.ni - 1) * z.Fi + 1, NJ = (z.nj - 1) * z.Fj + 1;
        const size_t nq = (size_t)NI * NJ;
        if (nq * (size_t)nb > ((size_t)1 << 31)) return fail(BSA_ERR_ARG, "zone export block too large");
        brm.resize(nq * nb);
        f1.resize(nq);
        f2.resize(nq);
        for (int qj = 0; qj < NJ; ++qj)
            for (int qi = 0; qi < NI; ++qi) {
                const size_t q = (size_t)qj * NI + qi;
                const double a = (double)qi / z.Fi, b = (double)qj / z.Fj;
                const double v1 = z.fi0 + a * z.dIi + b * z.dJi, v2 = z.fj0 + a * z.dIj + b * z.dJj;
                f1[q] = v1;
                f2[q] = v2;
                // cell corners and their bilinear weights (one corner on a lattice line)
                const int i0 = qi / z.Fi, j0 = qj / z.Fj;
                const double li = (double)(qi % z.Fi) / z.Fi, lj = (double)(qj % z.Fj) / z.Fj;
                const int i1 = li > 0.0 ? i0 + 1 : i0, j1 = lj > 0.0 ? j0 + 1 : j0;
                const double *B00 = bfm.data() + ((size_t)i0 * z.nj + j0) * nb;
                const double *B10 = bfm.data() + ((size_t)i1 * z.nj + j0) * nb;
                const double *B01 = bfm.data() + ((size_t)i0 * z.nj + j1) * nb;
                const double *B11 = bfm.data() + ((size_t)i1 * z.nj + j1) * nb;
                const double c00 = (1.0 - li) * (1.0 - lj), c10 = li * (1.0 - lj), c01 = (1.0 - li) * lj, c11 = li * lj;
                for (int m = 0; m < nm; ++m) {
                    frf_eval(hM[m], hK[m], hC[m], v1 * kPi2, H[2 * m], H[2 * m + 1]);
                    frf_eval(hM[m], hK[m], hC[m], v2 * kPi2, H[2 * nm + 2 * m], H[2 * nm + 2 * m + 1]);
                    frf_eval(hM[m], hK[m], hC[m], (v1 + v2) * kPi2, H[4 * nm + 2 * m], H[4 * nm + 2 * m + 1]);
                }
                double *out = brm.data() + q * nb;
                for (long long x = 0; x < nb; ++x) {
                    const int m = diag ? (int)x : (int)(x % nm);
                    const int nn = diag ? (int)x : (int)((x / nm) % nm);
                    const int o = diag ? (int)x : (int)(x / ((long long)nm * nm));
                    const double h2r = H[2 * nm + 2 * nn], h2i = H[2 * nm + 2 * nn + 1];
                    const double h3r = H[4 * nm + 2 * o], h3i = H[4 * nm + 2 * o + 1];
                    const double cr = h2r * h3r + h2i * h3i, ci = h2i * h3r - h2r * h3i;  // H_n conj H_o
                    const double fr = H[2 * m] * cr - H[2 * m + 1] * ci;
                    out[x] = fr * (c00 * B00[x] + c10 * B10[x] + c01 * B01[x] + c11 * B11[x]);
                }
            }
        if ((rc = brm_file_zone(1, NI, NJ)) || (rc = emit_brm((int)nq, f1.data(), f2.data(), brm.data()))) {
            brm_file_close(-1);
            return rc;
        }
        total += (long long)nq;
    }
    if ((rc0 = brm_file_close(total))) return rc0;
    return BSA_OK;
}

}  // namespace bsa

using bsa::eng;

extern "C" {

int bsa_gpu_mshZones(const bsa_zone *zones, int nz, double *m3mf, double *m3mr, double *npts) {
    bsa::Engine &E = eng();
    if (E.halted) return BSA_ERR_STATE;
    if (!zones || nz <= 0) return E.fail(BSA_ERR_ARG, "empty zone list");
    std::vector<bsa::ZoneDev> zd(nz);
    for (int k = 0; k < nz; ++k) zd[k] = bsa::zone_from_abi(zones[k]);
    return E.run_zones(zd, m3mf, m3mr, npts);
}

int bsa_gpu_mshGenerateZones(bsa_zone *zones, int cap, int *nz) {
    bsa::Engine &E = eng();
    if (E.halted) return BSA_ERR_STATE;
    std::vector<bsa::ZoneDev> zd;
    std::vector<int> pol;
    int rc = E.mesher_zones(zd, pol);
    if (rc) return rc;
    if (nz) *nz = (int)zd.size();
    for (int k = 0; k < (int)zd.size() && k < cap && zones; ++k) {
        const bsa::ZoneDev &d = zd[k];
        bsa_zone &z = zones[k];
        z.fi0 = d.fi0; z.fj0 = d.fj0; z.dIi = d.dIi; z.dIj = d.dIj; z.dJi = d.dJi; z.dJj = d.dJj;
        z.ni = d.ni; z.nj = d.nj; z.Fi = d.Fi; z.Fj = d.Fj; z.sym = d.sym; z.policy = pol[k];
    }
    return BSA_OK;
}

}  // extern "C"
