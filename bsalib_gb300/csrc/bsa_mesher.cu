// bsa_mesher.cu -- the Mesher analysis: zone layout on the host, all zones evaluated in one
// batched device pass (the FP64 contraction over every zone's BFM lattice points, with the
// bilinear BRM neighbourhood and the trapezoid zone weights in its epilogue).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/bsa_gpu.h"
#include "bsa_engine.cuh"

namespace bsa {

namespace {

// MPolicy ids and the BRM interpolation factors of MPolicy_fromID
// (src/bsa/meshing/policy/MPolicy.F90:34-43, 130-168).
enum { kPolPrePeak1 = 3, kPolPrePeak2 = 4, kPolPeak = 5, kPolBasin = 7, kPolPadExtern = 9 };

int brm_factor(int pol) {
    switch (pol) {
    case kPolPeak: return 4;
    case kPolPrePeak1:
    case kPolPrePeak2: return 2;
    default: return 2;
    }
}

// Lattice spacing of a 1-D interval relative to the background-zone spacing: the delta
// factors of MPolicy_fromID (PEAK 1, PRE_PEAK 2, external padding 8).
double delta_factor(int pol) {
    switch (pol) {
    case kPolPeak: return 1.0;
    case kPolPadExtern: return 8.0;
    default: return 2.0;
    }
}

struct Interval {
    double a, b;
    int pol;
};

}  // namespace

// Zone layout.  Restates prefetchZoneLimits_ (BsaMesherImpl.F90:1638-1859) with
// getActualPeakZoneExtensionLimits_ (:1864-1890) for the 1-D frontiers of the resonant peak
// zones, the background peak zone of PreMesh (:266-420; width max(U/L) * bkg_area_ext,
// bkg_base_rfmnt points per side) and the extension to max(natf) * max_area_ext
// (getMaxSpaceExtension_, :1626-1631).  The 2-D zones are the tensor product of those
// intervals on both axes (rectangular zones only; the reference's rotated crest and
// triangular zones are not generated).
int Engine::mesher_zones(std::vector<ZoneDev> &zones, std::vector<int> &policy) {
    int rc = validate();
    if (rc) return rc;
    if (set.bispsym != 0) return fail(BSA_ERR_UNSUPPORTED, "Mesher with spatial symmetry %d is not on this path", set.bispsym);
    if (!in.natf || !in.xsi) return fail(BSA_ERR_STATE, "natural frequencies / damping not set");
    if (!in.ubref) return fail(BSA_ERR_STATE, "zone mean wind speeds not set");
    if (set.bkgrfmt < 2) return fail(BSA_ERR_ARG, "background zone refinement must be >= 2");
    // background peak width: max over components of 1 / max_zones(L(c, 1, z) / Uref(z))
    // (validateAll_, BsaLibImpl.F90:503-518; computeBKGPeakWidths, StructureImpl.F90:225-260;
    // restricted to the first direction as bsa_setMaxBkgPeakRestriction(.true.))
    double bkgw = 0.0;
    for (int c = 0; c < 3; ++c) {
        double mx = 0.0;
        for (int z = 0; z < in.nz; ++z) {
            const double u = in.ubref[z];
            if (u != 0.0) mx = std::max(mx, in.L[(size_t)c + 9 * (size_t)z] / u);
        }
        if (mx > 0.0) bkgw = std::max(bkgw, 1.0 / mx);
    }
    if (!(bkgw > 0.0)) return fail(BSA_ERR_ARG, "background peak width is zero");
    const double base = bkgw * set.bkgaext;
    const double half = base / 2.0;
    const double d0 = base / (set.bkgrfmt - 1);

    // peak zone frontiers of the kept modes, ascending natural frequency
    std::vector<std::pair<double, double>> pk;
    double fmaxn = 0.0;
    for (int m : modes) {
        const double f = in.natf[m - 1], ext = in.xsi[m - 1] * f * set.genpaext;
        pk.push_back({f - ext, f + ext});
        fmaxn = std::max(fmaxn, f);
    }
    std::sort(pk.begin(), pk.end());
    const int NM = (int)pk.size();
    std::vector<double> lim;
    std::vector<int> pol;
    int skip = 0;
    while (skip < NM && pk[skip].second <= half) ++skip;
    if (skip < NM) {
        if (half < pk[skip].first) {
            lim = {pk[skip].first, pk[skip].second};
            pol = {kPolPrePeak1, kPolPeak};
        } else {
            lim = {pk[skip].second};
            pol = {kPolPeak};
        }
        for (int im = skip + 1; im < NM; ++im) {
            const double BF = pk[im].first, FF = pk[im].second;
            const int NL = (int)lim.size();
            if (BF < lim[NL - 1]) {
                if (NL == 2 && BF <= lim[NL - 2]) {
                    lim[NL - 2] = BF;
                    pol[NL - 2] = kPolPrePeak2;
                }
                lim[NL - 1] = FF;
                pol[NL - 1] = kPolPeak;
            } else {
                lim.push_back(BF);
                pol.push_back(kPolPrePeak2);
                lim.push_back(FF);
                pol.push_back(kPolPeak);
            }
        }
        lim.push_back(lim.back() + base * std::sqrt(2.0) / 4.0);  // maxF (PreMesh)
        pol.push_back(kPolPrePeak2);
    }
    const double max_ext = fmaxn * set.maxaext;
    if (!lim.empty() && max_ext > lim.back()) {
        lim.push_back(max_ext);
        pol.push_back(kPolPadExtern);
    }
    // 1-D intervals on one axis, mirrored: [-..., -half] ... [-half, half] ... [half, ...]
    std::vector<Interval> pos;
    double a = half;
    for (size_t k = 0; k < lim.size(); ++k) {
        if (lim[k] > a) pos.push_back({a, lim[k], pol[k]});
        a = std::max(a, lim[k]);
    }
    std::vector<Interval> axis;
    for (int k = (int)pos.size() - 1; k >= 0; --k) axis.push_back({-pos[k].b, -pos[k].a, pos[k].pol});
    const int center = (int)axis.size();
    axis.push_back({-half, half, kPolPeak});
    for (auto &iv : pos) axis.push_back(iv);
    auto npoints = [&](int k) {
        if (k == center) return set.bkgrfmt;
        const double len = axis[k].b - axis[k].a, dl = d0 * delta_factor(axis[k].pol);
        return std::max(2, (int)std::ceil(len / dl - 1e-9) + 1);
    };
    zones.clear();
    policy.clear();
    for (int ki = 0; ki < (int)axis.size(); ++ki)
        for (int kj = 0; kj < (int)axis.size(); ++kj) {
            const Interval &X = axis[ki], &Y = axis[kj];
            ZoneDev z{};
            z.ni = npoints(ki);
            z.nj = npoints(kj);
            z.fi0 = X.a;
            z.fj0 = Y.a;
            z.dIi = (X.b - X.a) / (z.ni - 1);
            z.dIj = 0.0;
            z.dJi = 0.0;
            z.dJj = (Y.b - Y.a) / (z.nj - 1);
            z.Fi = brm_factor(X.pol);
            z.Fj = brm_factor(Y.pol);
            z.wI = std::fabs(z.dIi) * kPi2;
            z.wJ = std::fabs(z.dJj) * kPi2;
            z.sym = 1.0;
            zones.push_back(z);
            const int p = (ki == center && kj == center) ? kPolPeak
                          : (X.pol == kPolPeak || Y.pol == kPolPeak) ? kPolPeak
                          : (X.pol == kPolPadExtern || Y.pol == kPolPadExtern) ? kPolPadExtern
                                                                                : kPolBasin;
            policy.push_back(p);
        }
    return BSA_OK;
}

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
    return run_zones(zones, m3mf, m3mr, nullptr);
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
