// bsa_io.cu -- the standalone driver's input files, read natively: bsa.bsadata (settings,
// getBsaData, app/bsa.F90:877-930) and bsa.extdata (structure, wind and modal data,
// getExtData, app/bsa.F90:696-871, written by generateBSAInputFiles_,
// src/bsa/BsaLibImpl.F90:2065-2155), then the driver's library controls and setter sequence
// (app/bsa.F90:544-606).  The arrays are owned by the library until bsa_Finalise.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iterator>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/bsa_gpu.h"
#include "bsa_engine.cuh"

namespace bsa {
namespace {

struct Stream {
    std::vector<char> buf;
    size_t pos = 0;
    bool ok = true;
    int i32() {
        int32_t v = 0;
        if (pos + 4 > buf.size()) { ok = false; return 0; }
        std::memcpy(&v, buf.data() + pos, 4);  // little-endian on every target of this library
        pos += 4;
        return v;
    }
    double f64() {
        double v = 0.0;
        if (pos + 8 > buf.size()) { ok = false; return 0.0; }
        std::memcpy(&v, buf.data() + pos, 8);
        pos += 8;
        return v;
    }
    std::vector<int> ivec(long long n) {
        std::vector<int> v(n > 0 ? n : 0);
        for (auto &x : v) x = i32();
        return v;
    }
    std::vector<double> dvec(long long n) {
        std::vector<double> v(n > 0 ? n : 0);
        for (auto &x : v) x = f64();
        return v;
    }
};

// Fortran list-directed reals may carry a d / D exponent.
double parse_real(const std::string &s) {
    std::string t = s;
    for (char &c : t)
        if (c == 'd' || c == 'D') c = 'e';
    return std::strtod(t.c_str(), nullptr);
}

}  // namespace
}  // namespace bsa

using bsa::eng;

extern "C" int bsa_loadInputFiles(const char *dir) {
    bsa::Engine &E = eng();
    if (E.halted) return BSA_ERR_STATE;
    if (!E.inited) return E.fail(BSA_ERR_STATE, "bsa_Init was not called");
    if (!dir) return E.fail(BSA_ERR_ARG, "no directory");
    const std::string d(dir);
    // ---------------- bsa.bsadata ----------------
    std::ifstream fs(d + "/bsa.bsadata");
    if (!fs) return E.fail(BSA_ERR_ARG, "cannot open %s/bsa.bsadata", dir);
    std::vector<std::string> lines;
    for (std::string ln; std::getline(fs, ln);) lines.push_back(ln);
    size_t li = 0;
    bool bad = false;
    auto next = [&]() -> std::string {
        if (li >= lines.size()) { bad = true; return "0"; }
        std::istringstream is(lines[li++]);
        std::string tok;
        is >> tok;
        return tok.empty() ? std::string("0") : tok;
    };
    auto label = [&]() { next(); };
    auto rint = [&]() { return (int)std::strtol(next().c_str(), nullptr, 10); };
    auto rflt = [&]() { return bsa::parse_real(next()); };
    label();
    const int suban = rint(), vers = rint(), defsc = rint(), ipsd = rint(), ibisp = rint(), onlyd = rint();
    const int bispsym = rint(), sym3d = rint(), test = rint();
    label();
    const int scalar = rint(), nfreqs = rint();
    const double df = rflt();
    label();
    const int svd = rint(), bkgrfmt = rint();
    const double bkgaext = rflt(), genpaext = rflt(), maxaext = rflt();
    const int fcov = rint(), dumpmod = rint();
    label();
    const int ndirs = rint();
    std::vector<int> dirs(ndirs > 0 && ndirs <= 3 ? ndirs : 0);
    for (auto &x : dirs) x = rint();
    label();
    const int ntc = rint();
    std::vector<int> tc(ntc > 0 && ntc <= 3 ? ntc : 0);
    for (auto &x : tc) x = rint();
    if (bad || dirs.empty() || tc.empty()) return E.fail(BSA_ERR_ARG, "bsa.bsadata is truncated or malformed");
    // ---------------- bsa.extdata ----------------
    std::ifstream fx(d + "/bsa.extdata", std::ios::binary);
    if (!fx) return E.fail(BSA_ERR_ARG, "cannot open %s/bsa.extdata", dir);
    bsa::Stream S;
    S.buf.assign(std::istreambuf_iterator<char>(fx), std::istreambuf_iterator<char>());
    const int nn = S.i32(), nlibs = S.i32(), nnl = S.i32(), nlibsl = S.i32();
    if (!S.ok || nn <= 0 || nlibs <= 0 || nnl <= 0 || nlibsl <= 0 || nnl > nn)
        return E.fail(BSA_ERR_ARG, "bsa.extdata: invalid dimensions");
    auto n_load = S.ivec(nnl);
    auto libs_load = S.ivec(nlibsl);
    auto coords = S.dvec(3LL * nn);
    const int i_varu = S.i32(), psd_type = S.i32(), i_vert = S.i32(), ndegw = S.i32();
    const double air = S.f64();
    auto rot = S.dvec(9);
    const int nz = S.i32();
    if (!S.ok || nz <= 0 || ndegw < 0) return E.fail(BSA_ERR_ARG, "bsa.extdata: invalid wind-zone data");
    auto zref = S.dvec(nz), ubref = S.dvec(nz), L = S.dvec(9LL * nz), sigma = S.dvec(3LL * nz);
    auto corrC = S.dvec(9LL * nz), corrEx = S.dvec(9LL * nz), lims = S.dvec(nz + 1LL), rotz = S.dvec(9LL * nz);
    auto incang = S.dvec(nz);
    auto wz = S.ivec(nn);
    auto walt = S.dvec(nn), unod = S.dvec(nn);
    const long long ncorr = ((long long)nn * nn + nn) / 2;
    auto corr = S.dvec(3 * ncorr);
    auto wfc = S.dvec((long long)nlibsl * (ndegw + 3) * nnl);
    const int ndofs = S.i32(), nm = S.i32();
    if (!S.ok || ndofs <= 0 || nm <= 0) return E.fail(BSA_ERR_ARG, "bsa.extdata: invalid modal dimensions");
    auto natf = S.dvec(nm), phi = S.dvec((long long)ndofs * nm), Mg = S.dvec(nm), Kg = S.dvec(nm);
    auto Cg = S.dvec((long long)nm * nm), xsi = S.dvec(nm);
    if (!S.ok) return E.fail(BSA_ERR_ARG, "bsa.extdata is truncated");
    if (S.pos != S.buf.size()) return E.fail(BSA_ERR_ARG, "bsa.extdata: %zu trailing bytes", S.buf.size() - S.pos);
    // ---------------- keep the arrays, then the driver's setter sequence ----------------
    E.own_i.clear();
    E.own_d.clear();
    auto I = [&](std::vector<int> &v) { E.own_i.push_back(std::move(v)); return E.own_i.back().data(); };
    auto D = [&](std::vector<double> &v) { E.own_d.push_back(std::move(v)); return E.own_d.back().data(); };
    E.own_i.reserve(8);
    E.own_d.reserve(24);
    int rc = BSA_OK;
#define CALL(x)                 \
    do {                        \
        if ((rc = (x))) return rc; \
    } while (0)
    // the driver's library controls (app/bsa.F90:544-552)
    CALL(bsa_doValidateZoneDeltas(0));
    CALL(bsa_setBfmMLR(0));
    CALL(bsa_setMaxBkgPeakRestriction(1));
    CALL(bsa_setPODNOfModesKept(0));
    if (suban) CALL(bsa_setAnalysisType(suban));
    if (vers) CALL(bsa_setVersion(vers));
    if (defsc) CALL(bsa_setScalingConv(defsc));
    CALL(bsa_setSpectraComputation(ipsd, ibisp));
    CALL(bsa_setSpectraExtension(onlyd));
    CALL(bsa_setSpatialSymmetry(bispsym));
    CALL(bsa_setSpectraSymmetries(sym3d));
    CALL(bsa_setTestMode(test));
    CALL(bsa_setupClassic(nfreqs, df));
    CALL(bsa_setClassicMode(scalar));
    CALL(bsa_setupMesher(svd, bkgrfmt, bkgaext, genpaext, maxaext, fcov, dumpmod));
    CALL(bsa_setWindDirections(I(dirs), ndirs));
    CALL(bsa_setWindTurbComps(I(tc), ntc));
    CALL(bsa_setTotalNOfNodes(nn));
    CALL(bsa_setNumOfNodalDOFs(nlibs));
    CALL(bsa_setLoadedNodes(I(n_load), nnl));
    CALL(bsa_setLoadedNodalDOFs(I(libs_load), nlibsl));
    CALL(bsa_setNodalCoords(nn, D(coords)));
    CALL(bsa_setWindVertProf(i_varu));
    CALL(bsa_setPSDType(psd_type));
    CALL(bsa_setWindAltDir(i_vert));
    CALL(bsa_setAirDensity(air));
    CALL(bsa_setWZMeanWindVel(D(ubref), nz));
    CALL(bsa_setWZRefAlt(D(zref), nz));
    CALL(bsa_setTurbWindScales(D(L), nz));
    CALL(bsa_setTurbWindSDT(D(sigma), nz));
    CALL(bsa_setNodalVel(D(unod), nn));
    CALL(bsa_setNodalWindZones(I(wz), nn));
    CALL(bsa_setNodalWindAltitudes(D(walt), nn));
    CALL(bsa_setSpatialNodalCorr(D(corr), ncorr));
    CALL(bsa_setWindFCoeffs(D(wfc), nlibsl, ndegw + 3, nnl));
    CALL(bsa_setModalInfo(ndofs, nm, D(phi), D(natf)));
    CALL(bsa_setModalMatrices(nm, D(Mg), D(Kg), D(Cg)));
    CALL(bsa_setTotDamping(D(xsi), nm));
#undef CALL
    (void)rot; (void)corrC; (void)corrEx; (void)lims; (void)rotz; (void)incang;
    return BSA_OK;
}
