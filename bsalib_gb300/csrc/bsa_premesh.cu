// bsa_premesh.cu -- the Mesher's zone layout (pre-mesh) and each zone's post-mesh lattice,
// restated from BsaLib so that the Mesher evaluates the reference's zones.
//
// Pre-mesh (PreMesh, src/bsa/meshing/BsaMesherImpl.F90:266-1393): the background peak zone
// centred at the origin, the four crest bands along the axes (one zone per zone limit and a
// closing one), then in the default scheme the four quadrants as nested L-shapes (a diagonal
// square and two side strips per limit), in the diagonal-crest scheme (bsa_setPremeshScheme(1),
// :924-1279) padding rectangles over the NE / SW quadrants and triangles and rotated rectangles
// along the SE / NW diagonals (MTriangZone, zones/MTriangZoneImpl.F90), and, with full
// coverage, four external padding bands up to max(natf) * max_area_ext.  Zone limits, policies and interest modes come
// from prefetchZoneLimits_ (:1638-1859) over the peak extensions of
// getActualPeakZoneExtensionLimits_ (:1864-1890).  The geometry follows MRectZone
// (zones/MRectZoneImpl.F90), M2DPolygZone (zones/M2DPolygZone.F90) and MPoint
// (point/MPoint.F90), with one zone object reused from zone to zone as the reference does, so
// that state a call does not set carries over; each parallel direction loop of the reference
// starts from a fresh object (OpenMP firstprivate), and so does each loop here.
//
// Post-mesh (interpolateRZ_HTPC_v3, zones/_shared_poly2d.fi:470-900): the dumped zone (init
// point, rotation, bases, refinements, policy, interest-mode pointer) gets its deltas back from
// bases / (n - 1), its BFM lattice refined by the policy's BFM factors (multi-level
// refinement, bsa_setBfmMLR) and, with bsa_doValidateZoneDeltas, re-refined until its step
// resolves the narrowest peak of its interest modes (neither in visual mode); the BRM lattice
// refines the BFM one by the policy's BRM factors.  The result is the device zone record the
// integration kernels read: the lattice the walk evaluates, from the init point with its
// coordinates exchanged for rot in [pi/2, pi) and [3 pi/2, 2 pi).  Triangles leave as their
// dump with the policy's factors; their walk is bsa_triang.cu's.
//
// Settings of the reference's standalone driver (app/bsa.F90:544-552) differ from the library
// defaults used here: bsa_loadInputFiles applies the driver's (no delta validation, no BFM
// multi-level refinement, background peak restricted to the first direction).
#include <algorithm>
#include <cmath>
#include <vector>

#include "../../include/bsa_gpu.h"
#include "bsa_engine.cuh"

namespace bsa {
namespace premesh {

// _CONSTANTS.F90:196-209
const double PI = 4.0 * std::atan(1.0);
const double PId2 = PI / 2.0, PIt3d2 = PI * (3.0 / 2.0), PIt2 = PI * 2.0;
constexpr double MACHINE_PRECISION = 1e-12;

// MPolicy ids and MPolicy_fromID (policy/MPolicy.F90:34-43, 130-168)
enum { kNull = 0, kDef = 1, kConst = 2, kPrePeak1 = 3, kPrePeak2 = 4, kPeak = 5, kCrest = 6, kBasin = 7,
       kPadIntern = 8, kPadExtern = 9 };

struct Policy {
    int dfI = 0, dfJ = 0, bfm_i = 1, bfm_j = 1, brm_i = 1, brm_j = 1, nlevs = 0, id = kNull;
};

Policy policy(int id) {
    auto P = [](int a, int b, int c, int d, int e, int f, int g, int h) {
        Policy p;
        p.dfI = a; p.dfJ = b; p.bfm_i = c; p.bfm_j = d; p.brm_i = e; p.brm_j = f; p.nlevs = g; p.id = h;
        return p;
    };
    switch (id) {
    case kNull: return P(0, 0, 0, 0, 0, 0, 0, kNull);
    case kConst: return P(1, 1, 1, 1, 1, 1, 1, kConst);
    case kPrePeak1: return P(1, 4, 4, 4, 4, 2, 1, kPrePeak1);
    case kPrePeak2: return P(1, 8, 2, 2, 4, 2, 1, kPrePeak2);
    case kPeak: return P(1, 1, 4, 4, 4, 4, 1, kPeak);
    case kCrest: return P(1, 4, 4, 4, 4, 2, 1, kCrest);
    case kBasin: return P(1, 4, 2, 2, 2, 2, 1, kBasin);
    case kPadIntern: return P(4, 4, 1, 1, 2, 2, 1, kPadIntern);
    case kPadExtern: return P(8, 8, 1, 1, 2, 2, 1, kPadExtern);
    default: return P(2, 2, 2, 2, 2, 2, 1, kDef);
    }
}

constexpr int CODE_PRE_PEAK_OK = -1, CODE_PRE_PEAK_KO = -2;  // BsaLibData.F90:248-257

struct Pt {
    double fi = 0.0, fj = 0.0;
};

double distance(const Pt &a, const Pt &b) {  // getPointsDistance
    const double dx = std::fabs(a.fi - b.fi), dy = std::fabs(a.fj - b.fj);
    return std::sqrt(dx * dx + dy * dy);
}

// MPoint getNewPointFromDistAndRot (rotations in [0, 2 pi] here)
Pt from_dist_rot(const Pt &p, double dist, double rot) {
    double dI, dJ;
    if (rot < PId2) {
        dI = std::sin(rot);
        dJ = std::cos(rot);
    } else if (rot < PI) {
        const double ang = rot - PId2;
        dI = std::cos(ang);
        dJ = -std::sin(ang);
    } else if (rot < PIt3d2) {
        const double ang = rot - PI;
        dI = -std::sin(ang);
        dJ = -std::cos(ang);
    } else {
        const double ang = rot - PIt3d2;
        dI = -std::cos(ang);
        dJ = std::sin(ang);
    }
    return Pt{dI * dist + p.fi, dJ * dist + p.fj};
}

// A dumped zone: what post-mesh reads back (MRectZone dumpRZ and DumpZone).
struct Dumped {
    Pt I;
    double rot, baseI, baseJ;
    int ni, nj, pol, id_im;
};

struct Fail {
    const char *msg;
};

// MRectZone_t with the state the pre-mesh reads and writes.
struct RZ {
    Pt I, E;
    double rot = 0.0, baseI = 0.0, baseJ = 0.0, dI = 0.0, dJ = 0.0;
    int ni = 0, nj = 0, pol = kNull, id_im = 0;

    void setRotation(double r) {  // M2DPolygZone setRotation (r < 2 pi here)
        if (r >= PIt2) r -= std::floor(r / PIt2) * PIt2;
        rot = r;
    }
    bool aligned() const { return rot == 0.0 || rot == PId2 || rot == PI || rot == PIt3d2; }
    void deduceDeltas() {  // deduceDeltas_rect
        dI = baseI / (ni - 1);
        dJ = baseJ / (nj - 1);
    }
    // setRefinements(ni, nj, force): its force flag is a saved local in the reference
    // (M2DPolygZone.F90), so after the first forced call every call behaves as forced; *sticky
    // carries that state through one layout.
    void setRefinements(int n_i, int n_j, bool force, bool *sticky) {
        if (force) *sticky = true;
        if (*sticky) {
            ni = n_i;
            nj = n_j;
        } else {
            ni = n_i % 2 == 0 ? n_i + 1 : n_i;
            nj = n_j % 2 == 0 ? n_j + 1 : n_j;
        }
        deduceDeltas();
    }
    void setDeltas(double dfi, double dfj) {  // setDeltas(.., adapt=.true.) -> deduceRefinements
        dI = dfi;
        dJ = dfj;
        int si = (int)std::floor(baseI / dI), sj = (int)std::floor(baseJ / dJ);
        if (si % 2 != 0) ++si;
        if (sj % 2 != 0) ++sj;
        if (si == 0) si = 1;
        if (sj == 0) sj = 1;
        dI = baseI / si;
        dJ = baseJ / sj;
        ni = si + 1;
        nj = sj + 1;
    }
    void setIEpts(const Pt &p) {  // loc = 'i'
        double c, s, di = 0.0, dj = 0.0;
        if (rot < PId2) {
            c = std::cos(rot); s = std::sin(rot);
            di = baseI * c + baseJ * s;
            dj = baseJ * c - baseI * s;
        } else if (rot < PI) {
            const double a = rot - PId2;
            c = std::cos(a); s = std::sin(a);
            di = baseJ * c - baseI * s;
            dj = -(baseJ * s + baseI * c);
        } else if (rot < PIt3d2) {
            const double a = rot - PI;
            c = std::cos(a); s = std::sin(a);
            di = -(baseJ * s + baseI * c);
            dj = -baseJ * c + baseI * s;
        } else if (rot < PIt2) {
            const double a = rot - PIt3d2;
            c = std::cos(a); s = std::sin(a);
            di = -baseJ * c + baseI * s;
            dj = baseJ * s + baseI * c;
        }
        I = p;
        E = Pt{p.fi + di, p.fj + dj};
    }
    // define(pt, loc, base_i, base_j): 'c' centres the zone on pt, 'i' starts it there
    void define(const Pt &p, char loc, double bi, double bj) {
        baseI = bi;
        baseJ = bj;
        if (loc == 'c') {
            I = Pt{p.fi - bi / 2, p.fj - bj / 2};
            E = Pt{p.fi + bi / 2, p.fj + bj / 2};
        } else {
            setIEpts(p);
        }
    }
    Pt getA() const { return from_dist_rot(I, baseJ, rot); }
    Pt getB() const { return from_dist_rot(I, baseI, rot > PIt3d2 ? rot - PIt3d2 : rot + PId2); }

    // getOtherBase: the end point from the side point pt (B for base_dir 'i', A for 'j') and
    // the known end coordinate; the forms per (side, known coordinate, quadrant) as written.
    void otherBase(const Pt &pt, char base_dir, char known, double coord) {
        const double kd = std::fabs(known == 'i' ? coord - pt.fi : coord - pt.fj);
        double cd = 0.0;
        if (kd >= MACHINE_PRECISION) {
            int q;
            double r;
            if (rot < PId2) { q = 1; r = rot; }
            else if (rot < PI) { q = 2; r = rot - PId2; }
            else if (rot < PIt3d2) { q = 3; r = rot - PI; }
            else { q = 4; r = rot - PIt3d2; }
            const double t = std::tan(r);
            if (base_dir == 'i' && known == 'i') {
                cd = q == 1 ? kd / t : q == 2 ? -kd * t : q == 3 ? -kd / t : kd * t;
            } else if (base_dir == 'i') {  // known 'j'
                cd = q == 1 ? kd * t : q == 2 ? kd / t : q == 3 ? -kd * t : -kd / t;
            } else if (known == 'i') {     // base_dir 'j'
                cd = q == 1 ? kd * t : q == 2 ? -kd / t : q == 3 ? -kd * t : kd / t;
            } else {                       // base_dir 'j', known 'j'
                cd = q == 1 ? kd / t : q == 2 ? -kd * t : q == 3 ? -kd / t : kd * t;
            }
        }
        const Pt Pe = known == 'i' ? Pt{coord, pt.fj + cd} : Pt{pt.fi + cd, coord};
        if (base_dir == 'i')
            baseJ = distance(pt, Pe);
        else
            baseI = distance(pt, Pe);
        E = Pe;
    }
    // defineFromEndPtCoordAndBase_forceDeltas
    void fromEndCoordAndBase(const Pt &Pi, double coord, char coord_ty, double base, char base_dir, double dfi,
                             double dfj) {
        I = Pi;
        double ang;
        if (base_dir == 'i') {
            baseI = base;
            ang = rot >= PIt3d2 ? rot - PIt3d2 : rot + PId2;
        } else {
            baseJ = base;
            ang = rot;
        }
        const Pt pt = from_dist_rot(I, base, ang);
        otherBase(pt, base_dir, coord_ty, coord);
        setDeltas(dfi, dfj);
    }
    // defineFromEndPtCoordAndBase_norm(.., called): without called, the deltas follow from the
    // refinements already set
    void fromEndCoordAndBaseNorm(const Pt &Pi, double coord, char coord_ty, double base, char base_dir, bool called) {
        I = Pi;
        double ang;
        if (base_dir == 'i') {
            baseI = base;
            ang = rot >= PIt3d2 ? rot - PIt3d2 : rot + PId2;
        } else {
            baseJ = base;
            ang = rot;
        }
        const Pt pt = from_dist_rot(I, base, ang);
        otherBase(pt, base_dir, coord_ty, coord);
        if (!called) deduceDeltas();
    }
    // defineFromDeltas_maxvalues(pt, 'i', dfi, dfj, maxF_i, maxF_j, force=.true.)
    void fromDeltasMax(const Pt &p, double dfi, double dfj, double mi, double mj) {
        if (!aligned()) throw Fail{"padding zone is not aligned with the frequency axes"};
        const double fi = p.fi, fj = p.fj;
        double bi = 0.0, bj = 0.0;
        const Fail bad{"external padding: max_area_ext does not reach beyond the last zone limit"};
        if (rot == 0.0) {
            if (mi <= fi || mj <= fj) throw bad;
            bi = mi - fi; bj = mj - fj;
        } else if (rot == PId2) {
            if (mi <= fi || mj >= fj) throw bad;
            bj = mi - fi; bi = fj - mj;
        } else if (rot == PI) {
            if (mi >= fi || mj >= fj) throw bad;
            bi = fi - mi; bj = fj - mj;
        } else {
            if (mi >= fi || mj <= fj) throw bad;
            bj = fi - mi; bi = mj - fj;
        }
        if (!(rot == 0.0 || rot == PI)) std::swap(dfi, dfj);
        int si = (int)std::ceil(bi / dfi), sj = (int)std::ceil(bj / dfj);
        dfi = bi / si;
        dfj = bj / sj;
        ni = si + 1;
        nj = sj + 1;
        dI = dfi;
        dJ = dfj;
        define(p, 'i', bi, bj);
    }
    Dumped dump() const { return Dumped{I, rot, baseI, baseJ, ni, nj, pol, id_im}; }
};

// MTriangZone_t (zones/MTriangZoneImpl.F90) with the state the pre-mesh reads and writes:
// corner C, A at the end of the J side CA, B at the end of the I side CB.
struct TZ {
    Pt C, A, B;
    double rot = 0.0;
    int ni = 0, nj = 0, pol = kNull, id_im = 0;

    void setRefinements(int n_i, int n_j, bool *sticky) {  // M2DPolygZone setRefinements, not forced
        if (*sticky) {
            ni = n_i;
            nj = n_j;
        } else {
            ni = n_i % 2 == 0 ? n_i + 1 : n_i;
            nj = n_j % 2 == 0 ? n_j + 1 : n_j;
        }
    }
    // defineFromPts_norm (:275-346): which of P1, P2 is A, then deduceRotation (:157-198)
    void define(const Pt &Cp, const Pt &P1, const Pt &P2) {
        if (ni == 0 || nj == 0) throw Fail{"missing triangle refinement information"};
        if (P1.fj > P2.fj || P1.fj < P2.fj) {
            A = P1; B = P2;
        } else if (P1.fj > Cp.fj) {
            if (P1.fi < P2.fi) { A = P1; B = P2; }
            else if (P2.fi < P1.fi) { A = P2; B = P1; }
            else throw Fail{"triangle collapsed into a segment"};
        } else if (P1.fj < Cp.fj) {
            if (P1.fi > P2.fi) { A = P1; B = P2; }
            else if (P2.fi > P1.fi) { A = P2; B = P1; }
            else throw Fail{"triangle collapsed into a segment"};
        } else {
            throw Fail{"three triangle points on one line"};
        }
        C = Cp;
        const double dx = A.fi - C.fi, dy = A.fj - C.fj;
        double ang = std::atan(std::fabs(dx) / std::fabs(dy));
        if (!(dx >= 0.0 && dy >= 0.0)) {
            if (dy < 0.0)
                ang = dx >= 0.0 ? PI - ang : PI + ang;
            else
                ang = ang > 1e-14 ? PIt2 - ang : 0.0;
        }
        rot = ang;
    }
    double baseI() const { return distance(C, B); }
    double baseJ() const { return distance(C, A); }
};

// M2DPolygZone getUnaryDeltas (M2DPolygZone.F90:172-226): the unit steps along the zone's I
// and J sides as the lattice walk adds them to (fi, fj).
void unary_deltas(double rot, double &Ii, double &Ij, double &Ji, double &Jj) {
    if (rot < PId2) {
        const double c = std::cos(rot), s = std::sin(rot);
        Ji = s; Jj = c; Ii = c; Ij = -s;
    } else if (rot < PI) {
        const double a = rot - PId2, c = std::cos(a), s = std::sin(a);
        Ji = -s; Jj = c; Ii = -c; Ij = -s;
    } else if (rot < PIt3d2) {
        const double a = rot - PI, c = std::cos(a), s = std::sin(a);
        Ji = -s; Jj = -c; Ii = -c; Ij = s;
    } else {
        const double a = rot - PIt3d2, c = std::cos(a), s = std::sin(a);
        Ji = s; Jj = -c; Ii = c; Ij = s;
    }
}

// The lattice walks of compute_rz_ / compute_TZ_iso_ and of both interpolations start from the
// zone's init point with its two coordinates exchanged when rot lies in [pi/2, pi) or
// [3 pi/2, 2 pi) (_shared_poly2d.fi:196-212, 873-900), and write the exported BRM points with
// the coordinates exchanged back (fi_ptr => fj).
bool swaps_base(double rot) { return (rot >= PId2 && rot < PI) || (rot >= PIt3d2 && rot < PIt2); }

}  // namespace premesh

int Engine::mesher_zones(std::vector<ZoneDev> &zones, std::vector<int> &policy_out, std::vector<TriDump> *tris,
                         std::vector<int> *order, std::vector<unsigned char> *swapped) {
    using namespace premesh;
    int rc = validate();
    if (rc) return rc;
    // spatial symmetry (validateAll_, BsaLibImpl.F90:488-498): none counts once, HALF lays out
    // the half plane f1 >= 0 and counts twice, FOURTH lays out the whole plane and counts four
    // times (the reference has no layout of its own for it)
    const bool half = set.bispsym == 2;
    const double isym = set.bispsym == 0 ? 1.0 : (double)set.bispsym;
    bool sticky = false;  // setRefinements' saved force flag
    if (!in.natf || !in.xsi) return fail(BSA_ERR_STATE, "natural frequencies / damping not set");
    if (!in.ubref) return fail(BSA_ERR_STATE, "zone mean wind speeds not set");
    // bkg_peak_width_(i, j) = 1 / max_z L(i, j, z) / U(z) (computeBKGPeakWidths,
    // StructureImpl.F90:225-260, from validateAll_, BsaLibImpl.F90:513-524); the background
    // peak width is its maximum, over the first direction only when restricted (PreMesh :302)
    double bkgw = 0.0;
    for (int j = 0; j < (bkg_restrict ? 1 : 3); ++j)
        for (int i = 0; i < 3; ++i) {
            double mx = -INFINITY;
            for (int z = 0; z < in.nz; ++z) mx = std::max(mx, in.L[(size_t)i + 3 * (size_t)j + 9 * (size_t)z] / in.ubref[z]);
            if (mx != 0.0 && std::isfinite(mx)) bkgw = std::max(bkgw, 1.0 / mx);
        }
    if (!(bkgw > 0.0)) return fail(BSA_ERR_ARG, "background peak width is zero");
    if (set.bkgrfmt < 2) return fail(BSA_ERR_ARG, "background zone refinement must be >= 2");
    const double base_i = bkgw * set.bkgaext;
    const double dS2_2 = base_i * (std::sqrt(2.0) / 2.0), d2S2_2 = dS2_2 / 2.0;
    double max_ext = -INFINITY;
    for (int m = 0; m < in.nm; ++m) max_ext = std::max(max_ext, in.natf[m]);
    max_ext *= set.maxaext;  // getMaxSpaceExtension_ (:1626-1631)

    // ---- prefetchZoneLimits_ / getActualPeakZoneExtensionLimits_ ----
    const int NM = (int)modes.size();
    std::vector<double> peak_ext(in.nm + 1, -1.0);  // peak_exts_(mode), 1-based
    std::vector<double> pbf(NM + 1), pff(NM + 1);
    for (int im = 1; im <= NM; ++im) {
        const int nmode = modes[im - 1];
        const double f = in.natf[nmode - 1], ext = in.xsi[nmode - 1] * f * set.genpaext;
        pbf[im] = f - ext;
        pff[im] = f + ext;
        peak_ext[nmode] = ext + ext;
    }
    const double bpw2 = base_i / 2.0;
    std::vector<double> lim(1, 0.0);   // 1-based
    std::vector<int> pol(1, kDef), IM(1, 0);
    int NLims = 0;
    {
        int skip = 1;
        while (pff[skip] <= bpw2) {
            ++skip;
            if (skip > NM) break;
        }
        skip -= 1;
        if (NM - skip > 0) {
            const int cap = (NM - skip) * 2 + 1;
            lim.assign(cap + 1, 0.0);
            pol.assign(cap + 1, kDef);
            IM.assign(201, 0);
            int NL, iim, jim;
            skip += 1;
            if (bpw2 < pbf[skip]) {
                lim[1] = pbf[skip]; lim[2] = pff[skip];
                NL = 2;
                pol[1] = kPrePeak1; pol[2] = kPeak;
                IM[1] = skip == 1 ? CODE_PRE_PEAK_OK : CODE_PRE_PEAK_KO;
                iim = 2; IM[iim] = 1;
                jim = 3; IM[jim] = modes[skip - 1];
            } else {
                lim[1] = pff[skip]; pol[1] = kPeak; NL = 1;
                IM[1] = 1; IM[2] = modes[skip - 1];
                iim = 1; jim = 2;
            }
            for (int im = skip + 1; im <= NM; ++im) {
                const int nmode = modes[im - 1];
                const double BF = pbf[im], FF = pff[im];
                if (jim + 3 > 200) return fail(BSA_ERR_UNSUPPORTED, "too many interest-mode entries for the zone layout");
                if (BF < lim[NL]) {
                    if (NL == 2 && BF <= lim[NL - 1]) {
                        lim[NL - 1] = BF; pol[NL - 1] = kPrePeak2;
                        lim[NL] = FF; pol[NL] = kPeak;
                    } else {
                        lim[NL] = FF; pol[NL] = kPeak;
                    }
                    IM[iim] += 1;
                    IM[++jim] = nmode;
                } else {
                    lim[++NL] = BF; pol[NL] = kPrePeak2;
                    lim[++NL] = FF; pol[NL] = kPeak;
                    iim = jim + 1; IM[iim] = CODE_PRE_PEAK_OK;
                    ++iim; IM[iim] = 1;
                    jim = iim + 1; IM[jim] = nmode;
                }
            }
            iim = jim + 1; IM[iim] = 1;
            jim = iim + 1; IM[jim] = modes[NM - 1];
            NLims = NL;
            lim.resize(NL + 2);
            pol.resize(NL + 2);
            IM.resize(jim + 1);
        }
    }

    // ---- pre-mesh ----
    std::vector<Dumped> dz;
    std::vector<TZ> dt;
    std::vector<int> seq;  // dump order: k >= 0 rectangle k, k < 0 triangle -k - 1
    // compute_rz_ (_shared_poly2d.fi:76-88, 433-449): a zone with a side of zero length is
    // skipped (not dumped); a zero delta aborts the reference
    auto emit = [&](const RZ &z) {
        if (z.baseI <= MACHINE_PRECISION || z.baseJ <= MACHINE_PRECISION) return;
        if (z.dI <= MACHINE_PRECISION || z.dJ <= MACHINE_PRECISION) throw Fail{"a zone delta is zero"};
        seq.push_back((int)dz.size());
        dz.push_back(z.dump());
    };
    // MTriangZone compute (MTriangZoneImpl.F90:489-510, _shared_poly2d.fi:78-80): isosceles,
    // equal refinements, or the reference aborts
    auto emit_tri = [&](const TZ &t) {
        if (!(std::fabs(t.baseJ() - t.baseI()) <= MACHINE_PRECISION)) throw Fail{"triangle must be isosceles"};
        if (t.ni != t.nj) throw Fail{"different triangle side refinements not allowed"};
        seq.push_back(-(int)dt.size() - 1);
        dt.push_back(t);
    };
    RZ bkgz;
    const double base_j = base_i;
    double base_ib = base_i;  // HALF halves the background zone's I side (PreMesh :372-378)
    if (half) {
        base_ib = base_i / 2.0;
        bkgz.define(Pt{0.0, -base_ib}, 'i', base_ib, base_j);
    } else {
        bkgz.define(Pt{0.0, 0.0}, 'c', base_i, base_j);
    }
    bkgz.pol = kPeak;
    bkgz.id_im = 0;
    {
        const int iost = set.bkgrfmt;
        if (half)
            bkgz.setRefinements((iost - 1) / 2 + 1, iost, false, &sticky);
        else
            bkgz.setRefinements(iost, iost, false, &sticky);
        if (half) {
            const int io2 = (bkgz.nj - 1) / 2 + 1;
            if (bkgz.ni != io2) bkgz.setRefinements(io2, bkgz.nj, true, &sticky);
        }
    }
    const double df_I_ref = bkgz.dI, df_J_ref = bkgz.dJ;
    if (!(std::fabs(df_I_ref - df_J_ref) < MACHINE_PRECISION))
        return fail(BSA_ERR_ARG, "freq deltas of the background peak zone differ");
    try {
        emit(bkgz);
        if (NLims > 0) {
            const int NLimsP1 = NLims + 1;
            const double maxF = lim[NLims] + d2S2_2;
            const int id_im_last = (int)IM.size() - 1 - 1;  // size(msh_ZoneLimsInterestModes) - 1
            lim[NLimsP1] = maxF;
            pol[NLimsP1] = kPrePeak2;
            std::vector<double> dlt1(NLimsP1 + 1), dlt2(NLimsP1 + 1);
            std::vector<int> ref1(NLimsP1 + 1), ref2(NLimsP1 + 1), imz(NLimsP1 + 1, 0);
            const double ROT[7] = {0.0, PIt3d2, 0.0, PId2, PI, PIt3d2, 0.0};  // ROTATIONS(1:6)
            const char CDIR[5] = {0, 'j', 'i', 'j', 'i'};                     // COORDS_DIR_CH
            const int LSIGN[5] = {0, 1, 1, -1, -1};                           // LIM_SIGN_DIRS
            const int LEFT[5] = {0, 1, -1, -1, 1};                            // LEFT_RZ_SIGNS
            Pt basePts[5] = {Pt{}, bkgz.getA(), bkgz.E, bkgz.getB(), bkgz.I};
            // crest bands (directions N, E, S, W)
            const int n_dirs = half ? 3 : 4;
            const double bases_i[5] = {0.0, base_ib, half ? base_j : base_ib, base_ib, base_ib};
            for (int idir = 1; idir <= n_dirs; ++idir) {
                RZ rz;
                rz.setRotation(ROT[idir + 1]);
                Pt ptI = basePts[idir];
                const char cdir = CDIR[idir];
                const int sgn = LSIGN[idir];
                const double bi_dir = bases_i[idir];
                int iim = 1;
                for (int ilim = 1; ilim <= NLims; ++ilim) {
                    const double l = lim[ilim];
                    const Policy P = premesh::policy(pol[ilim]);
                    const double dfI = df_I_ref * P.dfI, dfJ = df_J_ref * P.dfJ;
                    rz.pol = pol[ilim];
                    if (idir == 2) imz[ilim] = iim;
                    if (ilim == 1 || pol[ilim + 1] == kPeak) {
                        int nim = IM[iim];
                        if (nim < 0) nim = IM[++iim];
                        rz.id_im = iim;
                        iim = iim + nim + 1;
                    }
                    rz.fromEndCoordAndBase(ptI, sgn * l, cdir, bi_dir, 'i', dfI, dfJ);
                    if (idir == 1 || idir == 3)
                        ptI.fj += sgn * l - ptI.fj;
                    else
                        ptI.fi += sgn * l - ptI.fi;
                    if (idir == 2) {
                        ref1[ilim] = rz.ni; ref2[ilim] = rz.nj;
                        dlt1[ilim] = rz.dI; dlt2[ilim] = rz.dJ;
                    }
                    emit(rz);
                }
                const Policy P = premesh::policy(kPrePeak2);
                rz.pol = kPrePeak2;
                rz.id_im = id_im_last;
                rz.fromEndCoordAndBase(ptI, sgn * maxF, cdir, bi_dir, 'i', df_I_ref * P.dfI, df_J_ref * P.dfJ);
                if (idir == 2) {
                    ref1[NLimsP1] = rz.ni; ref2[NLimsP1] = rz.nj;
                    dlt1[NLimsP1] = rz.dI; dlt2[NLimsP1] = rz.dJ;
                }
                emit(rz);
            }
            imz[NLimsP1] = id_im_last;
            if (premesh_diag_crest) {
                // diagonal-crest scheme (BsaMesherImpl.F90:924-1279): an internal padding
                // rectangle over the NE (and SW) quadrant, and along the SE (and NW) diagonal
                // crest a triangle at the background zone's corner, then per zone limit a
                // rotated crest rectangle, two levelling triangles and two closing rectangles,
                // and a closing triangle at the far corner
                if (premesh_mode_base) throw Fail{"the BASE pre-mesh mode is not implemented by the reference"};
                const int ndiag = half ? 1 : 2;
                {
                    const Policy P = premesh::policy(kPadIntern);
                    for (int idir = 1; idir <= ndiag; ++idir) {
                        RZ rz;  // a copy of the master's zone object, interest-mode pointer 0
                        rz.setRotation(ROT[2 * idir]);
                        rz.pol = kPadIntern;
                        const double r = LSIGN[2 * idir] * maxF;
                        rz.fromDeltasMax(basePts[2 * idir], df_I_ref * P.dfI, df_J_ref * P.dfJ, r, r);
                        emit(rz);
                    }
                }
                Pt bpd[5] = {Pt{}, basePts[3], basePts[1], basePts[3], basePts[4]};
                const double trots[3] = {0.0, PId2 + PI / 4.0, PIt3d2 + PI / 4.0};
                for (int idir = 1; idir <= ndiag; ++idir) {
                    const int S = LSIGN[2 * idir];
                    const double tdel = dS2_2 * S;
                    TZ tz;
                    const double limI = bpd[idir].fi, limJ = bpd[idir].fj;
                    Pt ptI{limI + tdel, limJ}, ptA{limI, limJ - tdel};
                    tz.id_im = 1;
                    tz.setRefinements(bkgz.ni, bkgz.nj, &sticky);
                    tz.pol = kPeak;
                    tz.define(bpd[idir], ptI, ptA);
                    emit_tri(tz);
                    const double trot = trots[idir];
                    int k0 = 1;  // limits the first triangle covers (one count per direction loop)
                    while (std::fabs(ptI.fi) > lim[k0] && k0 <= NLims) ++k0;
                    const bool warn = k0 == NLims + 1;
                    const double rvals[2] = {trot - trots[1], trot + trots[1]};
                    int idrot = 0;
                    RZ rz;
                    int iim = 1;
                    for (int ilim = k0; ilim <= NLimsP1; ++ilim) {
                        const double l = lim[ilim];
                        rz.setRefinements(bkgz.ni, ref2[ilim], false, &sticky);
                        rz.id_im = iim;
                        rz.setRotation(trot);
                        rz.pol = pol[ilim];
                        rz.fromEndCoordAndBaseNorm(ptI, -l * S, 'j', base_ib, 'i', false);
                        emit(rz);
                        ptA = rz.getA();
                        const Pt ptB = rz.getB(), ptE = rz.E;
                        const int pl = pol[ilim] == kPeak ? kCrest : kBasin;
                        tz.id_im = iim;
                        const int nim = IM[iim];
                        iim += nim < 0 ? 1 : nim + 1;
                        ptI = Pt{l * S, rz.I.fj};
                        tz.setRefinements(rz.nj, rz.nj, &sticky);
                        tz.pol = pl;
                        tz.define(ptI, ptA, rz.I);
                        emit_tri(tz);
                        const double rtmp = tz.baseI();
                        const Policy dP = premesh::policy(pl);
                        rz.setRotation(rvals[idrot++ % 2]);
                        rz.pol = pl;
                        rz.fromEndCoordAndBase(Pt(rz.I), limJ, 'j', rtmp, 'i', dlt2[ilim] * dP.dfI, dlt2[ilim] * dP.dfJ);
                        emit(rz);
                        ptI = Pt{ptB.fi, -l * S};
                        tz.define(ptI, ptB, ptE);
                        emit_tri(tz);
                        rz.setRotation(rvals[idrot++ % 2]);
                        rz.fromEndCoordAndBase(Pt(tz.C), limI, 'i', rtmp, 'i', dlt2[ilim] * dP.dfI, dlt2[ilim] * dP.dfJ);
                        emit(rz);
                        ptI = ptA;
                    }
                    if (!warn) {  // closing triangle
                        const Policy dP = premesh::policy(kPeak);
                        tz.id_im = id_im_last;
                        tz.pol = kPeak;
                        tz.setRefinements(set.bkgrfmt * dP.dfI, set.bkgrfmt * dP.dfJ, &sticky);
                        const Pt c{maxF * S, -maxF * S};
                        tz.define(c, Pt{c.fi - dS2_2 * S, c.fj}, Pt{c.fi, c.fj + dS2_2 * S});
                        emit_tri(tz);
                    }
                }
            }
            // quadrants (scheme without diagonal crests, BsaMesherImpl.F90:743-920)
            if (!premesh_diag_crest) {
                const Pt p1 = basePts[1];
                basePts[1] = basePts[2]; basePts[2] = basePts[3]; basePts[3] = basePts[4]; basePts[4] = p1;
                const double init_freq = basePts[1].fi;
                const int main_refs = std::max(ref1[1], ref2[1]);
                const char bases_ch[5] = {0, 'i', 'j', 'i', 'j'};
                for (int idir = 1; idir <= (half ? 2 : 4); ++idir) {
                    RZ rz;
                    const double lrot = ROT[idir], mrot = ROT[idir + 1], rrot = ROT[idir + 2];
                    rz.setRotation(mrot);
                    rz.pol = pol[1];
                    Pt ptI = basePts[idir];
                    double rbase = lim[1] - init_freq;
                    if (rbase <= 0.0) throw Fail{"negative base of the first quadrant zone"};
                    rz.define(ptI, 'i', rbase, rbase);
                    rz.setRefinements(main_refs, main_refs, false, &sticky);
                    rz.id_im = 1;
                    emit(rz);
                    Pt ptE = rz.E;
                    const int lsgn = LEFT[idir], rsgn = LSIGN[idir];
                    const char lknown = bases_ch[idir], rknown = bases_ch[5 - idir];
                    for (int ilim = 2; ilim <= NLimsP1; ++ilim) {
                        rz.id_im = imz[ilim];
                        const double rl = lim[ilim];
                        rbase = rl - lim[ilim - 1];
                        ptI = ptE;
                        rz.pol = pol[ilim];
                        double dm = std::min(dlt1[ilim], dlt2[ilim]);
                        rz.setRotation(mrot);
                        rz.fromEndCoordAndBase(ptI, lsgn * rl, 'j', rbase, lknown, dm, dm);
                        emit(rz);
                        ptE = rz.E;
                        dm = dlt2[ilim];
                        rz.setRotation(lrot);
                        rz.fromEndCoordAndBase(ptI, lsgn * init_freq, lknown, rbase, 'i', dm, dm);
                        emit(rz);
                        rz.setRotation(rrot);
                        rz.fromEndCoordAndBase(ptI, rsgn * init_freq, rknown, rbase, 'j', dm, dm);
                        emit(rz);
                    }
                }
            }
            // external padding (BsaMesherImpl.F90:1286-1350)
            if (set.fcov == 1) {
                const Policy P = premesh::policy(kPadExtern);
                const double dfI = df_I_ref * P.dfI, dfJ = df_J_ref * P.dfJ;
                const Pt bp[5] = {Pt{}, Pt{half ? 0.0 : -maxF, maxF}, Pt{maxF, maxF}, Pt{maxF, -maxF},
                                  Pt{-maxF, -maxF}};
                const double mext[5] = {0.0, max_ext, max_ext, half ? 0.0 : max_ext, max_ext};
                for (int idir = 1; idir <= (half ? 3 : 4); ++idir) {
                    RZ rz;
                    rz.id_im = id_im_last;
                    rz.pol = kPadExtern;
                    rz.setRotation(ROT[idir + 1]);
                    rz.fromDeltasMax(bp[idir], dfI, dfJ, LSIGN[idir] * mext[idir], LEFT[idir] * max_ext);
                    emit(rz);
                }
            }
        }
    } catch (const Fail &f) {
        return fail(BSA_ERR_ARG, "zone layout: %s", f.msg);
    }

    // ---- post-mesh lattice of every zone (interpolateRZ_HTPC_v3, _shared_poly2d.fi:588-870) ----
    zones.clear();
    policy_out.clear();
    if (swapped) swapped->clear();
    for (const Dumped &d : dz) {
        if (d.ni < 2 || d.nj < 2) return fail(BSA_ERR_ARG, "zone with fewer than 2 lattice points per side");
        const double dI0 = d.baseI / (d.ni - 1), dJ0 = d.baseJ / (d.nj - 1);  // setRefinements(.., force)
        Policy P = premesh::policy(d.pol);
        if (!bfm_mlr) {  // disableZonePolicyBfmMLR (MZone.F90)
            P.nlevs = 0;
            P.bfm_i = 1;
            P.bfm_j = 1;
        }
        if (visual) P.nlevs = 0;  // the visual mode interpolates the BFM lattice as dumped
        int si = 1, sj = 1;
        for (int l = 0; l < P.nlevs; ++l) {
            si *= P.bfm_i;
            sj *= P.bfm_j;
        }
        double dIr = dI0 / si, dJr = dJ0 / sj;
        if (validate_deltas && !visual) {
            int idx = d.id_im == 0 ? 1 : d.id_im;
            int nim = IM.size() > (size_t)idx ? IM[idx] : 0;
            double dwI;
            if (nim == CODE_PRE_PEAK_OK) {
                dwI = bkgw;
            } else {
                if (nim < 0) nim = IM[++idx];
                dwI = INFINITY;
                for (int k = idx + 1; k <= idx + nim; ++k) dwI = std::min(dwI, peak_ext[IM[k]]);
            }
            const double dwJ = dwI;
            if (dIr > dwI / P.bfm_i) {
                while (dIr > dwI / P.bfm_i) dIr = dI0 / ++si;
            } else {
                while (dIr < dwI / P.bfm_i && si > 1) dIr = dI0 / --si;
            }
            if (dJr > dwJ / P.bfm_j) {
                while (dJr > dwJ / P.bfm_j) dJr = dJ0 / ++sj;
            } else {
                while (dJr < dwJ / P.bfm_j && sj > 1) dJr = dJ0 / --sj;
            }
        }
        double Ii, Ij, Ji, Jj;
        unary_deltas(d.rot, Ii, Ij, Ji, Jj);
        const bool sw = swaps_base(d.rot);
        ZoneDev z{};
        z.fi0 = sw ? d.I.fj : d.I.fi;
        z.fj0 = sw ? d.I.fi : d.I.fj;
        z.dIi = Ii * dIr; z.dIj = Ij * dIr;
        z.dJi = Ji * dJr; z.dJj = Jj * dJr;
        z.ni = (d.ni - 1) * si + 1;
        z.nj = (d.nj - 1) * sj + 1;
        z.Fi = P.brm_i;
        z.Fj = P.brm_j;
        z.wI = dIr * kPi2;
        z.wJ = dJr * kPi2;
        z.sym = isym;  // m3 += intg * i_bisp_sym_ (_shared_poly2d.fi:2117-2119)
        zones.push_back(z);
        policy_out.push_back(d.pol);
        if (swapped) swapped->push_back(sw ? 1 : 0);
    }
    // triangles: the policy's factors for the post-mesh walk (interpolateTZ_HTPC_v3 has no
    // delta validation); the walk itself is bsa_triang.cu's
    if (tris) {
        tris->clear();
        for (const TZ &t : dt) {
            Policy P = premesh::policy(t.pol);
            if (!bfm_mlr) {
                P.nlevs = 0;
                P.bfm_i = 1;
                P.bfm_j = 1;
            }
            TriDump d;
            d.Ci = t.C.fi; d.Cj = t.C.fj; d.Ai = t.A.fi; d.Aj = t.A.fj; d.Bi = t.B.fi; d.Bj = t.B.fj;
            d.rot = t.rot;
            d.sym = isym;
            d.n = t.ni;
            d.pol = t.pol;
            d.bfi = P.bfm_i; d.bfj = P.bfm_j; d.bri = P.brm_i; d.brj = P.brm_j; d.nlevs = P.nlevs;
            tris->push_back(d);
        }
    } else if (!dt.empty()) {
        return fail(BSA_ERR_UNSUPPORTED, "this entry takes rectangular zones only; the layout has triangles");
    }
    if (order) *order = seq;
    return BSA_OK;
}

}  // namespace bsa
