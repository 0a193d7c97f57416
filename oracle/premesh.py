"""Mesher zone layout (pre-mesh) and post-mesh lattices -- TEST INFRASTRUCTURE ONLY.

A second restatement, in Python, of the reference's zone layout, used by the tests to check the
library's (bsalib_gb300/csrc/bsa_premesh.cu) zone by zone:

* limits, policies and interest modes: prefetchZoneLimits_ and
  getActualPeakZoneExtensionLimits_ (src/bsa/meshing/BsaMesherImpl.F90:1638-1890);
* zones: PreMesh (:266-1393): background peak zone, crest bands (:450-730), quadrants
  (:743-920) or, in the diagonal-crest scheme, padding rectangles, triangles and rotated
  rectangles along the diagonals (:924-1279; triangle geometry in triang.py), external padding
  (:1286-1350);
* rectangle geometry: MRectZone (zones/MRectZoneImpl.F90: define, setIEpts, getOtherBase,
  defineFromEndPtCoordAndBase, defineFromDeltas_maxvalues, setDeltas / deduceRefinements,
  deduceDeltas), M2DPolygZone (setRefinements, getUnaryDeltas), MPoint
  (getNewPointFromDistAndRot), MPolicy_fromID (policy/MPolicy.F90:130-168);
* post-mesh refinement of every zone: interpolateRZ_HTPC_v3 (zones/_shared_poly2d.fi:588-870).

Each rectangle comes out as (fi0, fj0, dIi, dIj, dJi, dJj, ni, nj, Fi, Fj, policy, sym), the
lattice the integration evaluates (walked from the init point with its coordinates exchanged
for rot in [pi/2, pi) and [3 pi/2, 2 pi), _shared_poly2d.fi:873-900) and its weight (i_bisp_sym_: 1 without spatial symmetry, 2 for HALF,
whose layout covers f1 >= 0, 4 for FOURTH, whose layout is the whole plane).
"""
from __future__ import annotations

import math

PI = 4.0 * math.atan(1.0)
PId2, PIt3d2, PIt2 = PI / 2.0, PI * 1.5, PI * 2.0
MACHINE_PRECISION = 1e-12
PRE_OK, PRE_KO = -1, -2
NULL, DEF, CONST, PRE1, PRE2, PEAK, CREST, BASIN, PADI, PADE = range(10)

# MPolicy_fromID: (delta_fI, delta_fJ, bfm_i, bfm_j, brm_i, brm_j, n_levels)
POLICY = {NULL: (0, 0, 0, 0, 0, 0, 0), DEF: (2, 2, 2, 2, 2, 2, 1), CONST: (1, 1, 1, 1, 1, 1, 1),
          PRE1: (1, 4, 4, 4, 4, 2, 1), PRE2: (1, 8, 2, 2, 4, 2, 1), PEAK: (1, 1, 4, 4, 4, 4, 1),
          CREST: (1, 4, 4, 4, 4, 2, 1), BASIN: (1, 4, 2, 2, 2, 2, 1), PADI: (4, 4, 1, 1, 2, 2, 1),
          PADE: (8, 8, 1, 1, 2, 2, 1)}


def new_point(p, dist, rot):
    """MPoint getNewPointFromDistAndRot."""
    if rot < PId2:
        di, dj = math.sin(rot), math.cos(rot)
    elif rot < PI:
        a = rot - PId2
        di, dj = math.cos(a), -math.sin(a)
    elif rot < PIt3d2:
        a = rot - PI
        di, dj = -math.sin(a), -math.cos(a)
    else:
        a = rot - PIt3d2
        di, dj = -math.cos(a), math.sin(a)
    return (di * dist + p[0], dj * dist + p[1])


def dist(a, b):
    dx, dy = abs(a[0] - b[0]), abs(a[1] - b[1])
    return math.sqrt(dx * dx + dy * dy)


class Rect:
    """The MRectZone_t state the pre-mesh uses."""

    def __init__(self):
        self.I = (0.0, 0.0)
        self.E = (0.0, 0.0)
        self.rot = 0.0
        self.bI = self.bJ = 0.0
        self.dI = self.dJ = 0.0
        self.ni = self.nj = 0
        self.pol = NULL
        self.im = 0

    def quadrant(self):
        r = self.rot
        if r < PId2:
            return 1, r
        if r < PI:
            return 2, r - PId2
        if r < PIt3d2:
            return 3, r - PI
        return 4, r - PIt3d2

    def set_ie(self, p):
        q, a = self.quadrant()
        c, s = math.cos(a), math.sin(a)
        bI, bJ = self.bI, self.bJ
        if q == 1:
            di, dj = bI * c + bJ * s, bJ * c - bI * s
        elif q == 2:
            di, dj = bJ * c - bI * s, -(bJ * s + bI * c)
        elif q == 3:
            di, dj = -(bJ * s + bI * c), -bJ * c + bI * s
        else:
            di, dj = -bJ * c + bI * s, bJ * s + bI * c
        self.I = p
        self.E = (p[0] + di, p[1] + dj)

    def define(self, p, loc, bi, bj):
        self.bI, self.bJ = bi, bj
        if loc == "c":
            self.I = (p[0] - bi / 2, p[1] - bj / 2)
            self.E = (p[0] + bi / 2, p[1] + bj / 2)
        else:
            self.set_ie(p)

    def set_refinements(self, ni, nj, force, sticky):
        """M2DPolygZone setRefinements; its force flag is a saved local: after one forced call
        every call is forced (sticky[0] carries it through a layout)."""
        if force:
            sticky[0] = True
        if sticky[0]:
            self.ni, self.nj = ni, nj
        else:
            self.ni = ni + 1 if ni % 2 == 0 else ni
            self.nj = nj + 1 if nj % 2 == 0 else nj
        self.dI = self.bI / (self.ni - 1)
        self.dJ = self.bJ / (self.nj - 1)

    def set_deltas_adapt(self, dfi, dfj):
        si, sj = math.floor(self.bI / dfi), math.floor(self.bJ / dfj)
        si += si % 2
        sj += sj % 2
        si = si or 1
        sj = sj or 1
        self.dI, self.dJ = self.bI / si, self.bJ / sj
        self.ni, self.nj = si + 1, sj + 1

    def a_point(self):
        return new_point(self.I, self.bJ, self.rot)

    def b_point(self):
        return new_point(self.I, self.bI, self.rot - PIt3d2 if self.rot > PIt3d2 else self.rot + PId2)

    def other_base(self, pt, base_dir, known, coord):
        kd = abs(coord - (pt[0] if known == "i" else pt[1]))
        cd = 0.0
        if kd >= MACHINE_PRECISION:
            q, r = self.quadrant()
            t = math.tan(r)
            table = {("i", "i"): (kd / t if t else math.inf, -kd * t, -kd / t if t else -math.inf, kd * t),
                     ("i", "j"): (kd * t, kd / t if t else math.inf, -kd * t, -kd / t if t else -math.inf),
                     ("j", "i"): (kd * t, -kd / t if t else -math.inf, -kd * t, kd / t if t else math.inf),
                     ("j", "j"): (kd / t if t else math.inf, -kd * t, -kd / t if t else -math.inf, kd * t)}
            cd = table[(base_dir, known)][q - 1]
        pe = (coord, pt[1] + cd) if known == "i" else (pt[0] + cd, coord)
        if base_dir == "i":
            self.bJ = dist(pt, pe)
        else:
            self.bI = dist(pt, pe)
        self.E = pe

    def from_end_coord_base(self, p, coord, coord_ty, base, base_dir, dfi, dfj):
        self.I = p
        if base_dir == "i":
            self.bI = base
            ang = self.rot - PIt3d2 if self.rot >= PIt3d2 else self.rot + PId2
        else:
            self.bJ = base
            ang = self.rot
        self.other_base(new_point(self.I, base, ang), base_dir, coord_ty, coord)
        self.set_deltas_adapt(dfi, dfj)

    def set_rotation(self, r):
        """M2DPolygZone setRotation: r in [0, 2 pi)."""
        if r >= PIt2:
            r -= math.floor(r / PIt2) * PIt2
        self.rot = r

    def from_end_coord_base_norm(self, p, coord, coord_ty, base, base_dir, called):
        """defineFromEndPtCoordAndBase_norm: with called false the deltas follow from the
        refinements already set (deduceDeltas)."""
        self.I = p
        if base_dir == "i":
            self.bI = base
            ang = self.rot - PIt3d2 if self.rot >= PIt3d2 else self.rot + PId2
        else:
            self.bJ = base
            ang = self.rot
        self.other_base(new_point(self.I, base, ang), base_dir, coord_ty, coord)
        if not called:
            self.dI = self.bI / (self.ni - 1)
            self.dJ = self.bJ / (self.nj - 1)

    def from_deltas_max(self, p, dfi, dfj, mi, mj):
        fi, fj = p
        r = self.rot
        if r == 0.0:
            assert mi > fi and mj > fj
            bi, bj = mi - fi, mj - fj
        elif r == PId2:
            assert mi > fi and mj < fj
            bj, bi = mi - fi, fj - mj
        elif r == PI:
            assert mi < fi and mj < fj
            bi, bj = fi - mi, fj - mj
        else:
            assert mi < fi and mj > fj
            bj, bi = fi - mi, mj - fj
        if r not in (0.0, PI):
            dfi, dfj = dfj, dfi
        si, sj = math.ceil(bi / dfi), math.ceil(bj / dfj)
        self.ni, self.nj = si + 1, sj + 1
        self.dI, self.dJ = bi / si, bj / sj
        self.define(p, "i", bi, bj)

    def dump(self):
        return dict(I=self.I, rot=self.rot, bI=self.bI, bJ=self.bJ, ni=self.ni, nj=self.nj, pol=self.pol,
                    im=self.im)


def zone_limits(modes, natf, xsi, peak_area_ext, bpw2):
    """prefetchZoneLimits_ with getActualPeakZoneExtensionLimits_; 1-based lists."""
    nm = len(modes)
    lo = [None] + [natf[m - 1] - xsi[m - 1] * natf[m - 1] * peak_area_ext for m in modes]
    hi = [None] + [natf[m - 1] + xsi[m - 1] * natf[m - 1] * peak_area_ext for m in modes]
    skip = 1
    while hi[skip] <= bpw2:
        skip += 1
        if skip > nm:
            break
    skip -= 1
    if nm - skip == 0:
        return 0, None, None, None
    lim = [0.0] * (2 * (nm - skip) + 2)
    pol = [DEF] * (2 * (nm - skip) + 2)
    im = [0] * 201
    skip += 1
    if bpw2 < lo[skip]:
        lim[1], lim[2] = lo[skip], hi[skip]
        n = 2
        pol[1], pol[2] = PRE1, PEAK
        im[1] = PRE_OK if skip == 1 else PRE_KO
        iim, im[2] = 2, 1
        jim, im[3] = 3, modes[skip - 1]
    else:
        lim[1], pol[1], n = hi[skip], PEAK, 1
        im[1], im[2] = 1, modes[skip - 1]
        iim, jim = 1, 2
    for k in range(skip + 1, nm + 1):
        BF, FF = lo[k], hi[k]
        if BF < lim[n]:
            if n == 2 and BF <= lim[n - 1]:
                lim[n - 1], pol[n - 1] = BF, PRE2
            lim[n], pol[n] = FF, PEAK
            im[iim] += 1
            jim += 1
            im[jim] = modes[k - 1]
        else:
            lim[n + 1], pol[n + 1] = BF, PRE2
            lim[n + 2], pol[n + 2] = FF, PEAK
            n += 2
            iim = jim + 1
            im[iim] = PRE_OK
            iim += 1
            im[iim] = 1
            jim = iim + 1
            im[jim] = modes[k - 1]
    iim = jim + 1
    im[iim] = 1
    jim = iim + 1
    im[jim] = modes[nm - 1]
    return n, lim[: n + 2], pol[: n + 2], im[: jim + 1]


def layout(modes, natf, xsi, L, ubref, bkgrfmt, bkgaext, peak_area_ext, maxaext, fcov=1,
           validate=True, mlr=True, restrict=False, bispsym=0, diag=False, mode_base=False, visual=False):
    """Zones of the Mesher analysis in dump order: rectangles as (fi0, fj0, dIi, dIj, dJi, dJj,
    ni, nj, Fi, Fj, policy, sym), the lattice the walk evaluates; with diag (the diagonal-crest
    scheme) also triangles, as dicts (C, A, B, rot, n, pol, sym and the policy's BFM / BRM
    factors).  L: turbulence length scales (3, 3, nz) column-major flattened; ubref: zone mean
    speeds.  A condition the reference aborts on raises AssertionError or TriError."""
    from .triang import Tri
    nz = len(ubref)
    bkgw = 0.0
    for j in range(1 if restrict else 3):
        for i in range(3):
            mx = max(L[i + 3 * j + 9 * z] / ubref[z] for z in range(nz))
            if mx != 0.0:
                bkgw = max(bkgw, 1.0 / mx)
    base = bkgw * bkgaext
    d2 = base * (math.sqrt(2.0) / 2.0) / 2.0
    max_ext = max(natf) * maxaext
    NL, lim, pol, im = zone_limits(modes, natf, xsi, peak_area_ext, base / 2.0)
    peak_ext = {m: 2.0 * xsi[m - 1] * natf[m - 1] * peak_area_ext for m in modes}
    half = bispsym == 2
    isym = 1.0 if bispsym == 0 else float(bispsym)
    sticky = [False]
    bkg = Rect()
    base_b = base / 2.0 if half else base
    if half:
        bkg.define((0.0, -base_b), "i", base_b, base)
        bkg.set_refinements((bkgrfmt - 1) // 2 + 1, bkgrfmt, False, sticky)
        n2 = (bkg.nj - 1) // 2 + 1
        if bkg.ni != n2:
            bkg.set_refinements(n2, bkg.nj, True, sticky)
    else:
        bkg.define((0.0, 0.0), "c", base, base)
        bkg.set_refinements(bkgrfmt, bkgrfmt, False, sticky)
    bkg.pol, bkg.im = PEAK, 0
    dfI0, dfJ0 = bkg.dI, bkg.dJ
    dumped = []

    def emit(z):  # compute_rz_: a zone with an empty side is not dumped; a zero delta aborts
        if z.bI <= MACHINE_PRECISION or z.bJ <= MACHINE_PRECISION:
            return
        assert z.dI > MACHINE_PRECISION and z.dJ > MACHINE_PRECISION
        dumped.append(z.dump())

    emit(bkg)
    if NL > 0:
        P1 = NL + 1
        maxF = lim[NL] + d2
        last = len(im) - 1 - 1
        lim[P1], pol[P1] = maxF, PRE2
        ROT = [None, PIt3d2, 0.0, PId2, PI, PIt3d2, 0.0]
        CDIR = [None, "j", "i", "j", "i"]
        SGN = [None, 1, 1, -1, -1]
        LEFT = [None, 1, -1, -1, 1]
        base_pts = [None, bkg.a_point(), bkg.E, bkg.b_point(), bkg.I]
        refm = {}
        dlt = {}
        izm = {}
        bases = [None, base_b, base if half else base_b, base_b, base_b]
        for d in range(1, 4 if half else 5):                   # crest bands
            rz = Rect()
            rz.rot = ROT[d + 1]
            p = base_pts[d]
            iim = 1
            for k in range(1, NL + 1):
                P = POLICY[pol[k]]
                rz.pol = pol[k]
                if d == 2:
                    izm[k] = iim
                if k == 1 or pol[k + 1] == PEAK:
                    n = im[iim]
                    if n < 0:
                        iim += 1
                        n = im[iim]
                    rz.im = iim
                    iim += n + 1
                rz.from_end_coord_base(p, SGN[d] * lim[k], CDIR[d], bases[d], "i", dfI0 * P[0], dfJ0 * P[1])
                p = (p[0], p[1] + (SGN[d] * lim[k] - p[1])) if d in (1, 3) else (p[0] + (SGN[d] * lim[k] - p[0]), p[1])
                if d == 2:
                    refm[k], dlt[k] = (rz.ni, rz.nj), (rz.dI, rz.dJ)
                emit(rz)
            P = POLICY[PRE2]
            rz.pol, rz.im = PRE2, last
            rz.from_end_coord_base(p, SGN[d] * maxF, CDIR[d], bases[d], "i", dfI0 * P[0], dfJ0 * P[1])
            if d == 2:
                refm[P1], dlt[P1] = (rz.ni, rz.nj), (rz.dI, rz.dJ)
            emit(rz)
        izm[P1] = last
        if diag:                                                # BsaMesherImpl.F90:924-1279
            assert not mode_base, "BASE pre mesh mode not yet implemented"
            dS2_2 = 2.0 * d2

            def emit_tri(t):  # compute: isosceles, equal refinements
                t.check_compute()
                dumped.append(dict(tri=True, C=t.C, A=t.A, B=t.B, rot=t.rot, ni=t.ni, nj=t.nj, pol=t.pol,
                                   im=t.im))

            P = POLICY[PADI]
            for d in range(1, 2 if half else 3):               # internal padding NE (, SW)
                rz = Rect()
                rz.im = 0
                rz.set_rotation(ROT[2 * d])
                rz.pol = PADI
                r = SGN[2 * d] * maxF
                rz.from_deltas_max(base_pts[2 * d], dfI0 * P[0], dfJ0 * P[1], r, r)
                emit(rz)
            bpd = list(base_pts)
            bpd[2] = bpd[1]
            bpd[1] = bpd[3]
            trots = [None, PId2 + PI / 4.0, PIt3d2 + PI / 4.0]
            for d in range(1, 2 if half else 3):               # diagonal crests SE (, NW)
                S = SGN[2 * d]
                tdel = dS2_2 * S
                tz = Tri()
                limI, limJ = bpd[d]
                ptI = (limI + tdel, limJ)
                ptA = (limI, limJ - tdel)
                tz.im = 1
                tz.set_refinements(bkg.ni, bkg.nj, False, sticky)
                tz.pol = PEAK
                tz.define(bpd[d], ptI, ptA)
                emit_tri(tz)
                trot = trots[d]
                k0 = 1
                while abs(ptI[0]) > lim[k0] and k0 <= NL:
                    k0 += 1
                warn = k0 == NL + 1
                vals = [trot - trots[1], trot + trots[1]]
                rots = [vals[i % 2] for i in range(2 * P1)]
                idrot = 0
                rz = Rect()
                rz.im = 0
                iim = 1
                for k in range(k0, P1 + 1):
                    lk = lim[k]
                    rz.set_refinements(bkg.ni, refm[k][1], False, sticky)
                    rz.im = iim
                    rz.set_rotation(trot)
                    rz.pol = pol[k]
                    rz.from_end_coord_base_norm(ptI, -lk * S, "j", base_b, "i", False)
                    emit(rz)
                    ptA, ptB, ptE = rz.a_point(), rz.b_point(), rz.E
                    pl = CREST if pol[k] == PEAK else BASIN
                    tz.im = iim
                    n = im[iim]
                    iim += 1 if n < 0 else n + 1
                    ptI = (lk * S, rz.I[1])
                    tz.set_refinements(rz.nj, rz.nj, False, sticky)
                    tz.pol = pl
                    tz.define(ptI, ptA, rz.I)
                    emit_tri(tz)
                    rtmp = tz.base_i()
                    rz.set_rotation(rots[idrot])
                    idrot += 1
                    rz.pol = pl
                    dP = POLICY[pl]
                    rz.from_end_coord_base(rz.I, limJ, "j", rtmp, "i", dlt[k][1] * dP[0], dlt[k][1] * dP[1])
                    emit(rz)
                    ptI = (ptB[0], -lk * S)
                    tz.define(ptI, ptB, ptE)
                    emit_tri(tz)
                    rz.set_rotation(rots[idrot])
                    idrot += 1
                    rz.from_end_coord_base(tz.C, limI, "i", rtmp, "i", dlt[k][1] * dP[0], dlt[k][1] * dP[1])
                    emit(rz)
                    ptI = ptA
                if not warn:                                    # closing triangle
                    tz.im = last
                    tz.pol = PEAK
                    dP = POLICY[PEAK]
                    tz.set_refinements(bkgrfmt * dP[0], bkgrfmt * dP[1], False, sticky)
                    ptI = (maxF * S, -maxF * S)
                    tz.define(ptI, (ptI[0] - dS2_2 * S, ptI[1]), (ptI[0], ptI[1] + dS2_2 * S))
                    emit_tri(tz)
        bp = [None, base_pts[2], base_pts[3], base_pts[4], base_pts[1]]    # quadrants
        init = bp[1][0]
        mrefs = max(refm[1])
        bch = [None, "i", "j", "i", "j"]
        for d in range(1, (3 if half else 5) if not diag else 1):  # quadrants
            rz = Rect()
            rz.rot = ROT[d + 1]
            rz.pol = pol[1]
            rb = lim[1] - init
            assert rb > 0.0
            rz.define(bp[d], "i", rb, rb)
            rz.set_refinements(mrefs, mrefs, False, sticky)
            rz.im = 1
            emit(rz)
            pe = rz.E
            for k in range(2, P1 + 1):
                rz.im = izm[k]
                rb = lim[k] - lim[k - 1]
                p = pe
                rz.pol = pol[k]
                dm = min(dlt[k])
                rz.rot = ROT[d + 1]
                rz.from_end_coord_base(p, LEFT[d] * lim[k], "j", rb, bch[d], dm, dm)
                emit(rz)
                pe = rz.E
                dm = dlt[k][1]
                rz.rot = ROT[d]
                rz.from_end_coord_base(p, LEFT[d] * init, bch[d], rb, "i", dm, dm)
                emit(rz)
                rz.rot = ROT[d + 2]
                rz.from_end_coord_base(p, SGN[d] * init, bch[5 - d], rb, "j", dm, dm)
                emit(rz)
        if fcov == 1:                                           # external padding
            P = POLICY[PADE]
            bpp = [None, (0.0 if half else -maxF, maxF), (maxF, maxF), (maxF, -maxF), (-maxF, -maxF)]
            mext = [None, max_ext, max_ext, 0.0 if half else max_ext, max_ext]
            for d in range(1, 4 if half else 5):
                rz = Rect()
                rz.im, rz.pol, rz.rot = last, PADE, ROT[d + 1]
                rz.from_deltas_max(bpp[d], dfI0 * P[0], dfJ0 * P[1], SGN[d] * mext[d], LEFT[d] * max_ext)
                emit(rz)
    out = []
    for z in dumped:                                            # post-mesh lattices
        if z.get("tri"):                                        # interpolateTZ_HTPC_v3 (triang.py)
            _, _, bi, bj, ri, rj, lv = POLICY[z["pol"]]
            if not mlr:
                lv, bi, bj = 0, 1, 1
            out.append(dict(tri=True, C=z["C"], A=z["A"], B=z["B"], rot=z["rot"], ni=z["ni"], nj=z["nj"],
                            pol=z["pol"], sym=isym, bfi=bi, bfj=bj, bri=ri, brj=rj, nlevs=lv))
            continue
        dI0, dJ0 = z["bI"] / (z["ni"] - 1), z["bJ"] / (z["nj"] - 1)
        dfi, dfj, bi, bj, ri, rj, lv = POLICY[z["pol"]]
        if not mlr:
            lv, bi, bj = 0, 1, 1
        if visual:
            lv = 0
        si, sj = bi ** lv, bj ** lv
        dIr, dJr = dI0 / si, dJ0 / sj
        if validate and not visual:
            idx = z["im"] or 1
            n = im[idx] if im is not None else 0
            if n == PRE_OK:
                dw = bkgw
            else:
                if n < 0:
                    idx += 1
                    n = im[idx]
                dw = min((peak_ext[m] for m in im[idx + 1: idx + n + 1]), default=math.inf) if im else math.inf
            if dIr > dw / bi:
                while dIr > dw / bi:
                    si += 1
                    dIr = dI0 / si
            else:
                while dIr < dw / bi and si > 1:
                    si -= 1
                    dIr = dI0 / si
            if dJr > dw / bj:
                while dJr > dw / bj:
                    sj += 1
                    dJr = dJ0 / sj
            else:
                while dJr < dw / bj and sj > 1:
                    sj -= 1
                    dJr = dJ0 / sj
        # getUnaryDeltas (M2DPolygZone.F90:172-226) from the init point, its coordinates
        # exchanged for rot in [pi/2, pi) and [3 pi/2, 2 pi) (_shared_poly2d.fi:873-900)
        r = z["rot"]
        if r < PId2:
            c, s = math.cos(r), math.sin(r)
            ax = (c, -s, s, c)
        elif r < PI:
            a = r - PId2
            c, s = math.cos(a), math.sin(a)
            ax = (-c, -s, -s, c)
        elif r < PIt3d2:
            a = r - PI
            c, s = math.cos(a), math.sin(a)
            ax = (-c, s, -s, -c)
        else:
            a = r - PIt3d2
            c, s = math.cos(a), math.sin(a)
            ax = (c, s, s, -c)
        f0 = (z["I"][1], z["I"][0]) if (PId2 <= r < PI or PIt3d2 <= r < PIt2) else z["I"]
        out.append((f0[0], f0[1], ax[0] * dIr, ax[1] * dIr, ax[2] * dJr, ax[3] * dJr,
                    (z["ni"] - 1) * si + 1, (z["nj"] - 1) * sj + 1, ri, rj, z["pol"], isym))
    return out


def unmirror(z):
    """The geometric zone of an evaluated rectangle (the walk of a zone with rot in [pi/2, pi)
    or [3 pi/2, 2 pi) evaluates the mirror image of the zone through f1 = f2, whose lattice has
    the opposite orientation)."""
    fi0, fj0, dIi, dIj, dJi, dJj = z[:6]
    if dIi * dJj - dIj * dJi < 0.0:
        return (fj0, fi0, dIj, dIi, dJj, dJi) + tuple(z[6:])
    return tuple(z)


def layout_for(prob, modes, validate=True, mlr=True, restrict=False, diag=False, mode_base=False, visual=False):
    """layout() for a bsalib_gb300 Problem and its kept modes (1-based); spatial symmetry from
    prob.settings.bispsym."""
    import numpy as np
    s = prob.settings
    return layout([int(m) for m in modes], list(prob.natf), list(prob.xsi),
                  list(np.asarray(prob.L, dtype=float).reshape(-1, order="F")), list(prob.UBref), s.bkgrfmt,
                  s.bkgaext, s.genpaext, s.maxaext, s.fcov, validate, mlr, restrict, s.bispsym, diag, mode_base,
                  visual)
