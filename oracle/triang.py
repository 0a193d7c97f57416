"""Triangular Mesher zones -- TEST INFRASTRUCTURE ONLY.

A literal restatement, in Python, of the reference's triangular zone, used by the tests as the
checker of the library's triangle lattices (bsalib_gb300/csrc/bsa_triang.cu) and of their zone
integration on the device:

* geometry: MTriangZone (zones/MTriangZoneImpl.F90): defineFromPts_norm (:275-346, which of the
  two points is A), deduceRotation (:157-198), getRotatedUnaryDF (:209-261), baseI / baseJ,
  the isosceles check of compute (:489-510), getTriangZoneEquivNPts (:563-573);
* pre-mesh lattice: compute_TZ_iso_ (zones/_shared_poly2d.fi:40-454, triangle branches): the
  BFM points C..A along the J side, then lines parallel to CA of one point less each, the last
  one the B point; the walk starts from C with its coordinates exchanged for rot in [pi/2, pi)
  and [3 pi/2, 2 pi) (:196-212);
* post-mesh: interpolateTZ_HTPC_v3 (zones/_shared_poly2d.fi:470-2166, triangle branches): the
  multi-level BFM refinement of the policy (BFM evaluated at the refinement points), the linear
  interpolation of the BFM onto the BRM lattice of factor max(brm_i, brm_j) along J, along I
  and, past the lattice's diagonal, from the diagonal interpolant; the BRM at every point; the
  influence weights (corner dw^2 / 4, border / 2, centre 1, the two acute vertices dw^2 / 8)
  accumulated into the zone's m3mf / m3mr; the BRM export in the routine's write order.

The routine is followed step by step, with its brm(:, slot) work array and slot arithmetic, so
that whatever a slot holds when the routine reads or writes it is what the restatement reads or
writes.  Values are numpy vectors of one length (dim_bisp); bfm(fi, fj) and brm(fi, fj, bfm)
are supplied by the caller.
"""
from __future__ import annotations

import math

import numpy as np

from .premesh import MACHINE_PRECISION, PI, PId2, PIt2, PIt3d2, POLICY, dist

CST_PIt2 = PI * 2.0


class TriError(RuntimeError):
    """A condition the reference ends with bsa_Abort."""


def rotated_unary_df(rot):
    """getRotatedUnaryDF with both optional outputs: (dfI_var, dfJ_var, dfI_cst, dfJ_cst), the
    unit steps along CA (var) and along CB (cst)."""
    if rot <= PId2:
        vi, vj = math.sin(rot), math.cos(rot)
    elif rot <= PI:
        a = rot - PId2
        vi, vj = math.cos(a), -math.sin(a)
    elif rot <= PIt3d2:
        a = rot - PI
        vi, vj = -math.sin(a), -math.cos(a)
    else:
        a = rot - PIt3d2
        vi, vj = -math.cos(a), math.sin(a)
    if abs(vi) < MACHINE_PRECISION:
        vi = 0.0
    if abs(vj) < MACHINE_PRECISION:
        vj = 0.0
    ci, cj = vj, -vi
    if abs(ci) < MACHINE_PRECISION:
        ci = 0.0
    if abs(cj) < MACHINE_PRECISION:
        cj = 0.0
    return vi, vj, ci, cj


def swaps_base(rot):
    """The lattice walks exchange the start point's coordinates for these rotations."""
    return (PId2 <= rot < PI) or (PIt3d2 <= rot < PIt2)


class Tri:
    """MTriangZone_t: corner C, A at the end of the J side CA, B at the end of the I side CB."""

    def __init__(self):
        self.C = self.A = self.B = None
        self.rot = 0.0
        self.ni = self.nj = 0
        self.pol = 0
        self.im = 0

    def set_refinements(self, ni, nj, force, sticky):
        """M2DPolygZone setRefinements (its force flag is a saved local: sticky[0])."""
        if force:
            sticky[0] = True
        if sticky[0]:
            self.ni, self.nj = ni, nj
        else:
            self.ni = ni + 1 if ni % 2 == 0 else ni
            self.nj = nj + 1 if nj % 2 == 0 else nj

    def define(self, Cp, P1, P2):
        """defineFromPts_norm."""
        if self.ni == 0 or self.nj == 0:
            raise TriError("Missing refinement information")
        if P1[1] > P2[1] or P1[1] < P2[1]:
            self.A, self.B = P1, P2
        elif P1[1] > Cp[1]:
            if P1[0] < P2[0]:
                self.A, self.B = P1, P2
            elif P2[0] < P1[0]:
                self.A, self.B = P2, P1
            else:
                raise TriError("Triangle collapsed into a segment")
        elif P1[1] < Cp[1]:
            if P1[0] > P2[0]:
                self.A, self.B = P1, P2
            elif P2[0] > P1[0]:
                self.A, self.B = P2, P1
            else:
                raise TriError("Triangle collapsed into a segment")
        else:
            raise TriError("Three points are aligned on the same line")
        self.C = (float(Cp[0]), float(Cp[1]))
        self.deduce_rotation()

    def deduce_rotation(self):
        dx = self.A[0] - self.C[0]
        dy = self.A[1] - self.C[1]
        if dy == 0.0:
            ang = math.atan(math.inf) if dx != 0.0 else math.nan
        else:
            ang = math.atan(abs(dx) / abs(dy))
        if not (dx >= 0.0 and dy >= 0.0):
            if dy < 0.0:
                ang = PI - ang if dx >= 0.0 else PI + ang
            else:
                ang = PIt2 - ang if ang > 1e-14 else 0.0
        self.rot = ang

    def base_i(self):
        return dist(self.C, self.B)

    def base_j(self):
        return dist(self.C, self.A)

    def check_compute(self):
        """compute / compute_TZ_iso_ preconditions."""
        if not abs(self.base_j() - self.base_i()) <= MACHINE_PRECISION:
            raise TriError('Triangle must be "isosceles"')
        if self.ni != self.nj:
            raise TriError("Different sides' refinements not yet allowed")

    def tot_npts(self):
        return (self.ni * self.ni + self.ni) // 2

    def dump(self):
        return {"C": self.C, "A": self.A, "B": self.B, "rot": self.rot, "ni": self.ni, "nj": self.nj,
                "pol": self.pol, "im": self.im}


def equiv_npts(ni, nj):
    """getTriangZoneEquivNPts: int((ni nj + ni) / 2.0 in single precision)."""
    return int(np.float32(ni * nj + ni) / np.float32(2.0))


def lv0_points(t):
    """compute_TZ_iso_: the pre-mesh BFM points of a dumped triangle, in dump order."""
    n = t["ni"]
    Np_m1 = n - 1
    Nj_m1 = Np_m1
    df_cst = dist(t["C"], t["A"]) / Np_m1
    dJi, dJj, dIi, dIj = rotated_unary_df(t["rot"])
    dJi, dJj, dIi, dIj = dJi * df_cst, dJj * df_cst, dIi * df_cst, dIj * df_cst
    bi, bj = t["C"]
    if swaps_base(t["rot"]):
        bi, bj = bj, bi
    pts = []
    fi, fj = bi, bj
    pts.append((fi, fj))
    for _ in range(2, Nj_m1 + 1):
        fi += dJi
        fj += dJj
        pts.append((fi, fj))
    fi += dJi
    fj += dJj
    pts.append((fi, fj))
    for _ in range(2, Np_m1 + 1):
        Nj_m1 -= 1
        bi += dIi
        bj += dIj
        fi, fj = bi, bj
        pts.append((fi, fj))
        for _ in range(2, Nj_m1 + 1):
            fi += dJi
            fj += dJj
            pts.append((fi, fj))
        fi += dJi
        fj += dJj
        pts.append((fi, fj))
    bi += dIi
    bj += dIj
    pts.append((bi, bj))
    assert len(pts) == (n * n + n) // 2
    return pts


class _Arr:
    """A Fortran array of vectors, 1-based, zero-initialised, with its declared size."""

    def __init__(self, n, dim, name):
        self.n, self.name = n, name
        self.v = {}
        self.dim = dim
        self.oob = False

    def __getitem__(self, k):
        if not 1 <= k <= self.n:
            self.oob = True
        return self.v.get(k, np.zeros(self.dim))

    def __setitem__(self, k, val):
        if not 1 <= k <= self.n:
            self.oob = True
        self.v[k] = np.array(val, dtype=np.float64)


def interp(t, mlr, visual, bfm_undump, bfm, brm, write=None):
    """interpolateTZ_HTPC_v3 for the dumped triangle t (lv0_points order in bfm_undump); the
    policy's factors from t when the layout resolved them, else from its policy id and mlr.

    Returns (intg_bfm, intg, n_bfm_post, n_brm_post, oob): the zone's m3mf and m3mr
    contributions before the i_bisp_sym_ factor, the point counts the routine adds to
    msh_bfmpts_post_ / msh_brmpts_post_, and whether a work array was indexed outside its
    declared size.  write(f1, f2, value) receives the BRM export in the routine's order."""
    dim = len(bfm_undump[0])
    if "bfi" in t:  # factors already resolved by the layout (premesh.layout)
        bfi, bfj, bri, brj, nlev = t["bfi"], t["bfj"], t["bri"], t["brj"], t["nlevs"]
    else:
        _, _, bfi, bfj, bri, brj, nlev = POLICY[t["pol"]]
        if not mlr:
            nlev, bfi, bfj = 0, 1, 1
    nsi = nsj = 1
    if not visual:
        for _ in range(nlev):
            nsi *= bfi
            nsj *= bfj
    F = max(bri, brj)
    njOld = t["nj"] - 1
    df_cst = dist(t["C"], t["A"]) / njOld
    dJi0, dJj0, dIi0, dIj0 = rotated_unary_df(t["rot"])
    dIi0, dIj0, dJi0, dJj0 = dIi0 * df_cst, dIj0 * df_cst, dJi0 * df_cst, dJj0 * df_cst
    dfI0 = dfJ0 = df_cst
    npr_i, npr_j = nsi - 1, nsj - 1
    dIi_r, dIj_r, dJi_r, dJj_r = dIi0 / nsi, dIj0 / nsi, dJi0 / nsj, dJj0 / nsj
    dIi_b, dIj_b, dJi_b, dJj_b = dIi_r / F, dIj_r / F, dJi_r / F, dJj_r / F
    dfI_r = dfI0 / nsi
    dfI_b = dfI_r / F
    dfJ_r = dfJ0 / nsj
    dfJ_b = dfJ_r / F
    dw = dfI_r * CST_PIt2
    ctr_bfm = dw * dw
    brd_bfm = ctr_bfm / 2.0
    vtx_bfm = brd_bfm / 2.0
    dw = dfI_b * CST_PIt2
    ctr = dw * dw
    brd = ctr / 2.0
    vtx = brd / 2.0
    vtx_t, vtx_t_bfm = vtx / 2, vtx_bfm / 2
    ni_r, nj_r = t["ni"] - 1, t["nj"] - 1
    njOld = nj_r
    ni = ni_r * (nsi * F) + 1
    nj = nj_r * (nsj * F) + 1
    ni_r = ni_r * nsi + 1
    nj_r = nj_r * nsj + 1
    njNew_picurr = nj
    nipI = F - 1
    nipJ = nipI
    df_diag_old = math.sqrt(dfI0 ** 2 + dfJ0 ** 2)
    df_diag_ref = df_diag_old / nsi
    df_diag_b = df_diag_ref / F
    nPtsPost = equiv_npts(ni, nj)
    B = _Arr(nPtsPost, dim, "brm")
    left = _Arr(nj, dim, "bfm_new_left")
    right = _Arr(nj - nipJ - 1, dim, "bfm_new_right")
    itp = _Arr(nj, dim, "bfm_interp")
    fbI, gbI = t["C"]
    sw = swaps_base(t["rot"])
    if sw:
        fbI, gbI = gbI, fbI

    def put(k, fi, fj, v):  # getBRM_msh(brm(:, k:k), fi, fj, v)
        B[k] = brm(fi, fj, v)

    def out(fi, fj, v):  # write_brm_fptr_(fi_ptr, fj_ptr, ...)
        if write is not None:
            write(fj, fi, v) if sw else write(fi, fj, v)

    i_brm = 1
    fi, fj = fbI, gbI
    fbJ, gbJ = fi, fj
    tail = np.array(bfm_undump[0], dtype=np.float64)
    intg_bfm = tail * vtx_bfm
    left[1] = tail
    put(1, fi, fj, tail)
    out(fi, fj, B[1])
    intg = B[1] * vtx
    # first line (J direction, C to A)
    for pJhead in range(2, t["nj"] + 1):
        for _ in range(npr_j):
            fbJ += dJi_r
            gbJ += dJj_r
            head = bfm(fbJ, gbJ)
            intg_bfm = intg_bfm + head * brd_bfm
            dh, dt = dfJ_r, 0.0
            for _ in range(nipJ):
                fi += dJi_b
                fj += dJj_b
                dt += dfJ_b
                dh -= dfJ_b
                i_brm += 1
                left[i_brm] = (head * dt + tail * dh) / dfJ_r
                put(i_brm, fi, fj, left[i_brm])
                out(fi, fj, B[i_brm])
                intg = intg + B[i_brm] * brd
            fi += dJi_b
            fj += dJj_b
            i_brm += 1
            left[i_brm] = head
            put(i_brm, fi, fj, left[i_brm])
            out(fi, fj, B[i_brm])
            intg = intg + B[i_brm] * brd
            tail = head
        head = np.array(bfm_undump[pJhead - 1], dtype=np.float64)
        intg_bfm = intg_bfm + head * brd_bfm
        dh, dt = dfJ_r, 0.0
        for _ in range(nipJ):
            fi += dJi_b
            fj += dJj_b
            dt += dfJ_b
            dh -= dfJ_b
            i_brm += 1
            left[i_brm] = (head * dt + tail * dh) / dfJ_r
            put(i_brm, fi, fj, left[i_brm])
            out(fi, fj, B[i_brm])
            intg = intg + B[i_brm] * brd
        fi += dJi_b
        fj += dJj_b
        i_brm += 1
        left[i_brm] = head
        put(i_brm, fi, fj, left[i_brm])
        out(fi, fj, B[i_brm])
        intg = intg + B[i_brm] * brd
        tail = head
        fbJ, gbJ = fi, fj
    intg = intg - B[i_brm] * vtx_t
    intg_bfm = intg_bfm - tail * vtx_t_bfm
    i_bfm_old = t["nj"]
    # lines parallel to CA, one lv0 line at a time, each preceded by its BFM refinement lines
    for _pIcurr in range(2, t["ni"] + 1):
        for i_bfm_ref_i in range(1, npr_i + 1):
            i_brm_shift = i_brm
            njNew_tmp = njNew_picurr
            for _ in range(nipI):
                njNew_tmp -= 1
                i_brm_shift += njNew_tmp
            i_brm_write = i_brm_shift
            fbJ, gbJ = fbI + dIi_r, gbI + dIj_r
            fi, fj = fbJ, gbJ
            tail = bfm(fi, fj)
            intg_bfm = intg_bfm + tail * brd_bfm
            right[1] = tail
            i_brm_shift += 1
            put(i_brm_shift, fi, fj, right[1])
            intg = intg + B[i_brm_shift] * brd
            ij = 1
            for _pJhead in range(2, njOld + 1):
                for _ in range(npr_j):
                    fbJ += dJi_r
                    gbJ += dJj_r
                    head = bfm(fbJ, gbJ)
                    intg_bfm = intg_bfm + head * ctr_bfm
                    dh, dt = dfJ_r, 0.0
                    for _ in range(nipJ):
                        fi += dJi_b
                        fj += dJj_b
                        dt += dfJ_b
                        dh -= dfJ_b
                        ij += 1
                        right[ij] = (head * dt + tail * dh) / dfJ_r
                        i_brm_shift += 1
                        put(i_brm_shift, fi, fj, right[ij])
                        intg = intg + B[i_brm_shift] * ctr
                    fi += dJi_b
                    fj += dJj_b
                    ij += 1
                    right[ij] = head
                    i_brm_shift += 1
                    put(i_brm_shift, fi, fj, right[ij])
                    intg = intg + B[i_brm_shift] * ctr
                    tail = head
                fbJ += dJi_r
                gbJ += dJj_r
                head = bfm(fbJ, gbJ)
                intg_bfm = intg_bfm + head * vtx_bfm
                dh, dt = dfJ_r, 0.0
                for _ in range(nipJ):
                    fi += dJi_b
                    fj += dJj_b
                    dt += dfJ_b
                    dh -= dfJ_b
                    ij += 1
                    right[ij] = (head * dt + tail * dh) / dfJ_r
                    i_brm_shift += 1
                    put(i_brm_shift, fi, fj, right[ij])
                    intg = intg + B[i_brm_shift] * ctr
                fi += dJi_b
                fj += dJj_b
                ij += 1
                right[ij] = head
                i_brm_shift += 1
                put(i_brm_shift, fi, fj, right[ij])
                intg = intg + B[i_brm_shift] * ctr
                tail = head
            for _ in range(1, npr_j - (i_bfm_ref_i - 1) + 1):
                fbJ += dJi_r
                gbJ += dJj_r
                head = bfm(fbJ, gbJ)
                intg_bfm = intg_bfm + head * ctr_bfm
                dh, dt = dfJ_r, 0.0
                for _ in range(nipJ):
                    fi += dJi_b
                    fj += dJj_b
                    dt += dfJ_b
                    dh -= dfJ_b
                    ij += 1
                    right[ij] = (head * dt + tail * dh) / dfJ_r
                    i_brm_shift += 1
                    put(i_brm_shift, fi, fj, right[ij])
                    intg = intg + B[i_brm_shift] * ctr
                fi += dJi_b
                fj += dJj_b
                ij += 1
                right[ij] = head
                i_brm_shift += 1
                put(i_brm_shift, fi, fj, right[ij])
                intg = intg + B[i_brm_shift] * ctr
                tail = head
            njNew_piprev = njNew_picurr
            njNew_picurr = ij
            dfJ_oldtmp = dfJ0
            njtmp = nipJ
            intg = intg - B[i_brm_shift] * brd
            intg_bfm = intg_bfm - tail * brd_bfm
            dIcurr, dIprev = dfI_r, 0.0
            for pIprev in range(1, nipI + 1):
                dIprev += dfI_b
                dIcurr -= dfI_b
                for k in range(1, njNew_picurr + 1):
                    itp[k] = (left[k] * dIcurr + right[k] * dIprev) / dfI_r
                fi = fbI + dIi_b * pIprev
                fj = gbI + dIj_b * pIprev
                i_brm += 1
                put(i_brm, fi, fj, itp[1])
                out(fi, fj, B[i_brm])
                intg = intg + B[i_brm] * brd
                for pJtail in range(2, njNew_picurr + 1):
                    fi += dJi_b
                    fj += dJj_b
                    i_brm += 1
                    put(i_brm, fi, fj, itp[pJtail])
                    out(fi, fj, B[i_brm])
                    intg = intg + B[i_brm] * ctr
                head = (left[njNew_piprev] * (df_diag_b * pIprev) +
                        right[njNew_picurr] * (df_diag_b * (nipI + 1 - pIprev))) / df_diag_ref
                njtmp -= 1
                dfJ_oldtmp -= dfJ_b
                dh, dt = dfJ_oldtmp, 0.0
                ipos = njNew_picurr
                for _ in range(njtmp):
                    fi += dJi_b
                    fj += dJj_b
                    dt += dfJ_b
                    dh -= dfJ_b
                    ipos += 1
                    itp[ipos] = (head * dt + dh * itp[njNew_picurr]) / dfJ_oldtmp
                    i_brm += 1
                    put(i_brm, fi, fj, itp[ipos])
                    out(fi, fj, B[i_brm])
                    intg = intg + B[i_brm] * ctr
                fi += dJi_b
                fj += dJj_b
                i_brm += 1
                put(i_brm, fi, fj, head)
                out(fi, fj, B[i_brm])
                intg = intg + B[i_brm] * vtx_t
            fbI += dIi_r
            gbI += dIj_r
            fi, fj = fbI, gbI
            for _ in range(nj):
                i_brm_write += 1
                out(fi, fj, B[i_brm_write])
                fi += dJi_b
                fj += dJj_b
            for k in range(1, njNew_picurr + 1):
                left[k] = right[k]
            i_brm = i_brm_shift
        # the lv0 line
        i_brm_shift = i_brm
        njNew_tmp = njNew_picurr
        for _ in range(nipI):
            njNew_tmp -= 1
            i_brm_shift += njNew_tmp
        i_brm_write = i_brm_shift
        fbJ, gbJ = fbI + dIi_r, gbI + dIj_r
        fi, fj = fbJ, gbJ
        i_bfm_old += 1
        tail = np.array(bfm_undump[i_bfm_old - 1], dtype=np.float64)
        intg_bfm = intg_bfm + tail * brd_bfm
        right[1] = tail
        i_brm_shift += 1
        put(i_brm_shift, fi, fj, right[1])
        intg = intg + B[i_brm_shift] * brd
        ij = 1
        for _pJhead in range(2, njOld + 1):
            for _ in range(npr_j):
                fbJ += dJi_r
                gbJ += dJj_r
                head = bfm(fbJ, gbJ)
                intg_bfm = intg_bfm + head * ctr_bfm
                dh, dt = dfJ_r, 0.0
                for _ in range(nipJ):
                    fi += dJi_b
                    fj += dJj_b
                    dt += dfJ_b
                    dh -= dfJ_b
                    ij += 1
                    right[ij] = (head * dt + tail * dh) / dfJ_r
                    i_brm_shift += 1
                    put(i_brm_shift, fi, fj, right[ij])
                    intg = intg + B[i_brm_shift] * ctr
                fi += dJi_b
                fj += dJj_b
                ij += 1
                right[ij] = head
                i_brm_shift += 1
                put(i_brm_shift, fi, fj, right[ij])
                intg = intg + B[i_brm_shift] * ctr
                tail = head
            fi, fj = fbJ, gbJ
            fbJ += dJi_r
            gbJ += dJj_r
            i_bfm_old += 1
            head = np.array(bfm_undump[i_bfm_old - 1], dtype=np.float64)
            intg_bfm = intg_bfm + head * ctr_bfm
            dh, dt = dfJ_r, 0.0
            for _ in range(nipJ):
                fi += dJi_b
                fj += dJj_b
                dt += dfJ_b
                dh -= dfJ_b
                ij += 1
                right[ij] = (head * dt + tail * dh) / dfJ_r
                i_brm_shift += 1
                put(i_brm_shift, fi, fj, right[ij])
                intg = intg + B[i_brm_shift] * ctr
            fi += dJi_b
            fj += dJj_b
            ij += 1
            right[ij] = head
            i_brm_shift += 1
            put(i_brm_shift, fi, fj, right[ij])
            intg = intg + B[i_brm_shift] * ctr
            tail = head
        intg = intg - B[i_brm_shift] * brd
        intg_bfm = intg_bfm - tail * brd_bfm
        njNew_piprev = njNew_picurr
        njNew_picurr = ij
        dfJ_oldtmp = dfJ_r
        njtmp = nipJ
        dIcurr, dIprev = dfI_r, 0.0
        for pIprev in range(1, nipI + 1):
            dIprev += dfI_b
            dIcurr -= dfI_b
            for k in range(1, njNew_picurr + 1):
                itp[k] = (left[k] * dIcurr + right[k] * dIprev) / dfI_r
            fi = fbI + dIi_b * pIprev
            fj = gbI + dIj_b * pIprev
            i_brm += 1
            put(i_brm, fi, fj, itp[1])
            out(fi, fj, B[i_brm])
            intg = intg + B[i_brm] * brd
            for pJtail in range(2, nj + 1):  # nj, as written for this block
                fi += dJi_b
                fj += dJj_b
                i_brm += 1
                put(i_brm, fi, fj, itp[pJtail])
                out(fi, fj, B[i_brm])
                intg = intg + B[i_brm] * ctr
            head = (left[njNew_piprev] * (df_diag_b * pIprev) +
                    right[njNew_picurr] * (df_diag_b * (nipI + 1 - pIprev))) / df_diag_ref
            njtmp -= 1
            dfJ_oldtmp -= dfJ_b
            dh, dt = dfJ_oldtmp, 0.0
            ipos = njNew_picurr
            for _ in range(njtmp):
                fi += dJi_b
                fj += dJj_b
                dt += dfJ_b
                dh -= dfJ_b
                ipos += 1
                itp[ipos] = (head * dt + dh * itp[njNew_picurr]) / dfJ_oldtmp
                i_brm += 1
                put(i_brm, fi, fj, itp[ipos])
                out(fi, fj, B[i_brm])
                intg = intg + B[i_brm] * ctr
            fi += dJi_b
            fj += dJj_b
            i_brm += 1
            put(i_brm, fi, fj, head)
            out(fi, fj, B[i_brm])
            intg = intg + B[i_brm] * vtx_t
        i_brm = i_brm_shift
        fbI += dIi_r
        gbI += dIj_r
        fi, fj = fbI, gbI
        for _ in range(njNew_picurr):
            i_brm_write += 1
            out(fi, fj, B[i_brm_write])
            fi += dJi_b
            fj += dJj_b
        njOld -= 1
        for k in range(1, njNew_picurr + 1):
            left[k] = right[k]
    intg = intg - B[i_brm] * vtx_t
    intg_bfm = intg_bfm - tail * vtx_t_bfm
    oob = B.oob or left.oob or right.oob or itp.oob
    return intg_bfm, intg, equiv_npts(ni_r, nj_r), nPtsPost, oob


def zone(o, t, sym, mlr=True, visual=False, write=None):
    """One triangle's (m3mf, m3mr) contribution with the oracle's point bispectra (o: Oracle):
    the pre-mesh BFM, the post-mesh interpolation, times i_bisp_sym_."""
    undump = [o.msh_bfm(fi, fj) for fi, fj in lv0_points(t)]
    mf, mr, nb, nq, oob = interp(t, mlr, visual, undump, o.msh_bfm,
                                 lambda fi, fj, v: o.msh_brm(fi, fj, v).reshape(-1), write)
    return mf * sym, mr * sym, nb, nq, oob
