"""Triangular Mesher zones on the CPU: the oracle's literal restatement of the reference's
triangle (oracle/triang.py) and the library's host-side trace of it (bsa_gpu_mshTriangLattice,
bsalib_gb300/csrc/bsa_triang.cu), which the device integration consumes.

The trace is checked against the literal routine with vector-valued test functions standing in
for the force bispectrum and the FRF product, so every weight, interpolation share, coordinate
and export record is compared, not only totals."""
import math

import numpy as np
import pytest

from bsalib_gb300 import api
from bsalib_gb300.problem import bridge_deck, cantilever_tower, tall_building
from oracle import triang as T
from oracle.oracle import Oracle
from oracle.premesh import BASIN, CONST, CREST, PADI, PEAK, POLICY, PRE2, layout_for, unmirror

S2 = 0.3 / math.sqrt(2.0)
# (C, P1, P2): rotations 0, pi/2, 3 pi/2 and a 45-degree one
SHAPES = [((0.0, 0.0), (0.0, 0.4), (0.4, 0.0)), ((0.5, -0.5), (0.8, -0.5), (0.5, -0.8)),
          ((1.0, 1.0), (0.7, 1.0), (1.0, 1.3)), ((0.2, 0.1), (0.2 + S2, 0.1 + S2), (0.2 + S2, 0.1 - S2))]


def g(fi, fj):  # stands in for B_F(fi, fj)
    return np.array([1.0, fi, fj, fi * fi, fi * fj, math.sin(3 * fi) * math.cos(2 * fj)])


def h(fi, fj):  # stands in for the FRF product at (fi, fj)
    return np.array([1.0, math.cos(fi), math.sin(fj), fi + fj, 2.0, math.exp(-fi * fi)])


def tri(shape, n, pol):
    tz = T.Tri()
    tz.set_refinements(n, n, True, [False])
    tz.define(*shape)
    tz.pol = pol
    return tz


def to_abi(tz, n, pol):
    _, _, bi, bj, ri, rj, lv = POLICY[pol]
    return api.Triangle(Ci=tz.C[0], Cj=tz.C[1], Ai=tz.A[0], Aj=tz.A[1], Bi=tz.B[0], Bj=tz.B[1], rot=tz.rot,
                        sym=1.0, n=n, policy=pol, bfm_i=bi, bfm_j=bj, bfm_levels=lv, brm_i=ri, brm_j=rj, seq=0)


def test_oracle_const_policy_weights_cover_the_triangle():
    """Without refinement (policy CONST: BFM and BRM factors 1) the routine's weights add up to
    the triangle's area in (rad/s)^2, on the BFM and on the BRM lattice."""
    for shape in SHAPES:
        for n in (2, 3, 6):
            tz = tri(shape, n, CONST)
            t = tz.dump()
            one = lambda fi, fj: np.array([1.0])
            mf, mr, nb, nq, oob = T.interp(t, True, False, [one(*p) for p in T.lv0_points(t)], one,
                                           lambda fi, fj, v: v)
            area = (tz.base_i() * 2 * math.pi) ** 2 / 2
            assert mf[0] == pytest.approx(area, rel=1e-12) and mr[0] == pytest.approx(area, rel=1e-12)
            assert nb == nq == n * (n + 1) // 2 and not oob


def test_oracle_quirks():
    """The restated routine keeps the reference's behaviour: for rot in [pi/2, pi) the walk
    starts from C with its coordinates exchanged but steps along the geometric sides; with a BRM
    factor above 1 the pre-mesh line's interpolated lines run the full BRM line length, past
    the routine's brm(:, nPtsPost) work array."""
    tz = tri(SHAPES[1], 3, CONST)
    assert tz.rot == pytest.approx(math.pi / 2)
    pts = T.lv0_points(tz.dump())
    assert pts[0] == (tz.C[1], tz.C[0])
    assert pts[1][0] > pts[0][0] and pts[1][1] == pts[0][1]          # CA runs along +f1
    t = tri(SHAPES[0], 3, PADI).dump()                               # BRM factor 2
    one = lambda fi, fj: np.array([1.0])
    *_, oob = T.interp(t, True, False, [one(*p) for p in T.lv0_points(t)], one, lambda fi, fj, v: v)
    assert oob


def lib_eval(L):
    bf, q = L["bfm"], L["brm"]
    G = np.array([g(a, b) for a, b, _ in bf])
    mf = (bf[:, 2:3] * G).sum(0)
    vals = np.zeros((len(q), 6))
    for r in range(len(q)):
        k0, k1 = L["qptr"][r], L["qptr"][r + 1]
        vals[r] = h(q[r, 0], q[r, 1]) * (L["qc"][k0:k1, None] * G[L["qsrc"][k0:k1]]).sum(0)
    mr = (q[:, 2:3] * vals).sum(0)
    ex = [(L["exp"][e, 0], L["exp"][e, 1], vals[L["eq"][e]] if L["eq"][e] >= 0 else np.zeros(6))
          for e in range(len(L["eq"]))]
    return mf, mr, ex


@pytest.mark.parametrize("pol", [CONST, PADI, BASIN, CREST, PEAK, PRE2])
@pytest.mark.parametrize("visual", [False, True], ids=["run", "visual"])
def test_library_trace_vs_oracle(bsalib, pol, visual):
    """bsa_gpu_mshTriangLattice against the literal routine: m3mf / m3mr of the test functions,
    every export record (coordinates and value), the point counts and the work-array flag."""
    for shape in SHAPES:
        for n in (2, 3, 5):
            tz = tri(shape, n, pol)
            t = tz.dump()
            L = api.triangle_lattice(to_abi(tz, n, pol), visual)
            rec = []
            mf, mr, nb, nq, oob = T.interp(t, True, visual, [g(*p) for p in T.lv0_points(t)], g,
                                           lambda fi, fj, v: v * h(fi, fj), lambda a, b, v: rec.append((a, b, v)))
            lmf, lmr, lex = lib_eval(L)
            np.testing.assert_allclose(lmf, mf, rtol=1e-12, atol=1e-12 * np.abs(mf).max())
            np.testing.assert_allclose(lmr, mr, rtol=1e-12, atol=1e-12 * np.abs(mr).max())
            assert (nb, nq, oob) == (L["bfm_post"], L["brm_post"], L["oob"])
            assert len(rec) == len(lex)
            for (a1, a2, av), (b1, b2, bv) in zip(rec, lex):
                assert abs(a1 - b1) < 1e-12 and abs(a2 - b2) < 1e-12
                np.testing.assert_allclose(bv, av, rtol=1e-12, atol=1e-14)


def test_library_trace_rejects_bad_input(bsalib):
    t = to_abi(tri(SHAPES[0], 3, CONST), 3, CONST)
    t.n = 1
    with pytest.raises(api.BsaError):
        api.triangle_lattice(t)


def diag_cases():
    return [("tower", cantilever_tower(nodes=8)), ("building", tall_building(nodes=20, modes=6, nfreqs=9, df=0.5, seed=3))]


@pytest.mark.parametrize("name,prob", diag_cases(), ids=[c[0] for c in diag_cases()])
def test_diag_crest_layout_structure(name, prob):
    """The oracle's diagonal-crest scheme (BsaMesherImpl.F90:924-1279): background zone and
    crest bands as in the default scheme, padding rectangles over the NE / SW quadrants, and
    along each of the SE / NW diagonals a corner triangle, per zone limit a rotated crest
    rectangle with two levelling triangles and two closing rectangles, and a closing triangle;
    every triangle isosceles with equal refinements."""
    prob.settings.bispsym = 0
    o = Oracle(prob)
    zs = layout_for(prob, o.modes, diag=True)
    tris = [z for z in zs if isinstance(z, dict)]
    rects = [z for z in zs if not isinstance(z, dict)]
    base = layout_for(prob, o.modes)
    assert len(tris) > 0 and len(tris) % 2 == 0
    for t in tris:
        assert abs(T.dist(t["C"], t["A"]) - T.dist(t["C"], t["B"])) <= 1e-12 and t["ni"] == t["nj"]
    # the background zone and the first crest-band zones are the default scheme's
    assert [tuple(z) for z in rects[:5]] == [tuple(z) for z in base[:5]]
    # the crest rectangles along the diagonals step at 45 degrees to the axes
    rot = [z for z in rects if z[2] != 0.0 and abs(abs(z[2]) - abs(z[3])) < 1e-9 * abs(z[2])]
    assert len(rot) > 0


def test_diag_crest_half_symmetry_aborts():
    """With HALF spatial symmetry the background zone has unequal refinements, so the first
    diagonal triangle aborts the reference (compute_TZ_iso_, _shared_poly2d.fi:78-80)."""
    prob = cantilever_tower(nodes=8)
    prob.settings.bispsym = 2
    with pytest.raises(T.TriError):
        layout_for(prob, Oracle(prob).modes, diag=True)


def test_diag_crest_isosceles_abort():
    """A levelling triangle that is not isosceles aborts the reference (MTriangZoneImpl.F90:
    502-508): the bridge deck's limits make one."""
    prob = bridge_deck(nodes=40, modes=12, seed=5)
    prob.settings.bispsym = 0
    with pytest.raises(T.TriError, match="isosceles"):
        layout_for(prob, Oracle(prob).modes, diag=True)


def test_default_layout_mirrored_zones():
    """In the default scheme the zones with rot in [pi/2, pi) and [3 pi/2, 2 pi) are walked from
    the exchanged start point: their evaluated lattices are the mirror images (negative
    orientation) of the geometric zones, which tile the plane."""
    prob = cantilever_tower(nodes=8)
    prob.settings.bispsym = 0
    zs = layout_for(prob, Oracle(prob).modes)
    neg = [z for z in zs if z[2] * z[5] - z[3] * z[4] < 0.0]
    assert 0 < len(neg) < len(zs)
    for z in neg:
        u = unmirror(z)
        assert u[0] == z[1] and u[1] == z[0] and u[2] * u[5] - u[3] * u[4] > 0.0
