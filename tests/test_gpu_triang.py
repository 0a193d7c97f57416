"""Triangular Mesher zones and the diagonal-crest pre-mesh scheme on the GPU, against the
oracle's literal restatements (oracle/triang.py, oracle/premesh.py): the device integration of
triangles (the FP64 point kernel with each BFM point's listed BRM points), the library's layout
zone by zone, bsa_Run with the scheme, its split-precision run and its BRM export.
FP64 path: 1e-10 relative (max-norm)."""
import numpy as np
import pytest

from bsalib_gb300 import api
from bsalib_gb300.problem import cantilever_tower, tall_building
from oracle import triang as T
from oracle.oracle import Oracle
from oracle.premesh import BASIN, CONST, CREST, PEAK, POLICY, layout_for

pytestmark = pytest.mark.gpu
TOL = 1e-10
DRIVER = dict(validate=False, mlr=False, restrict=True)


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def _controls(s, ctl):
    s.lib.bsa_doValidateZoneDeltas(1 if ctl.get("validate", True) else 0)
    s.lib.bsa_setBfmMLR(1 if ctl.get("mlr", True) else 0)
    s.lib.bsa_setMaxBkgPeakRestriction(1 if ctl.get("restrict", False) else 0)


def tower():
    prob = cantilever_tower(nodes=5)
    prob.settings.suban = 2
    prob.settings.bkgrfmt = 6
    prob.settings.bispsym = 0
    return prob


def abi(t, sym=1.0):
    return api.Triangle(Ci=t["C"][0], Cj=t["C"][1], Ai=t["A"][0], Aj=t["A"][1], Bi=t["B"][0], Bj=t["B"][1],
                        rot=t["rot"], sym=sym, n=t["ni"], policy=t["pol"], bfm_i=t.get("bfi", POLICY[t["pol"]][2]),
                        bfm_j=t.get("bfj", POLICY[t["pol"]][3]), bfm_levels=t.get("nlevs", POLICY[t["pol"]][6]),
                        brm_i=t.get("bri", POLICY[t["pol"]][4]), brm_j=t.get("brj", POLICY[t["pol"]][5]), seq=0)


def test_triangles_vs_oracle(bsalib):
    """bsa_gpu_mshTriangles against the literal routine with the oracle's bispectra, for the
    four orientations and the policies the diagonal-crest scheme gives triangles."""
    prob = tower()
    o = Oracle(prob)
    shapes = [((0.05, 0.05), (0.05, 0.35), (0.35, 0.05)), ((0.3, -0.3), (0.5, -0.3), (0.3, -0.5)),
              ((-0.1, 0.2), (-0.3, 0.2), (-0.1, 0.4)), ((0.6, -0.6), (0.6, -0.9), (0.3, -0.6))]
    tris, mf, mr = [], 0.0, 0.0
    for k, shape in enumerate(shapes):
        pol = (CONST, BASIN, CREST, PEAK)[k]
        tz = T.Tri()
        tz.set_refinements(3, 3, True, [False])
        tz.define(*shape)
        tz.pol = pol
        t = tz.dump()
        a, b, *_ = T.zone(o, t, 2.0 if k == 1 else 1.0)
        mf, mr = mf + a, mr + b
        tris.append(abi(t, 2.0 if k == 1 else 1.0))
    s = api.BsaSession(prob)
    try:
        gf, gr, cnt = s.msh_triangles(tris)
    finally:
        s.close()
    assert rel(gf, mf) < TOL and rel(gr, mr) < TOL
    assert cnt[0] > 0 and cnt[1] > 0


@pytest.mark.parametrize("ctl", [dict(), DRIVER], ids=["library", "driver"])
def test_diag_layout_vs_oracle(bsalib, ctl):
    """bsa_setPremeshScheme(1): the library's rectangles and triangles against the oracle's
    restatement of the scheme, zone by zone in dump order."""
    for prob in (cantilever_tower(nodes=8), tall_building(nodes=20, modes=6, nfreqs=9, df=0.5, seed=3)):
        prob.settings.suban = 2
        prob.settings.bispsym = 0
        s = api.BsaSession(prob)
        try:
            _controls(s, ctl)
            s.set_premesh(diag_crest=True)
            zs = s.generate_zones()
            ts = s.generate_triangles()
        finally:
            s.close()
        ref = layout_for(prob, Oracle(prob).modes, diag=True, **ctl)
        rr = [z for z in ref if not isinstance(z, dict)]
        rt = [(k, z) for k, z in enumerate(ref) if isinstance(z, dict)]
        assert len(zs) == len(rr) and len(ts) == len(rt) > 0
        for z, r in zip(zs, rr):
            got = (z.fi0, z.fj0, z.dIi, z.dIj, z.dJi, z.dJj)
            assert np.allclose(got, r[:6], rtol=1e-12, atol=1e-14), (got, r)
            assert (z.ni, z.nj, z.Fi, z.Fj, z.policy, z.sym) == tuple(r[6:12])
        for t, (k, r) in zip(ts, rt):
            got = (t.Ci, t.Cj, t.Ai, t.Aj, t.Bi, t.Bj, t.rot)
            want = r["C"] + r["A"] + r["B"] + (r["rot"],)
            assert np.allclose(got, want, rtol=1e-12, atol=1e-14), (got, want)
            assert (t.n, t.policy, t.bfm_i, t.bfm_j, t.bfm_levels, t.brm_i, t.brm_j, t.seq) == \
                (r["ni"], r["pol"], r["bfi"], r["bfj"], r["nlevs"], r["bri"], r["brj"], k)


def oracle_mesher(o, ref):
    mf = np.zeros(o.nme ** 3)
    mr = np.zeros(o.nme ** 3)
    for z in ref:
        if isinstance(z, dict):
            a, b, *_ = T.zone(o, z, z["sym"])
        else:
            a, b = o.rect_zone(*z[:10], z[11])
        mf += a
        mr += b
    return mf, mr


def test_diag_mesher_run_vs_oracle(bsalib):
    """bsa_Run with the Mesher analysis in the diagonal-crest scheme equals the oracle's zone
    integration over the oracle's layout (rectangles and triangles)."""
    prob = tower()
    s = api.BsaSession(prob)
    try:
        _controls(s, DRIVER)
        s.set_premesh(diag_crest=True)
        out = s.run()
    finally:
        s.close()
    o = Oracle(prob)
    ref = layout_for(prob, o.modes, diag=True, **DRIVER)
    assert any(isinstance(z, dict) for z in ref)
    mf, mr = oracle_mesher(o, ref)
    assert rel(out["m3mf_msh"], mf) < TOL
    assert rel(out["m3mr_msh"], mr) < TOL


def test_diag_mesher_split_precision(bsalib):
    """The split-precision Mesher in the diagonal-crest scheme (axis-aligned rectangles on the
    tensor cores; rotated rectangles and triangles through the FP64 kernel) against FP64."""
    prob = tower()
    res = {}
    for prec in (api.PREC_FP64, api.PREC_BF16X3):
        s = api.BsaSession(prob, precision=prec)
        try:
            _controls(s, DRIVER)
            s.set_premesh(diag_crest=True)
            res[prec] = s.run()
        finally:
            s.close()
    for k in ("m3mf_msh", "m3mr_msh"):
        assert rel(res[api.PREC_BF16X3][k], res[api.PREC_FP64][k]) < 1e-4


def test_diag_mesher_export(bsalib):
    """The BRM export of the scheme: one block per zone in dump order; a triangle's block is the
    routine's write sequence (coordinates as written, the BRM the slot holds), against the
    oracle's literal routine with the oracle's bispectra."""
    prob = tower()
    got = []
    s = api.BsaSession(prob)
    try:
        _controls(s, DRIVER)
        s.set_premesh(diag_crest=True)
        s.set_export(lambda f1, f2, brm: got.append((f1.copy(), f2.copy(), brm.copy())))
        s.run()
        s.set_export(None)
    finally:
        s.close()
    o = Oracle(prob)
    ref = layout_for(prob, o.modes, diag=True, **DRIVER)
    assert len(got) == len(ref)
    k = next(i for i, z in enumerate(ref) if isinstance(z, dict))
    rec = []
    T.zone(o, ref[k], 1.0, write=lambda a, b, v: rec.append((a, b, v)))
    f1, f2, b = got[k]
    assert f1.size == len(rec)
    np.testing.assert_allclose(f1, [r[0] for r in rec], rtol=0, atol=1e-12)
    np.testing.assert_allclose(f2, [r[1] for r in rec], rtol=0, atol=1e-12)
    assert rel(b, np.array([r[2] for r in rec])) < TOL


def test_diag_half_symmetry_refused(bsalib):
    """HALF spatial symmetry: the first diagonal triangle has unequal refinements, which the
    reference aborts on; the library returns an error."""
    prob = tower()
    prob.settings.bispsym = 2
    s = api.BsaSession(prob)
    try:
        s.set_premesh(diag_crest=True)
        with pytest.raises(api.BsaError):
            s.run()
    finally:
        s.close()
