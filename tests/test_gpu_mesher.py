"""The Mesher path: rectangular zones (BFM lattice, bilinear BRM interpolation, trapezoid
zone weights) evaluated on the GPU in one batched pass, against the oracle's restatement of
the zone integration; the zone layout; and bsa_Run with the Mesher analysis.
FP64 path: 1e-10 relative (max-norm)."""
import numpy as np
import pytest

from bsalib_gb300 import api
from bsalib_gb300.problem import cantilever_tower, tall_building
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu
TOL = 1e-10


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def zone(fi0, fj0, dIi, dIj, dJi, dJj, ni, nj, Fi, Fj, sym=1.0):
    return api.Zone(fi0, fj0, dIi, dIj, dJi, dJj, ni, nj, Fi, Fj, sym, 0)


ZONES = [
    zone(-0.4, -0.4, 0.1, 0.0, 0.0, 0.1, 9, 9, 4, 4),              # background-like square
    zone(0.4, -0.4, 0.05, 0.0, 0.0, 0.2, 5, 5, 4, 2),              # crest-like strip
    zone(1.2, 0.6, 0.0, 0.15, -0.12, 0.0, 4, 6, 2, 3),             # swapped axes (rot 90)
    zone(-1.0, 1.0, 0.07, 0.07, 0.07, -0.07, 3, 4, 1, 2, 2.0),     # 45-degree lattice, sym 2
]


def test_zones_vs_oracle(bsalib):
    prob = tall_building(nodes=12, modes=4, nfreqs=5, df=0.3, seed=31)
    o = Oracle(prob)
    ref_f = np.zeros(o.nme ** 3)
    ref_r = np.zeros(o.nme ** 3)
    for z in ZONES:
        mf, mr = o.rect_zone(z.fi0, z.fj0, z.dIi, z.dIj, z.dJi, z.dJj, z.ni, z.nj, z.Fi, z.Fj, z.sym)
        ref_f += mf
        ref_r += mr
    s = api.BsaSession(prob)
    try:
        mf, mr, cnt = s.msh_zones(ZONES)
        st = s.stats()
    finally:
        s.close()
    assert rel(mf, ref_f) < TOL
    assert rel(mr, ref_r) < TOL
    nbfm = sum(z.ni * z.nj for z in ZONES)
    nbrm = sum(((z.ni - 1) * z.Fi + 1) * ((z.nj - 1) * z.Fj + 1) for z in ZONES)
    assert cnt[0] == nbfm and cnt[1] == nbrm and st.points == nbrm


def test_zone_with_unit_factors_is_plain_trapezoid(bsalib):
    """Fi = Fj = 1: the BRM lattice is the BFM lattice, so m3mr is the trapezoid sum of B_R."""
    prob = cantilever_tower(nfreqs=5, df=0.5, nodes=6)
    z = zone(-0.3, 0.2, 0.1, 0.0, 0.0, 0.15, 4, 3, 1, 1)
    s = api.BsaSession(prob)
    try:
        _, mr, _ = s.msh_zones([z])
        fi = np.array([z.fi0 + i * z.dIi for i in range(4) for j in range(3)])
        fj = np.array([z.fj0 + j * z.dJj for i in range(4) for j in range(3)])
        ti = np.array([0.5 if i in (0, 3) else 1.0 for i in range(4) for j in range(3)])
        tj = np.array([0.5 if j in (0, 2) else 1.0 for i in range(4) for j in range(3)])
        w = ti * tj * (0.1 * 2 * np.pi) * (0.15 * 2 * np.pi)
        _, mr2 = s.msh_moments(fi, fj, w)
    finally:
        s.close()
    assert rel(mr, mr2) < 1e-12


LAYOUT_CTL = [dict(), dict(validate=False, mlr=False, restrict=True)]


def _controls(s, ctl):
    s.lib.bsa_doValidateZoneDeltas(1 if ctl.get("validate", True) else 0)
    s.lib.bsa_setBfmMLR(1 if ctl.get("mlr", True) else 0)
    s.lib.bsa_setMaxBkgPeakRestriction(1 if ctl.get("restrict", False) else 0)


@pytest.mark.parametrize("ctl", LAYOUT_CTL, ids=["library", "driver"])
@pytest.mark.parametrize("sym", [0, 2, 4], ids=["full", "half", "fourth"])
def test_mesher_layout_vs_oracle(bsalib, ctl, sym):
    """The library's zone layout (pre-mesh and post-mesh lattices, spatial-symmetry weight)
    against the oracle's restatement, zone by zone."""
    from oracle.premesh import layout_for
    for prob in (cantilever_tower(nodes=8), tall_building(nodes=20, modes=6, nfreqs=9, df=0.5, seed=3)):
        prob.settings.suban = 2
        prob.settings.bispsym = sym
        s = api.BsaSession(prob)
        try:
            _controls(s, ctl)
            zs = s.generate_zones()
        finally:
            s.close()
        ref = layout_for(prob, Oracle(prob).modes, **ctl)
        assert len(zs) == len(ref)
        for z, r in zip(zs, ref):
            got = (z.fi0, z.fj0, z.dIi, z.dIj, z.dJi, z.dJj)
            assert np.allclose(got, r[:6], rtol=1e-12, atol=1e-14), (got, r)
            assert (z.ni, z.nj, z.Fi, z.Fj, z.policy, z.sym) == tuple(r[6:12])


def test_mesher_layout_covers_the_plane(bsalib):
    prob = cantilever_tower(nodes=8)
    prob.settings.suban = 2
    s = api.BsaSession(prob)
    try:
        zs = s.generate_zones()
    finally:
        s.close()
    assert len(zs) > 9
    area = sum(abs((z.ni - 1) * (z.nj - 1) * (z.dIi * z.dJj - z.dIj * z.dJi)) for z in zs)
    X = max(max(z.fi0, z.fi0 + (z.ni - 1) * z.dIi + (z.nj - 1) * z.dJi) for z in zs)
    assert np.isclose(area, (2 * X) ** 2, rtol=1e-10)
    assert np.isclose(X, prob.natf.max() * prob.settings.maxaext)


def test_mesher_run_vs_oracle_on_its_zones(bsalib):
    """bsa_Run with the Mesher analysis equals the oracle's zone integration over the same
    layout."""
    prob = cantilever_tower(nodes=5)
    prob.settings.suban = 2
    prob.settings.bkgrfmt = 6
    s = api.BsaSession(prob)
    try:
        _controls(s, LAYOUT_CTL[1])  # the driver's controls keep the oracle's lattice small
        out = s.run()
        zs = s.generate_zones()
    finally:
        s.close()
    o = Oracle(prob)
    ref_f = np.zeros(o.nme ** 3)
    ref_r = np.zeros(o.nme ** 3)
    for z in zs:
        mf, mr = o.rect_zone(z.fi0, z.fj0, z.dIi, z.dIj, z.dJi, z.dJj, z.ni, z.nj, z.Fi, z.Fj, z.sym)
        ref_f += mf
        ref_r += mr
    assert rel(out["m3mf_msh"], ref_f) < TOL
    assert rel(out["m3mr_msh"], ref_r) < TOL
    assert np.all(out["m3mr_cls"] == 0.0)  # analysis type 2 runs the Mesher only


def test_pod_truncation(bsalib):
    """Truncated POD (bsa_setPODNOfModesKept, bsa_setPODTruncationThreshold) against the
    oracle's restatement of getFM_full_tm_scalar_msh_POD_ with numpy's eigensolver; full-rank
    requests keep the direct form."""
    prob = tall_building(nodes=9, modes=3, nfreqs=4, df=0.5, seed=4)
    prob.settings.svd = 1  # the POD form (the reference's default Mesher function)
    o = Oracle(prob)
    fi, fj = np.array([0.3, -1.1, 0.05]), np.array([0.9, 0.4, 0.0])
    s = api.BsaSession(prob)
    try:
        L = s.lib
        assert L.bsa_setPODTruncationThreshold(100.0) == 0    # 100 % keeps every mode
        assert L.bsa_setPODNOfModesKept(prob.nnl) == 0
        bf, _ = s.msh_bispectra(fi, fj)
        for k in range(fi.size):
            assert rel(bf[k], o.direct_point(fi[k], fj[k])) < TOL
        for nkeep in (4, 1):
            assert L.bsa_setPODNOfModesKept(nkeep) == 0
            bf, _ = s.msh_bispectra(fi, fj)
            for k in range(fi.size):
                assert rel(bf[k], o.pod_point(fi[k], fj[k], nmodes=nkeep)) < 1e-9
        # the threshold takes precedence over the fixed count
        assert L.bsa_setPODTruncationThreshold(50.0) == 0
        bf, _ = s.msh_bispectra(fi, fj)
        for k in range(fi.size):
            assert rel(bf[k], o.pod_point(fi[k], fj[k], trunc_lim=0.5)) < 1e-9
    finally:
        s.close()


def test_pod_truncation_zones_split_precision(bsalib):
    """The split-precision zone path reads the same truncated expansions."""
    prob = tall_building(nodes=12, modes=4, nfreqs=5, df=0.3, seed=31)
    prob.settings.svd = 1
    out = {}
    for prec in (api.PREC_FP64, api.PREC_BF16X3):
        s = api.BsaSession(prob, precision=prec)
        try:
            assert s.lib.bsa_setPODNOfModesKept(3) == 0
            out[prec] = s.msh_zones(ZONES[:2])
        finally:
            s.close()
    full = api.BsaSession(prob, precision=api.PREC_FP64)
    try:
        mf_full, mr_full, _ = full.msh_zones(ZONES[:2])
    finally:
        full.close()
    assert rel(out[api.PREC_BF16X3][1], out[api.PREC_FP64][1]) < 1e-4
    assert rel(out[api.PREC_BF16X3][0], out[api.PREC_FP64][0]) < 1e-4
    assert rel(out[api.PREC_FP64][1], mr_full) > 1e-6


@pytest.mark.parametrize("prec,tol", [(api.PREC_FP64, 1e-10), (api.PREC_BF16X3, 1e-4)], ids=["fp64", "bf16x3"])
def test_mesher_export(bsalib, prec, tol):
    """bsa_setBispExportCallback in the Mesher analysis: one block per zone holding every BRM
    lattice point (i fastest, then j) with the bilinear interpolation of the zone's BFM lattice
    times the FRF product.  At the BFM lattice points it equals the point bispectra; summed
    with the zone integration weights it gives the analysis' m3mr (FP64 export; the analysis
    in the selected precision).  A zone whose walk exchanges its start point's coordinates
    (its evaluated lattice has negative orientation) is written with the exchange undone."""
    prob = cantilever_tower(nodes=5)
    prob.settings.suban = 2
    prob.settings.bkgrfmt = 6
    got = []
    s = api.BsaSession(prob, precision=prec)
    try:
        _controls(s, LAYOUT_CTL[1])
        zs = s.generate_zones()
        s.set_export(lambda f1, f2, brm: got.append((f1.copy(), f2.copy(), brm.copy())))
        out = s.run()
        s.set_export(None)
        ref = s.run()
        assert len(got) == len(zs)
        acc = np.zeros_like(out["m3mr_msh"])
        for z, (f1, f2, b) in zip(zs, got):
            NI, NJ = (z.ni - 1) * z.Fi + 1, (z.nj - 1) * z.Fj + 1
            assert f1.size == NI * NJ
            qi, qj = np.meshgrid(np.arange(NI), np.arange(NJ))  # qi fastest
            qi, qj = qi.ravel(), qj.ravel()
            a, c = qi / z.Fi, qj / z.Fj
            if z.dIi * z.dJj - z.dIj * z.dJi < 0.0:
                f1, f2 = f2, f1                        # back to the evaluated coordinates
            np.testing.assert_allclose(f1, z.fi0 + a * z.dIi + c * z.dJi, rtol=0, atol=1e-12)
            np.testing.assert_allclose(f2, z.fj0 + a * z.dIj + c * z.dJj, rtol=0, atol=1e-12)
            ti = np.where((qi == 0) | (qi == NI - 1), 0.5, 1.0)
            tj = np.where((qj == 0) | (qj == NJ - 1), 0.5, 1.0)
            wI = np.hypot(z.dIi, z.dIj) * 2 * np.pi / z.Fi
            wJ = np.hypot(z.dJi, z.dJj) * 2 * np.pi / z.Fj
            acc += (z.sym * wI * wJ * ti * tj) @ b
            lat = (qi % z.Fi == 0) & (qj % z.Fj == 0)
            _, br = s.msh_bispectra(f1[lat], f2[lat])
            assert rel(b[lat], br) < 1e-12
    finally:
        s.close()
    assert rel(acc, out["m3mr_msh"]) < tol
    assert rel(out["m3mr_msh"], ref["m3mr_msh"]) < 1e-12
