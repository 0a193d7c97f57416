"""Diagonal-only spectra (bsa_setSpectraExtension(1): same node, same mode) on the GPU
through the C-ABI, against the oracle's restatement of the reference's diagonal functions
(functionsImpl.F90:1123-1286, 1747-2101, 2460-2637).  FP64 path: 1e-10 relative (max-norm)."""
import dataclasses

import numpy as np
import pytest

from bsalib_gb300 import api
from bsalib_gb300.dist import MOMENT_KEYS, shard_rows
from bsalib_gb300.problem import cantilever_tower, tall_building
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu
TOL = 1e-10


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def diag(prob):
    prob.settings.onlyd = 1
    return prob


def two_dof(prob):
    nn, nm = prob.nn, prob.nm
    phi = np.zeros((2 * nn, nm), order="F")
    phi[0::2] = prob.phi
    phi[1::2] = 0.6 * prob.phi[::-1]
    wfc = np.zeros((2,) + prob.wfc.shape[1:], order="F")
    wfc[0] = prob.wfc[0]
    wfc[1] = 0.35 * prob.wfc[0]
    return dataclasses.replace(prob, nlibs=2, libs_load=np.array([1, 2], dtype=np.int32), phi=phi, wfc=wfc,
                               ndofs=2 * nn)


PROBLEMS = [
    ("tower", lambda: diag(cantilever_tower(nfreqs=9, df=0.25, nodes=12))),
    ("building_2tc", lambda: diag(tall_building(nodes=40, modes=6, nfreqs=9, df=0.3, seed=4))),
    ("tower_2dof", lambda: diag(two_dof(cantilever_tower(nfreqs=7, df=0.3, nodes=9)))),
]


@pytest.fixture
def session(bsalib):
    made = []

    def make(prob, **kw):
        s = api.BsaSession(prob, **kw)
        made.append(s)
        return s

    yield make
    for s in made:
        s.close()


@pytest.mark.parametrize("name,make", PROBLEMS)
def test_classic_diag_moments_vs_oracle(session, name, make):
    prob = make()
    s = session(prob)
    assert s.dims() == (s.nmodes(), s.nmodes())
    out = s.run()
    ref = Oracle(prob).classic_vect_diag(keep_bisp=False)
    for k in ("m2mf", "m2mr", "m2o2mr", "m3mf", "m3mr"):
        assert rel(out[k + "_cls"], ref[k]) < TOL, k


def test_classic_diag_bispectra_vs_oracle(session):
    prob = diag(tall_building(nodes=20, modes=5, nfreqs=7, df=0.3, seed=9))
    f, bf, br = session(prob).classic_bispectra()
    ref = Oracle(prob).classic_vect_diag()
    np.testing.assert_array_equal(f, ref["f"])
    assert rel(bf, ref["bf"]) < TOL
    assert rel(br, ref["br"]) < TOL


def test_classic_diag_scalar_vs_oracle(session):
    prob = diag(tall_building(nodes=24, modes=5, nfreqs=7, df=0.3, seed=3))
    prob.settings.scalar = 1
    out = session(prob).run()
    ref = Oracle(prob).classic_scalar_diag()
    for k in ("m2mf", "m2mr", "m2o2mr", "m3mf", "m3mr"):
        assert rel(out[k + "_cls"], ref[k]) < TOL, k


def test_diag_ignores_split_precision(session):
    """The diagonal-only contraction is O(K nm) per point and always runs in FP64."""
    prob = diag(tall_building(nodes=30, modes=8, nfreqs=9, df=0.3, seed=6))
    out = session(prob, precision=api.PREC_BF16X3).run()
    ref = Oracle(prob).classic_vect_diag(keep_bisp=False)
    assert rel(out["m3mr_cls"], ref["m3mr"]) < TOL


def test_diag_row_shards_sum_to_full_grid(bsalib):
    prob = diag(tall_building(nodes=30, modes=6, nfreqs=9, df=0.3, seed=12))
    s = api.BsaSession(prob)
    try:
        full = s.run()
        acc = {k: np.zeros_like(full[k]) for k in MOMENT_KEYS}
        for r in range(3):
            s.set_rows(*shard_rows(prob.classic_nf(), r, 3))
            part = s.run()
            for k in MOMENT_KEYS:
                acc[k] += part[k]
    finally:
        s.close()
    for k in MOMENT_KEYS:
        assert rel(acc[k], full[k]) < 1e-12, k


@pytest.mark.parametrize("name,make", PROBLEMS)
def test_mesher_diag_points_vs_oracle(session, name, make):
    prob = make()
    o = Oracle(prob)
    rng = np.random.default_rng(1)
    fi = rng.uniform(-2.0, 2.0, 37)
    fj = rng.uniform(-2.0, 2.0, 37)
    bfm, brm = session(prob).msh_bispectra(fi, fj)
    for p in range(fi.size):
        b = o.msh_bfm_diag(fi[p], fj[p])
        assert rel(bfm[p], b) < TOL
        assert rel(brm[p], o.msh_brm_diag(fi[p], fj[p], b)[:, 0]) < TOL


def test_mesher_diag_zones_and_run_vs_oracle(session):
    prob = diag(cantilever_tower(nodes=6))
    prob.settings.suban = 2
    prob.settings.bkgrfmt = 6
    s = session(prob)
    out = s.run()
    zs = s.generate_zones()
    mf, mr, _ = s.msh_zones(zs)
    o = Oracle(prob)
    ref_f, ref_r = np.zeros(o.nme), np.zeros(o.nme)
    for z in zs:
        a, b = o.rect_zone_diag(z.fi0, z.fj0, z.dIi, z.dIj, z.dJi, z.dJj, z.ni, z.nj, z.Fi, z.Fj, z.sym)
        ref_f += a
        ref_r += b
    assert rel(out["m3mf_msh"], ref_f) < TOL
    assert rel(out["m3mr_msh"], ref_r) < TOL
    assert rel(mr, ref_r) < TOL


def test_diag_skewness(session):
    prob = diag(cantilever_tower(nfreqs=9, df=0.25, nodes=12))
    s = session(prob)
    out = s.run()
    sk = s.skewness(out["m2mr_cls"], out["m3mr_cls"])
    o = Oracle(prob)
    assert rel(sk, o.skewness_diag(out["m2mr_cls"], out["m3mr_cls"])) < 1e-14
