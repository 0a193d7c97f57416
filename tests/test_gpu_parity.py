"""Parity of the CUDA path (through the C-ABI) with the oracle and the golden vectors.

Tolerance for the plain FP64 path: 1e-10 relative, max-norm over each tensor
(max|gpu - ref| / max|ref|), as the FP64 parity gate of the BFM path requires.
"""
import os

import numpy as np
import pytest

from bsalib_gb300 import api
from bsalib_gb300.problem import cantilever_tower, tall_building
from oracle.oracle import Oracle, classic_weights

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")
TOL = 1e-10


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


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


@pytest.mark.parametrize("name,prob", [
    ("tower6_nf9", cantilever_tower(nfreqs=5, df=0.5, nodes=6)),
    ("building8_2tc_nf7", tall_building(nodes=8, modes=3, nfreqs=4, df=0.5, seed=7)),
])
def test_classic_bispectra_golden(session, name, prob):
    g = np.load(os.path.join(GOLD, name + ".npz"))
    s = session(prob)
    f, bf, br = s.classic_bispectra()
    assert np.array_equal(f, g["f"])
    assert rel(bf, g["bf"]) < TOL
    assert rel(br, g["br"]) < TOL


@pytest.mark.parametrize("prob", [
    cantilever_tower(nfreqs=17, df=0.25, nodes=30),
    tall_building(nodes=40, modes=6, nfreqs=11, df=0.4, seed=11),
])
def test_classic_moments_vs_oracle(session, prob):
    o = Oracle(prob).classic_vect(keep_bisp=False)
    r = session(prob).run()
    for k in ("m2mf", "m2mr", "m2o2mr", "m3mf", "m3mr"):
        assert rel(r[k + "_cls"], o[k]) < TOL, k


def test_tower_full_grid_vs_oracle(session):
    """The 30-node tower on its full 129 x 129 grid (the reference's CPU-runnable case)."""
    prob = cantilever_tower()
    o = Oracle(prob).classic_vect(keep_bisp=False)
    s = session(prob)
    r = s.run()
    for k in ("m2mf", "m2mr", "m2o2mr", "m3mf", "m3mr"):
        assert rel(r[k + "_cls"], o[k]) < TOL, k
    sk = s.skewness(r["m2mr_cls"], r["m3mr_cls"])
    assert rel(sk, Oracle(prob).skewness(o["m2mr"], o["m3mr"])) < TOL
    assert s.stats().points == 129 * 129


def test_scalar_classic_vs_oracle(session):
    prob = cantilever_tower(nfreqs=6, df=0.4, nodes=9)
    prob.settings.scalar = 1
    o = Oracle(prob).classic_scalar()
    r = session(prob).run()
    for k in ("m2mf", "m2mr", "m2o2mr", "m3mf", "m3mr"):
        assert rel(r[k + "_cls"], o[k]) < TOL, k


def test_analytic_sum_frequency(session):
    """With the truncation switched off, S(f1+f2) is evaluated beyond the grid."""
    prob = cantilever_tower(nfreqs=5, df=0.5, nodes=6)
    s = session(prob, classic_truncation=False)
    f, bf, br = s.classic_bispectra()
    o = Oracle(prob)
    for i1, i2 in [(0, 0), (8, 8), (2, 7), (6, 5)]:
        ref = o.direct_point(f[i1], f[i2])
        assert rel(bf[i1, i2], ref) < TOL
        assert rel(br[i1, i2], ref * o.brm_factor(f[i1], f[i2])) < TOL


@pytest.mark.parametrize("psd_type", [2, 3, 5])
def test_psd_models(session, psd_type):
    prob = tall_building(nodes=10, modes=3, nfreqs=5, df=0.3, seed=1)
    prob.psd_type = psd_type
    o = Oracle(prob).classic_vect(keep_bisp=False)
    r = session(prob).run()
    if psd_type == 2:  # kaimalPSD_ is identically zero
        assert np.all(r["m3mr_cls"] == 0.0) and np.all(r["m2mf_cls"] == 0.0)
    else:
        for k in ("m2mf", "m3mf", "m3mr"):
            assert rel(r[k + "_cls"], o[k]) < TOL, k


def test_mesher_points_golden(session):
    g = np.load(os.path.join(GOLD, "tower6_points.npz"))
    s = session(cantilever_tower(nfreqs=5, df=0.5, nodes=6))
    bf, br = s.msh_bispectra(g["pts"][:, 0], g["pts"][:, 1])
    assert rel(bf, g["bf"]) < TOL
    assert rel(br, g["br"]) < TOL


def test_mesher_weighted_moments(session):
    prob = tall_building(nodes=16, modes=4, nfreqs=5, df=0.3, seed=2)
    o = Oracle(prob)
    rng = np.random.default_rng(0)
    fi = rng.uniform(-2, 2, 37)
    fj = rng.uniform(-2, 2, 37)
    w = rng.uniform(0.1, 1.0, 37)
    mf, mr = session(prob).msh_moments(fi, fj, w)
    bfs = np.stack([o.msh_bfm(a, b) for a, b in zip(fi, fj)])
    brs = np.stack([bfs[k] * o.brm_factor(a, b) for k, (a, b) in enumerate(zip(fi, fj))])
    assert rel(mf, w @ bfs) < TOL
    assert rel(mr, w @ brs) < TOL


def test_determinism(session):
    prob = tall_building(nodes=24, modes=5, nfreqs=9, df=0.3, seed=4)
    s = session(prob)
    a = s.run()
    b = s.run()
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def test_errors_are_codes_not_exits(bsalib):
    lib = bsalib
    assert lib.bsa_Init() == 0
    rc = lib.bsa_Run(*([None] * 7))
    assert rc == -2  # BSA_ERR_STATE: inputs missing
    assert b"not set" in lib.bsa_lastError()
    assert lib.bsa_setTestMode(1) == -2  # halted (sticky) until bsa_Finalise
    assert lib.bsa_Finalise() == 0
    assert lib.bsa_Init() == 0
    assert lib.bsa_setTestMode(7) == -1
    lib.bsa_Finalise()


def test_psd_type_without_model_is_rejected(session):
    prob = cantilever_tower(nfreqs=4, df=0.5, nodes=5)
    prob.psd_type = 4
    s = session(prob)
    with pytest.raises(api.BsaError, match="no model"):
        s.run()


def test_classic_weights_in_kernel(session):
    """m3 from the materialised spectra with the Q2 weights equals the fused reduction."""
    prob = tall_building(nodes=12, modes=4, nfreqs=6, df=0.3, seed=9)
    s = session(prob)
    f, bf, br = s.classic_bispectra()
    r = s.run()
    w = classic_weights(f.size, f[1] - f[0])
    assert rel(r["m3mf_cls"], np.einsum("ij,ijk->k", w, bf)) < 1e-12
    assert rel(r["m3mr_cls"], np.einsum("ij,ijk->k", w, br)) < 1e-12


def test_bsacl_abi_matches_oracle(bsalib):
    """The BsaCL entry points (bsacl.h) driven as BsaLibImpl.F90:266-303 and
    BsaClassicImpl.F90:74-88 drive them: m3mr over fi x fj with influence dfi*dfj*4pi^2."""
    import ctypes as C
    prob = tall_building(nodes=10, modes=3, nfreqs=4, df=0.5, seed=13)
    o = Oracle(prob)
    lib = bsalib
    keep = []

    def P(a, dt=np.float64):
        a = np.asfortranarray(np.asarray(a, dtype=dt))
        keep.append(a)
        return a.ctypes.data_as(C.c_void_p)

    lib.bsaclAcquirePSDId.argtypes = [C.c_uint32]
    lib.bsaclAcquirePSDId(prob.psd_type)
    lib.bsaclAcquireStructModMat(P(prob.phi), P(prob.natf), C.c_uint32(prob.ndofs), C.c_uint32(prob.nm))
    lib.bsaclAcquireModalMatrices(P(prob.Mg), P(prob.Cg), P(prob.Kg))
    lib.bsaclAcquireLoadedNodesList(P(prob.n_load, np.int32), C.c_uint32(prob.nnl))
    lib.bsaclAcquireTotalNOfNodes(C.c_uint32(prob.nn))
    lib.bsaclAcquireUsedModesList(P(o.modes, np.int32), C.c_uint32(o.nme))
    lib.bsaclAcquireWindCoeffs(P(prob.wfc), C.c_uint32(prob.nnl), C.c_uint32(1), C.c_uint32(6))
    lib.bsaclAcquirePhiTimesCMat(P(o.phitc), C.c_uint32(o.nme), C.c_uint32(prob.nnl), C.c_uint32(6))
    lib.bsaclAcquireTurbComponentsList(P(np.array(prob.settings.tc), np.int32), C.c_uint32(prob.ntc))
    lib.bsaclAcquireNodalCorrelation(P(prob.nod_corr), C.c_uint32(prob.nod_corr.shape[0]))
    lib.bsaclAcquireWindNodalVelocities(P(prob.u_node))
    lib.bsaclAcquireWindNodalWindZones(P(prob.wz_node, np.int32))
    lib.bsaclAcquireWindTurbScales(P(prob.L), C.c_uint32(prob.nz))
    lib.bsaclAcquireWindTurbStd(P(prob.sigma), C.c_uint32(prob.nz))
    assert lib.bsaclInit(1) == 0
    assert lib.bsaclInitDeviceMemory() == 0
    fi = np.linspace(-1.5, 1.5, 7)
    fj = np.linspace(-1.0, 1.0, 5)
    lib.bsaclAcquireComputationFreqs(C.c_uint(0), C.c_uint32(fi.size), P(fi), C.c_uint32(fj.size), P(fj))
    assert lib.bsaclSetKernelID(2) == 0
    res = np.zeros(o.nme ** 3)
    lib.bsaclRun.argtypes = [C.c_uint, C.c_size_t, C.c_void_p]
    assert lib.bsaclRun(0, res.size, res.ctypes.data_as(C.c_void_p)) == 0
    lib.bsaclFinalise()
    infl = (fi[1] - fi[0]) * (fj[1] - fj[0]) * 4 * np.pi ** 2
    ref = np.zeros_like(res)
    for a in fi:
        for b in fj:
            ref += infl * o.msh_bfm(a, b) * o.brm_factor(a, b)
    assert rel(res, ref) < TOL


@pytest.mark.parametrize("prec,tol", [(api.PREC_FP64, 1e-12), (api.PREC_BF16X3, 1e-6)])
def test_row_shards_sum_to_full_grid(prec, tol):
    """Contiguous row shards (the multi-GPU split) add up to the full Classic analysis."""
    from bsalib_gb300.dist import MOMENT_KEYS, shard_rows
    prob = tall_building(nodes=30, modes=6, nfreqs=9, df=0.3, seed=12)
    s = api.BsaSession(prob, precision=prec)
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
        assert rel(acc[k], full[k]) < tol, k


def test_controls_reset_by_finalise(bsalib):
    """A new session does not inherit the previous one's row shard or precision."""
    prob = tall_building(nodes=16, modes=4, nfreqs=7, df=0.3, seed=2)
    s = api.BsaSession(prob)
    full = s.run()
    s.set_rows(5, -1)
    s.set_precision(api.PREC_BF16X3)
    s.close()
    s2 = api.BsaSession(prob)
    try:
        again = s2.run()
        assert s2.stats().precision == api.PREC_FP64
    finally:
        s2.close()
    assert np.array_equal(again["m3mr_cls"], full["m3mr_cls"])
