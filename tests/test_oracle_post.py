"""CPU tests of the oracle's second-order post-processing (bsa_computeBRdecomp,
BsaLibImpl.F90:1292-1420; bsa_computePeakFactors, :1428-1517) against numpy restatements
written from the formulas.  No GPU."""
import numpy as np
import pytest

from bsalib_gb300.problem import cantilever_tower, tall_building
from oracle.oracle import Oracle

GAMMA = 0.5772


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("make", [lambda: cantilever_tower(nfreqs=9, df=0.25, nodes=10),
                                  lambda: tall_building(nodes=12, modes=4, nfreqs=7, df=0.3, seed=8)])
def test_br_decomp_vs_numpy(make):
    prob = make()
    o = Oracle(prob)
    nm = o.nme
    m2mf = np.random.default_rng(0).uniform(0.5, 2.0, nm * nm)
    bkg, res = o.br_decomp(m2mf)
    modes = o.modes - 1
    K = prob.Kg[modes]
    f = prob.natf[modes]
    sfm = np.zeros(nm)
    for tc in prob.settings.tc:
        L = o.phitc[:, :, tc - 1]
        for im in range(nm):
            sfm[im] += L[im] @ o.cross_psd(f[im], tc) @ L[im]
    assert rel(bkg, m2mf[[m * nm + m for m in range(nm)]] / K ** 2) < 1e-14
    assert rel(res, np.pi * 2 * np.pi * f * sfm / (2 * prob.xsi[modes] * K ** 2)) < 1e-12


def np_peaks(m2, m2o2, T, sk):
    beta = np.sqrt(2 * np.log(np.sqrt(m2o2 / m2) / (2 * np.pi) * T))
    g = GAMMA / beta + beta
    g4 = 1.5 * sk ** 2
    h40 = np.sqrt(1 + 1.5 * g4)
    h3 = sk / (4 + 2 * h40)
    h4 = (h40 - 1) / 18
    k = 1 / np.sqrt(1 + 2 * h3 ** 2 + 6 * h4 ** 2)
    common = h4 * (5.44 / beta ** 3 + 3 / beta * (np.pi ** 2 / 6 - GAMMA + GAMMA ** 2) + beta ** 3
                   + 3 * beta * (GAMMA - 1))
    odd = h3 * (beta ** 2 + 2 * GAMMA - 1 + 1.98 / beta ** 2)
    return g, k * (g + common + odd), k * (g + common - odd)


def test_peak_factors_vs_numpy():
    o = Oracle(cantilever_tower(nfreqs=5, df=0.4, nodes=4))
    m2 = np.array([1.0, 2.5, 0.3, 7.0])
    m2o2 = np.array([40.0, 300.0, 9.0, 2000.0])
    sk = np.array([0.2, -0.5, 0.0, 1.1])
    rc, g, pos, neg = o.peak_factors(m2, m2o2, 600.0, sk)
    assert rc == 0
    eg, ep, en = np_peaks(m2, m2o2, 600.0, sk)
    assert rel(g, eg) < 1e-14 and rel(pos, ep) < 1e-13 and rel(neg, en) < 1e-13
    rc, g2, _, _ = o.peak_factors(m2, m2o2, 600.0)
    assert rc == 0 and rel(g2, eg) < 1e-14


def test_peak_factors_skip_cases():
    o = Oracle(cantilever_tower(nfreqs=5, df=0.4, nodes=4))
    assert o.peak_factors(np.ones(3), np.zeros(3), 600.0)[0] == 1
    assert o.peak_factors(np.ones(3), np.full(3, 1e-4), 1.0)[0] == 2


@pytest.mark.parametrize("diag", [False, True])
def test_modal_recombination_vs_numpy(diag):
    """modalRecombination (app/bsa.F90:935-1053) restated in the oracle, against einsum sums
    written from the formulas: diag = sum_m M(m..m) phi_m^p, CCC = the full contraction."""
    prob = tall_building(nodes=12, modes=5, nfreqs=7, df=0.3, seed=8)
    o = Oracle(prob)
    nm = o.nme
    rng = np.random.default_rng(3)
    if diag:
        m2, m3, m2o2 = rng.uniform(0.5, 2, nm), rng.normal(size=nm), rng.uniform(0.5, 2, nm)
    else:
        A = rng.normal(size=(nm, nm))
        m2 = (A @ A.T + nm * np.eye(nm)).ravel(order="F")
        m3 = rng.normal(size=nm ** 3)
        m2o2 = (A.T @ A + np.eye(nm)).ravel(order="F")
    out = o.modal_recomb_all(m2, m3, m2o2)
    phi = prob.phi[:, o.modes - 1]
    if diag:
        e2, e3 = m2, m3
    else:
        M2, M3 = m2.reshape(nm, nm, order="F"), m3.reshape(nm, nm, nm, order="F")
        e2, e3 = np.diagonal(M2), np.array([M3[m, m, m] for m in range(nm)])
    d2 = (phi ** 2) @ e2
    d3 = (phi ** 3) @ e3
    assert rel(out["m2_diag"], d2) < 1e-13 and rel(out["m3_diag"], d3) < 1e-13
    assert rel(out["sk_diag"], d3 / d2 ** 1.5) < 1e-12
    if diag:
        assert "m2_ccc" not in out
        return
    c2 = np.einsum("dj,dk,jk->d", phi, phi, M2)
    c3 = np.einsum("di,dj,dk,ijk->d", phi, phi, phi, M3)
    co = np.einsum("dj,dk,jk->d", phi, phi, m2o2.reshape(nm, nm, order="F"))
    assert rel(out["m2_ccc"], c2) < 1e-12 and rel(out["m3_ccc"], c3) < 1e-12
    assert rel(out["m2o2_ccc"], co) < 1e-12
    assert rel(out["sk_ccc"], c3 / c2 ** 1.5) < 1e-11
    # the CCC branch of the older restatement agrees
    m2o, m3o, sko = o.modal_recomb(m2, m3)
    assert rel(out["m3_ccc"], m3o) < 1e-14 and rel(out["sk_ccc"], sko) < 1e-14
