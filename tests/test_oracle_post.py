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
