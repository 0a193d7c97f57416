"""Second-order post-processing through the C-ABI: bsa_computeBRdecomp (the resonant part's
modal force PSD at each natural frequency evaluated on the GPU) and bsa_computePeakFactors,
against the oracle.  FP64: 1e-10 relative."""
import dataclasses

import numpy as np
import pytest

from bsalib_gb300 import api
from bsalib_gb300.problem import cantilever_tower, tall_building
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu
TOL = 1e-10


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


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


@pytest.mark.parametrize("make,onlyd", [
    (lambda: cantilever_tower(nfreqs=9, df=0.25, nodes=14), 0),
    (lambda: tall_building(nodes=40, modes=6, nfreqs=9, df=0.3, seed=4), 0),
    (lambda: tall_building(nodes=40, modes=6, nfreqs=9, df=0.3, seed=4), 1),
    (lambda: two_dof(cantilever_tower(nfreqs=7, df=0.3, nodes=9)), 0),
])
def test_br_decomp_vs_oracle(bsalib, make, onlyd):
    prob = make()
    prob.settings.onlyd = onlyd
    s = api.BsaSession(prob)
    try:
        out = s.run()
        bkg, res = s.br_decomp(out["m2mf_cls"])
    finally:
        s.close()
    ebkg, eres = Oracle(prob).br_decomp(out["m2mf_cls"])
    assert rel(bkg, ebkg) < TOL
    assert rel(res, eres) < TOL


def test_peak_factors_vs_oracle(bsalib):
    prob = cantilever_tower(nfreqs=9, df=0.25, nodes=12)
    s = api.BsaSession(prob)
    try:
        out = s.run()
        nm = s.nmodes()
        d2 = [m * nm + m for m in range(nm)]
        d3 = [m + nm * m + nm * nm * m for m in range(nm)]
        sk = s.skewness(out["m2mr_cls"], out["m3mr_cls"])[d3]
        m2, m2o2 = out["m2mr_cls"][d2], out["m2o2mr_cls"][d2]
        rc, g, pos, neg = s.peak_factors(m2, m2o2, 600.0, sk)
        assert rc == api.BSA_OK
        rc0, g0, _, _ = s.peak_factors(m2, m2o2, 600.0)
        skip1 = s.peak_factors(m2, np.zeros_like(m2), 600.0)[0]
        skip2 = s.peak_factors(m2, m2o2, 1e-3)[0]
        after = s.run()  # a skipped call is a warning: the session is not halted
    finally:
        s.close()
    erc, eg, epos, eneg = Oracle(prob).peak_factors(m2, m2o2, 600.0, sk)
    assert erc == 0
    assert rel(g, eg) < 1e-14 and rel(pos, epos) < 1e-14 and rel(neg, eneg) < 1e-14
    assert rc0 == api.BSA_OK and rel(g0, eg) < 1e-14
    assert skip1 == 1 and skip2 == 1
    assert np.array_equal(after["m3mr_cls"], out["m3mr_cls"])


@pytest.mark.parametrize("onlyd", [0, 1])
def test_modal_recombination_vs_oracle(bsalib, onlyd):
    """bsa_modalRecombination (app/bsa.F90:935-1053) on the modal moments of an FP64 analysis,
    against the oracle's restatement: nodal m2 / m3 / m2o2 / skewness of both branches."""
    prob = tall_building(nodes=40, modes=6, nfreqs=9, df=0.3, seed=4)
    prob.settings = dataclasses.replace(prob.settings, onlyd=onlyd)
    s = api.BsaSession(prob, precision=api.PREC_FP64)
    try:
        r = s.run()
        got = s.modal_recombination(r["m2mr_cls"], r["m3mr_cls"], r["m2o2mr_cls"])
        no_m2o2 = s.modal_recombination(r["m2mr_cls"], r["m3mr_cls"])
    finally:
        s.close()
    ref = Oracle(prob).modal_recomb_all(r["m2mr_cls"], r["m3mr_cls"], r["m2o2mr_cls"])
    assert sorted(got) == sorted(ref)
    for k in ref:
        assert rel(got[k], ref[k]) < TOL, k
    assert np.all(no_m2o2["m2o2_diag"] == 0.0)
    assert rel(no_m2o2["m3_diag"], ref["m3_diag"]) < TOL
