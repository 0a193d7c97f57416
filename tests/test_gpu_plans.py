"""Every tile plan the autotuner may pick computes the same analysis: the Classic split
analysis under each valid (form, width) and the Mesher zone pass under each mode width give the
default plan's third moments to FP32 rounding (2e-6 relative; the summation order and the
padding differ, not the products)."""
import numpy as np
import pytest

from bsalib_gb300 import api
from bsalib_gb300.problem import bridge_deck, tall_building

pytestmark = pytest.mark.gpu
TOL = 2e-6


def rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def run(prob, plans, mesher=False):
    lib = api.load()
    assert lib.bsa_gpu_clearTilePlans() == 0
    for fam, val in plans:
        assert lib.bsa_gpu_setTilePlan(fam, 0, 1 << 30, 0, 1 << 30, 0, 1 << 30, val) == 0
    s = api.BsaSession(prob, precision=api.PREC_BF16X3)
    try:
        if mesher:
            s.use_driver_controls()
        r = s.run()
    finally:
        s.close()
        lib.bsa_gpu_loadTilePlans(None)
    return r["m3mr_msh" if mesher else "m3mr_cls"], r["m3mf_msh" if mesher else "m3mf_cls"]


@pytest.mark.parametrize("modes", [12, 20])
def test_classic_plans_agree(bsalib, modes):
    prob = tall_building(nodes=60, modes=modes, nfreqs=33, df=0.125, seed=9)
    ref = run(prob, [])
    cands = [[(api.PLAN_CLS_E_WIDTH, w)] for w in (16, 24, 32, 48) if w >= modes]
    cands += [[(api.PLAN_CLS_E_WIDTH, w), (api.PLAN_CLS_E_SPLIT, sp)] for w in (16, 24) if w >= modes for sp in (1, 2)]
    cands += [[(api.PLAN_CLS_FORM, 0), (api.PLAN_CLS_D_WIDTH, w)] for w in (16, 24, 32, 64) if w >= modes]
    for c in cands:
        mr, mf = run(prob, c)
        assert rel(mr, ref[0]) < TOL, c
        assert rel(mf, ref[1]) < TOL, c


def test_mesher_plans_agree(bsalib):
    prob = bridge_deck(nodes=120, modes=12)
    prob.settings.suban = 2
    ref = run(prob, [], mesher=True)
    for w in (24, 32):
        mr, mf = run(prob, [(api.PLAN_MSH_WIDTH, w)], mesher=True)
        assert rel(mr, ref[0]) < TOL, w
        assert rel(mf, ref[1]) < TOL, w
