"""The split-precision (BF16x3, FP32 accumulation) tcgen05 contraction against the plain
FP64 GPU path on the same inputs.

Tolerances (the mixed-precision bar of the BFM path): third moments within 1e-4 relative
(max-norm over the tensor) and response skewness within 1e-3 relative.
"""
import numpy as np
import pytest

from bsalib_gb300 import api
from bsalib_gb300.problem import cantilever_tower, tall_building

pytestmark = pytest.mark.gpu
TOL_M3 = 1e-4
TOL_SK = 1e-3


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def both(prob, truncation=True):
    out = {}
    for prec in (api.PREC_FP64, api.PREC_BF16X3):
        s = api.BsaSession(prob, precision=prec, classic_truncation=truncation)
        try:
            r = s.run()
            r["sk"] = s.skewness(r["m2mr_cls"], r["m3mr_cls"])
            r["stats"] = s.stats()
        finally:
            s.close()
        out[prec] = r
    return out[api.PREC_FP64], out[api.PREC_BF16X3]


CASES = [
    ("tower_nm4", cantilever_tower(nfreqs=17, df=0.25, nodes=30)),
    ("bldg_nm6_2tc", tall_building(nodes=40, modes=6, nfreqs=11, df=0.4, seed=11)),
    ("bldg_nm12", tall_building(nodes=64, modes=12, nfreqs=21, df=0.2, seed=3)),
    ("bldg_nm24", tall_building(nodes=100, modes=24, nfreqs=25, df=0.16, seed=5)),
    ("bldg_nm30", tall_building(nodes=50, modes=30, nfreqs=9, df=0.5, seed=8)),
    # more than 32 kept modes: the modes split into two halves of 32, each row swept twice
    ("bldg_nm33", tall_building(nodes=40, modes=33, nfreqs=11, df=0.4, seed=12)),
    ("bldg_nm40_2tc", tall_building(nodes=70, modes=40, nfreqs=13, df=0.3, seed=13)),
    ("bldg_nm64", tall_building(nodes=48, modes=64, nfreqs=9, df=0.5, seed=14)),
]


@pytest.mark.parametrize("name,prob", CASES, ids=[c[0] for c in CASES])
def test_mixed_matches_fp64(name, prob):
    ref, mix = both(prob)
    assert mix["stats"].precision == api.PREC_BF16X3
    assert rel(mix["m3mf_cls"], ref["m3mf_cls"]) < TOL_M3
    assert rel(mix["m3mr_cls"], ref["m3mr_cls"]) < TOL_M3
    assert rel(mix["sk"], ref["sk"]) < TOL_SK
    # second-order moments: FP64 sums of the FP32 factor table in the mixed run
    assert rel(mix["m2mr_cls"], ref["m2mr_cls"]) < 1e-6
    assert rel(mix["m2mf_cls"], ref["m2mf_cls"]) < 1e-6


def test_mixed_analytic_sum_frequency():
    prob = tall_building(nodes=48, modes=8, nfreqs=13, df=0.3, seed=21)
    ref, mix = both(prob, truncation=False)
    assert rel(mix["m3mr_cls"], ref["m3mr_cls"]) < TOL_M3


def test_mixed_uniform_weights():
    prob = tall_building(nodes=32, modes=10, nfreqs=9, df=0.3, seed=22)
    prob.settings.scalar = 1
    ref, mix = both(prob)
    assert rel(mix["m3mr_cls"], ref["m3mr_cls"]) < TOL_M3
    assert rel(mix["m3mf_cls"], ref["m3mf_cls"]) < TOL_M3


def test_mixed_building_129_grid():
    """The 400-node, 24-mode, two-component building on a 129 x 129 grid."""
    prob = tall_building(nfreqs=65, df=4.0 / 64)
    ref, mix = both(prob)
    assert rel(mix["m3mr_cls"], ref["m3mr_cls"]) < TOL_M3
    assert rel(mix["sk"], ref["sk"]) < TOL_SK


@pytest.mark.parametrize("modes", [16, 40])
def test_mixed_is_deterministic(modes):
    prob = tall_building(nodes=40, modes=modes, nfreqs=17, df=0.25, seed=30)
    s = api.BsaSession(prob, precision=api.PREC_BF16X3)
    try:
        a = s.run()["m3mr_cls"]
        b = s.run()["m3mr_cls"]
    finally:
        s.close()
    assert np.array_equal(a, b)


def test_mixed_more_than_32_modes_with_symmetry_and_shards():
    """Two mode halves combined with the central symmetry and row shards."""
    prob = tall_building(nodes=40, modes=36, nfreqs=13, df=0.3, seed=31)
    ref, _ = both(prob)
    s = api.BsaSession(prob, precision=api.PREC_BF16X3)
    try:
        s.set_symmetry(True)
        sym = s.run()["m3mr_cls"]
        s.set_symmetry(False)
        nf = prob.classic_nf()
        parts = []
        for r0, r1 in ((0, 7), (7, nf)):
            s.set_rows(r0, r1)
            parts.append(s.run()["m3mr_cls"])
    finally:
        s.close()
    assert rel(sym, ref["m3mr_cls"]) < TOL_M3
    assert rel(parts[0] + parts[1], ref["m3mr_cls"]) < TOL_M3


@pytest.mark.parametrize("modes", [6, 12, 24])
def test_symmetric_d1_matches_the_full_form(modes):
    """A launch over the whole grid forms D1 for the columns c >= r only and adds term 1's
    mirror at (c, r); row shards run the full form.  Same moments up to FP32 summation order."""
    prob = tall_building(nodes=40, modes=modes, nfreqs=17, df=0.25, seed=32)
    s = api.BsaSession(prob, precision=api.PREC_BF16X3)
    try:
        full = s.run()
        nf = prob.classic_nf()
        parts = []
        for r0, r1 in ((0, 11), (11, nf)):
            s.set_rows(r0, r1)
            parts.append(s.run())
    finally:
        s.close()
    for k in ("m3mr_cls", "m3mf_cls"):
        assert rel(full[k], parts[0][k] + parts[1][k]) < 2e-6, k


@pytest.mark.parametrize("nodes,modes,nfreqs,tc", [(30, 4, 33, (1,)), (60, 8, 41, (1, 3)), (80, 12, 65, (1, 3)),
                                                     (100, 16, 33, (1,)), (120, 24, 49, (1, 3)), (70, 28, 25, (1, 3)),
                                                     (90, 40, 21, (1,)), (64, 48, 17, (1, 3))])
def test_e_form_matches_the_d_form(bsalib, nodes, modes, nfreqs, tc):
    """The E form (one GEMM family over half the grid pairs, six contributions per product;
    above 24 kept modes in two mode halves) against the D1 / D3 form on the same grid: the
    same products, summed in another order (FP32 partials), so 2e-6 relative."""
    import dataclasses
    prob = tall_building(nodes=nodes, modes=modes, nfreqs=nfreqs, df=4.0 / (nfreqs - 1), seed=nodes)
    prob.settings = dataclasses.replace(prob.settings, tc=tc)
    out = []
    for form in (1, 0):
        s = api.BsaSession(prob, precision=api.PREC_BF16X3)
        try:
            s.set_classic_form(form)
            out.append(s.run())
        finally:
            s.close()
    for k in ("m3mr_cls", "m3mf_cls"):
        assert rel(out[0][k], out[1][k]) < 2e-6, k
