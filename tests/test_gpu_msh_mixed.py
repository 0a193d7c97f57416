"""The Mesher zones in the split precision: axis-aligned zones through the BF16x3 tensor-core
contraction (three GEMM families, FP32 term tensors) and the FP32 zone integration with
FP64-evaluated FRF, against the FP64 zone path on the same zones.  Tolerance: 1e-4 relative
(max-norm) on the third moments, the bar the split precision is held to."""
import numpy as np
import pytest

from bsalib_gb300 import api
from bsalib_gb300.problem import cantilever_tower, tall_building

pytestmark = pytest.mark.gpu
TOL = 1e-4


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def zone(fi0, fj0, dIi, dIj, dJi, dJj, ni, nj, Fi, Fj, sym=1.0):
    return api.Zone(fi0, fj0, dIi, dIj, dJi, dJj, ni, nj, Fi, Fj, sym, 0)


ZONES = [
    zone(-0.4, -0.4, 0.1, 0.0, 0.0, 0.1, 9, 9, 4, 4),              # square
    zone(0.4, -0.4, 0.05, 0.0, 0.0, 0.2, 5, 13, 4, 2),             # long lines (several N tiles)
    zone(1.2, 0.6, 0.0, 0.15, -0.12, 0.0, 4, 6, 2, 3),             # swapped axes
    zone(-1.0, 1.0, 0.07, 0.07, 0.07, -0.07, 3, 4, 1, 2, 2.0),     # rotated: FP64 kernel
    zone(0.25, 0.3, 0.02, 0.0, 0.0, 0.03, 2, 2, 1, 1),             # one cell
]


def both(prob, fn):
    out = []
    for prec in (api.PREC_FP64, api.PREC_BF16X3):
        s = api.BsaSession(prob, precision=prec)
        try:
            out.append(fn(s))
        finally:
            s.close()
    return out


@pytest.mark.parametrize("nodes,modes", [(12, 4), (13, 7), (40, 11), (30, 24)])
def test_zones_mixed_vs_fp64(bsalib, nodes, modes):
    prob = tall_building(nodes=nodes, modes=modes, nfreqs=5, df=0.3, seed=31)
    (f64, c64), (mix, cmx) = both(prob, lambda s: (s.msh_zones(ZONES)[:2], s.msh_zones(ZONES)[2]))
    assert rel(mix[0], f64[0]) < TOL
    assert rel(mix[1], f64[1]) < TOL
    assert np.array_equal(c64, cmx)


def test_mesher_run_mixed_vs_fp64(bsalib):
    prob = cantilever_tower(nodes=30)
    prob.settings.suban = 2
    f64, mix = both(prob, lambda s: s.run())
    assert rel(mix["m3mr_msh"], f64["m3mr_msh"]) < TOL
    assert rel(mix["m3mf_msh"], f64["m3mf_msh"]) < TOL


def test_mesher_run_mixed_building(bsalib):
    prob = tall_building(nodes=60, modes=8, nfreqs=9, df=0.3, seed=5)
    prob.settings.suban = 2
    prob.settings.bkgrfmt = 8
    f64, mix = both(prob, lambda s: s.run())
    assert rel(mix["m3mr_msh"], f64["m3mr_msh"]) < TOL
    assert rel(mix["m3mf_msh"], f64["m3mf_msh"]) < TOL
