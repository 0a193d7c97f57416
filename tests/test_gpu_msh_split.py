"""A Mesher zone too large for one pass of the split-precision path is evaluated as strips of
lattice lines sharing their boundary lines: the integrals equal the FP64 zone path's on the
whole zone (split-precision tolerance), and its per-zone diagonal moments are the sum over the
strips."""
import numpy as np
import pytest

from bsalib_gb300 import api
from bsalib_gb300.problem import tall_building

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def test_oversized_zone_in_strips(bsalib):
    prob = tall_building(nodes=20, modes=4, nfreqs=9, df=0.3, seed=6)
    prob.settings.suban = 2
    n = 1001  # 1.0 M BFM points: above the one-pass point cap
    z = api.Zone(0.05, -0.6, 0.9 / (n - 1), 0.0, 0.0, 0.9 / (n - 1), n, n, 1, 1, 1.0, 0)
    half = (n - 1) // 2
    za = api.Zone(0.05, -0.6, 0.9 / (n - 1), 0.0, 0.0, 0.9 / (n - 1), half + 1, n, 1, 1, 1.0, 0)
    zb = api.Zone(0.05 + half * 0.9 / (n - 1), -0.6, 0.9 / (n - 1), 0.0, 0.0, 0.9 / (n - 1), n - half, n, 1, 1,
                  1.0, 0)
    s = api.BsaSession(prob, precision=api.PREC_FP64)
    try:
        mf64, mr64, cnt = s.msh_zones([z])
    finally:
        s.close()
    s = api.BsaSession(prob, precision=api.PREC_BF16X3)
    try:
        mf, mr, cnt2 = s.msh_zones([z])
        _, mr_d, zd = s.msh_zones_diag([z])
        _, _, zd2 = s.msh_zones_diag([za, zb])
    finally:
        s.close()
    assert cnt[0] == cnt2[0] == n * n
    assert rel(mf, mf64) < 1e-4 and rel(mr, mr64) < 1e-4
    assert rel(mr_d, mr) < 1e-5
    assert rel(zd[0], zd2.sum(axis=0)) < 1e-5


def test_small_pass_budget_blocks_and_strips(bsalib):
    """With a small pass budget (bsa_gpu_setMesherPassBytes) a zone runs as blocks of columns and
    strips of lines sharing their boundary lattice lines: the same integrals as the FP64 zone
    path, zones of both lattice orientations, and the per-zone moments the sum over the pieces."""
    prob = tall_building(nodes=20, modes=4, nfreqs=9, df=0.3, seed=6)
    prob.settings.suban = 2
    zs = [api.Zone(0.05, -0.6, 0.9 / 120, 0.0, 0.0, 0.9 / 300, 121, 301, 2, 1, 1.0, 0),
          api.Zone(-0.7, 0.1, 0.0, 0.6 / 200, 0.8 / 90, 0.0, 201, 91, 1, 2, 2.0, 0)]
    s = api.BsaSession(prob, precision=api.PREC_FP64)
    try:
        mf64, mr64, cnt = s.msh_zones(zs)
    finally:
        s.close()
    s = api.BsaSession(prob, precision=api.PREC_BF16X3)
    try:
        _, mr_whole, zd_whole = s.msh_zones_diag(zs)
        api.check(s.lib.bsa_gpu_setMesherPassBytes(8e6), "bsa_gpu_setMesherPassBytes")
        mf, mr, cnt2 = s.msh_zones(zs)
        _, mr_d, zd = s.msh_zones_diag(zs)
    finally:
        s.lib.bsa_gpu_setMesherPassBytes(0.0)
        s.close()
    assert cnt[0] == cnt2[0] and cnt[1] == cnt2[1]
    assert rel(mf, mf64) < 1e-4 and rel(mr, mr64) < 1e-4
    assert rel(mr_d, mr_whole) < 1e-5
    assert rel(zd, zd_whole) < 1e-5
