"""bsa_gpu_setClassicSymmetry: the Classic analysis on the rows f1 <= 0 of the symmetric grid
(rows f1 < 0 with twice their weight) gives the full grid's moments: FP64 to 1e-12 (the
summation order alone differs), the split precision to 1e-6 against its own full-grid run."""
import numpy as np
import pytest

from bsalib_gb300 import api
from bsalib_gb300.dist import MOMENT_KEYS, shard_rows
from bsalib_gb300.problem import cantilever_tower, tall_building

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def runs(prob, prec=api.PREC_FP64, **kw):
    s = api.BsaSession(prob, precision=prec, **kw)
    try:
        full = s.run()
        s.set_symmetry(True)
        half = s.run()
        pts = s.stats().points
    finally:
        s.close()
    return full, half, pts


@pytest.mark.parametrize("trunc", [True, False])
def test_symmetric_half_grid_fp64(bsalib, trunc):
    prob = tall_building(nodes=30, modes=6, nfreqs=9, df=0.3, seed=13)
    full, half, pts = runs(prob, classic_truncation=trunc)
    nf = prob.classic_nf()
    assert pts == ((nf + 1) // 2) * nf
    for k in ("m3mf_cls", "m3mr_cls", "m2mf_cls", "m2mr_cls", "m2o2mr_cls"):
        assert rel(half[k], full[k]) < 1e-12, k


def test_symmetric_half_grid_split_precision(bsalib):
    prob = tall_building(nodes=60, modes=12, nfreqs=33, df=0.1, seed=14)
    full, half, _ = runs(prob, api.PREC_BF16X3)
    assert rel(half["m3mr_cls"], full["m3mr_cls"]) < 1e-6
    assert rel(half["m3mf_cls"], full["m3mf_cls"]) < 1e-6


def test_symmetric_diagonal_and_scalar(bsalib):
    prob = cantilever_tower(nfreqs=9, df=0.25, nodes=12)
    prob.settings.onlyd = 1
    full, half, _ = runs(prob)
    assert rel(half["m3mr_cls"], full["m3mr_cls"]) < 1e-12
    prob = cantilever_tower(nfreqs=9, df=0.25, nodes=12)
    prob.settings.scalar = 1
    full, half, _ = runs(prob)
    assert rel(half["m3mr_cls"], full["m3mr_cls"]) < 1e-12


def test_symmetric_row_shards_sum(bsalib):
    prob = tall_building(nodes=30, modes=6, nfreqs=9, df=0.3, seed=12)
    s = api.BsaSession(prob)
    try:
        full = s.run()
        s.set_symmetry(True)
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


def test_one_sided_grid_ignores_the_switch(bsalib):
    prob = tall_building(nodes=20, modes=4, nfreqs=9, df=0.3, seed=3)
    prob.settings.defsc = 2
    full, half, _ = runs(prob)
    assert rel(half["m3mr_cls"], full["m3mr_cls"]) < 1e-14
