"""Per-point accuracy of the split-precision (BF16x3, FP32 accumulation) Classic path against
the plain FP64 path, at the benchmark's configuration: the 400-node, 24-mode, two-component
building on its full 1025 x 1025 grid.

bsa_gpu_clsBispectraAt returns, in BF16x3, the analysis's own per-point values: the E-form
tensor-core products of the whole grid with the epilogue writing the listed points'
bispectra instead of the moments.  The bars are the split path's: 1e-4 relative (max-norm per
tensor over the sampled points) on the force and the response bispectra
(functionsImpl.F90:1494-1538 and :1598-1738).  A small-grid test samples every point and checks
that the per-point values, integrated with the Classic weights (intgSpectraVect_), give the
E form's own third moments: the sampled epilogue writes exactly what the moment epilogue sums."""
import numpy as np
import pytest

from bsalib_gb300 import api
from bsalib_gb300.problem import tall_building

pytestmark = pytest.mark.gpu
TOL_BISP = 1e-4


def maxrel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def sample(nf, n, seed):
    rng = np.random.default_rng(seed)
    flat = rng.choice(nf * nf, size=n, replace=False)
    return (flat % nf).astype(np.int32), (flat // nf).astype(np.int32)


@pytest.mark.parametrize("modes", [24, 40])
def test_split_point_bispectra_full_grid(bsalib, modes):
    prob = tall_building(modes=modes)
    nf = prob.classic_nf()
    assert nf == 1025
    i1, i2 = sample(nf, 2048, 11 + modes)
    out = {}
    for prec in (api.PREC_FP64, api.PREC_BF16X3):
        s = api.BsaSession(prob, precision=prec)
        try:
            out[prec] = s.classic_points(i1, i2)
        finally:
            s.close()
    (bf64, br64), (bfx, brx) = out[api.PREC_FP64], out[api.PREC_BF16X3]
    assert np.all(np.isfinite(bfx)) and np.all(np.isfinite(brx))
    assert maxrel(bfx, bf64) < TOL_BISP
    assert maxrel(brx, br64) < TOL_BISP


def classic_weights(nf, d):
    w1 = np.ones(nf)
    w1[0] = w1[-1] = 0.5
    W = np.outer(w1, w1)
    W[0, 0] = W[0, -1] = W[-1, 0] = W[-1, -1] = -0.5   # the reference's vertex weight
    return W * d * d


@pytest.mark.parametrize("modes", [12, 24, 30])
def test_sampled_epilogue_integrates_to_the_moments(bsalib, modes):
    prob = tall_building(nodes=40, modes=modes, nfreqs=33, df=0.125, seed=3)
    nf = prob.classic_nf()
    I1, I2 = np.meshgrid(np.arange(nf), np.arange(nf), indexing="ij")
    i1, i2 = I1.ravel().astype(np.int32), I2.ravel().astype(np.int32)
    s = api.BsaSession(prob, precision=api.PREC_BF16X3)
    try:
        bf, br = s.classic_points(i1, i2)
        r = s.run()
    finally:
        s.close()
    W = classic_weights(nf, prob.settings.df * 2 * np.pi)[i1, i2]
    mf, mr = W @ bf, W @ br
    assert maxrel(mf, r["m3mf_cls"]) < 1e-5
    assert maxrel(mr, r["m3mr_cls"]) < 1e-5
    # and the per-point values against the FP64 path's on this grid
    s = api.BsaSession(prob, precision=api.PREC_FP64)
    try:
        bf64, br64 = s.classic_points(i1, i2)
    finally:
        s.close()
    assert maxrel(bf, bf64) < TOL_BISP
    assert maxrel(br, br64) < TOL_BISP


def test_point_bispectra_fp64_match_the_materialised_grid(bsalib):
    prob = tall_building(nodes=16, modes=4, nfreqs=9, df=0.3, seed=5)
    s = api.BsaSession(prob, precision=api.PREC_FP64)
    try:
        f, bfg, brg = s.classic_bispectra()
        nf = f.size
        i1, i2 = sample(nf, 40, 2)
        bf, br = s.classic_points(i1, i2)
    finally:
        s.close()
    assert maxrel(bf, bfg[i1, i2]) < 1e-12
    assert maxrel(br, brg[i1, i2]) < 1e-12
