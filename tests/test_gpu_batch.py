"""The batched Classic sweep (bsa_gpu_batch*) against one bsa_Run per case.

Each case of a batch must give the moments its own split-precision analysis gives.  Up to 48
kept modes on odd grids both use the E form of the contraction (each product of one GEMM
family feeding the three terms at up to six grid points); the batch flushes its FP32 partials
at other points and adds them with atomics, so third moments agree to ~1e-7.  The batch's
D1 / D3 form (`Sweep.run(form=0)`, and every case above 48 modes or on an even grid) sums the
same products in another order: ~1e-6 from the E form (both lie ~3e-6 from the FP64 path).
The bar is 1e-5 relative (max-norm, 10x inside the split-precision bar).  Second moments
agree to 1e-12.  Against the FP64 path the mixed-precision bar holds
(third moments 1e-4 relative).  Cases of every FRF-table width (8, 16, 24, 32 kept modes, and
two halves of 32 above that),
different grids and load sizes share one batch; the library's own inputs are left as they
were.
"""
import copy

import numpy as np
import pytest

from bsalib_gb300 import api
from bsalib_gb300.problem import cantilever_tower, random_structure, tall_building

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def single(prob, prec):
    s = api.BsaSession(prob, precision=prec)
    try:
        return s.run()
    finally:
        s.close()


CASES = [
    cantilever_tower(nfreqs=17, df=0.25, nodes=30),
    tall_building(nodes=64, modes=12, nfreqs=21, df=0.2, seed=3),
    tall_building(nodes=100, modes=24, nfreqs=25, df=0.16, seed=5),
    tall_building(nodes=50, modes=30, nfreqs=9, df=0.5, seed=8),
    random_structure(11, nodes=(60, 60), modes=(7, 7), nfreq_grid=(65, 65)),
    random_structure(12, nodes=(230, 230), modes=(16, 16), nfreq_grid=(129, 129)),
    random_structure(13, nodes=(40, 40), modes=(5, 5), nfreq_grid=(33, 33)),
    random_structure(14, nodes=(150, 150), modes=(20, 20), nfreq_grid=(97, 97)),
    # more than 32 kept modes: two mode halves per grid row
    random_structure(15, nodes=(90, 90), modes=(40, 40), nfreq_grid=(33, 33)),
    tall_building(nodes=48, modes=64, nfreqs=9, df=0.5, seed=14),
]


@pytest.fixture(scope="module")
def batch(bsalib):
    sw = api.Sweep()
    for p in CASES:
        sw.add(p)
    out, total = sw.run()
    sw.clear()
    return out, total


def test_batch_matches_single_analyses(batch):
    out, _ = batch
    assert len(out) == len(CASES)
    for k, p in enumerate(CASES):
        ref = single(p, api.PREC_BF16X3)
        assert out[k]["nm"] ** 3 == ref["m3mr_cls"].size
        assert rel(out[k]["m3mr"], ref["m3mr_cls"]) < 1e-5, k
        assert rel(out[k]["m3mf"], ref["m3mf_cls"]) < 1e-5, k
        assert rel(out[k]["m2mr"], ref["m2mr_cls"]) < 1e-12, k


def test_batch_d_form_matches_the_e_form(bsalib, batch):
    """The whole batch again in the D1 / D3 form (k_bfm_batch with symmetric D1 up to 24
    modes): the same moments to the split-precision reassociation."""
    out, _ = batch
    sw = api.Sweep()
    for p in CASES:
        sw.add(p)
    outd, _ = sw.run(form=0)
    sw.clear()
    for k in range(len(CASES)):
        assert rel(outd[k]["m3mr"], out[k]["m3mr"]) < 1e-5, k
        assert rel(outd[k]["m3mf"], out[k]["m3mf"]) < 1e-5, k
        assert rel(outd[k]["m2mr"], out[k]["m2mr"]) < 1e-12, k


def test_batch_within_mixed_bar_of_fp64(batch):
    out, _ = batch
    for k in (1, 3, 5, 8):
        ref = single(CASES[k], api.PREC_FP64)
        assert rel(out[k]["m3mr"], ref["m3mr_cls"]) < 1e-4, k
        assert rel(out[k]["m3mf"], ref["m3mf_cls"]) < 1e-4, k


def test_batch_latencies(batch):
    out, total = batch
    ms = np.array([o["ms"] for o in out])
    assert np.all(ms > 0.0)
    assert np.all(ms <= total)


def test_batch_wind_cases_of_one_structure(bsalib):
    # one structure under three mean wind speeds: the same modes, different forces
    probs = [random_structure(21, nodes=(120, 120), modes=(10, 10), nfreq_grid=(65, 65), U_mean=u)
             for u in (20.0, 30.0, 45.0)]
    sw = api.Sweep()
    for p in probs:
        sw.add(p)
    out, _ = sw.run()
    sw.clear()
    for k, p in enumerate(probs):
        ref = single(p, api.PREC_BF16X3)
        assert rel(out[k]["m3mr"], ref["m3mr_cls"]) < 1e-5
    v = [float(np.max(np.abs(o["m3mr"]))) for o in out]
    assert v[0] < v[1] < v[2]


def test_batch_leaves_current_inputs(bsalib):
    p = tall_building(nodes=64, modes=12, nfreqs=21, df=0.2, seed=3)
    s = api.BsaSession(p, precision=api.PREC_FP64)
    try:
        before = s.run()
        sw = api.Sweep()
        sw.add_current()
        other = copy.deepcopy(CASES[2])
        # a case set up through the setters of the same library instance
        s2 = api.BsaSession(other, precision=api.PREC_BF16X3)
        sw.add_current()
        s2.close()
        s = api.BsaSession(p, precision=api.PREC_FP64)
        sw.run()
        after = s.run()
        sw.clear()
    finally:
        s.close()
    assert rel(after["m3mr_cls"], before["m3mr_cls"]) < 1e-12
    assert rel(after["m2mr_cls"], before["m2mr_cls"]) < 1e-12


def test_batch_rejects_unsupported_cases(bsalib):
    sw = api.Sweep()
    big = tall_building(nodes=60, modes=70, nfreqs=9, df=0.5, seed=2)
    s = api.BsaSession(big, precision=api.PREC_BF16X3)
    try:
        with pytest.raises(api.BsaError, match="64 kept modes"):
            sw.add_current()
    finally:
        s.close()
    d = copy.deepcopy(CASES[1])
    d.settings.onlyd = 1
    s = api.BsaSession(d, precision=api.PREC_BF16X3)
    try:
        with pytest.raises(api.BsaError, match="full-tensor"):
            sw.add_current()
    finally:
        s.close()
    with pytest.raises(api.BsaError, match="empty batch"):
        sw.run()
