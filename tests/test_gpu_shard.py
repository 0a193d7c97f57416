"""Shards of one Classic analysis (bsa_gpu_setClassicShard): the moments of the shards sum to
the whole analysis's, in FP64 (contiguous row blocks) and in the split precision's E form
(interleaved product rows) and D1 / D3 form (row blocks).  The split forms' sums differ from the
whole run only by the FP32 accumulation order (2e-6); FP64 to 1e-12."""
import numpy as np
import pytest

from bsalib_gb300 import api
from bsalib_gb300.problem import tall_building

pytestmark = pytest.mark.gpu
KEYS = ("m2mf_cls", "m2mr_cls", "m3mf_cls", "m3mr_cls")


def rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


@pytest.mark.parametrize("prec,form,tol", [(api.PREC_FP64, 1, 1e-12), (api.PREC_BF16X3, 1, 2e-6),
                                           (api.PREC_BF16X3, 0, 2e-6)])
@pytest.mark.parametrize("n", [2, 3])
def test_shards_sum_to_the_whole_analysis(bsalib, prec, form, tol, n):
    prob = tall_building(nodes=40, modes=12, nfreqs=33, df=0.125, seed=3)
    s = api.BsaSession(prob, precision=prec)
    try:
        s.set_classic_form(form)
        full = s.run()
        tot = {k: np.zeros_like(full[k]) for k in KEYS}
        for r in range(n):
            s.set_shard(r, n)
            part = s.run()
            for k in KEYS:
                tot[k] += part[k]
        s.set_shard(0, 1)
        again = s.run()
    finally:
        s.close()
    for k in KEYS:
        assert rel(tot[k], full[k]) < (1e-12 if k.startswith("m2") else tol), k
        assert rel(again[k], full[k]) < 1e-12, k
