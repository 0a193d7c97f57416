"""Device blocks kept across bsa_Init ... bsa_Finalise cycles (bsa_gpu_releaseDeviceCache):
an analysis on reused blocks gives the same bits as the first one, before and after the cache
is freed."""
import numpy as np
import pytest

from bsalib_gb300 import api
from bsalib_gb300.problem import cantilever_tower, tall_building

pytestmark = pytest.mark.gpu


def analysis(prob, prec):
    s = api.BsaSession(prob, precision=prec)
    try:
        return s.run()
    finally:
        s.close()


@pytest.mark.parametrize("prec", [api.PREC_FP64, api.PREC_BF16X3])
def test_reused_blocks_same_results(bsalib, prec):
    big = tall_building(nodes=64, modes=12, nfreqs=33, df=0.2, seed=3)
    small = cantilever_tower(nodes=30)
    first = analysis(big, prec)
    analysis(small, prec)  # leaves blocks of other sizes in the cache
    again = analysis(big, prec)
    for k in ("m3mr_cls", "m3mf_cls", "m2mr_cls"):
        assert np.array_equal(first[k], again[k]), k
    assert bsalib.bsa_gpu_releaseDeviceCache() == 0
    fresh = analysis(big, prec)
    for k in ("m3mr_cls", "m3mf_cls", "m2mr_cls"):
        assert np.array_equal(first[k], fresh[k]), k
