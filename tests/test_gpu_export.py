"""bsa_setBispExportCallback: the Classic response bispectra streamed to a callback during
bsa_Run, in the reference's loop order (f1 fastest, then f2), equal to the materialised
bispectra and to the oracle; the moments of the exporting run equal the plain FP64 run's."""
import numpy as np
import pytest

from bsalib_gb300 import api
from bsalib_gb300.problem import tall_building
from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("prec", [api.PREC_FP64, api.PREC_BF16X3])
def test_export_stream_matches_materialised(bsalib, prec):
    prob = tall_building(nodes=16, modes=4, nfreqs=7, df=0.3, seed=21)
    got = []
    s = api.BsaSession(prob, precision=prec)
    try:
        s.set_export(lambda f1, f2, brm: got.append((f1, f2, brm)))
        out = s.run()
        s.set_export(None)
        s.set_precision(api.PREC_FP64)
        ref = s.run()
        f, bf, br = s.classic_bispectra()
    finally:
        s.close()
    f1 = np.concatenate([g[0] for g in got])
    f2 = np.concatenate([g[1] for g in got])
    b = np.concatenate([g[2] for g in got])
    nf = f.size
    assert f1.size == nf * nf
    np.testing.assert_array_equal(f1, np.tile(f, nf))
    np.testing.assert_array_equal(f2, np.repeat(f, nf))
    # br from classic_bispectra is [i1][i2][mno]; the stream is i1 fastest
    assert rel(b, br.transpose(1, 0, 2).reshape(nf * nf, -1)) < 1e-12
    assert rel(b, Oracle(prob).classic_vect()["br"].transpose(1, 0, 2).reshape(nf * nf, -1)) < 1e-10
    assert rel(out["m3mr_cls"], ref["m3mr_cls"]) < 1e-12
    assert rel(out["m3mf_cls"], ref["m3mf_cls"]) < 1e-12
