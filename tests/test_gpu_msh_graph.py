"""The split-precision Mesher zone pass as one CUDA graph (bsa_gpu_setMesherGraphs): the graph
and the kernel-by-kernel launch give the same moments (to the 1e-12 by which the zone sums'
order can move them), and the statistics count one graph per zone pass."""
import numpy as np
import pytest

from bsalib_gb300 import api
from bsalib_gb300.problem import bridge_deck

pytestmark = pytest.mark.gpu


def test_graph_and_direct_launch_agree(bsalib):
    prob = bridge_deck(nodes=160, modes=10)
    out = {}
    for on in (1, 0):
        s = api.BsaSession(prob, precision=api.PREC_BF16X3)
        try:
            s.use_driver_controls()
            assert s.lib.bsa_gpu_setMesherGraphs(on) == 0
            r = s.run()
            st = s.stats()
            out[on] = (r["m3mr_msh"], r["m3mf_msh"], st.graphs, st.kernels)
        finally:
            s.close()
    assert out[1][2] >= 1 and out[0][2] == 0
    assert out[1][3] == out[0][3]
    rel = lambda a, b: float(np.max(np.abs(a - b)) / np.max(np.abs(b)))
    assert rel(out[1][0], out[0][0]) < 1e-12 and rel(out[1][1], out[0][1]) < 1e-12


def test_device_and_host_expansion_agree(bsalib):
    """The zone pass expanded on the device (hash-table frequencies, tasks and work queue built by
    kernels) and on the host give the same moments to FP32 rounding (the A rows' frequencies
    differ by under 5e-13 Hz), and the device expansion is deterministic run to run."""
    prob = bridge_deck(nodes=160, modes=10)
    out = {}
    for dev in (1, 0, 1):
        s = api.BsaSession(prob, precision=api.PREC_BF16X3)
        try:
            s.use_driver_controls()
            assert s.lib.bsa_gpu_setMesherExpansion(dev) == 0
            r = s.run()
            out.setdefault(dev, []).append((r["m3mr_msh"], r["m3mf_msh"]))
        finally:
            s.close()
    rel = lambda a, b: float(np.max(np.abs(a - b)) / np.max(np.abs(b)))
    (d0, d1), (h0, h1) = out[1][0], out[0][0]
    assert rel(d0, h0) < 1e-6 and rel(d1, h1) < 1e-6
    assert rel(out[1][1][0], d0) < 1e-12 and rel(out[1][1][1], d1) < 1e-12
