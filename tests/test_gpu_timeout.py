"""The bounded device waits, exercised without a fault: bsa_gpu_setWaitTest makes CTA 0 of the
next split-precision Classic analysis (E form) omit one accumulator-ready signal, so that
CTA's epilogue wait runs out of its 2 s budget, every other wait of the launch sees the error
flag and gives up, in-flight copies and MMAs land, TMEM is freed and the kernel returns.  The
host reports BSA_ERR_TIMEOUT, the library halts until bsa_Finalise, and the next analysis in a
new session runs normally on the same context."""
import time

import numpy as np
import pytest

from bsalib_gb300 import api
from bsalib_gb300.problem import tall_building

pytestmark = pytest.mark.gpu


def test_wait_budget_runs_out_and_the_context_stays_usable(bsalib):
    prob = tall_building(nodes=40, modes=12, nfreqs=33, df=0.125, seed=3)
    s = api.BsaSession(prob, precision=api.PREC_BF16X3)
    try:
        ref = s.run()["m3mr_cls"]
    finally:
        s.close()
    s = api.BsaSession(prob, precision=api.PREC_BF16X3)
    try:
        assert bsalib.bsa_gpu_setWaitTest(3) == 0
        t0 = time.perf_counter()
        with pytest.raises(api.BsaError) as exc:
            s.run()
        dt = time.perf_counter() - t0
        assert "ran out of its budget" in str(exc.value)
        assert exc.value.code == -5          # BSA_ERR_TIMEOUT
        assert dt < 30.0
        assert s.lib.bsa_gpu_setPrecision(1) == -2   # halted (BSA_ERR_STATE) until bsa_Finalise
    finally:
        s.close()
    s = api.BsaSession(prob, precision=api.PREC_BF16X3)
    try:
        again = s.run()["m3mr_cls"]
    finally:
        s.close()
    assert float(np.max(np.abs(again - ref)) / np.max(np.abs(ref))) < 1e-12
