"""bsa_loadInputFiles: the driver's bsa.bsadata / bsa.extdata read by the library itself give
the same analysis as the same problem set through the setters with the driver's Mesher
controls (bitwise)."""
import ctypes as C

import numpy as np
import pytest

from bsalib_gb300 import api
from bsalib_gb300.problem import tall_building, write_inputs

pytestmark = pytest.mark.gpu


def test_input_files_round_trip(bsalib, tmp_path):
    prob = tall_building(nodes=24, modes=5, nfreqs=7, df=0.3, seed=8)
    prob.settings.suban = 3  # Classic and Mesher
    write_inputs(prob, str(tmp_path))
    s = api.BsaSession(prob)
    try:
        s.use_driver_controls()   # bsa_loadInputFiles applies the driver's Mesher controls
        ref = s.run()
    finally:
        s.close()
    L = api.load()
    assert L.bsa_Init() == 0
    try:
        assert L.bsa_loadInputFiles(str(tmp_path).encode()) == 0, L.bsa_lastError()
        nm = C.c_int(0)
        assert L.bsa_getNModesEff(C.byref(nm)) == 0
        d2, d3 = nm.value ** 2, nm.value ** 3
        out = {k: np.zeros(d2) for k in ("m2mf_cls", "m2mr_cls", "m2o2mr_cls")}
        out.update({k: np.zeros(d3) for k in ("m3mf_msh", "m3mr_msh", "m3mf_cls", "m3mr_cls")})
        p = lambda a: a.ctypes.data_as(C.c_void_p)
        rc = L.bsa_Run(p(out["m2mf_cls"]), p(out["m2mr_cls"]), p(out["m2o2mr_cls"]), p(out["m3mf_msh"]),
                       p(out["m3mr_msh"]), p(out["m3mf_cls"]), p(out["m3mr_cls"]))
        assert rc == 0, L.bsa_lastError()
    finally:
        L.bsa_Finalise()
    for k in out:
        assert np.array_equal(out[k], ref[k]), k


def test_missing_files_are_an_error(bsalib, tmp_path):
    L = api.load()
    assert L.bsa_Init() == 0
    try:
        assert L.bsa_loadInputFiles(str(tmp_path / "nowhere").encode()) == -1
        assert b"cannot open" in L.bsa_lastError()
    finally:
        L.bsa_Finalise()
