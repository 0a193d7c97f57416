"""The response-bispectrum export files of bsa_Run (visual mode and base export mode,
src/bsa/BsaLibImpl.F90:119-233, 1764-1913): header and zone records, and every exported value
against the library's own bispectra (the materialised Classic grid; the Mesher's export
callback, which receives the same per-zone BRM lattices) to float32 rounding."""
import numpy as np
import pytest

from bsalib_gb300 import api, brmfile
from bsalib_gb300.problem import cantilever_tower, tall_building

pytestmark = pytest.mark.gpu


def f32rel(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def test_classic_visual_modal(bsalib, tmp_path, monkeypatch):
    monkeypatch.chdir(tmp_path)
    prob = cantilever_tower(nfreqs=9, df=0.25, nodes=12)
    s = api.BsaSession(prob, precision=api.PREC_FP64)
    try:
        f, bf, br = s.classic_bispectra()
        nm = s.nmodes()
        s.set_visual([2, 1, 3], modal=True)
        s.run()
    finally:
        s.close()
    d = brmfile.read(tmp_path / "bsaexport_cls.brm")
    nf = f.size
    assert (d["nm"], list(d["modes"]), d["ncomb"], d["nzones"], d["npts"]) == (3, [2, 1, 3], 1, 1, nf * nf)
    z = d["zones"][0]
    assert (z["id"], z["nI"], z["nJ"]) == (1, nf, nf)
    vis = (3 - 1) * nm * nm + (1 - 1) * nm + (2 - 1)
    want = br[:, :, vis].T.ravel()   # f1 fastest, then f2 (the reference's j-outer loop)
    assert np.allclose(z["f1"], np.tile(f, nf).astype(np.float32))
    assert np.allclose(z["f2"], np.repeat(f, nf).astype(np.float32))
    assert f32rel(z["values"][:, 0], want) < 1e-6


def mesher_export(prob, tmp_path, monkeypatch, setup):
    monkeypatch.chdir(tmp_path)
    got = []
    s = api.BsaSession(prob, precision=api.PREC_FP64)
    try:
        s.use_driver_controls()
        s.set_export(lambda f1, f2, brm: got.append((f1, f2, brm)))
        setup(s)
        s.run()
        nm = s.nmodes()
    finally:
        s.close()
    return got, nm


def test_mesher_base_export(bsalib, tmp_path, monkeypatch):
    prob = tall_building(nodes=12, modes=3, nfreqs=9, df=0.25, seed=5)
    prob.settings.suban = 2
    got, nm = mesher_export(prob, tmp_path, monkeypatch, lambda s: s.set_brm_export_mode(1))
    d = brmfile.read(tmp_path / "bsaexport_msh.brm")
    assert d["nm"] == nm and d["ncomb"] == nm ** 3 and d["nzones"] == len(got) == len(d["zones"])
    assert d["npts"] == nm   # the count record is rewritten in visual mode only
    for z, (f1, f2, brm) in zip(d["zones"], got):
        assert z["nI"] * z["nJ"] == f1.size
        assert np.allclose(z["f1"], f1.astype(np.float32)) and np.allclose(z["f2"], f2.astype(np.float32))
        assert f32rel(z["values"], brm) < 1e-6


def test_mesher_visual_nodal(bsalib, tmp_path, monkeypatch):
    prob = tall_building(nodes=12, modes=3, nfreqs=9, df=0.25, seed=5)
    prob.settings.suban = 2
    node, dof = 7, 1
    got, nm = mesher_export(prob, tmp_path, monkeypatch, lambda s: s.set_visual([node, dof, 1], modal=False))
    d = brmfile.read(tmp_path / "bsaexport_msh.brn")
    assert (d["nm"], list(d["modes"]), d["ncomb"]) == (2, [node, dof], 1)
    assert d["npts"] == sum(f1.size for f1, _, _ in got)
    from oracle.oracle import Oracle
    modes = Oracle(prob).modes - 1
    phi = prob.phi[(node - 1) * prob.nlibs + (dof - 1), modes]
    # getBRN_full_scalar_ as the reference reads it: m = MODES(in), so phi_n phi_n phi_o
    w = np.einsum("n,o->no", phi * phi, phi)
    W = np.broadcast_to(w[None], (nm, nm, nm)).reshape(-1, order="F")
    for z, (f1, f2, brm) in zip(d["zones"], got):
        assert f32rel(z["values"][:, 0], brm @ W) < 1e-5
