"""bsa.extdata / bsa.bsadata round trips and the synthetic structures (CPU)."""
import numpy as np

from bsalib_gb300.problem import (cantilever_tower, read_inputs, tall_building, write_inputs,
                                  packed_coherence, random_structure)


def _same(a, b):
    for f in ("nn", "nlibs", "ndegw", "ndofs", "nm", "psd_type", "i_varu", "i_vert"):
        assert getattr(a, f) == getattr(b, f), f
    for f in ("n_load", "libs_load", "coords", "Zref", "UBref", "L", "sigma", "corrC", "corrEx", "lims",
              "rotW2G_z", "incang", "wz_node", "wAlt_node", "u_node", "nod_corr", "wfc", "natf", "phi",
              "Mg", "Kg", "Cg", "xsi"):
        x, y = getattr(a, f), getattr(b, f)
        assert x.shape == y.shape, f
        assert np.array_equal(x, y), f


def test_extdata_bsadata_round_trip(tmp_path):
    p = tall_building(nodes=12, modes=4, nfreqs=9, df=0.25, seed=5)
    write_inputs(p, str(tmp_path))
    q = read_inputs(str(tmp_path))
    _same(p, q)
    assert q.settings == p.settings


def test_extdata_size_matches_reader_order(tmp_path):
    p = cantilever_tower(nodes=7)
    write_inputs(p, str(tmp_path))
    nn, nnl, nz, nm = p.nn, p.nnl, p.nz, p.nm
    expect = 4 * 4 + 4 * (nnl + 1) + 8 * 3 * nn + 4 * 4 + 8 + 8 * 9 + 4 \
        + 8 * (nz + nz + 9 * nz + 3 * nz + 9 * nz + 9 * nz + nz + 1 + 9 * nz + nz) \
        + 4 * nn + 8 * (nn + nn + 3 * (nn * nn + nn) // 2 + 6 * nnl) \
        + 4 * 2 + 8 * (nm + nn * nm + nm + nm + nm * nm + nm)
    assert (tmp_path / "bsa.extdata").stat().st_size == expect


def test_tower_configuration():
    p = cantilever_tower()
    assert p.nn == 30 and p.nm == 4 and p.classic_nf() == 129
    assert np.all(np.max(np.abs(p.phi), axis=0) == 1.0)
    z = p.coords[2]
    assert np.isclose(z[-1], 100.0)
    assert np.allclose(p.u_node, 30 * (z / 10) ** 0.16)
    assert np.allclose(p.wfc[0, 0], 1.22 * 2 * p.u_node) and np.allclose(p.wfc[0, 3], 0.5 * 1.22 * 2)


def test_building_configuration():
    p = tall_building()
    assert p.nn == 400 and p.nm == 24 and p.classic_nf() == 1025 and p.settings.tc == (1, 3)
    assert np.all(np.max(np.abs(p.phi), axis=0) == 1.0)
    assert np.all((p.xsi >= 0.01) & (p.xsi <= 0.02))


def test_packed_coherence_index():
    z = np.array([0.0, 1.0, 3.0])
    U = np.array([10.0, 10.0, 10.0])
    c = packed_coherence(z, U, 10.0)
    # util_getCorrVectIndex: id = (ni-1)*N + nj - (ni^2-ni)/2, 1-based, nj >= ni
    idx = lambda i, j: (i - 1) * 3 + j - (i * i - i) // 2
    assert np.isclose(c[idx(1, 3) - 1], np.exp(-10 * 3 / 10))
    assert np.isclose(c[idx(2, 3) - 1], np.exp(-10 * 2 / 10))
    assert c[idx(2, 2) - 1] == 1.0


def test_random_structures_are_valid():
    for s in range(5):
        p = random_structure(s)
        assert np.all(np.max(np.abs(p.phi), axis=0) == 1.0)
        assert p.classic_nf() % 2 == 1
