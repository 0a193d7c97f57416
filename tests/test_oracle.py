"""CPU tests of the oracle (the C restatement of the reference) against the golden vectors
and the independent numpy restatements.  No GPU."""
import os

import numpy as np
import pytest

from bsalib_gb300.problem import cantilever_tower, tall_building
from oracle.oracle import Oracle, classic_weights

GOLD = os.path.join(os.path.dirname(__file__), "golden")
RTOL = 1e-12  # oracle vs its numpy cross-check: same FP64 math, different summation order


def rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


@pytest.mark.parametrize("name,prob", [
    ("tower6_nf9", cantilever_tower(nfreqs=5, df=0.5, nodes=6)),
    ("building8_2tc_nf7", tall_building(nodes=8, modes=3, nfreqs=4, df=0.5, seed=7)),
])
def test_classic_vect_matches_golden(name, prob):
    g = np.load(os.path.join(GOLD, name + ".npz"))
    o = Oracle(prob)
    r = o.classic_vect()
    np.testing.assert_allclose(r["f"], g["f"], rtol=0, atol=0)
    assert rel(r["bf"], g["bf"]) < RTOL
    assert rel(r["br"], g["br"]) < RTOL
    assert rel(r["m3mf"], g["m3mf"]) < RTOL
    assert rel(r["m3mr"], g["m3mr"]) < RTOL


def test_mesher_direct_matches_golden():
    g = np.load(os.path.join(GOLD, "tower6_points.npz"))
    o = Oracle(cantilever_tower(nfreqs=5, df=0.5, nodes=6))
    for k, (a, b) in enumerate(g["pts"]):
        assert rel(o.msh_bfm(a, b), g["bf"][k]) < RTOL
        br = o.msh_brm(np.array([a]), np.array([b]), o.msh_bfm(a, b))[:, 0]
        assert rel(br, g["br"][k]) < RTOL


def test_pod_full_rank_equals_direct():
    """getFM_full_tm_scalar_msh_POD_ with every POD mode kept is the direct form."""
    o = Oracle(tall_building(nodes=10, modes=3, nfreqs=4, df=0.5, seed=3))
    for a, b in [(0.3, 0.9), (-1.1, 0.4)]:
        assert rel(o.pod_point(a, b), o.direct_point(a, b)) < 1e-10


def test_pod_count_quirk():
    """getNPODModesByThreshold_ as built with dsyev (ascending eigenvalues): it inspects the
    two smallest eigenvalues, so it keeps 1 POD mode unless the second smallest reaches the
    limit."""
    from oracle.oracle import pod_count
    assert pod_count([1e-9, 1e-6, 0.5, 2.0], 0.05) == 1          # usual: one mode
    assert pod_count([1e-9, 0.2, 0.5, 2.0], 0.05) == 0           # eig(2) >= 0.05 * 2
    assert pod_count([0.3, 0.3, 0.3], 0.05) == 1                 # all equal
    assert pod_count([0.2, 0.3, 0.5, 2.0], 0.05) == 0            # reference reads eig(0): 0 here


def _truncated(o, f, tc, n):
    D, V = np.linalg.eigh(o.cross_psd(f, tc))
    return (V[:, -n:] * D[-n:]) @ V[:, -n:].T


def test_pod_truncated_is_direct_with_truncated_spectra():
    """The truncated POD sum equals the direct triple sum with each S(f) replaced by its
    expansion over the kept eigenpairs -- the identity the device path is built on (the A
    table of the Mesher frequencies from the truncated S)."""
    o = Oracle(tall_building(nodes=9, modes=3, nfreqs=4, df=0.5, seed=4))
    nm = o.nme
    for f1, f2, nkeep in [(0.3, 0.9, 4), (-1.1, 0.4, 2)]:
        pod = o.pod_point(f1, f2, nmodes=nkeep)
        out = np.zeros((nm, nm, nm))
        for tc in o.prob.settings.tc:
            l = o.phitc[:, :, tc - 1]
            q = o.phitc[:, :, tc + 2]
            S1, S2, S3 = (_truncated(o, f, tc, nkeep) for f in (f1, f2, f1 + f2))
            t1 = np.einsum("mi,nj,ok,ij,ik->mno", q, l, l, S1, S2)
            t2 = np.einsum("mi,nj,ok,ij,jk->mno", l, q, l, S3, S2)
            t3 = np.einsum("mi,nj,ok,jk,ik->mno", l, l, q, S1, S3)
            out += 2.0 * (t1 + t2 + t3)
        assert rel(pod, out.reshape(-1, order="F")) < 1e-10
        assert rel(pod, o.direct_point(f1, f2)) > 1e-6   # the truncation changes the result
    # threshold form: one POD mode per spectrum where the second smallest eigenvalue is below
    # the limit (the quirk above), none where it reaches it
    pod1 = o.pod_point(0.3, 0.9, trunc_lim=0.5)
    assert rel(pod1, o.pod_point(0.3, 0.9, nmodes=1)) < 1e-12
    assert not np.any(o.pod_point(0.3, 0.9, trunc_lim=1e-12))


def test_scalar_classic_is_uniform_weight_sum():
    """Scalar Classic (BsaClassicImpl.F90:255-363): every pair weighted dw^2."""
    p = cantilever_tower(nfreqs=4, df=0.5, nodes=5)
    o = Oracle(p)
    v = o.classic_vect()
    s = o.classic_scalar()
    dw2 = ((v["f"][1] - v["f"][0]) * 2 * np.pi) ** 2
    assert rel(s["m3mf"], v["bf"].sum(axis=(0, 1)) * dw2) < RTOL
    assert rel(s["m3mr"], v["br"].sum(axis=(0, 1)) * dw2) < RTOL


def test_classic_weights_quirk():
    """Q2: vertices weigh -d^2/2, borders d^2/2, interior d^2."""
    w = classic_weights(5, 0.25)
    d2 = (0.25 * 2 * np.pi) ** 2
    assert np.isclose(w[0, 0], -0.5 * d2) and np.isclose(w[4, 4], -0.5 * d2)
    assert np.isclose(w[0, 2], 0.5 * d2) and np.isclose(w[2, 2], d2)


def test_grid_and_overrides():
    p = cantilever_tower()
    o = Oracle(p)
    f = o.freqs()
    assert f.size == 129 and f[0] == -2.0 and f[-1] == 2.0
    # outside test mode a too-coarse df is overridden by min(xsi*f)/5 (BsaClassicImpl.F90:458-530)
    g = o.freqs(test_mode=0)
    df_ref = np.min(p.xsi * p.natf) / 5
    assert np.isclose(g[1] - g[0], df_ref)
    assert g[-1] >= p.natf.max()


def test_psd_models_known_values():
    """Closed-form values of the nodal PSD models at f = 0 (WindPSDImpl.F90:149-316)."""
    p = cantilever_tower(nodes=3)
    o = Oracle(p)
    U = p.u_node[0]
    sig = p.sigma[0, 0]
    L = p.L[0, 0, 0]
    s0 = o.psd(np.array([0.0]), 1)[0, 0]
    assert np.isclose(s0, 4 * sig * sig * L / U / (4 * np.pi))
    p.psd_type = 5
    assert o.__class__(p).psd(np.array([0.0]), 1)[0, 0] == 0.0
    p.psd_type = 2
    assert np.all(o.__class__(p).psd(np.linspace(-1, 1, 5), 1) == 0.0)


def test_mode_validation_drops_unnormalised():
    """Q7: a mode whose max|Phi| != 1 is skipped (BsaLibImpl.F90:545-599)."""
    p = cantilever_tower(nodes=6)
    p.phi = p.phi.copy(order="F")
    p.phi[:, 1] *= 0.5
    o = Oracle(p)
    assert list(o.modes) == [1, 3, 4]


def test_skewness_and_recombination():
    p = cantilever_tower(nfreqs=4, df=0.5, nodes=5)
    o = Oracle(p)
    r = o.classic_vect(keep_bisp=False)
    sk = o.skewness(r["m2mr"], r["m3mr"])
    nm = o.nme
    m2 = r["m2mr"].reshape(nm, nm)
    sig = np.sqrt(np.diag(m2))
    ref = r["m3mr"].reshape(nm, nm, nm, order="F") / np.einsum("i,j,k->ijk", sig, sig, sig)
    assert rel(sk, ref.reshape(-1, order="F")) < 1e-13
    m2n, m3n, skn = o.modal_recomb(r["m2mr"], r["m3mr"])
    phi = p.phi[:, o.modes - 1]
    m3r = np.einsum("di,dj,dk,ijk->d", phi, phi, phi, r["m3mr"].reshape(nm, nm, nm, order="F"))
    assert rel(m3n, m3r) < 1e-12
