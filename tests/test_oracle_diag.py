"""CPU tests of the oracle's diagonal-only spectra (i_only_diag_ = 1: same node, same mode)
against an independent numpy restatement written from the projected coefficients:

  Classic  B_m(f1,f2) = 2 sum_{tc,node} Q_m L_m^2 [S(f1)S(f2) + S(f1+f2)S(f2) + S(f1)S(f1+f2)]
  Mesher   B_m(f1,f2) = 2 sum_{tc,node} Q_m L_m^2 [S(f1)S(f2) + S(f1)S(f2)^2 + S(f1)^2 S(f2)]

(the Mesher form is the reference's own, functionsImpl.F90:1160-1166: S(f1+f2) is never read).
The oracle loops over the loaded-DOF triple with the raw coefficients; the product of the
three projected sums must equal it, so a two-DOF-per-node structure is tested too.  No GPU."""
import dataclasses

import numpy as np
import pytest

from bsalib_gb300.problem import cantilever_tower, tall_building
from oracle.oracle import Oracle, classic_weights

RTOL = 1e-12


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def two_dof(prob):
    """The same structure with two loaded DOFs per node (DOF 2: scaled shapes and its own
    force coefficients); mode shapes keep max |phi| = 1 on DOF 1."""
    nn, nm = prob.nn, prob.nm
    phi = np.zeros((2 * nn, nm), order="F")
    phi[0::2] = prob.phi
    phi[1::2] = 0.6 * prob.phi[::-1]
    wfc = np.zeros((2,) + prob.wfc.shape[1:], order="F")
    wfc[0] = prob.wfc[0]
    wfc[1] = 0.35 * prob.wfc[0]
    return dataclasses.replace(prob, nlibs=2, libs_load=np.array([1, 2], dtype=np.int32), phi=phi, wfc=wfc,
                               ndofs=2 * nn)


PROBLEMS = [
    ("tower", lambda: cantilever_tower(nfreqs=6, df=0.35, nodes=7)),
    ("building_2tc", lambda: tall_building(nodes=9, modes=4, nfreqs=5, df=0.4, seed=11)),
    ("tower_2dof", lambda: two_dof(cantilever_tower(nfreqs=5, df=0.4, nodes=6))),
]


def weights(o, prob):
    """(W3, W2, tc list): W3 = Q L^2 and W2 = L^2 per component, (nm, nnl)."""
    out = []
    for tc in prob.settings.tc:
        L = o.phitc[:, :, tc - 1]
        Q = o.phitc[:, :, tc + 2]
        out.append((tc, Q * L * L, L * L))
    return out


def np_classic_diag(o, prob, f):
    nf = f.size
    npad = (nf - 1) // 2
    bf = np.zeros((nf, nf, o.nme))
    psd = np.zeros((nf, o.nme))
    for tc, W3, W2 in weights(o, prob):
        S = o.psd(f, tc)
        idx = np.arange(nf)[:, None] + np.arange(nf)[None, :] - npad
        S12 = np.where(((idx >= 0) & (idx < nf))[..., None], S[np.clip(idx, 0, nf - 1)], 0.0)
        g = S[:, None, :] * S[None, :, :] + S12 * S[None, :, :] + S[:, None, :] * S12
        bf += 2 * np.einsum("ijn,mn->ijm", g, W3)
        psd += S @ W2.T
    H = np.array([o.frf(2 * np.pi * x) for x in f])                     # (nf, nm)
    H12 = np.array([[o.frf(2 * np.pi * a + 2 * np.pi * b) for b in f] for a in f])
    br = bf * np.real(H[:, None, :] * H[None, :, :] * np.conj(H12))
    pr = psd * np.abs(H) ** 2
    return bf, br, psd, pr


def np_mesher_diag(o, prob, fi, fj):
    b = np.zeros(o.nme)
    for tc, W3, _ in weights(o, prob):
        s1 = o.psd(np.array([fi]), tc)[0]
        s2 = o.psd(np.array([fj]), tc)[0]
        g = s1 * s2 + s1 * s2 * s2 + s1 * s1 * s2
        b += 2 * W3 @ g
    return b


@pytest.mark.parametrize("name,make", PROBLEMS)
def test_classic_vect_diag_vs_numpy(name, make):
    prob = make()
    o = Oracle(prob)
    r = o.classic_vect_diag()
    f = r["f"]
    bf, br, psd, pr = np_classic_diag(o, prob, f)
    assert rel(r["bf"], bf) < RTOL
    assert rel(r["br"], br) < RTOL
    w = classic_weights(f.size, f[1] - f[0])
    assert rel(r["m3mf"], np.einsum("ij,ijm->m", w, bf)) < RTOL
    assert rel(r["m3mr"], np.einsum("ij,ijm->m", w, br)) < RTOL
    d = (f[1] - f[0]) * 2 * np.pi
    wf = np.full(f.size, d)
    wf[0] = wf[-1] = d / 2
    assert rel(r["m2mf"], wf @ psd) < RTOL
    assert rel(r["m2mr"], wf @ pr) < RTOL
    assert rel(r["m2o2mr"], (wf * (2 * np.pi * f) ** 2) @ pr) < RTOL


@pytest.mark.parametrize("name,make", PROBLEMS[:2])
def test_classic_scalar_diag_vs_numpy(name, make):
    prob = make()
    o = Oracle(prob)
    f = o.freqs()
    r = o.classic_scalar_diag(f)
    bf, br, psd, pr = np_classic_diag(o, prob, f)
    d = (f[1] - f[0]) * 2 * np.pi
    assert rel(r["m3mf"], bf.sum(axis=(0, 1)) * d * d) < RTOL
    assert rel(r["m3mr"], br.sum(axis=(0, 1)) * d * d) < RTOL
    assert rel(r["m2mr"], pr.sum(axis=0) * d) < RTOL


def test_diag_is_the_node_and_mode_diagonal_of_the_full_tensor():
    """With one loaded node the full tensor's (m, m, m) entries are the diagonal spectra."""
    prob = cantilever_tower(nfreqs=5, df=0.4, nodes=1)
    o = Oracle(prob)
    full = o.classic_vect()
    diag = o.classic_vect_diag()
    nm = o.nme
    mmm = [m + nm * m + nm * nm * m for m in range(nm)]
    assert rel(diag["bf"], full["bf"][:, :, mmm]) < RTOL
    assert rel(diag["m3mr"], full["m3mr"][mmm]) < RTOL


@pytest.mark.parametrize("name,make", PROBLEMS)
def test_mesher_diag_vs_numpy(name, make):
    prob = make()
    o = Oracle(prob)
    pts = [(0.3, 0.7), (-0.45, 0.2), (1.1, -1.6), (0.0, 0.25)]
    for a, b in pts:
        bf = o.msh_bfm_diag(a, b)
        assert rel(bf, np_mesher_diag(o, prob, a, b)) < RTOL
        br = o.msh_brm_diag(a, b, bf)[:, 0]
        H1, H2, H3 = o.frf(2 * np.pi * a), o.frf(2 * np.pi * b), o.frf(2 * np.pi * (a + b))
        assert rel(br, bf * np.real(H1 * H2 * np.conj(H3))) < RTOL


def test_rect_zone_diag_unit_factors_is_trapezoid():
    prob = tall_building(nodes=6, modes=3, nfreqs=5, df=0.4, seed=5)
    o = Oracle(prob)
    ni, nj, dI, dJ = 4, 3, 0.1, 0.15
    mf, mr = o.rect_zone_diag(-0.3, 0.2, dI, 0.0, 0.0, dJ, ni, nj, 1, 1, 2.0)
    ef, er = np.zeros(o.nme), np.zeros(o.nme)
    for i in range(ni):
        for j in range(nj):
            a, b = -0.3 + i * dI, 0.2 + j * dJ
            w = 2.0 * (dI * 2 * np.pi) * (dJ * 2 * np.pi) * (0.5 if i in (0, ni - 1) else 1) * \
                (0.5 if j in (0, nj - 1) else 1)
            bf = o.msh_bfm_diag(a, b)
            ef += w * bf
            er += w * o.msh_brm_diag(a, b, bf)[:, 0]
    assert rel(mf, ef) < RTOL
    assert rel(mr, er) < RTOL


def test_skewness_diag():
    o = Oracle(cantilever_tower(nfreqs=5, df=0.4, nodes=5))
    m2 = np.array([2.0, 3.0, 0.5, 1.5])[: o.nme]
    m3 = np.array([0.3, -0.2, 0.05, 0.9])[: o.nme]
    assert rel(o.skewness_diag(m2, m3), m3 / m2 ** 1.5) < 1e-15
