"""The oracle pinned against the reference's own Classic kernel: BsaCL's OpenCL C kernel
(BsaCL/src/bsacl.cl, kernel 2) compiled for the host from the reference tree by
oracle/bsacl_ref.py and run there (oracle/bsacl_ref_driver.c), on small structures with one
wind zone (the kernel reads one turbulence intensity and scale per component), the same
coherence for every component (it reads the first component's) and the u component (it
evaluates the u form of the von Karman spectrum for every component, where the Fortran uses
the v and w forms; test_kernel_uses_the_u_form_for_w shows the difference).

* nodal wind PSD (von Karman, Davenport): the kernel's evalFct against orc_eval_psd;
* m3mr and the force bispectrum summed over frequency pairs, with the host code's integration
  weight (bsacl.c:1362-1366), against the oracle's point BFM / BRM (orc_msh_bfm_direct,
  orc_msh_brm).

Tolerance 2e-7 relative (max-norm): the kernel writes its PSD constants as float literals
(70.7f, 2.f/3.f), which moves its PSD by up to 4.3e-8 from the FP64 values.  The kernel as
shipped (its _use_optimised_loop_ branch) leaves out the node triples (k, k, j), (k, j, k),
(j, k, k), k < j: it matches the oracle's three terms summed over the other triples, while its
plain-loop branch matches the oracle's full triple sum, the reference's Fortran form.  Runs
only where the reference tree is present (this container, not the GPU host)."""
import dataclasses
import itertools

import numpy as np
import pytest

from bsalib_gb300.problem import cantilever_tower, tall_building
from oracle import bsacl_ref
from oracle.oracle import Oracle

pytestmark = pytest.mark.skipif(not bsacl_ref.available(), reason="reference BsaCL source not present")
TOL = 2e-7


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def one_zone(p):
    p.sigma[:, :] = p.sigma[:, :1]
    p.L[:, :, :] = p.L[:, :, :1]
    return p


def tower(psd_type=1):
    p = one_zone(cantilever_tower(nfreqs=9, df=0.125, nodes=5))
    p.psd_type = psd_type
    return p


def building():
    p = one_zone(tall_building(nodes=6, modes=3, nfreqs=9, df=0.125, seed=7))
    p.settings = dataclasses.replace(p.settings, tc=(1,))
    return p


def kernel_args(p, o):
    m = o.modes - 1
    scl = np.array([p.L[0, 0, 0], p.L[1, 0, 0], p.L[2, 0, 0]])
    return dict(tc=np.array(p.settings.tc), nodes_load=p.n_load, phitc=o.phitc, nod_corr=p.nod_corr[:, 0],
                u=p.u_node, scl=scl, std=p.sigma[:, 0].copy(), winz=p.wz_node, Mg=p.Mg[m],
                Cg=p.Cg[np.ix_(m, m)], Kg=p.Kg[m])


def run_kernel(p, o, fi, fj, plain_loop, frf=True):
    ref = bsacl_ref.BsaclRef(len(p.settings.tc), p.nnl, o.nme, p.nn, fi.size, fj.size, p.psd_type, plain_loop)
    a = kernel_args(p, o)
    if not frf:  # H = 1: the force bispectrum
        a.update(Mg=np.zeros(o.nme), Cg=np.zeros((o.nme, o.nme)), Kg=np.ones(o.nme))
    return ref.m3mr(a["tc"], a["nodes_load"], a["phitc"], a["nod_corr"], a["u"], a["scl"], a["std"], a["winz"],
                    a["Mg"], a["Cg"], a["Kg"], fi, fj)


def weight(fi, fj):
    return (fi[1] - fi[0]) * (fj[1] - fj[0]) * 4.0 * np.pi ** 2


def bfm_triples(p, o, f1, f2, triples):
    """The oracle's three BFM terms (functionsImpl.F90:1494-1538) over a set of node triples."""
    nm = o.nme
    out = np.zeros((nm, nm, nm))
    for tc in p.settings.tc:
        l, q = o.phitc[:, :, tc - 1], o.phitc[:, :, tc + 2]
        S1, S2, S3 = o.cross_psd(f1, tc), o.cross_psd(f2, tc), o.cross_psd(f1 + f2, tc)
        for (i, j, k) in triples:
            out += 2.0 * (np.einsum("m,n,o->mno", q[:, i], l[:, j], l[:, k]) * S1[i, j] * S2[i, k]
                          + np.einsum("m,n,o->mno", l[:, i], q[:, j], l[:, k]) * S3[i, j] * S2[j, k]
                          + np.einsum("m,n,o->mno", l[:, i], l[:, j], q[:, k]) * S1[j, k] * S3[i, k])
    return out.reshape(-1, order="F")


def shipped_triples(n):
    t = [(k, k, k) for k in range(n)]
    for k in range(n):
        for j in range(k + 1, n):
            t += [(j, j, k), (j, k, j), (k, j, j)]
            for i in range(j + 1, n):
                t += list(set(itertools.permutations((i, j, k))))
    return t


@pytest.mark.parametrize("psd_type", [1, 5])
def test_nodal_psd(psd_type):
    p = tower(psd_type)
    o = Oracle(p)
    f = np.array([-0.7, -0.2, 0.05, 0.3, 1.1])
    ref = bsacl_ref.BsaclRef(1, p.nnl, o.nme, p.nn, f.size, f.size, psd_type)
    S = o.psd(f, 1)
    k = np.array([[ref.psd(x, p.L[0, 0, 0], p.sigma[0, 0], p.u_node[n]) for n in range(p.nnl)] for x in f])
    assert rel(k, S) < TOL


@pytest.mark.parametrize("make", [tower, building])
def test_plain_loop_kernel_matches_the_oracle(make):
    p = make()
    o = Oracle(p)
    fi = np.linspace(-0.6, 0.6, 5)
    fj = np.linspace(-0.45, 0.45, 4)
    w = weight(fi, fj)
    bf = sum(o.msh_bfm(x, y) for y in fj for x in fi) * w
    br = sum(o.msh_brm(x, y, o.msh_bfm(x, y))[:, 0] for y in fj for x in fi) * w
    assert rel(run_kernel(p, o, fi, fj, True, frf=False), bf) < TOL
    assert rel(run_kernel(p, o, fi, fj, True), br) < TOL


def test_shipped_kernel_sums_fewer_node_triples():
    p = tower()
    o = Oracle(p)
    f = np.linspace(-0.5, 0.5, 4)
    w = weight(f, f)
    t = shipped_triples(p.nnl)
    assert len(t) == p.nnl ** 3 - 3 * p.nnl * (p.nnl - 1) // 2
    part = sum(bfm_triples(p, o, x, y, t) for y in f for x in f) * w
    full = sum(o.msh_bfm(x, y) for y in f for x in f) * w
    got = run_kernel(p, o, f, f, False, frf=False)
    assert rel(got, part) < TOL
    assert rel(got, full) > 1e-2  # the shipped kernel is not the Fortran form


def test_kernel_uses_the_u_form_for_w():
    p = one_zone(tall_building(nodes=6, modes=3, nfreqs=9, df=0.125, seed=7))
    o = Oracle(p)
    f = np.array([-0.7, -0.2, 0.05, 0.3, 1.1])
    ref = bsacl_ref.BsaclRef(2, p.nnl, o.nme, p.nn, f.size, f.size, 1)
    for tc, same in ((1, True), (3, False)):
        S = o.psd(f, tc)
        k = np.array([[ref.psd(x, p.L[tc - 1, 0, 0], p.sigma[tc - 1, 0], p.u_node[n]) for n in range(p.nnl)]
                      for x in f])
        assert (rel(k, S) < TOL) == same
