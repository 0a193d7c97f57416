"""Generate tests/golden/bsacl_ref.npz (run from the repository root where the reference tree
is present: `python tests/golden/make_bsacl_golden.py`).

The numbers are the reference's own: its BsaCL Classic kernel (BsaCL/src/bsacl.cl, kernel 2)
compiled for the host and run by oracle/bsacl_ref.py, with the reference's host-side
integration weight (bsacl.c:1362-1366).  Per case: the frequency vectors fi, fj, and the
force (H = 1) and response m3 sums over the pairs fi x fj, from the kernel's full
triple-loop branch (the reference's Fortran form) and from the kernel as shipped (its
optimised loop, which leaves out the node triples (k, k, j), (k, j, k), (j, k, k), k < j).
The problems are rebuilt by tests from `case_problem(name)`.

Per-pair-group cases (GROUP_CASES): the 30-node tower of the Classic tower workload (four
modes, one wind zone per node with the zones' turbulence collapsed to one intensity and scale,
as the kernel reads) on 16 x 64 = 1024 frequency pairs of its 129-point grid, von Karman and
Davenport spectra.  For them the file holds the kernel's per-work-group partials (16 pairs
each, fi fastest: group g is every fi at fj[g]), from its full triple-loop branch, as shipped
(float PSD literals) and with the two literals written in double precision (oracle/bsacl_ref.py,
exact_literals).  The Davenport case uses positive frequencies only: the kernel's plain-loop
branch evaluates that spectrum with f where the Fortran (WindPSDImpl.F90:283-316) and the
kernel's shipped branch use |f|.
"""
import dataclasses
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from bsalib_gb300.problem import cantilever_tower, tall_building  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "bsacl_ref.npz")


def one_zone(p):
    """One wind zone (the kernel reads one turbulence intensity and scale per component)."""
    p.sigma[:, :] = p.sigma[:, :1]
    p.L[:, :, :] = p.L[:, :, :1]
    return p


def case_problem(name):
    if name == "tower5":
        return one_zone(cantilever_tower(nfreqs=9, df=0.125, nodes=5))
    if name == "building6":
        p = one_zone(tall_building(nodes=6, modes=3, nfreqs=9, df=0.125, seed=7))
        p.settings = dataclasses.replace(p.settings, tc=(1,))
        return p
    raise KeyError(name)


CASES = {"tower5": (np.linspace(-0.6, 0.6, 5), np.linspace(-0.45, 0.45, 4)),
         "building6": (np.linspace(-0.9, 0.6, 6), np.linspace(-0.5, 0.7, 5))}

# the tower's Classic grid: 129 points on [-2, 2] Hz
_F = (np.arange(129) - 64) / 32.0
GROUP_CASES = {"tower30_vk": (_F[4::8], _F[1::2]),          # 16 x 64, both signs
               "tower30_dav": (_F[68::4], _F[65:129])}      # 16 x 64, f > 0


def group_problem(name):
    p = one_zone(cantilever_tower())
    if name == "tower30_dav":
        p.psd_type = 5
    elif name != "tower30_vk":
        raise KeyError(name)
    return p


def _group_run(job):
    name, exact, frf = job
    from oracle import bsacl_ref
    from oracle.oracle import Oracle
    fi, fj = GROUP_CASES[name]
    p = group_problem(name)
    o = Oracle(p)
    m = o.modes - 1
    scl = np.array([p.L[0, 0, 0], p.L[1, 0, 0], p.L[2, 0, 0]])
    args = [np.array(p.settings.tc), p.n_load, o.phitc, p.nod_corr[:, 0], p.u_node, scl, p.sigma[:, 0].copy(),
            p.wz_node]
    h = [p.Mg[m], p.Cg[np.ix_(m, m)], p.Kg[m]] if frf else [np.zeros(o.nme), np.zeros((o.nme, o.nme)),
                                                              np.ones(o.nme)]
    ref = bsacl_ref.BsaclRef(len(p.settings.tc), p.nnl, o.nme, p.nn, fi.size, fj.size, p.psd_type, True, exact)
    g = ref.groups(*args, *h, fi, fj)
    return f"{name}_{'exact' if exact else 'shipped'}_{'mr' if frf else 'mf'}_groups", g[: fi.size * fj.size // 16]


def main():
    from oracle import bsacl_ref
    from oracle.oracle import Oracle
    out = {}
    for name, (fi, fj) in CASES.items():
        p = case_problem(name)
        o = Oracle(p)
        m = o.modes - 1
        scl = np.array([p.L[0, 0, 0], p.L[1, 0, 0], p.L[2, 0, 0]])
        args = [np.array(p.settings.tc), p.n_load, o.phitc, p.nod_corr[:, 0], p.u_node, scl, p.sigma[:, 0].copy(),
                p.wz_node]
        frf = [p.Mg[m], p.Cg[np.ix_(m, m)], p.Kg[m]]
        one = [np.zeros(o.nme), np.zeros((o.nme, o.nme)), np.ones(o.nme)]
        for plain, tag in ((True, "plain"), (False, "shipped")):
            ref = bsacl_ref.BsaclRef(len(p.settings.tc), p.nnl, o.nme, p.nn, fi.size, fj.size, p.psd_type, plain)
            out[f"{name}_{tag}_m3mr"] = ref.m3mr(*args, *frf, fi, fj)
            out[f"{name}_{tag}_m3mf"] = ref.m3mr(*args, *one, fi, fj)
        out[f"{name}_fi"], out[f"{name}_fj"] = fi, fj
    import multiprocessing as mp
    jobs = [(n, e, r) for n in GROUP_CASES for e in (False, True) for r in (False, True)]
    with mp.get_context("spawn").Pool(2) as pool:
        for key, g in pool.imap_unordered(_group_run, jobs):
            out[key] = g
            print(key, g.shape, flush=True)
    for name, (fi, fj) in GROUP_CASES.items():
        out[f"{name}_fi"], out[f"{name}_fj"] = fi, fj
    np.savez_compressed(OUT, **out)
    print("wrote", OUT)


if __name__ == "__main__":
    main()
