"""Against the reference's own numbers: tests/golden/bsacl_ref.npz holds the m3 sums of the
reference's BsaCL Classic kernel run on the host (tests/golden/make_bsacl_golden.py) over
frequency pairs of two small structures.  The oracle's point BFM / BRM and the library's
point-set moments (bsa_gpu_mshMoments, FP64) must give them with the reference's host weight
dInfl = dfi dfj 4 pi^2 on every pair.

Tolerance 2e-7 relative (max-norm): the kernel writes its PSD constants as float literals,
which moves its spectra by up to 4.3e-8.  The kernel's plain triple loop is the reference's
Fortran form; the shipped kernel (optimised loop, fewer node triples) differs from both by
percents, which one test records.

The 30-node tower cases (von Karman with frequencies of both signs, Davenport with positive
ones; 1024 pairs of the tower's 129-point grid) hold the kernel's partial of every work group
of 16 pairs, so the comparison is group by group (the finest output the kernel has), not
only summed.  With the kernel's two float literals written in double precision the oracle
gives its partials to 1e-12 and the library's FP64 path to 1e-10 (the plain path's parity bar);
as shipped, to 2e-7."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden"))
from make_bsacl_golden import CASES, GROUP_CASES, case_problem, group_problem  # noqa: E402

G = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "bsacl_ref.npz"))
TOL = 2e-7


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


def pairs(name):
    fi, fj = G[f"{name}_fi"], G[f"{name}_fj"]
    FI, FJ = np.meshgrid(fi, fj, indexing="xy")
    w = (fi[1] - fi[0]) * (fj[1] - fj[0]) * 4.0 * np.pi ** 2
    return FI.ravel().copy(), FJ.ravel().copy(), np.full(FI.size, w)


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_gives_the_reference_kernel_sums(name):
    from oracle.oracle import Oracle
    o = Oracle(case_problem(name))
    fi, fj, w = pairs(name)
    mf = sum(w[k] * o.msh_bfm(fi[k], fj[k]) for k in range(fi.size))
    mr = sum(w[k] * o.msh_brm(fi[k], fj[k], o.msh_bfm(fi[k], fj[k]))[:, 0] for k in range(fi.size))
    assert rel(mf, G[f"{name}_plain_m3mf"]) < TOL
    assert rel(mr, G[f"{name}_plain_m3mr"]) < TOL


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_library_gives_the_reference_kernel_sums(bsalib, name):
    from bsalib_gb300 import api
    s = api.BsaSession(case_problem(name), precision=api.PREC_FP64)
    try:
        fi, fj, w = pairs(name)
        mf, mr = s.msh_moments(fi, fj, w)
    finally:
        s.close()
    assert rel(mf, G[f"{name}_plain_m3mf"]) < TOL
    assert rel(mr, G[f"{name}_plain_m3mr"]) < TOL


@pytest.mark.parametrize("name", sorted(CASES))
def test_shipped_kernel_differs_from_the_fortran_form(name):
    assert rel(G[f"{name}_shipped_m3mf"], G[f"{name}_plain_m3mf"]) > 1e-3


TOL_EXACT_ORACLE = 1e-12
TOL_EXACT_GPU = 1e-10


def group_pairs(name):
    """Pairs of a group case in the kernel's order (fi fastest): group g = every fi at fj[g]."""
    fi, fj = G[f"{name}_fi"], G[f"{name}_fj"]
    FI, FJ = np.meshgrid(fi, fj, indexing="xy")
    return FI.ravel().copy(), FJ.ravel().copy()


def rel_groups(a, b):
    """Largest per-group max-norm relative difference over the groups (rows)."""
    return float(max(np.max(np.abs(x - y)) / max(np.max(np.abs(y)), 1e-300) for x, y in zip(a, b)))


def to_groups(per_pair):
    return per_pair.reshape(-1, 16, per_pair.shape[-1]).sum(axis=1)


@pytest.mark.parametrize("name", sorted(GROUP_CASES))
def test_oracle_gives_the_reference_kernel_groups(name):
    from oracle.oracle import Oracle
    o = Oracle(group_problem(name))
    fi, fj = group_pairs(name)
    bf = np.array([o.msh_bfm(x, y) for x, y in zip(fi, fj)])
    br = np.array([o.msh_brm(x, y, b)[:, 0] for x, y, b in zip(fi, fj, bf)])
    assert fi.size == 1024 and G[f"{name}_exact_mf_groups"].shape == (64, 64)
    assert rel_groups(to_groups(bf), G[f"{name}_exact_mf_groups"]) < TOL_EXACT_ORACLE
    assert rel_groups(to_groups(br), G[f"{name}_exact_mr_groups"]) < TOL_EXACT_ORACLE
    assert rel_groups(to_groups(bf), G[f"{name}_shipped_mf_groups"]) < TOL
    assert rel_groups(to_groups(br), G[f"{name}_shipped_mr_groups"]) < TOL


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(GROUP_CASES))
def test_library_gives_the_reference_kernel_groups(bsalib, name):
    from bsalib_gb300 import api
    s = api.BsaSession(group_problem(name), precision=api.PREC_FP64)
    try:
        fi, fj = group_pairs(name)
        bf, br = s.msh_bispectra(fi, fj)
    finally:
        s.close()
    assert rel_groups(to_groups(bf), G[f"{name}_exact_mf_groups"]) < TOL_EXACT_GPU
    assert rel_groups(to_groups(br), G[f"{name}_exact_mr_groups"]) < TOL_EXACT_GPU
    assert rel_groups(to_groups(bf), G[f"{name}_shipped_mf_groups"]) < TOL
    assert rel_groups(to_groups(br), G[f"{name}_shipped_mr_groups"]) < TOL
