"""Adaptive zone refinement: the plain criterion, and the learned form with the packaged
proposer (bsalib_gb300/data/proposer.npz), on structures of its held-out set.  The learned
form must reach the plain criterion's final mesh (same third moments, 1e-10) while
evaluating fewer lattice points; both in the split precision."""
import numpy as np
import pytest

from bsalib_gb300 import api
from bsalib_gb300.refine import DEFAULT_WEIGHTS, Proposer, Refiner, zone_points
from bsalib_gb300.train_proposer import structure

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300))


@pytest.mark.parametrize("seed", [100000, 100003, 100011])
def test_learned_reaches_the_plain_mesh_with_fewer_points(bsalib, seed):
    prop, thr, tol = Proposer.load(DEFAULT_WEIGHTS)
    s = api.BsaSession(structure(seed), precision=api.PREC_BF16X3)
    try:
        plain_r = Refiner(s, tol, 2)             # switches the session to the pre-mesh lattices
        level0 = zone_points(s.generate_zones())
        plain = plain_r.run()
        learned = Refiner(s, tol, 2).run(proposer=prop, threshold=thr)
    finally:
        s.close()
        prop.close()
    assert plain.points > 2 * level0          # every zone judged once more, plus the final integration
    assert learned.points < plain.points
    assert sorted((z.fi0, z.fj0, z.ni, z.nj) for z in learned.final_zones) == \
        sorted((z.fi0, z.fj0, z.ni, z.nj) for z in plain.final_zones)
    assert rel(learned.m3mr, plain.m3mr) < 1e-10


def test_plain_criterion_keeps_coarse_zones_within_tolerance(bsalib):
    """With a tolerance nothing reaches, no zone is refined: the final mesh is the layout."""
    s = api.BsaSession(structure(7), precision=api.PREC_BF16X3)
    try:
        ref = Refiner(s, 1e9, 2)
        zs = s.generate_zones()
        out = ref.run()
        mf, mr, _ = s.msh_zones(zs)
    finally:
        s.close()
    assert out.refined == 0 and out.zones == len(zs)
    assert rel(out.m3mr, mr) < 1e-12
