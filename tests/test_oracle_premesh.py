"""The oracle's restatement of the Mesher zone layout: the zones tile the square
[-max(natf) max_area_ext, +...]^2 without overlap, and the layout has the reference's structure
(background zone, crest bands, quadrant L-shapes, external padding)."""
import numpy as np
import pytest

from bsalib_gb300.problem import bridge_deck, cantilever_tower, random_structure, tall_building
from oracle.oracle import Oracle
from oracle.premesh import layout_for, unmirror, zone_limits


def corners(z):
    fi0, fj0, dIi, dIj, dJi, dJj, ni, nj = unmirror(z)[:8]
    a = np.array([fi0, fj0])
    u = np.array([dIi, dIj]) * (ni - 1)
    v = np.array([dJi, dJj]) * (nj - 1)
    return a, u, v


def cases():
    t = cantilever_tower(nodes=8)
    b = tall_building(nodes=20, modes=6, nfreqs=9, df=0.5, seed=3)
    d = bridge_deck(nodes=40, modes=12, seed=5)
    r = random_structure(7, nodes=(30, 30), modes=(8, 8), nfreq_grid=(65, 65))
    return [("tower", t), ("building", b), ("bridge", d), ("random", r)]


@pytest.mark.parametrize("name,prob", cases(), ids=[c[0] for c in cases()])
@pytest.mark.parametrize("ctl", [dict(), dict(validate=False, mlr=False, restrict=True)], ids=["lib", "driver"])
@pytest.mark.parametrize("sym", [0, 2], ids=["full", "half"])
def test_layout_tiles_the_square(name, prob, ctl, sym):
    prob.settings.bispsym = sym
    o = Oracle(prob)
    zs = layout_for(prob, o.modes, **ctl)
    X = prob.natf.max() * prob.settings.maxaext
    area = sum(abs(u[0] * v[1] - u[1] * v[0]) for _, u, v in map(corners, zs))
    lo = 0.0 if sym == 2 else -X                 # HALF lays out f1 >= 0
    assert np.isclose(area, (X - lo) * 2 * X, rtol=1e-10)
    assert all(z[11] == (2.0 if sym == 2 else 1.0) for z in zs)
    rng = np.random.default_rng(1)
    pts = np.column_stack([rng.uniform(lo, X, 4000), rng.uniform(-X, X, 4000)])
    cnt = np.zeros(len(pts), dtype=int)
    for z in zs:
        a, u, v = corners(z)
        M = np.array([u, v]).T
        st = np.linalg.solve(M, (pts - a).T).T
        cnt += np.all((st > 1e-9) & (st < 1 - 1e-9), axis=1)
    assert np.all(cnt <= 1)                    # no overlap
    assert np.mean(cnt == 1) > 0.999           # covered (up to points on zone borders)
    for z in zs:
        assert z[6] >= 2 and z[7] >= 2 and z[8] >= 1 and z[9] >= 1


def test_layout_structure():
    prob = tall_building(nodes=20, modes=6, nfreqs=9, df=0.5, seed=3)
    o = Oracle(prob)
    s = prob.settings
    zs = layout_for(prob, o.modes)
    # background width from the turbulence scales, limits from the peak bands
    L = np.asarray(prob.L).reshape(3, 3, -1, order="F")
    bkgw = max(1.0 / max(L[i, j, z] / prob.UBref[z] for z in range(L.shape[2])) for i in range(3) for j in range(3))
    NL, lim, pol, im = zone_limits([int(m) for m in o.modes], list(prob.natf), list(prob.xsi), s.genpaext,
                                   bkgw * s.bkgaext / 2)
    assert len(zs) == 1 + 4 * (NL + 1) + 4 * (1 + 3 * NL) + 4
    bkg = zs[0]
    assert np.isclose(bkg[0], -bkgw * s.bkgaext / 2) and bkg[10] == 5   # PEAK policy
