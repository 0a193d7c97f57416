"""Generate the golden fixtures in this folder (run from the repository root:
`python tests/golden/make_golden.py`).

BsaLib ships no tests, fixtures or golden vectors, and its Fortran sources cannot be
compiled here, so these vectors come from the independent numpy restatement in
oracle/oracle.py (`direct_point`: the plain nodal triple sum of
functionsImpl.F90:1494-1538 with numpy einsum; `brm_factor`: the FRF product of
functionsImpl.F90:1031-1115; the Classic edge weights of BsaClassicImpl.F90:596-632).
They pin the C oracle and, through it, the GPU path.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from bsalib_gb300.problem import cantilever_tower, tall_building  # noqa: E402
from oracle.oracle import Oracle, classic_weights  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))


def classic_case(name, prob):
    o = Oracle(prob)
    f = o.freqs()
    nf = f.size
    nm = o.nme
    bf = np.zeros((nf, nf, nm ** 3))
    br = np.zeros((nf, nf, nm ** 3))
    for i1 in range(nf):
        for i2 in range(nf):
            trunc = abs(f[i1] + f[i2]) > f[-1] * (1 + 1e-12) or (f[i1] + f[i2]) < f[0] * (1 + 1e-12)
            s12 = [np.zeros((prob.nnl, prob.nnl))] * prob.ntc if trunc else None
            bf[i1, i2] = o.direct_point(f[i1], f[i2], s12)
            br[i1, i2] = bf[i1, i2] * o.brm_factor(f[i1], f[i2])
    w = classic_weights(nf, f[1] - f[0], prob.settings.defsc)
    np.savez_compressed(os.path.join(OUT, name + ".npz"), f=f, bf=bf, br=br,
                        m3mf=np.einsum("ij,ijk->k", w, bf), m3mr=np.einsum("ij,ijk->k", w, br))


def mesher_case(name, prob, pts):
    o = Oracle(prob)
    bf = np.stack([o.direct_point(a, b) for a, b in pts])
    br = np.stack([bf[k] * o.brm_factor(a, b) for k, (a, b) in enumerate(pts)])
    np.savez_compressed(os.path.join(OUT, name + ".npz"), pts=np.array(pts), bf=bf, br=br)


if __name__ == "__main__":
    classic_case("tower6_nf9", cantilever_tower(nfreqs=5, df=0.5, nodes=6))
    classic_case("building8_2tc_nf7", tall_building(nodes=8, modes=3, nfreqs=4, df=0.5, seed=7))
    mesher_case("tower6_points", cantilever_tower(nfreqs=5, df=0.5, nodes=6),
                [(0.7, -0.3), (1.25, 0.5), (-2.5, 3.0), (0.0, 0.0), (4.1, 0.05)])
    print("written to", OUT)
