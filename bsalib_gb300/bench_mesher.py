"""Timing tool: the Mesher analysis (zone layout + zone integration) of a structure, run a few
times (also the command the committed ncu summaries under profiles/ were taken with).

  python -m bsalib_gb300.bench_mesher [--structure bridge|building|tower] [--nodes N]
                                        [--modes M] [--precision bf16x3|fp64] [--steps 2]
                                        [--max-zones N] [--synthetic N]

Prints the zone and lattice-point counts and, per run, the library statistics and the
response-bispectrum (BRM lattice) points per second.
"""
import argparse
import time

from . import api, build
from .problem import bridge_deck, cantilever_tower, tall_building


def make(a):
    if a.structure == "bridge":
        return bridge_deck(nodes=a.nodes or 1200, modes=a.modes or 60)
    if a.structure == "building":
        p = tall_building(nodes=a.nodes or 400, modes=a.modes or 24, nfreqs=65, df=0.0625)
    else:
        p = cantilever_tower(nodes=a.nodes or 30)
    p.settings.suban = 2
    return p


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--structure", default="bridge", choices=["bridge", "building", "tower"])
    ap.add_argument("--nodes", type=int, default=0)
    ap.add_argument("--modes", type=int, default=0)
    ap.add_argument("--precision", default="bf16x3", choices=["bf16x3", "fp64"])
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--zones-only", action="store_true")
    ap.add_argument("--synthetic", type=int, default=0,
                    help="evaluate this many seeded synthetic zones (problem.synthetic_zones) instead of the layout")
    ap.add_argument("--max-zones", type=int, default=0,
                    help="evaluate only the first N zones of the layout (a small case of the same zones)")
    ap.add_argument("--controls", default="driver", choices=["driver", "library"],
                    help="Mesher controls: the standalone driver's (default) or the library's")
    a = ap.parse_args()
    build.build()
    prob = make(a)
    prec = api.PREC_BF16X3 if a.precision == "bf16x3" else api.PREC_FP64
    s = api.BsaSession(prob, precision=prec)
    try:
        if a.controls == "driver":
            s.use_driver_controls()
        if a.synthetic:
            from .problem import synthetic_zones
            zs = synthetic_zones(prob, a.synthetic)
        else:
            zs = s.generate_zones()
            if a.max_zones:
                zs = zs[:a.max_zones]
        nbfm = sum(z.ni * z.nj for z in zs)
        nbrm = sum(((z.ni - 1) * z.Fi + 1) * ((z.nj - 1) * z.Fj + 1) for z in zs)
        print(f"{a.structure}: {prob.nnl} nodes, {s.nmodes()} modes, {len(zs)} zones, "
              f"{nbfm} BFM points, {nbrm} BRM points", flush=True)
        if a.zones_only:
            return
        for _ in range(a.steps):
            t0 = time.perf_counter()
            if a.synthetic or a.max_zones:
                s.msh_zones(zs)
            else:
                s.run()
            wall = time.perf_counter() - t0
            st = s.stats()
            print(f"  {st.ms_total:.1f} ms total (device), {wall * 1e3:.1f} ms wall, {st.ms_gemm:.1f} ms contraction "
                  f"kernel, {st.kernels} kernels, {st.graphs} graphs, {st.points / (st.ms_total * 1e-3):.4g} BRM pts/s",
                  flush=True)
    finally:
        s.close()


if __name__ == "__main__":
    main()
