"""Timing tool: the Classic analysis of the tall-building workload, run a few times (also the
command the committed ncu summaries under profiles/ were taken with).

  python -m bsalib_gb300.bench_classic [--nfreqs 513] [--steps 2] [--precision bf16x3]

Defaults give the full 400-node, 24-mode, two-component building on the 1025 x 1025 grid;
--nfreqs 65 gives the same structure on a 129 x 129 grid (a few hundred MB on the device).
Prints one line of library statistics per run.
"""
import argparse

from . import api, build
from .problem import tall_building


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--nfreqs", type=int, default=513)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--precision", default="bf16x3", choices=["bf16x3", "fp64"])
    ap.add_argument("--modes", type=int, default=24, help="kept modes of the building")
    a = ap.parse_args()
    build.build()
    prob = tall_building(modes=a.modes, nfreqs=a.nfreqs, df=4.0 / (a.nfreqs - 1))
    prec = api.PREC_BF16X3 if a.precision == "bf16x3" else api.PREC_FP64
    s = api.BsaSession(prob, precision=prec)
    try:
        for _ in range(a.steps):
            s.run()
            st = s.stats()
            print(f"grid {prob.classic_nf()}^2: {st.ms_total:.3f} ms total, {st.ms_gemm:.3f} ms contraction kernel, "
                  f"{st.kernels} kernels")
    finally:
        s.close()


if __name__ == "__main__":
    main()
