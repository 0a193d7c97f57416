"""Parametric sweep of Classic analyses: one batched evaluation against one bsa_Run per case.

  python -m bsalib_gb300.sweep [--structures 8] [--winds 8] [--seed0 5000] [--json out.json]

Cases are seeded random cantilevers (`problem.random_structure`: nodes 30-600, kept modes
4-40, Classic grids of 129-513 points), each under `winds` mean wind speeds spread evenly
over 15-50 m/s.  The batch is evaluated once untimed
and once timed (device time of the whole sweep and wall time of the call); each case is then
run on its own with the split precision, the sequential baseline.  Reported: aggregate Classic
grid points per second of both, the per-case completion latencies inside the batched launch
(p50 / p99) and the largest relative difference of any case's third moments between the two.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import api, build
from .problem import random_structure


def cases(structures, winds, seed0):
    us = np.linspace(15.0, 50.0, winds) if winds > 1 else [30.0]
    return [random_structure(seed0 + k, nodes=(30, 600), modes=(4, 40), nfreq_grid=(129, 513), U_mean=float(u))
            for k in range(structures) for u in us]


def run(structures=8, winds=8, seed0=5000, check=True):
    probs = cases(structures, winds, seed0)
    n = len(probs)
    sw = api.Sweep()
    for p in probs:
        sw.add(p)
    sw.run()  # warm-up (module load, allocations)
    t0 = time.perf_counter()
    out, dev_ms = sw.run()
    wall_ms = (time.perf_counter() - t0) * 1e3
    st = api.Stats()
    api.check(api.load().bsa_gpu_getStats(api.C.byref(st)), "bsa_gpu_getStats")
    batch_gemm_ms, batch_kernels = st.ms_gemm, st.kernels
    sw.clear()
    pts = float(sum(o["nf"] ** 2 for o in out))
    seq_ms, seq_gemm_ms, worst = 0.0, 0.0, 0.0
    if check:
        for k, p in enumerate(probs):
            s = api.BsaSession(p, precision=api.PREC_BF16X3)
            try:
                r = s.run()
                seq_ms += s.stats().ms_total
                seq_gemm_ms += s.stats().ms_gemm
            finally:
                s.close()
            ref = r["m3mr_cls"]
            worst = max(worst, float(np.max(np.abs(out[k]["m3mr"] - ref)) / np.max(np.abs(ref))))
    lat = np.array([o["ms"] for o in out])
    res = {"cases": n, "structures": structures, "winds": winds, "points": pts, "modes_min": min(o["nm"] for o in out),
           "modes_max": max(o["nm"] for o in out), "batch_device_ms": dev_ms, "batch_wall_ms": wall_ms,
           "batch_pts_per_s": pts / (dev_ms * 1e-3), "batch_contraction_launch_ms": batch_gemm_ms,
           "batch_kernels": batch_kernels, "latency_p50_ms": float(np.percentile(lat, 50)),
           "latency_p99_ms": float(np.percentile(lat, 99))}
    if check:
        res.update({"sequential_device_ms": seq_ms, "sequential_contraction_launch_ms": seq_gemm_ms, "sequential_pts_per_s": pts / (seq_ms * 1e-3),
                    "speedup_device": seq_ms / dev_ms, "m3mr_rel_batch_vs_single_max": worst})
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--structures", type=int, default=8)
    ap.add_argument("--winds", type=int, default=8)
    ap.add_argument("--seed0", type=int, default=5000)
    ap.add_argument("--no-check", action="store_true", help="skip the one-analysis-per-case baseline")
    ap.add_argument("--json", default="")
    a = ap.parse_args()
    build.build()
    res = run(a.structures, a.winds, a.seed0, check=not a.no_check)
    if a.json:
        with open(a.json, "w") as fh:
            fh.write(json.dumps(res))
    print(json.dumps(res))


if __name__ == "__main__":
    main()
