"""Parametric sweep of Classic analyses: one batched evaluation against one bsa_Run per case.

  python -m bsalib_gb300.sweep [--structures 8] [--winds 8] [--seed0 5000] [--json out.json]

Cases are seeded random cantilevers (`problem.random_structure`: nodes 30-600, kept modes
4-40, Classic grids of 129-513 points), each under `winds` mean wind speeds spread evenly
over 15-50 m/s.  The batch is evaluated once untimed
and once timed (device time of the whole sweep and wall time of the call); each case is then
run on its own with the split precision, the sequential baseline.  Reported: aggregate Classic
grid points per second of both, the per-case completion latencies inside the batched launch
(p50 / p99) and the largest relative difference of any case's third moments between the two.

The plain FP64 GPU path is measured beside it on a seeded subset of the cases (`fp64_cases`):
per case the FP64 kernel at `fp64_points` seeded grid points, whose rate (points per second
of that case) gives the case's full-grid FP64 time; the sweep's FP64 time is the subset's
total scaled by cases / subset size.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import api, build
from .problem import random_structure


class Cases:
    """The sweep's cases, built on demand (a case's nodal tables are a few MB): case c is
    structure seed0 + c // winds under the (c % winds)-th mean wind speed."""

    def __init__(self, structures, winds, seed0):
        self.us = np.linspace(15.0, 50.0, winds) if winds > 1 else np.array([30.0])
        self.structures, self.seed0 = structures, seed0

    def __len__(self):
        return self.structures * len(self.us)

    def __getitem__(self, c):
        if not 0 <= c < len(self):
            raise IndexError(c)
        w = len(self.us)
        return random_structure(self.seed0 + c // w, nodes=(30, 600), modes=(4, 40), nfreq_grid=(129, 513),
                                U_mean=float(self.us[c % w]))

    def __iter__(self):
        return (self[c] for c in range(len(self)))


def cases(structures, winds, seed0):
    return Cases(structures, winds, seed0)


def fp64_estimate(probs, ncase, npts, seed=1):
    """The plain FP64 GPU path on `ncase` seeded cases, `npts` seeded grid points each."""
    rng = np.random.default_rng(seed)
    pick = sorted(rng.choice(len(probs), size=min(ncase, len(probs)), replace=False).tolist())
    t_full, pts_full, rel_sample = 0.0, 0.0, []
    for k in pick:
        p = probs[k]
        nf = p.classic_nf()
        f = (np.arange(nf) - (nf - 1) // 2) * p.settings.df
        i1, i2 = rng.integers(nf, size=npts), rng.integers(nf, size=npts)
        s = api.BsaSession(p, precision=api.PREC_FP64)
        try:
            s.msh_moments(f[i1], f[i2], np.ones(npts))  # warm (A table, module load)
            s.msh_moments(f[i1], f[i2], np.ones(npts))
            ms = s.stats().ms_total
        finally:
            s.close()
        t_full += nf * nf * ms / npts  # this case's full grid at its measured FP64 rate
        pts_full += nf * nf
    scale = len(probs) / len(pick)
    return {"cases_sampled": len(pick), "points_per_case": npts, "est_sweep_ms": t_full * scale,
            "value": pts_full / (t_full * 1e-3), "unit": "pts/s",
            "method": "FP64 kernel at seeded grid points of a seeded subset of the cases; each case's full grid "
                      "at its measured rate, summed and scaled to all cases"}


def run(structures=8, winds=8, seed0=5000, check=True, fp64_cases=0, fp64_points=512):
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
    if fp64_cases:
        fp = fp64_estimate(probs, fp64_cases, fp64_points)
        res["fp64_gpu_path"] = fp
        res["speedup_batch_vs_fp64"] = fp["est_sweep_ms"] / dev_ms
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--structures", type=int, default=8)
    ap.add_argument("--winds", type=int, default=8)
    ap.add_argument("--seed0", type=int, default=5000)
    ap.add_argument("--no-check", action="store_true", help="skip the one-analysis-per-case baseline")
    ap.add_argument("--fp64-cases", type=int, default=0, help="cases of the FP64 GPU path estimate (0: none)")
    ap.add_argument("--json", default="")
    a = ap.parse_args()
    build.build()
    res = run(a.structures, a.winds, a.seed0, check=not a.no_check, fp64_cases=a.fp64_cases)
    if a.json:
        with open(a.json, "w") as fh:
            fh.write(json.dumps(res))
    print(json.dumps(res))


if __name__ == "__main__":
    main()
