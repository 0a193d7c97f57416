"""Train the zone-refinement proposer on records of the plain refinement criterion and
compare the learned form with the plain one on held-out structures.

  python -m bsalib_gb300.train_proposer [--train 2000] [--test 200] [--tol 1e-3]
                                        [--thr-cap 0.02] [--out proposer.npz] [--json r.json]

Structures are seeded random cantilevers (`problem.random_structure`) drawn as the learned
refinement configuration specifies: nodes uniform 50-800, modes 5-60, natural frequencies
log-uniform 0.05-5 Hz, damping 0.3-3 %, U 15-50 m/s, I_u 0.08-0.2; training seeds 0 .. train-1,
held-out seeds 100000 .. 100000 + test - 1.
Training records come from the plain criterion on the training seeds; the held-out seeds
are evaluated with both forms in the split precision, and the plain form's final zone set
once more with the FP64 path, the reference for the errors.  Skewness uses the second
moments of the same structure (Classic PSD integration, FP64).
"""
from __future__ import annotations

import argparse
import copy
import json
import time

import numpy as np

from . import api, build
from .problem import random_structure
from .refine import Proposer, Refiner


def structure(seed):
    p = random_structure(seed, nodes=(50, 800), modes=(5, 60), nfreq_grid=(129, 129))
    p.settings.suban = 2
    return p


def second_moments(prob):
    q = copy.deepcopy(prob)
    q.settings.suban, q.settings.ibisp = 1, 0
    s = api.BsaSession(q, precision=api.PREC_FP64)
    try:
        return s.run()["m2mr_cls"]
    finally:
        s.close()


def skew(nm, m2, m3):
    sig = np.sqrt(np.abs(np.diag(m2.reshape(nm, nm))))
    return m3 / np.einsum("i,j,k->ijk", sig, sig, sig).reshape(-1, order="F")


def layout_refused(err):
    """The reference's pre-mesh aborts on this structure as well (BsaMesherImpl.F90:809-810,
    "Negative base."): its first quadrant zone would have no extent.  A refinement level whose
    zone pass does not fit the device memory is skipped the same way (and reported)."""
    return "negative base" in str(err) or "out of memory" in str(err)


def records(seeds, tol, levels, skipped=None, budget_s=None, done=None):
    X, Y, E = [], [], []
    t0 = time.perf_counter()
    for n, seed in enumerate(seeds):
        if budget_s is not None and time.perf_counter() - t0 > budget_s:
            break
        if done is not None:
            done.append(seed)
        if n and n % 100 == 0:
            print(f"records: {n} structures, {time.perf_counter() - t0:.0f} s", flush=True)
        s = api.BsaSession(structure(seed), precision=api.PREC_BF16X3)
        try:
            out = Refiner(s, tol, levels).run(keep_records=True)
        except api.BsaError as e:
            if not layout_refused(e):
                raise
            if skipped is not None:
                skipped.append(seed)
            continue
        finally:
            s.close()
        if out.records is not None:
            X.append(out.records[0])
            Y.append(out.records[1])
            E.append(out.records[2])
    return np.concatenate(X), np.concatenate(Y), np.concatenate(E)


def brm_points(zones):
    return int(sum(((z.ni - 1) * z.Fi + 1) * ((z.nj - 1) * z.Fj + 1) for z in zones))


def compare(prop, thr, seeds, tol, levels, fp64_every=1, budget_s=None):
    """Plain and learned refinement of each held-out structure in the split precision (device
    time and host wall time of each run), and, on every fp64_every-th structure, the plain
    FP64 GPU path integrating the plain criterion's final mesh (the error reference)."""
    rows = []
    rel = lambda x, y: float(np.max(np.abs(x - y)) / np.max(np.abs(y)))
    t0 = time.perf_counter()
    for k, seed in enumerate(seeds):
        if budget_s is not None and time.perf_counter() - t0 > budget_s:
            break
        if k and k % 20 == 0:
            print(f"compare: {k} structures, {time.perf_counter() - t0:.0f} s", flush=True)
        prob = structure(seed)
        s = api.BsaSession(prob, precision=api.PREC_BF16X3)
        try:
            nm = s.nmodes()
            t0 = time.perf_counter()
            plain = Refiner(s, tol, levels).run()
            t1 = time.perf_counter()
            learned = Refiner(s, tol, levels).run(proposer=prop, threshold=thr)
            t2 = time.perf_counter()
        except api.BsaError as e:
            if not layout_refused(e):
                raise
            rows.append({"seed": seed, "skipped": "out of device memory" if "out of memory" in str(e) else
                         "the reference's pre-mesh refuses the layout (negative base)"})
            continue
        finally:
            s.close()
        row = {"seed": seed, "modes": nm, "nodes": prob.nnl,
               "plain_points": plain.points, "learned_points": learned.points,
               "plain_ms": plain.ms, "learned_ms": learned.ms,
               "plain_wall_s": t1 - t0, "learned_wall_s": t2 - t1,
               "final_brm_points": brm_points(learned.final_zones),
               "m3mr_rel_learned_vs_plain": rel(learned.m3mr, plain.m3mr)}
        if k % fp64_every == 0:
            s64 = api.BsaSession(prob, precision=api.PREC_FP64)
            try:
                s64.use_driver_controls()
                _, mr64, _ = s64.msh_zones(plain.final_zones)
                ms64 = s64.stats().ms_total
            finally:
                s64.close()
            m2 = second_moments(prob)
            row.update({"fp64_final_ms": ms64, "plain_final_brm_points": brm_points(plain.final_zones),
                        "m3mr_rel_learned_vs_fp64": rel(learned.m3mr, mr64),
                        "skew_rel_learned_vs_fp64": rel(skew(nm, m2, learned.m3mr), skew(nm, m2, mr64)),
                        "skew_rel_plain_vs_fp64": rel(skew(nm, m2, plain.m3mr), skew(nm, m2, mr64))})
        rows.append(row)
    return rows


def summary(rows):
    """Medians of the per-structure ratios and the aggregate rates."""
    skipped = [r["seed"] for r in rows if "skipped" in r]
    rows = [r for r in rows if "skipped" not in r]
    f = [r for r in rows if "fp64_final_ms" in r]
    out = {"points_ratio_learned_over_plain_median": float(np.median([r["learned_points"] / r["plain_points"]
                                                                      for r in rows])),
           "time_ratio_learned_over_plain_median": float(np.median([r["learned_ms"] / r["plain_ms"] for r in rows])),
           "wall_ratio_learned_over_plain_median": float(np.median([r["learned_wall_s"] / r["plain_wall_s"]
                                                                    for r in rows])),
           "exact_match_fraction": float(np.mean([r["m3mr_rel_learned_vs_plain"] < 1e-10 for r in rows])),
           "m3mr_rel_learned_vs_plain_max": float(max(r["m3mr_rel_learned_vs_plain"] for r in rows)),
           "evaluated_structures": len(rows), "skipped_structures": skipped}
    if f:
        pts = sum(r["plain_final_brm_points"] for r in f)
        learned_rate = sum(r["final_brm_points"] for r in f) / (sum(r["learned_ms"] for r in f) * 1e-3)
        fp64_rate = pts / (sum(r["fp64_final_ms"] for r in f) * 1e-3)
        out.update({"fp64_structures": len(f),
                    "skew_rel_learned_vs_fp64_max": float(max(r["skew_rel_learned_vs_fp64"] for r in f)),
                    "skew_rel_plain_vs_fp64_max": float(max(r["skew_rel_plain_vs_fp64"] for r in f)),
                    "learned_brm_pts_per_s": learned_rate, "fp64_brm_pts_per_s": fp64_rate,
                    "pts_per_s_ratio_learned_over_fp64": learned_rate / fp64_rate,
                    "wall_ratio_fp64_over_learned": sum(r["fp64_final_ms"] for r in f) /
                    sum(r["learned_ms"] for r in f)})
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--train", type=int, default=2000)
    ap.add_argument("--test", type=int, default=200)
    ap.add_argument("--fp64-every", type=int, default=1,
                    help="the FP64 reference on every k-th held-out structure (1: all)")
    ap.add_argument("--tol", type=float, default=1e-3)
    ap.add_argument("--levels", type=int, default=2)
    ap.add_argument("--epochs", type=int, default=40)
    ap.add_argument("--thr-cap", type=float, default=0.02, help="upper bound of the proposal threshold")
    ap.add_argument("--out", default="")
    ap.add_argument("--json", default="")
    ap.add_argument("--records", default="", help="write the training records (features, label, change)")
    ap.add_argument("--record-budget-s", type=float, default=None,
                    help="stop drawing training structures after this many seconds (the count used is reported)")
    ap.add_argument("--compare-budget-s", type=float, default=None,
                    help="stop the held-out comparison after this many seconds (the count used is reported)")
    a = ap.parse_args()
    build.build()
    t0 = time.perf_counter()
    skipped_train, used_train = [], []
    X, Y, E = records(range(a.train), a.tol, a.levels, skipped_train, a.record_budget_s, used_train)
    t_rec = time.perf_counter() - t0
    if a.records:
        np.savez(a.records, X=X, Y=Y, E=E)
    prop = Proposer()
    t0 = time.perf_counter()
    loss = prop.fit(X, E, a.tol, epochs=a.epochs)
    t_fit = time.perf_counter() - t0
    p = prop(X)
    # threshold: half the lowest probability any needed refinement of the training records
    # received, and at most thr_cap (every one of them proposed, with a margin for unseen
    # structures)
    thr = float(min(0.5 * np.min(p[Y > 0.5]), a.thr_cap)) if np.any(Y > 0.5) else a.thr_cap
    recall = float(np.mean(p[Y > 0.5] > thr)) if np.any(Y > 0.5) else 1.0
    skipped = float(np.mean(p[Y < 0.5] <= thr)) if np.any(Y < 0.5) else 0.0
    t0 = time.perf_counter()
    rows = compare(prop, thr, range(100000, 100000 + a.test), a.tol, a.levels, a.fp64_every, a.compare_budget_s)
    t_cmp = time.perf_counter() - t0
    res = {"train_structures": len(used_train), "train_requested": a.train, "train_skipped": skipped_train,
           "test_structures": len(rows), "test_requested": a.test,
           "records": int(len(Y)),
           "positive_fraction": float(Y.mean()), "record_s": t_rec, "fit_s": t_fit, "compare_s": t_cmp,
           "final_train_loss": loss, "threshold": thr, "train_recall": recall, "train_skipped_negatives": skipped,
           **summary(rows), "rows": rows}
    if a.out:
        prop.save(a.out, thr, a.tol)
    prop.close()
    if a.json:
        with open(a.json, "w") as fh:
            fh.write(json.dumps(res))
    print(json.dumps({k: v for k, v in res.items() if k != "rows"}))


if __name__ == "__main__":
    main()
