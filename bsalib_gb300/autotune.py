"""Autotuner of the split-precision contractions' tile plans (bsa_gpu_setTilePlan).

  python -m bsalib_gb300.autotune [--out bsalib_gb300/data/tile_plans.txt] [--reps 2] [--quick]

For each bucket of kept modes nm and of K (= turbulence components x loaded nodes), and for
the Classic analysis also of grid points per axis, it builds a seeded synthetic structure of
the bucket's size, times every candidate plan (CUDA-event device time of the whole split
analysis, the best of `reps` runs after one warm-up run), and writes the fastest per bucket
to the table libbsagpu.so loads at first use (data/tile_plans.txt beside the library).

  Classic (tall building, bsa_Run in BF16x3): every combination of the form (E form where it
  applies, D1 / D3 form) and of that form's FRF-table width that holds the modes (E widths 16
  and 24 in one pass or two); the table records the best form, the best E width and its pass
  count, and the best D1 / D3 width of each bucket.
  Mesher (bridge deck, the standalone driver's Mesher controls, bsa_Run with analysis type 2 in
  BF16x3): the mode width NMT of the zone kernel, every multiple of 8 from nm up to nm + 16.

Each bucket's representative case takes the top of its mode range (the tightest fit of the
narrowest width) and a representative K and grid size.  The table keeps the measured times as
comments.
"""
from __future__ import annotations

import argparse
import datetime
import json
import os

import numpy as np

from . import api, build
from .problem import bridge_deck, tall_building

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_OUT = os.path.join(HERE, "data", "tile_plans.txt")

NM_RANGES = [(1, 8), (9, 12), (13, 16), (17, 20), (21, 24), (25, 28), (29, 32), (33, 40), (41, 48), (49, 56),
             (57, 64)]
K_RANGES = [(1, 500, 300), (501, 1500, 800), (1501, 1 << 30, 2400)]        # (lo, hi, representative K)
NF_RANGES = [(1, 300, 129), (301, 700, 513), (701, 1 << 30, 1025)]        # (lo, hi, representative grid)
E_WIDTHS = (8, 16, 24, 32, 48)
D_WIDTHS = (8, 16, 24, 32, 64)
FAMILY = {"cls_form": api.PLAN_CLS_FORM, "cls_e_width": api.PLAN_CLS_E_WIDTH, "cls_d_width": api.PLAN_CLS_D_WIDTH,
          "msh_width": api.PLAN_MSH_WIDTH, "cls_e_split": api.PLAN_CLS_E_SPLIT}


def _set(lib, fam, val):
    """A catch-all plan of one family (every nm, K, nf) ahead of the table."""
    api.check(lib.bsa_gpu_setTilePlan(FAMILY[fam], 0, 1 << 30, 0, 1 << 30, 0, 1 << 30, int(val)),
              "bsa_gpu_setTilePlan")


def _time(prob, reps, plans, mesher=False):
    lib = api.load()
    api.check(lib.bsa_gpu_clearTilePlans(), "bsa_gpu_clearTilePlans")
    for fam, val in plans.items():
        _set(lib, fam, val)
    s = api.BsaSession(prob, precision=api.PREC_BF16X3)
    try:
        if mesher:
            s.use_driver_controls()
        s.run()
        best = min((s.run(), s.stats().ms_total)[1] for _ in range(reps))
    finally:
        s.close()
    return best


def classic_candidates(nm):
    c = []
    if nm <= 48:
        for w in E_WIDTHS:
            if nm <= w <= max(8, 2 * nm):
                # 16 and 24 in one pass or in two of half the modes (32 and 48 are always two)
                c += [{"cls_form": 1, "cls_e_width": w, "cls_e_split": sp} for sp in ((1, 2) if w in (16, 24) else (0,))]
    c += [{"cls_form": 0, "cls_d_width": w} for w in D_WIDTHS if nm <= w <= max(8, 2 * nm)]
    return c


def tune_classic(reps, quick):
    rows = []
    for (nlo, nhi) in NM_RANGES:
        for (klo, khi, K) in K_RANGES:
            for (flo, fhi, nf) in NF_RANGES:
                if quick and (nf > 129 or K > 300):
                    continue
                prob = tall_building(nodes=K // 2, modes=nhi, nfreqs=(nf + 1) // 2, df=4.0 / ((nf - 1) // 2),
                                     seed=31)
                res = []
                for cand in classic_candidates(nhi):
                    res.append((_time(prob, reps, cand), cand))
                res.sort(key=lambda r: r[0])
                best_e = min((r for r in res if r[1]["cls_form"] == 1), key=lambda r: r[0], default=None)
                best_d = min((r for r in res if r[1]["cls_form"] == 0), key=lambda r: r[0])
                rows.append({"nm": (nlo, nhi), "K": (klo, khi), "nf": (flo, fhi), "rep": (nhi, K, nf),
                             "form": res[0][1]["cls_form"], "e_width": best_e[1]["cls_e_width"] if best_e else None,
                             "e_split": best_e[1]["cls_e_split"] if best_e and best_e[1]["cls_e_split"] else None,
                             "d_width": best_d[1]["cls_d_width"],
                             "times_ms": [(round(t, 3), c) for t, c in res]})
                print(json.dumps(rows[-1]), flush=True)
    return rows


def tune_mesher(reps, quick):
    rows = []
    for (nlo, nhi) in NM_RANGES:
        for (klo, khi, K) in K_RANGES:
            if quick and K > 300:
                continue
            prob = bridge_deck(nodes=K // 2, modes=nhi)
            base = ((nhi + 7) // 8) * 8
            res = [(_time(prob, reps, {"msh_width": w}, mesher=True), w) for w in range(base, min(64, base + 16) + 1, 8)]
            res.sort()
            rows.append({"nm": (nlo, nhi), "K": (klo, khi), "rep": (nhi, K), "width": res[0][1],
                         "times_ms": [(round(t, 3), w) for t, w in res]})
            print(json.dumps(rows[-1]), flush=True)
    return rows


def write_table(path, cls_rows, msh_rows, note):
    lines = ["# Tile plans of the split-precision contractions, written by python -m bsalib_gb300.autotune",
             f"# {note}",
             "# family nm_lo nm_hi k_lo k_hi nf_lo nf_hi value   # measured ms of the candidates (value: ms)"]
    for fam, key in (("cls_form", "form"), ("cls_e_width", "e_width"), ("cls_e_split", "e_split"),
                     ("cls_d_width", "d_width")):
        for r in cls_rows:
            if r[key] is None:
                continue
            t = "; ".join(f"{c}: {ms}" for ms, c in r["times_ms"])
            lines.append(f"{fam} {r['nm'][0]} {r['nm'][1]} {r['K'][0]} {r['K'][1]} {r['nf'][0]} {r['nf'][1]} "
                         f"{r[key]}   # {t}")
    for r in msh_rows:
        t = "; ".join(f"{w}: {ms}" for ms, w in r["times_ms"])
        lines.append(f"msh_width {r['nm'][0]} {r['nm'][1]} {r['K'][0]} {r['K'][1]} 0 {1 << 30} {r['width']}   # {t}")
    os.makedirs(os.path.dirname(path), exist_ok=True)
    with open(path, "w") as fh:
        fh.write("\n".join(lines) + "\n")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=DEFAULT_OUT)
    ap.add_argument("--reps", type=int, default=2)
    ap.add_argument("--quick", action="store_true", help="small buckets only (a smoke run of the search)")
    ap.add_argument("--skip-mesher", action="store_true")
    a = ap.parse_args()
    build.build()
    cls_rows = tune_classic(a.reps, a.quick)
    msh_rows = [] if a.skip_mesher else tune_mesher(a.reps, a.quick)
    gpu = ""
    try:
        import torch
        gpu = torch.cuda.get_device_name(0)
    except Exception:
        pass
    note = f"{gpu or 'GPU'}, {datetime.date.today().isoformat()}, best of {a.reps} runs after one warm-up"
    write_table(a.out, cls_rows, msh_rows, note)
    api.check(api.load().bsa_gpu_loadTilePlans(None), "bsa_gpu_loadTilePlans")
    print("wrote", a.out)


if __name__ == "__main__":
    main()
