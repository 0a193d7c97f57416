"""Adaptive zone refinement for the Mesher, with the learned refinement proposer.

The plain criterion refines every zone once more (its lattice steps halved, the BRM factors
kept) and keeps the refinement where the zone's own mode-diagonal response moments
m3mr(m, m, m) change by more than `tol` relative to the largest total one (elsewhere the
current lattice is kept); refined zones are judged again at the next level, up to
`max_levels`.  It therefore evaluates every zone at every level it reaches plus one more.

The learned form evaluates the next level only for the zones the proposer network
(bsa_mlp_*, BF16 weights, trained on the device) predicts to need it; the plain criterion
still judges every proposal, and zones not proposed keep their current lattice.  Both end
with one integration of their final zone set.

Zone features (cheap, known before the next level is evaluated): distance of the zone's f1,
f2 and f1 + f2 intervals to the nearest resonance in half-power bandwidths, lattice steps per
bandwidth, lattice size, BRM factors, level, the zone's share of the total diagonal moments
and the change it showed at its previous refinement.
"""
from __future__ import annotations

import dataclasses
import os
from typing import Optional, Tuple

import numpy as np

from . import api

NFEAT = 13
# proposer trained by train_proposer.py on 600 seeded random structures (tol 1e-3, 2 levels)
DEFAULT_WEIGHTS = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "proposer.npz")


def refine_zone(z: api.Zone) -> api.Zone:
    """The same zone with its BFM lattice steps halved (BRM factors kept)."""
    return api.Zone(z.fi0, z.fj0, z.dIi / 2, z.dIj / 2, z.dJi / 2, z.dJj / 2, 2 * (z.ni - 1) + 1,
                    2 * (z.nj - 1) + 1, z.Fi, z.Fj, z.sym, z.policy)


def zone_points(zones) -> int:
    return int(sum(z.ni * z.nj for z in zones))


def _interval_dist(lo, hi, f, bw):
    """Distance of [lo, hi] (absolute frequencies) to the resonances f_m, in bandwidths, and
    the bandwidth of the nearest one."""
    a, b = min(abs(lo), abs(hi)), max(abs(lo), abs(hi))
    if lo <= 0.0 <= hi:
        a = 0.0
    d = np.where(f < a, a - f, np.where(f > b, f - b, 0.0)) / bw
    k = int(np.argmin(d))
    return float(d[k]), float(bw[k])


def features(z: api.Zone, level: int, zd: np.ndarray, tot_max: float, e_prev: float, natf, xsi) -> np.ndarray:
    f = np.asarray(natf, dtype=np.float64)
    bw = np.maximum(np.asarray(xsi) * f, 1e-9)
    i_lo, i_hi = sorted((z.fi0, z.fi0 + (z.ni - 1) * z.dIi + (z.nj - 1) * z.dJi))
    j_lo, j_hi = sorted((z.fj0, z.fj0 + (z.ni - 1) * z.dIj + (z.nj - 1) * z.dJj))
    dI, bI = _interval_dist(i_lo, i_hi, f, bw)
    dJ, bJ = _interval_dist(j_lo, j_hi, f, bw)
    dS, bS = _interval_dist(i_lo + j_lo, i_hi + j_hi, f, bw)
    hI = np.hypot(z.dIi, z.dIj) / bI
    hJ = np.hypot(z.dJi, z.dJj) / bJ
    hS = (np.hypot(z.dIi, z.dIj) + np.hypot(z.dJi, z.dJj)) / bS
    share = float(np.max(np.abs(zd))) / max(tot_max, 1e-300)
    return np.array([np.log1p(dI), np.log1p(dJ), np.log1p(dS), np.log(hI), np.log(hJ),
                     np.log(z.ni * z.nj), np.log(z.Fi * z.Fj), float(level),
                     np.log10(share + 1e-12), np.log10(e_prev + 1e-12),
                     np.log1p(min(dI, dJ)), np.log1p(dI + dJ), np.log(hS)], dtype=np.float64)


@dataclasses.dataclass
class Outcome:
    m3mf: np.ndarray
    m3mr: np.ndarray
    points: int            # BFM lattice points evaluated: judging levels and final integration
    ms: float              # device time of every evaluation
    zones: int             # final zone count
    refined: int           # zone refinements kept
    records: Optional[Tuple[np.ndarray, np.ndarray, np.ndarray]] = None  # features, label, change
    final_zones: Optional[list] = None


class Refiner:
    """Adaptive refinement of the pre-mesh zones.  It stands in for the reference's fixed
    refinement policies, so the session is switched to the driver's Mesher controls (no delta
    validation, no BFM multi-level refinement): the level-0 zones are the pre-mesh lattices."""

    def __init__(self, session: api.BsaSession, tol: float = 1e-3, max_levels: int = 2):
        session.use_driver_controls()
        self.s = session
        self.tol = tol
        self.max_levels = max_levels
        kept = np.nonzero(np.max(np.abs(session.prob.phi), axis=0) == 1.0)[0]  # the library's mode rule
        self.natf = session.prob.natf[kept]
        self.xsi = session.prob.xsi[kept]
        self.points = 0
        self.ms = 0.0

    def _eval(self, zones):
        mf, mr, zd = self.s.msh_zones_diag(zones)
        self.points += zone_points(zones)
        self.ms += self.s.stats().ms_total
        return mf, mr, zd

    def run(self, proposer=None, threshold: float = 0.5, keep_records: bool = False) -> Outcome:
        self.points, self.ms = 0, 0.0
        active = list(self.s.generate_zones())
        _, _, zd = self._eval(active)
        tot_max = float(np.max(np.abs(zd.sum(axis=0))))
        e_prev = np.zeros(len(active))
        final, refined = [], 0
        feats, labels, errs = [], [], []
        for level in range(self.max_levels):
            if not active:
                break
            F = np.stack([features(z, level, zd[k], tot_max, e_prev[k], self.natf, self.xsi)
                          for k, z in enumerate(active)])
            prop = np.ones(len(active), dtype=bool) if proposer is None else proposer(F) > threshold
            final += [z for k, z in enumerate(active) if not prop[k]]
            idx = np.nonzero(prop)[0]
            if idx.size == 0:
                active = []
                break
            cand = [refine_zone(active[k]) for k in idx]
            _, _, zd1 = self._eval(cand)
            e = np.max(np.abs(zd1 - zd[idx]), axis=1) / max(tot_max, 1e-300)
            if keep_records:
                feats.append(F[idx])
                labels.append((e > self.tol).astype(float))
                errs.append(e)
            more = e > self.tol
            refined += int(np.count_nonzero(more))
            # the change stays within tolerance: the current lattice is kept
            final += [active[k] for k, m in zip(idx, more) if not m]
            active = [c for c, m in zip(cand, more) if m]
            zd = zd1[more]
            e_prev = e[more]
        final += active
        mf, mr, _ = self._eval(final)
        rec = None
        if keep_records and feats:
            rec = (np.concatenate(feats), np.concatenate(labels), np.concatenate(errs))
        return Outcome(mf, mr, self.points, self.ms, len(final), refined, rec, final)


class Proposer:
    """The network with its input standardisation."""

    def __init__(self, width: int = 128, seed: int = 1):
        self.net = api.Mlp(NFEAT, width, seed)
        self.mu = np.zeros(NFEAT)
        self.sd = np.ones(NFEAT)

    def fit(self, X, err, tol: float, epochs: int = 40, batch: int = 512, lr: float = 1e-3, seed: int = 7):
        """Soft targets y = sigmoid((log10 e - log10 tol) / 0.3): the network grades how far a
        zone's refinement change is from the tolerance; records within a factor 30 of the
        tolerance or above it weigh 20x."""
        self.mu = X.mean(axis=0)
        self.sd = X.std(axis=0) + 1e-6
        Xn = (X - self.mu) / self.sd
        y = 1.0 / (1.0 + np.exp(-(np.log10(err + 1e-15) - np.log10(tol)) / 0.3))
        w = np.where(err > tol / 30.0, 20.0, 1.0)
        return self.net.train(Xn, y, w, epochs=epochs, batch=batch, lr=lr, seed=seed)

    def save(self, path, threshold, tol):
        np.savez(path, params=self.net.params(), mu=self.mu, sd=self.sd, threshold=threshold, tol=tol)

    @classmethod
    def load(cls, path):
        d = np.load(path)
        p = cls()
        p.net.set_params(d["params"])
        p.mu, p.sd = d["mu"], d["sd"]
        return p, float(d["threshold"]), float(d["tol"])

    def __call__(self, F):
        return self.net.forward((F - self.mu) / self.sd)

    def close(self):
        self.net.close()
