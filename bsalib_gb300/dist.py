"""Sharding the Classic grid across processes (one GPU each).

The (f1, f2) points are independent, so a Classic analysis splits into contiguous blocks of
grid rows (f1 index); every rank evaluates its rows and the NM^2 / NM^3 moment vectors are
summed once at the end (the only exchange of the path).  `torch.distributed` with any
backend carries the sum (NCCL between GPUs, gloo on CPU).
"""
from __future__ import annotations

from typing import Dict, Tuple

import numpy as np

MOMENT_KEYS = ("m2mf_cls", "m2mr_cls", "m2o2mr_cls", "m3mf_cls", "m3mr_cls")


def shard_rows(nf: int, rank: int, world: int) -> Tuple[int, int]:
    """Contiguous block of grid rows [r0, r1) for `rank` of `world` (sizes differ by <= 1)."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("invalid rank / world size")
    base, extra = divmod(nf, world)
    r0 = rank * base + min(rank, extra)
    r1 = r0 + base + (1 if rank < extra else 0)
    return r0, r1


def sum_moments(parts: Dict[str, np.ndarray], dist=None, device="cpu") -> Dict[str, np.ndarray]:
    """Sum each moment vector over the ranks of the default process group (FP64)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return {k: np.array(v, dtype=np.float64) for k, v in parts.items()}
    import torch
    out = {}
    for k in sorted(parts):
        t = torch.tensor(np.ascontiguousarray(parts[k], dtype=np.float64), device=device)
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
        out[k] = t.cpu().numpy()
    return out


def run_classic_sharded(session, dist=None, device="cuda") -> Dict[str, np.ndarray]:
    """One Classic analysis split over the ranks of the default process group
    (bsa_gpu_setClassicShard: contiguous row blocks, interleaved product rows in the split
    precision's E form), the moments summed over the ranks."""
    rank, world = (dist.get_rank(), dist.get_world_size()) if dist is not None and dist.is_initialized() else (0, 1)
    session.set_shard(rank, world)
    out = session.run()
    return sum_moments({k: out[k] for k in MOMENT_KEYS}, dist, device)
