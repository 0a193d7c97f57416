"""Multi-process sharding of the Classic grid (CPU, gloo, world size 2): the row shards
partition the grid, and the rank-local moment sums add up to the full grid's.  The
per-shard moments come from the oracle's bispectra, so no GPU is needed."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from bsalib_gb300.dist import shard_rows, sum_moments


def test_shards_partition_the_rows():
    for nf in (1, 2, 7, 129, 1025):
        for world in (1, 2, 3, 8):
            if world > nf:
                continue
            rows = []
            for r in range(world):
                r0, r1 = shard_rows(nf, r, world)
                assert r1 > r0
                rows.extend(range(r0, r1))
            assert rows == list(range(nf))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, ret):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    from bsalib_gb300.problem import cantilever_tower
    from oracle.oracle import Oracle, classic_weights
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        prob = cantilever_tower(nfreqs=6, df=0.4, nodes=7)
        r = Oracle(prob).classic_vect()
        f = r["f"]
        w = classic_weights(f.size, f[1] - f[0])
        r0, r1 = shard_rows(f.size, rank, world)
        part = {"m3mf_cls": np.einsum("ij,ijk->k", w[r0:r1], r["bf"][r0:r1]),
                "m3mr_cls": np.einsum("ij,ijk->k", w[r0:r1], r["br"][r0:r1])}
        tot = sum_moments(part, dist)
        ret[rank] = (tot["m3mf_cls"], tot["m3mr_cls"], r["m3mf"], r["m3mr"])
    finally:
        dist.destroy_process_group()


def test_gloo_two_ranks_sum_to_full_grid():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as mgr:
        ret = mgr.dict()
        port = _free_port()
        procs = [ctx.Process(target=_worker, args=(r, 2, port, ret)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(timeout=240)
            assert p.exitcode == 0
        for rank in range(2):
            mf, mr, ref_f, ref_r = ret[rank]
            assert np.max(np.abs(mf - ref_f)) / np.max(np.abs(ref_f)) < 1e-12
            assert np.max(np.abs(mr - ref_r)) / np.max(np.abs(ref_r)) < 1e-12
