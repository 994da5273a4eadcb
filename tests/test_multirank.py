"""The multi-rank path of bench.py on CPU: two `gloo` ranks shard the batches
with no data-path collective (weak scaling) and combine their figures the
way the bench does (slowest rank's time, summed counts)."""
from __future__ import annotations

import os
import sys

import pytest

from conftest import ROOT

sys.path.insert(0, ROOT)


def _rank(rank: int, world: int, port: int, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    mine = bench.rank_batches(rank, world, 16)
    sites = sum(len(bench.batch_sites(b, 16)) for b in mine)
    seconds = 10.0 + rank                     # the slower rank sets the job's time
    res = bench.reduce_over_ranks(dist, seconds, [sites, 2000 * sites], "cpu")
    out.put((rank, mine, res))
    dist.destroy_process_group()


def test_two_gloo_ranks_shard_and_reduce():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (_, b0, r0), (_, b1, r1) = got
    import bench
    assert sorted(b0 + b1) == list(range(16)) and not set(b0) & set(b1)
    n_sites = len(bench.grid_sites())
    assert r0 == r1 == [11.0, n_sites, 2000 * n_sites]
