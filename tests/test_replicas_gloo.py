"""Multi-rank (replicas-only) bookkeeping on CPU: two gloo ranks split the slices of a stack.

Slices are independent, so the N>1 path has no data-path collective: each rank reconstructs its
own block of slices and only the timing crosses ranks (barrier, max over ranks, unit total).
Here the per-rank work is the oracle's CPU reconstruction of small slices, standing in for the
device kernels, so that partition, aggregation and result assembly are checked without a GPU.
"""
from __future__ import annotations

import os
import socket
import time

import numpy as np
import pytest

from recview_gb300.replicas import shard

N_SLICES, W, V = 5, 48, 40


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _case(s: int):
    from tests.rvtest import fbp_case
    return fbp_case(1000 + s, W, V, (W - 1) / 2.0 + 0.25 * s)


def _rank_main(rank: int, world: int, port: int, outdir: str):
    import torch.distributed as dist
    from recview_gb300 import replicas
    from tests.rvtest import Oracle
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ora = Oracle()
        mine = replicas.shard(N_SLICES, world, rank)
        replicas.barrier()
        t0 = time.perf_counter()
        slices = {s: ora.reconstruct(_case(s)) for s in mine}
        if rank == 1:
            time.sleep(0.2)                     # make rank 1 the slow one
        dt = time.perf_counter() - t0
        replicas.barrier()
        rate, total, tmax = replicas.aggregate_rate(len(mine), dt)
        np.savez(os.path.join(outdir, f"rank{rank}.npz"), dt=dt, rate=rate, total=total, tmax=tmax,
                 ids=np.array(list(mine), np.int64),
                 **{f"s{s}": v for s, v in slices.items()})
    finally:
        dist.destroy_process_group()


def test_shard_partitions_exactly():
    for n in (0, 1, 5, 64, 1000):
        for world in (1, 2, 3, 8):
            parts = [shard(n, world, r) for r in range(world)]
            flat = [i for p in parts for i in p]
            assert flat == list(range(n))
            sizes = [len(p) for p in parts]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard(4, 2, 2)


def test_single_process_helpers_are_identity():
    from recview_gb300 import replicas
    replicas.barrier()
    assert replicas.max_over_ranks(1.5) == 1.5
    assert replicas.aggregate_rate(3, 2.0) == (1.5, 3, 2.0)


def test_two_gloo_ranks_split_slices(tmp_path, oracle):
    import torch.multiprocessing as mp
    world = 2
    mp.start_processes(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world,
                       start_method="spawn", join=True)
    got = [np.load(tmp_path / f"rank{r}.npz") for r in range(world)]
    ids = [list(g["ids"]) for g in got]
    assert sorted(ids[0] + ids[1]) == list(range(N_SLICES)) and not set(ids[0]) & set(ids[1])
    # whole-job figures: every rank agrees on the total units and on the slowest rank's time
    tmax = max(float(g["dt"]) for g in got)
    for g in got:
        assert int(g["total"]) == N_SLICES
        assert float(g["tmax"]) == pytest.approx(tmax)
        assert float(g["rate"]) == pytest.approx(N_SLICES / tmax)
    assert float(got[1]["dt"]) >= 0.2
    # the assembled slices equal a single-process run
    for r, g in enumerate(got):
        for s in ids[r]:
            assert np.array_equal(g[f"s{s}"], oracle.reconstruct(_case(s)))
