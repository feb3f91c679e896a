"""Channel sharding across ranks, exercised with two gloo ranks on the CPU:
the union of the ranks' row ranges is the batch, and per-rank filtering plus
gather_rows equals filtering the whole batch on one rank (the per-rank work
here is the CPU oracle; with one GPU per rank each rank calls the library)."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from scir_gb300.sharding import shard_rows


@pytest.mark.parametrize("batch,world", [(10, 2), (7, 3), (1, 4), (0, 2), (16384, 8)])
def test_shard_rows_partition(batch, world):
    rows = []
    sizes = []
    for r in range(world):
        a, b = shard_rows(batch, world, r)
        rows += list(range(a, b))
        sizes.append(b - a)
    assert rows == list(range(batch))
    assert max(sizes) - min(sizes) <= 1


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import torch
    import torch.distributed as dist

    import oracle as O
    from scir_gb300.sharding import gather_rows, shard_rows

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        rng = np.random.default_rng(0)
        x = rng.uniform(-1, 1, (9, 500)).astype(np.float32)
        taps = rng.standard_normal(17).astype(np.float32)
        a, b = shard_rows(x.shape[0], world, rank)
        local = torch.from_numpy(O.fir1d_batched_f32(x[a:b], taps)) if b > a else \
            torch.zeros((0, 500))
        full = gather_rows(local, x.shape[0])
        out[rank] = bool(np.array_equal(full.numpy(), O.fir1d_batched_f32(x, taps)))
    finally:
        dist.destroy_process_group()


def test_two_rank_gloo_sharding():
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert out[0] and out[1]


def _max_worker(rank, world, port, out):
    import torch
    import torch.distributed as dist

    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # each rank's own time; every rank must get the slowest one
        out[rank] = bench.max_over_ranks(torch, 1.5 * (rank + 1), "cpu", world)
    finally:
        dist.destroy_process_group()


def test_benchmark_time_is_the_max_over_ranks():
    import torch

    import bench
    assert bench.max_over_ranks(torch, 2.25, "cpu", 1) == 2.25
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_max_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    assert out[0] == 3.0 and out[1] == 3.0
