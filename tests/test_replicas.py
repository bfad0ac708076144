"""Multi-process (gloo, world_size 2, CPU) checks of the replica paths.

The step does not shard on one grid, so N GPUs run N independent replicas: bench.py times
each and reports the slowest rank's time (max over ranks) with the whole-job cell count; the
ensemble splits its runs across ranks by cost.  These run the same helpers over gloo.
"""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def _port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist

    import bench
    import fen_gb300 as F

    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = bench.max_over_ranks(10.0 + 5.0 * rank, dist, "cpu")
    value = bench.replica_throughput(world, 1000, 20, ms)
    sizes = np.array([64, 96, 128, 192, 256] * 7)
    mine = F.partition_runs(sizes, world)[rank]
    import torch

    cost = torch.tensor([float(np.sum(sizes[mine].astype(np.int64) ** 2))], dtype=torch.float64)
    costs = [torch.zeros(1, dtype=torch.float64) for _ in range(world)]
    dist.all_gather(costs, cost)
    ids = torch.zeros(len(sizes), dtype=torch.int64)
    ids[torch.from_numpy(mine)] = 1
    dist.all_reduce(ids)
    if rank == 0:
        np.save(out, np.array([ms, value, *[c.item() for c in costs], ids.min().item(), ids.max().item()]))
    dist.destroy_process_group()


def test_replica_timing_and_ensemble_partition(tmp_path):
    out = str(tmp_path / "r.npy")
    mp.spawn(_worker, args=(2, _port(), out), nprocs=2, join=True)
    ms, value, c0, c1, idmin, idmax = np.load(out)
    assert ms == 15.0                          # max over ranks
    assert value == pytest.approx(2 * 1000 * 20 / 0.015 / 1e6)
    assert idmin == 1 and idmax == 1           # every run on exactly one rank
    assert abs(c0 - c1) <= 256 * 256           # balanced within one largest run


def test_partition_covers_runs_once():
    import fen_gb300 as F

    sizes = np.random.Generator(np.random.PCG64(5)).choice([64, 96, 128, 192, 256], size=512)
    for world in (1, 2, 4, 8):
        parts = F.partition_runs(sizes, world)
        allr = np.sort(np.concatenate(parts))
        assert np.array_equal(allr, np.arange(512))
        loads = [np.sum(sizes[p].astype(np.int64) ** 2) for p in parts]
        assert max(loads) - min(loads) <= 256 * 256
