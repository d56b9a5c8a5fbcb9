"""The N > 1 bench path (replicas, one process per GPU): whole-job throughput = rays summed over ranks
divided by the slowest rank's time. Checked with two gloo ranks on CPU (127.0.0.1)."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    rays = 1_000_000.0 * (rank + 1)     # rank 0 casts 1M rays in 2 ms, rank 1 casts 2M rays in 5 ms
    ms = 2.0 + 3.0 * rank
    out[rank] = bench.aggregate_over_ranks(rays, ms, dist)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_aggregation_gloo():
    world = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    for r in range(world):
        rays, ms, mrays = res[r]
        assert rays == 3_000_000.0 and ms == 5.0
        assert abs(mrays - 3_000_000.0 / 5e-3 / 1e6) < 1e-9


def test_single_process_aggregation():
    import bench
    assert bench.aggregate_over_ranks(2e6, 4.0) == (2e6, 4.0, 500.0)
