"""Replica sharding and the cross-rank aggregation, on CPU with gloo
(world size 2): no GPU and no solver needed."""
import os
import socket

import pytest
import torch.multiprocessing as mp

from sweeping_fd_weno_gb300.replicas import aggregate, shard


def test_shard_covers_every_instance_once_and_balances():
    costs = [n * n for n in (128, 640, 300, 512, 129, 256, 640, 200, 333)]
    for world in (1, 2, 3, 4, 8):
        parts = [shard(costs, r, world) for r in range(world)]
        flat = sorted(k for p in parts for k in p)
        assert flat == list(range(len(costs)))
        loads = [sum(costs[k] for k in p) for p in parts]
        assert max(loads) - min(loads) <= max(costs)
        assert parts == [shard(costs, r, world) for r in range(world)]  # deterministic


def test_shard_rejects_bad_rank():
    with pytest.raises(ValueError):
        shard([1.0], 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r did (r + 1) * 1e6 updates in (r + 2) seconds
        out[rank] = aggregate((rank + 1) * 1e6, rank + 2.0)
    finally:
        dist.destroy_process_group()


def test_aggregate_over_two_gloo_ranks():
    world = 2
    with mp.get_context("spawn").Manager() as mgr:
        out = mgr.dict()
        mp.start_processes(_worker, args=(world, _free_port(), out), nprocs=world,
                           start_method="spawn")
        res = dict(out)
    for r in range(world):
        tu, tt, v = res[r]
        assert tu == 3e6 and tt == 3.0 and v == 1e6


def test_aggregate_without_a_process_group():
    assert aggregate(10.0, 2.0) == (10.0, 2.0, 5.0)
