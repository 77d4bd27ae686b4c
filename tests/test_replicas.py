"""The N > 1 path of bench.py on the CPU: independent replicas, one per
rank, joined only by the timing reduction (max of the ranks' times, sum of
their particles) -- the path does not shard, so there is no data-path
collective.  Two gloo ranks on 127.0.0.1."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    n_local = [1000, 3000][rank]
    secs = [2.0, 4.0][rank]
    value, tmax = bench.aggregate_replicas(n_local, 10, secs, world, device="cpu")
    out[rank] = (value, tmax)
    dist.barrier()
    dist.destroy_process_group()


def test_replica_aggregation_two_ranks():
    port = _free_port()
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_rank, args=(2, port, out), nprocs=2, start_method="spawn", join=True)
    for r in (0, 1):
        value, tmax = out[r]
        assert tmax == 4.0
        assert value == pytest.approx((1000 + 3000) * 10 / 4.0)


def test_single_rank_needs_no_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.aggregate_replicas(500, 4, 2.0, 1) == (1000.0, 2.0)
