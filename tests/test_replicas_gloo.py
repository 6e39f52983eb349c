"""Replica timing across ranks (bench.py's N>1 path) with the gloo backend on CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ws, r, local = bench.dist_env()
    assert (ws, r, local) == (world, rank, rank)
    bench.barrier(ws)
    ms = 10.0 + 5.0 * rank          # rank 1 is the slow replica
    ms_max = bench.max_over_ranks(ms, ws, torch.device("cpu"))
    out[rank] = ms_max
    dist.destroy_process_group()


def test_max_over_ranks_two_replicas():
    world = 2
    port = _free_port()
    manager = mp.get_context("spawn").Manager()
    out = manager.dict()
    mp.start_processes(_worker, args=(world, port, out), nprocs=world, join=True, start_method="spawn")
    assert dict(out) == {0: 15.0, 1: 15.0}
