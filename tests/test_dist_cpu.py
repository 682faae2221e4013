"""Multi-rank host logic of bench.py on CPU (gloo, world size 2).

The hot path shards over independent cells with no data-path collective
(replicas): each rank solves its own seeded cell, and only the timing is
reduced (max over ranks) after a barrier.  No GPU is used here.
"""
import os
import socket

import pytest

from conftest import ROOT


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import sys

    sys.path.insert(0, ROOT)
    import torch.distributed as dist

    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    bench.barrier(world)
    t = bench.max_over_ranks(world, 1.0 + rank)
    seed = bench.rank_seed(rank)
    mask = bench.workload_mask(16, seed)
    out[rank] = (t, seed, mask.tobytes())
    dist.destroy_process_group()


def test_replicas_gloo_world2():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    port = _free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    assert out[0][0] == out[1][0] == 2.0  # max over ranks
    assert out[0][1] != out[1][1]          # one distinct cell per rank
    assert out[0][2] != out[1][2]          # (same porosity, different voxels)
