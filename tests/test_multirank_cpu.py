"""The multi-rank path on CPU (gloo, world size 2): lower-state batches are disjoint
shards with no data exchange, and the reported step time is the slowest rank's."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import sys
    import torch.distributed as dist
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    first = bench.lower_first(rank, 2000, 11000)
    t = bench.max_over_ranks(10.0 + rank, dist, "cpu")
    out[rank] = (first, t)
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_shard_and_max():
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    mp.start_processes(_worker, args=(2, port, out), nprocs=2, start_method="spawn", join=True)
    (f0, t0), (f1, t1) = out[0], out[1]
    assert (f0, f1) == (0, 2000)          # disjoint consecutive batches
    assert t0 == t1 == 11.0               # max over ranks


def test_shards_disjoint_then_wrap():
    import bench
    firsts = [bench.lower_first(r, 2000, 11000) for r in range(8)]
    assert firsts[:5] == [0, 2000, 4000, 6000, 8000]
    assert firsts[5] == 0                 # beyond 5 disjoint batches: replicas
    assert bench.lower_first(0, 64, 10) == 0
