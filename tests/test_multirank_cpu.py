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


def _shard_worker(rank, world, port, out):
    """One rank: its own lower-state range of a block pair, amplitudes from the oracle's
    restatement of the reference loop (MultiGpuManager::ExecuteHalfLs per lower state), then
    its line-list shard as the reference prints it; the shards meet only on rank 0."""
    import sys
    import numpy as np
    import torch.distributed as dist
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for sub in ("", "gain-mpi_gb300", "oracle"):
        sys.path.insert(0, os.path.join(root, sub))
    import oracle
    import synth
    import threej
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    p = synth.make_problem(16, [2, 3], "c4", blocks=[(2, 0), (3, 1)])
    bI, bF = p.blocks[(0, 0)], p.blocks[(1, 1)]
    nI, nF = bI.vecs.shape[0], bF.vecs.shape[0]
    # contiguous shards by lower-state index (the reference orders its output the same way)
    bounds = [nI * r // world for r in range(world + 1)]
    lo = list(range(bounds[rank], bounds[rank + 1]))
    up = list(range(nF))
    amp = oracle.run_pair(p, 0, 0, 1, 1, lo, up, threej.threej_table(11), 11, oracle.REF, 1)
    text, n = oracle.line_list(amp, bI.energies[lo], bF.energies[up], lo, up, 2, 3, 0, 1)
    shards = [None] * world
    dist.all_gather_object(shards, (text, n))
    if rank == 0:
        full_lo = list(range(nI))
        amp_all = oracle.run_pair(p, 0, 0, 1, 1, full_lo, up, threej.threej_table(11), 11, oracle.REF, 1)
        whole, n_all = oracle.line_list(amp_all, bI.energies, bF.energies, full_lo, up, 2, 3, 0, 1)
        out["result"] = (b"".join(s[0] for s in shards) == whole, sum(s[1] for s in shards) == n_all,
                         all(s[1] > 0 for s in shards))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_line_list_shards_concatenate_to_the_single_rank_list():
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    mp.start_processes(_shard_worker, args=(2, port, out), nprocs=2, start_method="spawn", join=True)
    assert out["result"] == (True, True, True)
