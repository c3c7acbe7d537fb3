"""Multi-GPU is replicas only: every rank runs its own shard of independent pairs, and the
only cross-rank traffic is the benchmark's timing reduction.  This checks that host path
with two gloo ranks on the CPU: the reductions, and that ranks get disjoint seeded inputs."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import bench

    class A:
        pairs = 64
    r, w = bench.dist_init(A)
    assert (r, w) == (rank, world)
    bench.barrier(w)
    mx = bench.allmax(10.0 + rank, w)
    sm = bench.allsum(100 + rank, w)
    wl = bench.Workload("cfg0", A, r)
    out[rank] = (mx, sm, bytes(wl.sets[0].qbuf[:256]))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    world, port = 2, _free_port()
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_rank_main, args=(world, port, out), nprocs=world, start_method="spawn", join=True)
    assert out[0][0] == out[1][0] == 11.0           # max over ranks
    assert out[0][1] == out[1][1] == 201.0          # sum over ranks
    assert out[0][2] != out[1][2]                   # each rank has its own shard of pairs
