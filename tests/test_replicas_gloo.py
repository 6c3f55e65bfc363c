"""The N-replica timing of bench.py on CPU ranks (gloo, world size 2): each
rank times its own replica, the job time is the maximum over ranks and the
value counts every replica's atoms."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port),
                      RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    r, w, local = bench.dist_env()
    assert (r, w, local) == (rank, world, rank)
    ms = 10.0 + 5.0 * rank            # rank 1 is the slow one
    t = bench.replica_time(ms, w)
    out[rank] = (t, bench.replica_value(1000, 4, t, w))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_timing_two_ranks():
    port = _free_port()
    with mp.get_context("spawn").Manager() as m:  # no fork of this process
        out = m.dict()
        mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    assert res[0][0] == res[1][0] == 15.0          # max over ranks
    assert res[0][1] == res[1][1] == 2 * 1000 * 4 / 0.015


def test_single_replica_is_local_time():
    import bench
    assert bench.replica_time(12.5, 1) == 12.5
    assert bench.replica_value(10, 2, 1000.0, 1) == 20.0
