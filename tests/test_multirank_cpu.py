"""Two ranks on the gloo backend (CPU): the benchmark's whole-job aggregation for
replicas -- every rank gets the slowest rank's time, and the job rate counts the
rays of all ranks over it -- and a rank that never joins makes the rendezvous fail
with an error instead of hanging."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, ms_by_rank, out):
    import sys
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms, rate = bench.job_rate(ms_by_rank[rank], 1_000_000, world)
    out[rank] = (ms, rate)
    dist.barrier()
    dist.destroy_process_group()


def test_job_rate_takes_the_slowest_rank():
    world = 2
    ms_by_rank = [8.0, 10.0]
    with mp.Manager() as m:
        out = m.dict()
        mp.start_processes(_worker, args=(world, _free_port(), ms_by_rank, out), nprocs=world, start_method="spawn")
        res = dict(out)
    for r in range(world):
        ms, rate = res[r]
        assert ms == 10.0
        assert abs(rate - 2 * 1_000_000 / 10e-3 / 1e6) < 1e-9


def test_single_rank_needs_no_process_group():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    assert bench.job_rate(5.0, 1_000_000, 1) == (5.0, 200.0)


def _lonely(rank, world, port):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    from datetime import timedelta
    if rank == 1:
        return                      # this rank never joins
    dist.init_process_group("gloo", rank=rank, world_size=world, timeout=timedelta(seconds=3))


def test_missing_rank_fails_the_rendezvous():
    with pytest.raises(Exception):
        mp.start_processes(_lonely, args=(2, _free_port()), nprocs=2, start_method="spawn")
