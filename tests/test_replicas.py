"""bench.py's multi-replica logic on CPU: two gloo ranks, barrier, max over
ranks, and the whole-job throughput from the slowest rank."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    import torch
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    bench.barrier(ws)
    ms = 10.0 * (rank + 1)  # rank 1 is the slower one
    ms_max = bench.max_over_ranks(ws, ms, torch.device("cpu"))
    out[rank] = (ms_max, bench.job_mlups(ws, 1000, 50, ms_max))
    bench.barrier(ws)
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    out = mp.Manager().dict()
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    for r in range(2):
        ms_max, mlups = out[r]
        assert ms_max == 20.0
        assert abs(mlups - 2 * 1000 * 50 / 0.020 / 1e6) < 1e-9
