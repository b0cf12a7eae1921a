"""bench.py's N > 1 arithmetic (independent replicas, one per GPU: the slowest rank's time and the
whole-job MLUPS) on two gloo ranks on the CPU."""
import os
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        dt = bench.replica_time(1.0 + 0.5 * rank, world, dist, torch, "cpu")
        out[rank] = (dt, bench.replica_mlups(1000, 10, dt, world))
    finally:
        dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank():
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    mp.start_processes(_rank, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
    assert out[0] == out[1]
    dt, mlups = out[0]
    assert dt == 1.5
    assert abs(mlups - 2 * 1000 * 10 / 1.5 / 1e6) < 1e-15
