"""The N > 1 path of bench.py (replicas, one rank per GPU): the whole-job
rate is every rank's units over the slowest rank's time. Two gloo ranks on
CPU."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    rate, slowest = bench.job_rate(10, 1.0 + rank, world)  # rank r took 1 + r seconds for 10 units
    out.put((rank, rate, slowest))
    dist.destroy_process_group()


def test_job_rate_takes_the_slowest_rank():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    for rank, rate, slowest in got:
        assert slowest == pytest.approx(2.0)
        assert rate == pytest.approx(20 / 2.0)


def test_job_rate_single_rank():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.job_rate(9, 3.0, 1) == (3.0, 3.0)
