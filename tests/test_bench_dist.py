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


def _partition_rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    from gisbdw_gb300 import graphs as G
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    graphs = G.config2_graphs()
    mine = [graphs[i].name for i in bench.partition_graphs(graphs, world)[rank]]
    # every rank reports its share; the job rate sums the units over the slowest time
    rate, slowest = bench.job_rate_total(len(mine), 1.0 + rank, world)
    out.put((rank, mine, rate, slowest))
    dist.destroy_process_group()


def test_partition_splits_the_workload_over_gloo_ranks():
    """--partition: two gloo ranks split the nine headline graphs between
    them — every graph once, the loads (2^n per graph) balanced — and the
    whole-job rate is the sum of their solves over the slower rank's time."""
    import torch.multiprocessing as mp
    sys.path.insert(0, ROOT)
    from gisbdw_gb300 import graphs as G
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_partition_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(2))
    names = [n for _, mine, _, _ in got for n in mine]
    graphs = G.config2_graphs()
    assert sorted(names) == sorted(g.name for g in graphs)
    cost = {g.name: 2 ** g.n for g in graphs}
    loads = [sum(cost[n] for n in mine) for _, mine, _, _ in got]
    assert max(loads) - min(loads) <= max(cost.values())
    for _, _, rate, slowest in got:
        assert slowest == pytest.approx(2.0) and rate == pytest.approx(len(graphs) / 2.0)


def test_partition_is_deterministic_and_complete():
    sys.path.insert(0, ROOT)
    import bench
    from gisbdw_gb300 import graphs as G
    graphs = G.config3_graphs(count=50, seed=2)
    for world in (1, 3, 8):
        parts = bench.partition_graphs(graphs, world)
        assert parts == bench.partition_graphs(graphs, world)
        assert sorted(i for p in parts for i in p) == list(range(len(graphs)))
