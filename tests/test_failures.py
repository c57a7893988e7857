"""Failure detection without a GPU fault: every failure is made on the host
(an injected allocation failure, a stalled dependency, an abort request) and
the library must report it as a status and leave the handle usable. Calls go
through the C ABI (libgtd.so via ctypes)."""
import threading
import time

import numpy as np
import pytest

from gisbdw_gb300 import DynamicGPU, Handle, _lib
from gisbdw_gb300 import graphs as G
from gisbdw_gb300.treedepth import NO_RESULT
from gisbdw_gb300.validate import check_tree

pytestmark = pytest.mark.gpu


@pytest.fixture
def fresh():
    """A new handle (no buffers yet, so the first solve allocates)."""
    h = Handle(0)
    yield h
    _lib.inject_fault(_lib.FAULT_NONE, 0)
    h.close()


def _oom(fn):
    with pytest.raises(_lib.GtdError) as e:
        fn()
    assert e.value.status == 3, e.value  # GTD_OOM


def test_allocation_failure_single_dp(fresh, port):
    g = G.gnp_connected(20, 0.3, 2)
    for nth in (1, 2):  # the table, then the flags
        _lib.inject_fault(_lib.FAULT_ALLOC, nth)
        _oom(lambda: fresh.dp_solve(g.adj64(), g.n))
        _lib.inject_fault(_lib.FAULT_NONE, 0)
        td, parent, _, _ = fresh.dp_solve(g.adj64(), g.n)
        otd, opar = port.dp_solve(g)
        assert td == otd and parent.tolist() == opar.tolist()
        fresh.close()
        fresh.__init__(0)


def test_allocation_failure_batch_and_bnb(fresh):
    gs = G.config3_graphs(count=40, seed=9)
    want, _, _ = fresh.dp_solve_batch(gs)
    small = [G.grid(4, 4), G.tree_plus_edges(20, 3, 1)]
    bref = fresh.bnb_solve_batch(small, deadline_ns=30 * 10**9)
    big = G.config3_graphs(count=300, seed=10)  # a larger pool: the batch must allocate again
    _lib.inject_fault(_lib.FAULT_ALLOC, 1)
    _oom(lambda: fresh.dp_solve_batch(big))
    _lib.inject_fault(_lib.FAULT_NONE, 0)
    td, _, _ = fresh.dp_solve_batch(gs)
    assert td.tolist() == want.tolist()
    # the branch and bound: a batch larger than the last one allocates
    more = small + [G.cycle(11), G.grid(3, 6)]
    _lib.inject_fault(_lib.FAULT_ALLOC, 1)
    _oom(lambda: fresh.bnb_solve_batch(more, deadline_ns=30 * 10**9))
    _lib.inject_fault(_lib.FAULT_NONE, 0)
    res = fresh.bnb_solve_batch(more, deadline_ns=30 * 10**9)
    assert np.all(res["status"] == 0)
    dtd, _, _ = fresh.dp_solve_batch(more)
    assert res["td"][:2].tolist() == bref["td"].tolist() and res["td"].tolist() == dtd.tolist()


def test_class_layer_swallows_oom_like_the_reference():
    """DynamicCPU::operator() catches std::bad_alloc and leaves no result
    (dynamic_cpu.hpp:52-56); GetTDDecomp then returns the UINT_MAX sentinel
    (dynamic_cpu.hpp:79-80)."""
    d = DynamicGPU()
    g = G.gnp_connected(21, 0.3, 5)
    _lib.inject_fault(_lib.FAULT_ALLOC, 1)
    try:
        d(g)
    finally:
        _lib.inject_fault(_lib.FAULT_NONE, 0)
    assert d.Result().treedepth == NO_RESULT and d.GetElimination(g.n, g.n, 0) == []
    d(g)
    r = d.Result()
    assert r.treedepth != NO_RESULT and check_tree(g, r.treedepth, r.parent)


def test_abort_stops_a_running_search_and_handle_recovers(fresh):
    """gtd_abort from another thread ends a branch-and-bound call that would
    otherwise run for its whole 60 s deadline (random 3-regular graphs are not
    proven in that time): the call returns GTD_ABORTED within seconds."""
    gs = [g for g in G.config4_graphs(count=12) if g.name.startswith("reg3")]
    out = {}

    def run():
        t0 = time.perf_counter()
        try:
            fresh.bnb_solve_batch(gs, deadline_ns=60 * 10**9)
            out["status"] = 0
        except _lib.GtdError as e:
            out["status"] = e.status
        out["s"] = time.perf_counter() - t0

    th = threading.Thread(target=run)
    th.start()
    time.sleep(2.0)
    fresh.abort()
    th.join(timeout=90)
    assert not th.is_alive()
    assert out["status"] == 5, out  # GTD_ABORTED
    assert out["s"] < 20, out
    res = fresh.bnb_solve_batch([G.cycle(9)], deadline_ns=10**10)
    assert res["status"][0] == 0 and res["td"][0] == 5


def test_abort_stops_a_waiting_dp_solve(fresh):
    """A DP solve whose first tile is never taken (the injected stall) would
    wait 30 s for its dependencies; gtd_abort from another thread ends it with
    GTD_ABORTED within seconds, and the next solve is exact."""
    g = G.gnp_connected(22, 0.25, 6)
    out = {}

    def run():
        t0 = time.perf_counter()
        try:
            fresh.dp_solve(g.adj64(), g.n, timeout_ns=30 * 10**9)
            out["status"] = 0
        except _lib.GtdError as e:
            out["status"] = e.status
        out["s"] = time.perf_counter() - t0

    _lib.inject_fault(_lib.FAULT_STALL, 1)
    th = threading.Thread(target=run)
    th.start()
    time.sleep(1.0)
    fresh.abort()
    th.join(timeout=60)
    assert not th.is_alive()
    assert out["status"] == 5 and out["s"] < 10, out  # GTD_ABORTED
    td, _, _, _ = fresh.dp_solve(g.adj64(), g.n)
    assert td == fresh.dp_solve(g.adj64(), g.n, tile_bits=8)[0]
