"""Subset DP on the GPU (K1) against the oracle: bit-exact treedepth, parent
array and GetElimination order, full tables, edge cases and error paths.
Calls go through the C ABI (libgtd.so via ctypes)."""
import math

import numpy as np
import pytest

from gisbdw_gb300 import DynamicGPU, InvalidArgument, _lib
from gisbdw_gb300 import graphs as G

pytestmark = pytest.mark.gpu


def small_graphs():
    gs = [G.path(n) for n in (2, 3, 5, 8, 13, 21)]
    gs += [G.cycle(n) for n in (3, 4, 7, 12, 16)]
    gs += [G.complete(n) for n in (2, 3, 6, 10, 14)]
    gs += [G.star(n) for n in (2, 9, 17)]
    gs += [G.chordal_cycle(n) for n in (10, 15)]
    gs += [G.grid(3, 4), G.grid(4, 5)]
    gs += [G.sparse_connected(n, s) for n in (8, 12, 16, 20) for s in range(2)]
    gs += [G.gnp_connected(n, p, s) for n in (10, 15, 19) for p in (0.2, 0.5) for s in range(2)]
    gs += [G.tree_plus_edges(n, k, 7) for n, k in ((11, 0), (17, 4), (22, 9))]
    gs += [G.grid_deleted(n, 0.1, 3) for n in (12, 20)]
    gs += [G.Graph(6, [(0, 1), (2, 3), (3, 4)], name="disconnected6"),
           G.Graph(9, [], name="empty9"),
           G.Graph(12, [(0, 11), (1, 10), (2, 9), (3, 4), (4, 5), (5, 3)], name="forest12")]
    gs.append(G.config1_graph())
    return gs


def _full(n):
    return (1 << n) - 1


@pytest.mark.parametrize("tile_bits", [0, 8, 12])
def test_dp_matches_oracle(handle, port, tile_bits):
    for g in small_graphs():
        td, parent, order, stats = handle.dp_solve(g.adj64(), g.n, tile_bits=tile_bits)
        T = port.dp_table(g)
        otd, opar = port.tree_from_table(g, T)
        assert td == otd, g.name
        assert parent.tolist() == opar.tolist(), g.name
        assert order.tolist() == port.get_elimination(g, T, _full(g.n)), g.name
        assert port.check_valid(g, td, parent, allow_forest=not g.is_connected()), g.name


def test_dp_matches_reference_golden(handle, golden):
    """Against the reference's own DynamicCPUImprov outputs (fixtures)."""
    for e in golden("ref_solvers.json"):
        g = G.Graph(e["n"], [tuple(x) for x in e["edges"]])
        td, parent, order, _ = handle.dp_solve(g.adj64(), g.n)
        assert td == e["dp_cpu_improv"]["td"], e["name"]
        assert parent.tolist() == e["dp_cpu_improv"]["parent"], e["name"]


def _permute_to_masks(raw, n, lb):
    S = np.arange(1 << n, dtype=np.int64)
    idx = np.array([_lib.table_index(n, lb, int(s)) for s in S], dtype=np.int64)
    return raw[idx]


def _connected_flags(g):
    adj = g.adjacency_masks()
    out = np.zeros(1 << g.n, dtype=bool)
    for S in range(1, 1 << g.n):
        low = S & -S
        reach, frontier = low, low
        while frontier:
            nb = 0
            f = frontier
            while f:
                b = f & -f
                nb |= adj[b.bit_length() - 1]
                f ^= b
            nb &= S & ~reach
            reach |= nb
            frontier = nb
        out[S] = reach == S
    return out


@pytest.mark.parametrize("tile_bits", [8, 10, 12])
def test_full_table_matches_oracle(handle, port, tile_bits):
    for g in [G.gnp_connected(13, 0.3, 1), G.sparse_connected(14, 2), G.grid(3, 5),
              G.Graph(12, [(0, 1), (1, 2), (5, 6), (8, 9), (9, 10), (10, 8)])]:
        handle.dp_solve(g.adj64(), g.n, tile_bits=tile_bits)
        raw, n, lb = handle.dp_read_table()
        assert n == g.n
        tab = _permute_to_masks(raw, n, lb)
        T = port.dp_table(g)
        assert np.array_equal(tab >> 1, T), g.name
        conn = _connected_flags(g)
        conn[0] = False
        assert np.array_equal((tab & 1).astype(bool)[1:], conn[1:]), g.name


def test_dp_larger_graphs_match_oracle(handle, port):
    for n, p, s in ((24, 0.2, 1), (26, 0.15, 2)):
        g = G.gnp_connected(n, p, s)
        td, parent, order, _ = handle.dp_solve(g.adj64(), g.n)
        otd, opar = port.dp_solve(g, nthreads=8)
        assert td == otd and parent.tolist() == opar.tolist(), g.name


@pytest.mark.slow
@pytest.mark.parametrize("idx", range(9))
def test_dp_config2_bit_exact(handle, port, idx):
    """The headline workload's graphs (n = 28, 30, 32 and the 5 x 6 grid):
    treedepth, parent array and GetElimination order bit-exact against the
    oracle's restatement of DynamicGPU (multi-threaded on the host)."""
    import os
    g = G.config2_graphs()[idx]
    td, parent, order, _ = handle.dp_solve(g.adj64(), g.n)
    T = port.dp_table(g, nthreads=os.cpu_count() or 8)
    otd, opar = port.tree_from_table(g, T)
    assert td == otd, g.name
    assert parent.tolist() == opar.tolist(), g.name
    assert order.tolist() == port.get_elimination(g, T, _full(g.n)), g.name


def test_dp_config2_sized_properties(handle, port):
    """n = 30: no oracle table in seconds; check size-independent facts:
    the tree is valid with height = td, the elimination order replays to the
    same tree, td lies between the edge lower bound and a heuristic."""
    g = G.config2_graphs()[1]
    td, parent, order, stats = handle.dp_solve(g.adj64(), g.n)
    assert port.check_valid(g, td, parent)
    etd, epar = port.elimination_tree(g, order)
    assert etd == td and epar.tolist() == parent.tolist()
    assert port.edge_lower_bound(g.n, g.m) <= td <= port.heuristic(g, 0)[0]
    assert stats["dp_ms"] > 0


@pytest.mark.parametrize("n", [34, 36])
def test_dp_maximum_sizes(handle, port, n):
    """The largest tables (16 and 64 GiB): the same size-independent facts on
    a sparse random graph, and closed forms at the maximum n."""
    g = G.gnp_connected(n, 0.12, 7)
    td, parent, order, _ = handle.dp_solve(g.adj64(), g.n)
    assert port.check_valid(g, td, parent)
    etd, epar = port.elimination_tree(g, order)
    assert etd == td and epar.tolist() == parent.tolist()
    assert port.edge_lower_bound(g.n, g.m) <= td <= port.heuristic(g, 0)[0]
    assert handle.dp_solve(G.path(n).adj64(), n)[0] == math.ceil(math.log2(n + 1))
    assert handle.dp_solve(G.cycle(n).adj64(), n)[0] == 1 + math.ceil(math.log2(n))
    if n == 34:
        # 8-bit tiles: 26 high vertices, the most the tile map allows (every
        # lane of the warp decode and child ranking in use)
        td8, parent8, _, _ = handle.dp_solve(g.adj64(), g.n, tile_bits=8)
        assert td8 == td and parent8.tolist() == parent.tolist()
    # treedepths above 32: the largest byte values and OR + AND sums the
    # reduction meets (K_n: td n; K_n minus a perfect matching: td n - 1)
    td, parent, _, _ = handle.dp_solve(G.complete(n).adj64(), n)
    assert td == n and port.check_valid(G.complete(n), td, parent)
    cp = G.Graph(n, [(u, v) for u in range(n) for v in range(u + 1, n) if not (u % 2 == 0 and v == u + 1)],
                 name=f"cocktail{n}")
    td, parent, _, _ = handle.dp_solve(cp.adj64(), n)
    assert td == n - 1 and port.check_valid(cp, td, parent)


def test_dp_closed_forms(handle):
    for n in (3, 7, 15, 16, 31, 32):
        assert handle.dp_solve(G.path(n).adj64(), n)[0] == math.ceil(math.log2(n + 1))
    for n in (5, 17, 30):
        assert handle.dp_solve(G.cycle(n).adj64(), n)[0] == 1 + math.ceil(math.log2(n))
    assert handle.dp_solve(G.complete(20).adj64(), 20)[0] == 20
    assert handle.dp_solve(G.star(25).adj64(), 25)[0] == 2


def test_dp_query_get_elimination(handle, port):
    g = G.gnp_connected(16, 0.3, 5)
    handle.dp_solve(g.adj64(), g.n)
    T = port.dp_table(g)
    rng = np.random.default_rng(0)
    for _ in range(20):
        mask = int(rng.integers(1, 1 << g.n))
        td, order = handle.dp_query(mask)
        assert td == T[mask]
        assert order == port.get_elimination(g, T, mask)


def test_class_layer_mirrors_reference(port):
    from math import comb
    g = G.sparse_connected(14, 1)
    d = DynamicGPU()
    d(g)
    T = port.dp_table(g)
    assert d.GetElimination(g.n, g.n, 0) == port.get_elimination(g, T, _full(g.n))
    # subset of colex rank `code` among the 5-subsets
    code = 123
    from oracle import Port
    s = Port().decode(g.n, 5, code)
    mask = sum(1 << v for v in s)
    assert d.GetElimination(g.n, 5, code) == port.get_elimination(g, T, mask)
    r = d.Result()
    assert r.treedepth == T[_full(g.n)] and r.parent[r.root] == -1


def test_dp_invalid_inputs(handle):
    adj = G.path(5).adj64()
    bad = adj.copy()
    bad[2] |= np.uint64(1 << 2)  # self loop
    with pytest.raises(InvalidArgument):
        handle.dp_solve(bad, 5)
    asym = adj.copy()
    asym[0] |= np.uint64(1 << 4)
    with pytest.raises(InvalidArgument):
        handle.dp_solve(asym, 5)
    with pytest.raises(InvalidArgument):
        handle.dp_solve(np.zeros(40, dtype=np.uint64), 37)
    with pytest.raises(InvalidArgument):
        handle.dp_solve(np.zeros(1, dtype=np.uint64), 0)
    td, parent, order, _ = handle.dp_solve(np.zeros(1, dtype=np.uint64), 1)
    assert td == 1 and parent.tolist() == [-1]
    # the handle stays usable after rejected calls
    assert handle.dp_solve(adj, 5)[0] == 3


def test_dp_wait_bound_runs_out_and_context_stays_usable(handle, port):
    """A dependency wait that can never be satisfied (the injected stall:
    the level-0 tile is never computed) must end at its bound with
    GTD_TIMEOUT, and the next solve on the same handle must be exact."""
    g = G.gnp_connected(24, 0.2, 3)
    _lib.inject_fault(_lib.FAULT_STALL, 1)
    try:
        with pytest.raises(_lib.DeadlineExceeded):
            handle.dp_solve(g.adj64(), g.n, timeout_ns=200_000_000)
    finally:
        _lib.inject_fault(_lib.FAULT_NONE, 0)
    td, parent, _, _ = handle.dp_solve(g.adj64(), g.n)
    otd, opar = port.dp_solve(g, nthreads=8)
    assert td == otd and parent.tolist() == opar.tolist()


def test_dp_device_path_reports_timeout_at_sync(handle):
    """The asynchronous entry point reports the same timeout at gtd_sync."""
    import torch
    g = G.gnp_connected(22, 0.25, 4)
    d_adj = torch.from_numpy(g.adj64().view(np.int64)).cuda()
    d_out = torch.zeros(2 + 2 * g.n, dtype=torch.int32, device="cuda")
    _lib.inject_fault(_lib.FAULT_STALL, 1)
    try:
        handle.dp_solve_device(d_adj.data_ptr(), g.n, d_out.data_ptr(), d_out[2:].data_ptr(),
                               timeout_ns=200_000_000)
        with pytest.raises(_lib.DeadlineExceeded):
            handle.sync()
    finally:
        _lib.inject_fault(_lib.FAULT_NONE, 0)
    handle.dp_solve_device(d_adj.data_ptr(), g.n, d_out.data_ptr(), d_out[2:].data_ptr())
    handle.sync()
    assert int(d_out[0].item()) == handle.dp_solve(g.adj64(), g.n)[0]
