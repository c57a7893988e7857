"""Stress test of the subset DP's tile publication. A tile is published by a
warp barrier and one gpu-scope release store of its ready flag (no separate
fence); readers acquire the flag, then load the tile. Before each solve here
the table is filled with 0xFF (gtd_inject_fault, FAULT_POISON): treedepth
127, a value no solve writes. A tile read before its producer's stores were
visible would hand a child byte 0xFF to the OR / AND reduction, whose sum
then exceeds 126, so that subset's treedepth comes out >= 63 > n: the
full-table comparison with the oracle below checks every byte. Small tiles
give thousands of tiles per level, so many warps wait on tiles that are
being published at that moment."""
import numpy as np
import pytest

from gisbdw_gb300 import _lib
from gisbdw_gb300 import graphs as G

pytestmark = pytest.mark.gpu


def _natural_index(n, lb):
    """Position in the tiled table of every subset mask 0 .. 2^n - 1."""
    nh = n - lb
    tile = np.array([_lib.table_index(n, lb, h << lb) >> lb for h in range(1 << nh)], dtype=np.int64)
    S = np.arange(1 << n, dtype=np.int64)
    return (tile[S >> lb] << lb) | (S & ((1 << lb) - 1))


@pytest.mark.parametrize("tile_bits,sizes", [(8, (18, 20, 21, 22)), (11, (21, 22, 23))])
def test_poisoned_tables_match_oracle(handle, port, tile_bits, sizes):
    index = {}
    for i in range(16):
        n = sizes[i % len(sizes)]
        g = G.gnp_connected(n, (0.12, 0.2, 0.3)[i % 3], 500 + i) if i % 4 else G.grid_deleted(n, 0.1, 500 + i)
        _lib.inject_fault(_lib.FAULT_POISON, 1)
        try:
            td, parent, order, _ = handle.dp_solve(g.adj64(), g.n, tile_bits=tile_bits)
        finally:
            _lib.inject_fault(_lib.FAULT_NONE, 0)
        raw, tn, lb = handle.dp_read_table()
        assert tn == g.n and lb == tile_bits
        if (g.n, lb) not in index:
            index[(g.n, lb)] = _natural_index(g.n, lb)
        tab = raw[index[(g.n, lb)]]
        T = port.dp_table(g, nthreads=8)
        bad = np.flatnonzero((tab >> 1) != T)
        assert bad.size == 0, (g.name, bad[:8].tolist(), tab[bad[:8]].tolist())
        otd, opar = port.tree_from_table(g, T)
        assert td == otd and parent.tolist() == opar.tolist(), g.name


def test_poisoned_batches_match_oracle(handle, port):
    """The batched launch (tickets level-major across graphs), poisoned
    before the first launch and before a CUDA-graph replay of the same
    shape."""
    gs = [G.gnp_connected(n, 0.25, 700 + n) for n in range(12, 21)] * 24
    expect = {}
    for g in gs:
        if g.name not in expect:
            expect[g.name] = port.dp_solve(g)
    for call in range(2):
        _lib.inject_fault(_lib.FAULT_POISON, 1)
        try:
            td, parents, stats = handle.dp_solve_batch(gs, tile_bits=8)
        finally:
            _lib.inject_fault(_lib.FAULT_NONE, 0)
        if call:
            assert stats["graph_replayed"] == 1
        for g, t, par in zip(gs, td, parents):
            otd, opar = expect[g.name]
            assert t == otd and par.tolist() == opar.tolist(), (call, g.name)
