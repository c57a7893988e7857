"""The bottom-up union-find heuristic DP (the reference's
BottomUpHeuristicGPU, bottom_up_heuristic_gpu_algorithm.cu:57-258): the
oracle's restatement on small known answers (CPU), and the GPU kernel
(gtd_bottom_up, through the C ABI) bit-exact against the oracle: the same
elimination order, tree and height."""
import numpy as np
import pytest

from gisbdw_gb300 import _lib
from gisbdw_gb300 import graphs as G


def test_oracle_bottom_up_known_answers(port):
    # P3: the middle vertex is added last (the root over both ends)
    td, par, order = port.bottom_up(G.path(3))
    assert (td, order, par.tolist()) == (2, [1, 0, 2], [1, -1, 1])
    # a star: the centre last; the leaves follow in ascending order
    td, par, order = port.bottom_up(G.star(6))
    assert td == 2 and order == [0, 1, 2, 3, 4, 5]
    # a clique: every forest is a path, the first vertex is added last
    td, par, order = port.bottom_up(G.complete(5))
    assert td == 5 and order == [0, 1, 2, 3, 4]
    # edgeless: height 1, the lowest vertex comes first at every level
    td, par, order = port.bottom_up(G.Graph(4, []))
    assert td == 1 and order == [0, 1, 2, 3] and par.tolist() == [-1] * 4


def test_oracle_bottom_up_is_an_upper_bound(port):
    for g in [G.gnp_connected(n, p, s) for n in (8, 12, 15) for p in (0.2, 0.4) for s in range(2)] + \
             [G.grid(3, 4), G.cycle(11), G.tree_plus_edges(14, 3, 1)]:
        td, par, order = port.bottom_up(g)
        T = port.dp_table(g)
        assert td >= int(T[(1 << g.n) - 1]), g.name
        assert sorted(order) == list(range(g.n))
        assert port.check_valid(g, td, par, allow_forest=not g.is_connected()), g.name


def _family():
    gs = [G.path(n) for n in (2, 5, 9, 16)] + [G.cycle(n) for n in (3, 8, 13)]
    gs += [G.complete(n) for n in (2, 6, 9)] + [G.star(12), G.grid(3, 5), G.grid(4, 4)]
    gs += [G.gnp_connected(n, p, s) for n in (10, 14, 18, 20) for p in (0.15, 0.3, 0.5) for s in range(2)]
    gs += [G.tree_plus_edges(n, k, 3) for n, k in ((12, 2), (17, 6), (20, 10))]
    gs += [G.grid_deleted(n, 0.1, 5) for n in (15, 19)]
    gs += [G.Graph(7, [(0, 1), (2, 3), (3, 4)], name="disconnected7"), G.Graph(1, [], name="single")]
    return gs


@pytest.mark.gpu
def test_bottom_up_gpu_matches_oracle(handle, port):
    for g in _family():
        td, par, order = handle.bottom_up(g)
        otd, opar, oorder = port.bottom_up(g)
        assert order.tolist() == oorder, g.name
        assert td == otd and par.tolist() == opar.tolist(), g.name


@pytest.mark.gpu
def test_bottom_up_gpu_config3_sample_and_large_n(handle, port):
    for g in G.config3_graphs(count=24, seed=12):
        if g.n <= 20:
            td, par, order = handle.bottom_up(g)
            otd, opar, oorder = port.bottom_up(g)
            assert order.tolist() == oorder and td == otd, g.name
    # up to the 32-vertex limit: a valid tree no lower than the exact treedepth
    for g in (G.config2_graphs()[0], G.grid(5, 6), G.sparse_connected(32, 3)):
        td, par, order = handle.bottom_up(g)
        assert sorted(order.tolist()) == list(range(g.n))
        assert port.check_valid(g, td, par), g.name
        assert td >= handle.dp_solve(g.adj64(), g.n, want_order=False)[0], g.name
        etd, epar = port.elimination_tree(g, order)
        assert etd == td and epar.tolist() == par.tolist()


@pytest.mark.gpu
def test_bottom_up_beyond_its_limit_gives_no_result(handle):
    with pytest.raises(_lib.GtdError) as e:
        handle.bottom_up(G.path(33))
    assert e.value.status == 7  # GTD_NO_RESULT, the reference's no-result sentinel
    assert handle.bottom_up(G.path(7))[0] == 3


@pytest.mark.gpu
def test_reference_chain_is_the_bnbgpu_incumbent(handle):
    """HighestDegree(Variance(BottomUp)) (main.cpp:178-186): never above any
    of its three heuristics, and equal to the best of them."""
    from gisbdw_gb300.treedepth import reference_chain
    for g in G.config3_graphs(count=12, seed=4) + [G.grid(4, 6)]:
        td, par = reference_chain(handle, g)
        parts = [handle.bottom_up(g)[0], _lib.heuristic(g, 2)[0], _lib.heuristic(g, 1)[0]]
        assert td == min(parts), g.name
