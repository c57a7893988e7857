"""Batched subset DP on the GPU: one persistent launch over many graphs of
uneven size, checked graph by graph against the oracle (bit-exact td and
parent arrays), CUDA-graph replay, padding of graphs smaller than a tile,
invalid members, and the autotuner."""
import numpy as np
import pytest

from gisbdw_gb300 import InvalidArgument, _lib
from gisbdw_gb300 import graphs as G

pytestmark = pytest.mark.gpu


def mixed_batch():
    gs = G.config3_graphs(count=60, seed=9)
    gs += [G.path(3), G.cycle(5), G.complete(7), G.star(9), G.Graph(4, [(0, 1)], name="disc4"),
           G.Graph(1, [], name="single")]
    return gs


@pytest.mark.parametrize("tile_bits", [8, 10, 12])
def test_batch_matches_oracle(handle, port, tile_bits):
    gs = mixed_batch()
    td, parents, stats = handle.dp_solve_batch(gs, tile_bits=tile_bits)
    assert stats["tile_bits"] == tile_bits
    for g, t, par in zip(gs, td, parents):
        T = port.dp_table(g)
        otd, opar = port.tree_from_table(g, T)
        assert t == otd, g.name
        assert par.tolist() == opar.tolist(), g.name


def test_batch_graph_replay_same_shape_new_content(handle, port):
    a = [G.gnp_connected(14, 0.3, s) for s in range(8)]
    td_a, par_a, st_a = handle.dp_solve_batch(a, tile_bits=10)
    # same shape, new contents: the same graphs relabelled, then other graphs
    for b in ([G.relabel(g, list(reversed(range(g.n)))) for g in a],
              [G.gnp_connected(14, 0.2, 100 + s) for s in range(8)]):
        td_b, par_b, st_b = handle.dp_solve_batch(b, tile_bits=10)
        assert st_b["graph_replayed"] == 1
        for g, t, par in zip(b, td_b, par_b):
            otd, opar = port.dp_solve(g)
            assert t == otd and par.tolist() == opar.tolist()
    td_a2, par_a2, _ = handle.dp_solve_batch(a, tile_bits=10, use_cuda_graph=False)
    assert td_a2.tolist() == td_a.tolist()


def test_batch_config3_sample_matches_single_solves(handle):
    gs = G.config3_graphs(count=48, seed=3)
    td, parents, stats = handle.dp_solve_batch(gs)
    for g, t, par in zip(gs, td, parents):
        t1, p1, _, _ = handle.dp_solve(g.adj64(), g.n)
        assert t == t1 and par.tolist() == p1.tolist(), g.name
    assert stats["subsets"] == sum(1 << g.n for g in gs)


def test_batch_rejects_invalid_member(handle):
    gs = [G.path(6), G.cycle(7)]
    descs, pool = _lib.pack_batch(gs)
    pool[2] |= np.uint64(1 << 2)  # self loop in graph 0
    with pytest.raises(InvalidArgument):
        handle.dp_solve_batch(gs, packed=(descs, pool))
    td, _, _ = handle.dp_solve_batch(gs)
    assert td.tolist() == [3, 4]


def test_autotune_then_batch(handle, port):
    rates, eff = handle.dp_autotune(10, 12, with_mixed=True)
    assert rates.shape == (3, 5) and np.all(rates > 0)
    assert eff.shape == (5,) and np.all(eff > 0)
    gs = [G.gnp_connected(n, 0.3, n) for n in (10, 11, 12)]
    td, parents, stats = handle.dp_solve_batch(gs)
    assert 8 <= stats["tile_bits"] <= 12
    for g, t in zip(gs, td):
        assert t == port.dp_solve(g)[0]


def _rates_favouring(choice, n_min=2, n_max=24):
    """Synthetic autotuner rates (rows n_min..n_max, columns tile bits 8..12)
    that make the planner pick choice(n) tile bits for n vertices."""
    r = np.ones((n_max - n_min + 1, 5), dtype=np.float32)
    for n in range(n_min, n_max + 1):
        r[n - n_min, choice(n) - 8] = 1e4
    return r


@pytest.mark.parametrize("choice", [lambda n: 8 if n <= 16 else 12,
                                    lambda n: 9 + n % 3,
                                    lambda n: 11 if n >= 20 else 10])
def test_batch_tile_bits_per_n_match_oracle(port, choice):
    """Tile sizes per vertex count in one launch (the mixed-size kernel):
    every graph bit-exact against the oracle, the plan reported per n, and a
    CUDA-graph replay with new contents still exact."""
    from gisbdw_gb300 import Handle
    h = Handle(0)
    h.dp_set_rates(2, _rates_favouring(choice), mixed_eff=np.ones(5))
    gs = mixed_batch() + [G.gnp_connected(n, 0.3, 40 + n) for n in range(8, 25)]
    gs = [g for g in gs if g.n >= 2]
    td, parents, stats = h.dp_solve_batch(gs)
    want = {g.n: choice(g.n) for g in gs}
    assert stats["tile_bits_by_n"] == want
    assert stats["tile_bits"] == max(want.values())
    for g, t, par in zip(gs, td, parents):
        otd, opar = port.dp_solve(g)
        assert t == otd and par.tolist() == opar.tolist(), g.name
    other = [G.relabel(g, list(reversed(range(g.n)))) for g in gs]
    td2, par2, st2 = h.dp_solve_batch(other)
    assert st2["graph_replayed"] == 1
    for g, t, par in zip(other, td2, par2):
        otd, opar = port.dp_solve(g)
        assert t == otd and par.tolist() == opar.tolist(), g.name
    h.close()


def test_planner_never_mixes_without_a_measured_gain(port):
    """Rates favouring different sizes per n but a mixed-kernel efficiency
    that eats the gain: one size for every graph."""
    from gisbdw_gb300 import Handle
    h = Handle(0)
    r = _rates_favouring(lambda n: 10 if n <= 16 else 11)
    r[r == 1] = 9e3  # every size nearly as good
    h.dp_set_rates(2, r, mixed_eff=np.full(5, 0.5))
    gs = [G.gnp_connected(n, 0.3, 60 + n) for n in range(12, 22)]
    td, parents, stats = h.dp_solve_batch(gs)
    assert len(set(stats["tile_bits_by_n"].values())) == 1
    for g, t in zip(gs, td):
        assert t == port.dp_solve(g)[0]
    h.close()
