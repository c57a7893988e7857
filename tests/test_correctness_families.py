"""The reference's cross-solver correctness harness (CTF.CorrectnessTest,
Treedepth/test/correctness/correctness_unittest.cpp:33-76) over its own
families (:78-125: paths 7-21, chordal cycles 10-15, cycles 7-16, sparse
random connected graphs n = 8-18 with p = ln n / n; fixed seeds here, the
reference draws time(0)): every GPU solver of this library — the subset DP,
the batched DP, the branch and bound seeded by the reference's bnbGPU chain
HighestDegree(Variance(BottomUp)) — gives the treedepth of the oracle's
DynamicCPUImprov restatement, and every tree is valid (CheckIfTdDecompIsValid,
common/utils/utils.hpp:50-86)."""
import numpy as np
import pytest

from gisbdw_gb300 import graphs as G
from gisbdw_gb300.treedepth import reference_chain

pytestmark = pytest.mark.gpu


def families():
    gs = [G.path(n) for n in (7, 8, 10, 12, 14, 16, 21)]
    gs += [G.chordal_cycle(n) for n in range(10, 16)]
    gs += [G.cycle(n) for n in range(7, 17)]
    gs += [G.sparse_connected(n, s) for s in (0, 1, 2) for n in (8, 9, 10, 14, 15, 16, 17, 18)]
    return gs


def test_every_solver_agrees_on_the_reference_families(handle, port):
    gs = families()
    want = [port.dp_improv(g)[0] for g in gs]
    btd, bpar, _ = handle.dp_solve_batch(gs)
    seeds = [reference_chain(handle, g) for g in gs]
    res = handle.bnb_solve_batch(gs, seeds=seeds, deadline_ns=60 * 10**9)
    assert np.all(res["status"] == 0)
    for i, g in enumerate(gs):
        td, par, _, _ = handle.dp_solve(g.adj64(), g.n)
        assert td == want[i] == int(btd[i]) == int(res["td"][i]), g.name
        for t, p in ((td, par), (int(btd[i]), bpar[i]), (int(res["td"][i]), res["parents"][i]),
                     (seeds[i][0], seeds[i][1])):
            assert port.check_valid(g, t, p), g.name
        assert seeds[i][0] >= want[i], g.name  # a heuristic never beats the exact value


@pytest.mark.slow
def test_batched_dp_at_headline_sizes_matches_single_solves(handle):
    """One batch holding graphs of n = 28, 30 and 32 (4 GiB table) next to
    small ones: every graph's td and parent array equal the single-graph
    solver's."""
    gs = G.config2_graphs()[:3] + [G.grid(5, 6), G.cycle(12), G.sparse_connected(20, 4)]
    td, parents, stats = handle.dp_solve_batch(gs)
    assert stats["subsets"] == sum(1 << g.n for g in gs)
    for g, t, par in zip(gs, td, parents):
        st, sp, _, _ = handle.dp_solve(g.adj64(), g.n, want_order=False)
        assert int(t) == st and par.tolist() == sp.tolist(), g.name
