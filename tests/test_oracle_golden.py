"""The oracle (oracle/gtd_oracle.c) against the reference's own outputs.

The fixtures were produced by the reference's CPU solvers compiled unchanged
(tests/golden/make_golden.py); these tests pin the C restatement to them."""
import numpy as np
import pytest

from gisbdw_gb300 import graphs as G


def _graph(e):
    return G.Graph(e["n"], [tuple(x) for x in e["edges"]], name=e["name"])


def test_dp_improv_matches_reference(port, golden):
    for e in golden("ref_solvers.json"):
        g = _graph(e)
        td, par = port.dp_improv(g)
        ref = e["dp_cpu_improv"]
        assert td == ref["td"], e["name"]
        assert par.tolist() == ref["parent"], e["name"]


def test_dp_table_tree_matches_reference(port, golden):
    for e in golden("ref_solvers.json"):
        g = _graph(e)
        td, par = port.dp_solve(g, nthreads=2)
        assert td == e["dp_cpu_improv"]["td"], e["name"]
        assert par.tolist() == e["dp_cpu_improv"]["parent"], e["name"]
        if "dp_cpu" in e:
            assert par.tolist() == e["dp_cpu"]["parent"], e["name"]
        assert port.check_valid(g, td, par)


def test_bnb_matches_reference(port, golden):
    n = 0
    for e in golden("ref_solvers.json"):
        if "bnb_cpu" not in e:
            continue
        g = _graph(e)
        st, td, par, nodes = port.bnb(g, 0, 0)
        assert st == 0
        assert td == e["bnb_cpu"]["td"], e["name"]
        assert par.tolist() == e["bnb_cpu"]["parent"], e["name"]
        n += 1
    assert n > 50


def test_heuristics_match_reference(port, golden):
    for e in golden("ref_solvers.json"):
        g = _graph(e)
        for k, ref in e["heuristics"].items():
            td, par = port.heuristic(g, int(k))
            assert td == ref["td"], (e["name"], k)
            assert par.tolist() == ref["parent"], (e["name"], k)


def test_elimination_tree_known_answers(port, golden):
    for e in golden("elimination_tree.json"):
        g = _graph(e)
        if "order" in e:
            td, par = port.elimination_tree(g, e["order"])
            assert td == e["expected_depth"] == e["reference"]["td"]
            assert par.tolist() == e["reference"]["parent"]
            tree = {tuple(sorted((int(p), v))) for v, p in enumerate(par) if p >= 0}
            assert tree == {tuple(sorted(x)) for x in e["expected_tree_edges"]}
            assert par[e["order"][0]] == -1
        else:  # P3 B&B case
            st, td, par, _ = port.bnb(g, 1, 2)
            assert td == e["expected_depth"] == e["reference"]["td"]
            assert int(np.flatnonzero(par == -1)[0]) == e["expected_root"]


def test_set_encoder(port, golden):
    enc = golden("set_encoder.json")
    for n, row in enumerate(enc["nchoosek"]):
        for k, v in enumerate(row):
            assert port.nchoosek(n, k) == v
    for n, k, code, s, code2 in enc["sets"]:
        assert port.decode(n, k, code) == s
        assert port.encode(s) == code == code2


def test_edge_lower_bound_exhaustive(port, golden):
    """Integer form vs the reference's double formula, every n <= 128."""
    steps = golden("edge_lower_bound.json")
    for n_s, st in steps.items():
        n = int(n_s)
        bounds = [e for e, _ in st] + [n * (n - 1) // 2 + 1]
        for i, (e0, d) in enumerate(st):
            for e in {e0, bounds[i + 1] - 1}:
                assert port.edge_lower_bound(n, e) == d, (n, e)
        # the reference's value is also monotone in e and ends at n
        assert st[-1][1] == n if n > 1 else True


def test_validator_rejects_bad_trees(port):
    g = G.cycle(6)
    td, par = port.dp_solve(g)
    assert port.check_valid(g, td, par)
    assert not port.check_valid(g, td + 1, par)
    bad = par.copy()
    root = int(np.flatnonzero(bad == -1)[0])
    leaf = [v for v in range(6) if v not in set(bad.tolist())][0]
    bad[root] = leaf  # cycle
    assert not port.check_valid(g, td, bad)
    flat = np.full(6, 0, dtype=np.int32)
    flat[0] = -1
    assert not port.check_valid(g, 2, flat)  # star tree misses cycle edges


def test_dp_closed_forms(port):
    import math
    for n in range(1, 20):
        assert port.dp_solve(G.path(n))[0] == math.ceil(math.log2(n + 1))
        assert port.dp_solve(G.complete(min(n, 12)))[0] == min(n, 12)
    for n in range(3, 18):
        assert port.dp_solve(G.cycle(n))[0] == 1 + math.ceil(math.log2(n))
    for n in range(2, 15):
        assert port.dp_solve(G.star(n))[0] == 2
