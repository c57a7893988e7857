"""Generates the golden fixtures in this folder from the REFERENCE's own CPU
solvers, compiled unchanged from the reference sources against the Boost-API
shim (oracle/Makefile target ``ref`` -> oracle/_ref/libgtdref.so).

Run where the reference sources exist:
    make -C oracle ref && python tests/golden/make_golden.py

Outputs (JSON, committed):
  ref_solvers.json      per graph: edges and the reference's DynamicCPU,
                        DynamicCPUImprov, BranchAndBound(EdgeLowerBound,
                        HighestDegree(Variance)) results and its heuristics
  elimination_tree.json the EliminationTree known answers of the reference's
                        unit tests (elimination_tree_unittest.cpp:29-270),
                        replayed through the reference class
  set_encoder.json      NChooseK / Encode / Decode vectors for n < 16
                        (set_encoder_unittest.cpp:16-116 range)
  edge_lower_bound.json for every n <= 128 the smallest e at which
                        EdgeLowerBound::Get reaches each value d
"""
from __future__ import annotations

import itertools
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from oracle import Ref  # noqa: E402
from gisbdw_gb300 import graphs as G  # noqa: E402


def res(t):
    rc, td, root, parent = t
    return {"rc": rc, "td": td, "root": root, "parent": [int(x) for x in parent]}


def solver_graphs():
    gs = [G.path(n) for n in range(2, 22)]
    gs += [G.cycle(n) for n in range(3, 17)]
    gs += [G.chordal_cycle(n) for n in range(10, 16)]
    gs += [G.complete(n) for n in range(2, 10)]
    gs += [G.star(n) for n in range(2, 12)]
    gs += [G.grid(r, c) for r, c in ((2, 3), (3, 3), (3, 4), (4, 4))]
    gs += [G.sparse_connected(n, s) for n in range(8, 19) for s in range(3)]
    gs += [G.gnp_connected(n, p, s) for n in (10, 12) for p in (0.2, 0.4, 0.6) for s in range(2)]
    gs += [G.tree_plus_edges(n, k, s) for n in (10, 14, 18) for k in (0, 3, 6) for s in range(2)]
    gs += [G.grid_deleted(n, 0.1, s) for n in (10, 14, 18) for s in range(2)]
    gs.append(G.config1_graph())
    return gs


def main():
    R = Ref()
    out = []
    for g in solver_graphs():
        entry = {"name": g.name, "n": g.n, "edges": [list(e) for e in g.edges]}
        entry["dp_cpu_improv"] = res(R.dp_cpu_improv(g))
        if g.n <= 20:
            entry["dp_cpu"] = res(R.dp_cpu(g))
        dense = g.m > 2.2 * g.n
        if g.n <= 18 and not (dense and g.n > 10):
            entry["bnb_cpu"] = res(R.bnb_cpu(g, 0, 0))
        entry["heuristics"] = {str(k): res(R.heuristic(g, k)) for k in (0, 2, 3)}
        out.append(entry)
        print(g.name, entry["dp_cpu_improv"]["td"], flush=True)
    with open(os.path.join(HERE, "ref_solvers.json"), "w") as f:
        json.dump(out, f, separators=(",", ":"))

    # EliminationTree known answers (elimination_tree_unittest.cpp:29-270):
    # graph, elimination order, expected depth, expected tree edges.
    cases = [
        ("C5", G.cycle(5), [0, 3, 2, 4, 1], 4, [(0, 3), (2, 3), (1, 2), (3, 4)]),
        ("TwoCycles", G.Graph(7, [(0, 1), (1, 2), (2, 0), (2, 3), (3, 6), (6, 5), (5, 4), (4, 6)]),
         [3, 6, 4, 5, 2, 1, 0], 4, [(2, 3), (3, 6), (4, 6), (4, 5), (1, 2), (1, 0)]),
        ("PathSimple", G.path(4), [3, 2, 1, 0], 4, [(0, 1), (1, 2), (2, 3)]),
        ("PathOptimal", G.path(7), [3, 1, 5, 0, 2, 4, 6], 3, [(1, 3), (3, 5), (0, 1), (1, 2), (4, 5), (5, 6)]),
    ]
    et = []
    for name, g, order, depth, tree in cases:
        r = res(R.elimination_tree(g, order))
        et.append({"name": name, "n": g.n, "edges": [list(e) for e in g.edges], "order": order,
                   "expected_depth": depth, "expected_tree_edges": [list(e) for e in tree],
                   "reference": r})
    # P3 of branch_and_bound_unittest.cpp:36-45: td 2, root 1.
    et.append({"name": "P3_bnb", "n": 3, "edges": [[0, 1], [1, 2]], "expected_depth": 2, "expected_root": 1,
               "reference": res(R.bnb_cpu(G.path(3), 1, 2))})
    with open(os.path.join(HERE, "elimination_tree.json"), "w") as f:
        json.dump(et, f, indent=1)

    enc = {"nchoosek": [[R.nchoosek(n, k) for k in range(0, n + 1)] for n in range(0, 34)], "sets": []}
    for n in range(1, 16):
        for k in range(0, n + 1):
            for code in range(0, R.nchoosek(n, k), max(1, R.nchoosek(n, k) // 7)):
                s = R.decode(n, k, code)
                enc["sets"].append([n, k, code, s, R.encode(s)])
    with open(os.path.join(HERE, "set_encoder.json"), "w") as f:
        json.dump(enc, f, separators=(",", ":"))

    lb = {}
    for n in range(1, 129):
        emax = n * (n - 1) // 2
        steps = []
        prev = None
        for e in range(0, emax + 1):
            d = R.edge_lower_bound(n, e)
            if d != prev:
                steps.append([e, d])
                prev = d
        lb[str(n)] = steps
    with open(os.path.join(HERE, "edge_lower_bound.json"), "w") as f:
        json.dump(lb, f, separators=(",", ":"))


if __name__ == "__main__":
    main()
