"""Command line with the reference's interface (Treedepth/main.cpp:75-228):

    python -m gisbdw_gb300.cli -a dynGPU -o OUTDIR graph1.gviz [graph2.gviz ...]

For every input graph (the reference's text format: "v;" vertex lines and
"u -- v" edge lines, main.cpp:130-143) it prints the same progress lines and
writes OUTDIR/<name>_<suffix>.out (the statistics JSON of statistics.hpp:19-30,
values as strings like Boost's property-tree writer) and <that>.gviz (the
elimination tree as an undirected graphviz graph, like boost::write_graphviz).

Algorithms: dynGPU (exact subset DP, n <= 36), bnbGPU (exact branch and
bound, connected graphs, n <= 104, seeded by the reference's bnbGPU chain
HighestDegree(Variance(BottomUp))), highestDegreeHeur, varianceHeur and
hdVarianceHeur (the greedy heuristics, host) and bottomUpHeur (the bottom-up
union-find heuristic DP, GPU, n <= 32). The reference's CPU solvers (dynCPU,
dynCPUImprov, bnbCPU) and the spanning-tree heuristic are not part of this
library; naming them is an error.
"""
from __future__ import annotations

import argparse
import json
import os
import random
import sys
import time
from typing import List, Sequence

import numpy as np

from . import _lib
from .graphs import Graph, from_text

ALGORITHMS = ("dynGPU", "bnbGPU", "highestDegreeHeur", "varianceHeur", "hdVarianceHeur", "bottomUpHeur")
NOT_PROVIDED = ("dynCPU", "dynCPUImprov", "bnbCPU", "spanningTreeHeur")
_HEURISTIC_KIND = {"hdVarianceHeur": 0, "highestDegreeHeur": 1, "varianceHeur": 2}


def graph_name(path: str) -> str:
    """File name without every extension (main.cpp:148-150)."""
    name = os.path.basename(path)
    while "." in name and not name.startswith("."):
        name = name.rsplit(".", 1)[0]
    return name


def graphviz(parent: Sequence[int]) -> str:
    """The elimination tree as boost::write_graphviz writes an undirected
    graph: vertex lines, then one "p--c ;" line per tree edge."""
    out = ["graph G {"]
    out += [f"{v};" for v in range(len(parent))]
    out += [f"{int(p)}--{v} ;" for v, p in enumerate(parent) if p >= 0]
    out.append("}")
    return "\n".join(out) + "\n"


def statistics(algorithm: str, name: str, elapsed: float, td: int, root: int, g: Graph) -> str:
    """statistics.hpp:19-30 as JSON; Boost's writer stores every value as a
    string."""
    root_obj = {"algorithmType": algorithm, "graphName": name, "timeElapsed": repr(elapsed),
                "treedepth": str(td), "root": str(root), "edges": str(g.m), "vertices": str(g.n)}
    return json.dumps(root_obj, indent=4) + "\n"


def solve(algorithm: str, g: Graph, handle=None):
    """(treedepth, parent array) of g by `algorithm`."""
    if algorithm in _HEURISTIC_KIND:
        return _lib.heuristic(g, _HEURISTIC_KIND[algorithm])
    if handle is None:
        handle = _lib.Handle(0)
    if algorithm == "dynGPU":
        td, parent, _, _ = handle.dp_solve(g.adj64(), g.n, want_order=False)
        return td, parent
    if algorithm == "bottomUpHeur":
        td, parent, _ = handle.bottom_up(g)
        return td, parent
    if algorithm == "bnbGPU":
        from .treedepth import reference_chain
        res = handle.bnb_solve_batch([g], seeds=[reference_chain(handle, g)])
        if res["status"][0] != 0:
            raise _lib.DeadlineExceeded(int(res["status"][0]), "branch and bound deadline reached")
        return int(res["td"][0]), res["parents"][0]
    raise ValueError(f"unknown algorithm {algorithm}")


def run(algorithm: str, inputs: Sequence[str], output_dir: str, out=sys.stdout) -> List[str]:
    if algorithm in NOT_PROVIDED:
        raise SystemExit(f"{algorithm} is a CPU solver of the reference and is not part of this library; "
                         f"use one of {', '.join(ALGORITHMS)}")
    if algorithm not in ALGORITHMS:
        raise SystemExit("Wrong algorithm option specified.")
    if not os.path.isdir(output_dir):
        raise SystemExit(f"output directory {output_dir} does not exist")
    for path in inputs:
        if not os.path.isfile(path):
            raise SystemExit(f"input graph {path} does not exist")
    handle = None if algorithm in _HEURISTIC_KIND else _lib.Handle(0)
    written = []
    for path in inputs:
        with open(path) as f:
            name = graph_name(path)
            g = from_text(f.read(), name=name)
        print(f"Processing graph {name}", file=out)
        print(f"Algorithm: {algorithm}", file=out)
        print(f"Vertices: {g.n}", file=out)
        print(f"Edges: {g.m}", file=out)
        t0 = time.perf_counter()
        td, parent = solve(algorithm, g, handle)
        elapsed = round(time.perf_counter() - t0, 3)
        roots = [v for v in range(g.n) if parent[v] < 0]
        print(f"Elapsed time: {elapsed} seconds", file=out)
        print(f"Treedepth: {td}", file=out)
        suffix = f"{int(time.time())}{random.randrange(2**31)}"
        stats_path = os.path.join(output_dir, f"{name}_{suffix}.out")
        print(f"Output written to: {stats_path}\n", file=out)
        with open(stats_path, "w") as f:
            f.write(statistics(algorithm, name, elapsed, int(td), roots[0] if roots else 0, g))
        with open(stats_path + ".gviz", "w") as f:
            f.write(graphviz(np.asarray(parent)))
        written.append(stats_path)
    if handle is not None:
        handle.close()
    return written


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="gisbdw_gb300.cli", description=__doc__.split("\n\n")[0])
    ap.add_argument("-a", "--algorithm", required=True, help=", ".join(ALGORITHMS))
    ap.add_argument("-o", "--output", required=True, help="output directory")
    ap.add_argument("-i", "--input", action="append", default=[], help="input graph (repeatable)")
    ap.add_argument("inputs", nargs="*", help="input graphs")
    args = ap.parse_args(argv)
    inputs = args.input + args.inputs
    if not inputs:
        ap.error("no input graph")
    run(args.algorithm, inputs, args.output)
    return 0


if __name__ == "__main__":
    sys.exit(main())
