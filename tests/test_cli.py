"""The command line with the reference's interface (Treedepth/main.cpp):
argument handling and the .out / .gviz outputs on CPU (host heuristics), the
exact GPU algorithms against the oracle."""
import json
import os

import pytest

from gisbdw_gb300 import cli
from gisbdw_gb300 import graphs as G
from gisbdw_gb300.validate import check_tree


def _write(tmp_path, g, name):
    p = tmp_path / f"{name}.gviz"
    p.write_text(G.to_text(g))
    return str(p)


def _read_outputs(path):
    stats = json.loads(open(path).read())
    tree = G.from_text(open(path + ".gviz").read())
    return stats, tree


def test_heuristic_run_writes_reference_outputs(tmp_path):
    g = G.grid(3, 4)
    src = _write(tmp_path, g, "grid3x4")
    out = tmp_path / "out"
    out.mkdir()
    [path] = cli.run("hdVarianceHeur", [src], str(out), out=open(os.devnull, "w"))
    stats, tree = _read_outputs(path)
    assert stats["graphName"] == "grid3x4" and stats["algorithmType"] == "hdVarianceHeur"
    assert stats["vertices"] == "12" and stats["edges"] == str(g.m)
    td = int(stats["treedepth"])
    parent = [-1] * g.n
    text = open(path + ".gviz").read()  # edges are written parent--child
    for line in text.splitlines():
        if "--" in line:
            p, c = line.rstrip(" ;").split("--")
            parent[int(c)] = int(p)
    assert tree.n == g.n and check_tree(g, td, parent)
    assert parent[int(stats["root"])] == -1


def test_arguments(tmp_path):
    g = G.path(5)
    src = _write(tmp_path, g, "p5")
    with pytest.raises(SystemExit):
        cli.run("dynCPU", [src], str(tmp_path))  # a reference CPU solver: not in this library
    with pytest.raises(SystemExit):
        cli.run("nope", [src], str(tmp_path))
    with pytest.raises(SystemExit):
        cli.run("varianceHeur", [src], str(tmp_path / "missing"))
    assert cli.graph_name("/a/b/c.graph.gviz") == "c"
    assert cli.main(["-a", "highestDegreeHeur", "-o", str(tmp_path), "-i", src]) == 0


@pytest.mark.gpu
@pytest.mark.parametrize("algorithm", ["dynGPU", "bnbGPU"])
def test_exact_algorithms_match_oracle(tmp_path, port, algorithm):
    gs = [G.gnp_connected(14, 0.3, 3), G.grid(4, 4), G.cycle(11)]
    srcs = [_write(tmp_path, g, f"g{i}") for i, g in enumerate(gs)]
    out = tmp_path / "out"
    out.mkdir()
    paths = cli.run(algorithm, srcs, str(out), out=open(os.devnull, "w"))
    for g, path in zip(gs, paths):
        stats, _ = _read_outputs(path)
        assert int(stats["treedepth"]) == port.dp_solve(g)[0]


@pytest.mark.gpu
def test_bottom_up_heuristic_run_matches_oracle(tmp_path, port):
    gs = [G.gnp_connected(15, 0.3, 4), G.grid(3, 5)]
    srcs = [_write(tmp_path, g, f"b{i}") for i, g in enumerate(gs)]
    out = tmp_path / "out"
    out.mkdir()
    paths = cli.run("bottomUpHeur", srcs, str(out), out=open(os.devnull, "w"))
    for g, path in zip(gs, paths):
        stats, _ = _read_outputs(path)
        assert int(stats["treedepth"]) == port.bottom_up(g)[0]
        assert stats["algorithmType"] == "bottomUpHeur"
