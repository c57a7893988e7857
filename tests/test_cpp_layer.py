"""The header-only C++ layer (include/gtd/treedepth.hpp) compiles against a
Boost-style graph and, on the GPU, reproduces the reference's calling
pattern: same treedepth and GetElimination order as the oracle."""
import os
import subprocess

import pytest

from gisbdw_gb300 import build as B
from gisbdw_gb300 import graphs as G

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "test_treedepth.cpp")


def _compile(tmp_path):
    B.build()
    exe = str(tmp_path / "test_treedepth")
    cmd = ["g++", "-std=c++17", "-O1", "-I" + os.path.join(ROOT, "include"),
           "-I" + os.path.join(ROOT, "oracle", "shim"), SRC, "-o", exe,
           "-L" + B.OUT_DIR, "-lgtd", "-Wl,-rpath," + B.OUT_DIR]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    return exe


def test_cpp_layer_compiles(tmp_path):
    assert os.path.exists(_compile(tmp_path))


@pytest.mark.gpu
def test_cpp_layer_matches_oracle(tmp_path, port):
    exe = _compile(tmp_path)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split("\n")
    for line, g in zip(out, [G.path(7), G.cycle(5)]):
        vals = [int(x) for x in line.split()]
        T = port.dp_table(g)
        td, par = port.tree_from_table(g, T)
        assert vals[0] == td
        assert vals[2:] == port.get_elimination(g, T, (1 << g.n) - 1)
        assert par[vals[1]] == -1
    assert out[2] == "invalid_argument"
    for line, want in zip(out[3:5], (3, 4)):
        tag, t, td, root = line.split()
        assert tag == "bnb" and int(t) == want and int(td) == want
    assert out[5] == "invalid_argument"
    assert out[6] == "heur 3 4"
    assert out[7] == f"oom 0 {2**32 - 1} 0"  # no result, UINT_MAX sentinel, empty order
    assert out[8] == "after 1 5"  # td(P20) = ceil(log2(21))
