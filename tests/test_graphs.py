"""Generators and the reference's text format."""
import numpy as np

from gisbdw_gb300 import graphs as G


def test_generators_deterministic():
    a = G.config1_graph()
    b = G.config1_graph()
    assert a.edges == b.edges and a.n == 20 and a.is_connected()
    c4a = G.config4_graphs(count=6)
    c4b = G.config4_graphs(count=6)
    assert [g.edges for g in c4a] == [g.edges for g in c4b]
    for g in c4a:
        assert 40 <= g.n <= 64 and g.is_connected()
        assert 2.5 <= 2 * g.m / g.n <= 5.5


def test_config_families_connected():
    for g in G.config3_graphs(count=30):
        assert 10 <= g.n <= 24 and g.is_connected()
    for g in G.config2_graphs():
        assert g.n in (28, 30, 32) and g.is_connected()
    for g in G.config5_graphs(count=12):
        assert 20 <= g.n <= 80 and g.is_connected()


def test_text_roundtrip():
    g = G.chordal_cycle(12)
    h = G.from_text(G.to_text(g))
    assert h.n == g.n and h.edges == g.edges


def test_text_vertex_count_grows_with_edges():
    # the reference's vecS graph grows on add_edge (main.cpp:138-143)
    h = G.from_text("graph G {\n0;\n1;\n0 -- 1;\n1 -- 4;\n}\n")
    assert h.n == 5 and h.edges == [(0, 1), (1, 4)]


def test_masks():
    g = G.grid(3, 3)
    adj = g.adj64()
    assert all(((int(adj[v]) >> v) & 1) == 0 for v in range(9))
    a2 = g.adj128()
    assert np.all(a2[0::2] == adj) and np.all(a2[1::2] == 0)
