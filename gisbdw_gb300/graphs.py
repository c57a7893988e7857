"""Graphs: representation, the reference's text format, and seeded generators.

A :class:`Graph` is ``n`` vertices ``0..n-1`` plus a sorted list of undirected
edges ``(u, v)`` with ``u < v`` (no self loops, no parallel edges), the same
simple-graph semantics as the reference's
``boost::adjacency_list<mapS, vecS, undirectedS>`` (Treedepth/main.cpp:77-78).

Generators are deterministic: every random draw comes from a counter-based
splitmix64 stream (``Rng``), so the same (family, n, seed) gives the same edge
list on every machine. Connected families resample with the next attempt
number until the graph is connected, mirroring the ``++seed`` loop of the
reference's ``RandomConnectedGraph`` (Treedepth/common/utils/graph_gen.hpp:16-24).
The reference draws from Boost's ``sorted_erdos_renyi_iterator``; those graphs
are not reproducible without Boost, so parity is always computed on the same
explicit edge list fed to both solvers.
"""
from __future__ import annotations

import math
import re
from dataclasses import dataclass, field
from typing import Iterable, List, Sequence, Tuple

import numpy as np

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def _mix(z: np.ndarray) -> np.ndarray:
    with np.errstate(over="ignore"):
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


class Rng:
    """Counter-based splitmix64: draw i of stream ``seed`` is
    ``mix(seed + (i + 1) * golden)``; vectorised with numpy uint64."""

    def __init__(self, *key: int):
        s = np.uint64(0x243F6A8885A308D3)
        for k in key:
            with np.errstate(over="ignore"):
                s = _mix(np.array([s ^ np.uint64(k & 0xFFFFFFFFFFFFFFFF)], dtype=np.uint64))[0]
        self.seed = s
        self.counter = 0

    def u64(self, count: int) -> np.ndarray:
        idx = np.arange(self.counter + 1, self.counter + 1 + count, dtype=np.uint64)
        self.counter += count
        with np.errstate(over="ignore"):
            return _mix(self.seed + idx * _GOLDEN)

    def uniform(self, count: int) -> np.ndarray:
        return (self.u64(count) >> np.uint64(11)).astype(np.float64) * (2.0 ** -53)

    def randint(self, lo: int, hi: int, count: int = 1) -> np.ndarray:
        """Integers uniform in [lo, hi] (inclusive)."""
        span = np.uint64(hi - lo + 1)
        return (self.u64(count) % span).astype(np.int64) + lo

    def permutation(self, n: int) -> np.ndarray:
        return np.argsort(self.u64(n), kind="stable")


@dataclass
class Graph:
    n: int
    edges: List[Tuple[int, int]] = field(default_factory=list)
    name: str = ""

    def __post_init__(self):
        es = set()
        for u, v in self.edges:
            u, v = int(u), int(v)
            if u == v:
                raise ValueError(f"self loop at vertex {u}")
            if not (0 <= u < self.n and 0 <= v < self.n):
                raise ValueError(f"edge ({u}, {v}) out of range for n={self.n}")
            es.add((min(u, v), max(u, v)))
        self.edges = sorted(es)

    @property
    def m(self) -> int:
        return len(self.edges)

    def adjacency_masks(self) -> List[int]:
        adj = [0] * self.n
        for u, v in self.edges:
            adj[u] |= 1 << v
            adj[v] |= 1 << u
        return adj

    def adj64(self) -> np.ndarray:
        """Adjacency as uint64 masks (n <= 64)."""
        if self.n > 64:
            raise ValueError("adj64 needs n <= 64")
        return np.array(self.adjacency_masks(), dtype=np.uint64)

    def adj128(self) -> np.ndarray:
        """Adjacency as 2 x uint64 words per vertex (lo, hi), n <= 128."""
        if self.n > 128:
            raise ValueError("adj128 needs n <= 128")
        out = np.zeros(2 * self.n, dtype=np.uint64)
        for v, a in enumerate(self.adjacency_masks()):
            out[2 * v] = a & 0xFFFFFFFFFFFFFFFF
            out[2 * v + 1] = a >> 64
        return out

    def edge_array(self) -> np.ndarray:
        return np.array(self.edges, dtype=np.int32).reshape(-1, 2)

    def is_connected(self) -> bool:
        return len(components(self)) <= 1

    def degrees(self) -> np.ndarray:
        d = np.zeros(self.n, dtype=np.int64)
        for u, v in self.edges:
            d[u] += 1
            d[v] += 1
        return d


def components(g: Graph) -> List[int]:
    """Connected components as bit masks, ordered by smallest vertex."""
    adj = g.adjacency_masks()
    rest = (1 << g.n) - 1
    out = []
    while rest:
        low = rest & -rest
        reach, frontier = low, low
        while frontier:
            nb = 0
            f = frontier
            while f:
                b = f & -f
                nb |= adj[b.bit_length() - 1]
                f ^= b
            nb &= rest & ~reach
            reach |= nb
            frontier = nb
        out.append(reach)
        rest &= ~reach
    return out


# ---------------------------------------------------------------------------
# The reference's text format (Treedepth/main.cpp:130-143): vertex lines
# "<id>;" and edge lines "<u> -- <v>", e.g. a DOT "graph G { 0; 1; 0 -- 1; }".
# ---------------------------------------------------------------------------

_VERTEX_RE = re.compile(r"^\s*(\d+)\s*;\s*$", re.M)
_EDGE_RE = re.compile(r"(\d+)\s*--\s*(\d+)")


def to_text(g: Graph) -> str:
    lines = ["graph G {"]
    lines += [f"{v};" for v in range(g.n)]
    lines += [f"{u} -- {v};" for u, v in g.edges]
    lines.append("}")
    return "\n".join(lines) + "\n"


def from_text(text: str, name: str = "") -> Graph:
    """Parses the reference's graph text. The vertex count is the larger of
    the number of vertex lines and 1 + the largest id on an edge line, which
    is what the reference's vecS graph ends up with after add_edge grows it
    (main.cpp:138-143)."""
    nv = len(_VERTEX_RE.findall(text))
    edges = [(int(a), int(b)) for a, b in _EDGE_RE.findall(text)]
    n = max([nv] + [max(u, v) + 1 for u, v in edges])
    return Graph(n, edges, name=name)


# ---------------------------------------------------------------------------
# Families. The closed-form ones follow graph_gen.hpp:25-82.
# ---------------------------------------------------------------------------

def path(n: int) -> Graph:
    return Graph(n, [(i, i + 1) for i in range(n - 1)], name=f"path{n}")


def cycle(n: int) -> Graph:
    return Graph(n, [(i, i + 1) for i in range(n - 1)] + [(0, n - 1)], name=f"cycle{n}")


def complete(n: int) -> Graph:
    return Graph(n, [(j, i) for i in range(n) for j in range(i)], name=f"complete{n}")


def star(n: int) -> Graph:
    return Graph(n, [(0, i) for i in range(1, n)], name=f"star{n}")


def chordal_cycle(n: int) -> Graph:
    """Cycle plus chords (0, n/3) and (0, 2n/3) (graph_gen.hpp:77-82)."""
    g = cycle(n)
    return Graph(n, g.edges + [(0, n // 3), (0, 2 * n // 3)], name=f"chordal_cycle{n}")


def grid(rows: int, cols: int) -> Graph:
    e = []
    for r in range(rows):
        for c in range(cols):
            v = r * cols + c
            if c + 1 < cols:
                e.append((v, v + 1))
            if r + 1 < rows:
                e.append((v, v + cols))
    return Graph(rows * cols, e, name=f"grid{rows}x{cols}")


MAX_ATTEMPTS = 100000


def gnp(n: int, p: float, seed: int, attempt: int = 0) -> Graph:
    """Erdos-Renyi G(n, p): pair (u, v), u < v, in lexicographic order, kept
    when its uniform draw is below p."""
    rng = Rng(1, n, int(round(p * 1e9)), seed, attempt)
    iu, iv = np.triu_indices(n, 1)
    keep = rng.uniform(len(iu)) < p
    return Graph(n, list(zip(iu[keep].tolist(), iv[keep].tolist())), name=f"gnp{n}_{p}_{seed}")


def gnp_connected(n: int, p: float, seed: int) -> Graph:
    """G(n, p) resampled (attempt 0, 1, ...) until connected."""
    for attempt in range(MAX_ATTEMPTS):
        g = gnp(n, p, seed, attempt)
        if g.is_connected():
            g.name = f"gnp{n}_p{p:g}_s{seed}"
            return g
    raise RuntimeError(f"G({n},{p}) seed {seed}: no connected sample")


def sparse_connected(n: int, seed: int) -> Graph:
    """RandomSparseConnectedGraph: p = ln(n)/n (graph_gen.hpp:25-27)."""
    return gnp_connected(n, math.log(n) / n, seed)


def _prufer_tree(n: int, rng: Rng) -> List[Tuple[int, int]]:
    if n == 1:
        return []
    if n == 2:
        return [(0, 1)]
    seq = rng.randint(0, n - 1, n - 2).tolist()
    degree = [1] * n
    for x in seq:
        degree[x] += 1
    edges = []
    import heapq
    leaves = [v for v in range(n) if degree[v] == 1]
    heapq.heapify(leaves)
    for x in seq:
        leaf = heapq.heappop(leaves)
        edges.append((leaf, x))
        degree[x] -= 1
        if degree[x] == 1:
            heapq.heappush(leaves, x)
    u = heapq.heappop(leaves)
    v = heapq.heappop(leaves)
    edges.append((u, v))
    return edges


def tree_plus_edges(n: int, k: int, seed: int) -> Graph:
    """Random labelled tree (Pruefer sequence) plus k distinct extra edges."""
    rng = Rng(2, n, k, seed)
    edges = set((min(a, b), max(a, b)) for a, b in _prufer_tree(n, rng))
    target = min(len(edges) + k, n * (n - 1) // 2)
    while len(edges) < target:
        a, b = rng.randint(0, n - 1, 2).tolist()
        if a != b:
            edges.add((min(a, b), max(a, b)))
    return Graph(n, sorted(edges), name=f"tree{n}_k{k}_s{seed}")


def grid_deleted(n: int, rate: float, seed: int) -> Graph:
    """The first n vertices (row-major) of a rows x cols grid with
    rows = floor(sqrt(n)), each edge deleted with probability ``rate``;
    resampled until connected."""
    rows = max(1, int(math.isqrt(n)))
    cols = -(-n // rows)
    base = [(u, v) for u, v in grid(rows, cols).edges if u < n and v < n]
    for attempt in range(MAX_ATTEMPTS):
        rng = Rng(3, n, int(rate * 1e6), seed, attempt)
        keep = rng.uniform(len(base)) >= rate
        g = Graph(n, [e for e, k in zip(base, keep) if k], name=f"grid{n}_d{rate:g}_s{seed}")
        if g.is_connected():
            return g
    raise RuntimeError("grid_deleted: no connected sample")


def random_geometric(n: int, mean_degree: float, seed: int) -> Graph:
    """Random geometric graph in the unit square, radius
    sqrt(d / (pi (n - 1))) for expected mean degree d (boundary effects make
    it a little lower). Resampled until connected; after 64 failed attempts
    the components of the last sample are joined by their closest pairs."""
    r = math.sqrt(mean_degree / (math.pi * (n - 1)))
    for attempt in range(64):
        rng = Rng(4, n, int(mean_degree * 1e6), seed, attempt)
        xy = rng.uniform(2 * n).reshape(n, 2)
        d2 = ((xy[:, None, :] - xy[None, :, :]) ** 2).sum(-1)
        iu, iv = np.triu_indices(n, 1)
        keep = d2[iu, iv] <= r * r
        g = Graph(n, list(zip(iu[keep].tolist(), iv[keep].tolist())))
        if g.is_connected():
            g.name = f"rgg{n}_d{mean_degree:.2f}_s{seed}"
            return g
    edges = list(g.edges)
    comps = components(g)
    while len(comps) > 1:
        a = [v for v in range(n) if comps[0] >> v & 1]
        b = [v for v in range(n) if not (comps[0] >> v & 1)]
        sub = d2[np.ix_(a, b)]
        i, j = np.unravel_index(np.argmin(sub), sub.shape)
        edges.append((a[i], b[j]))
        g = Graph(n, edges)
        comps = components(g)
    g.name = f"rgg{n}_d{mean_degree:.2f}_s{seed}_joined"
    return g


def random_regular3(n: int, seed: int) -> Graph:
    """Random 3-regular simple connected graph (configuration model with
    rejection). n must be even."""
    if n % 2:
        raise ValueError("3-regular graphs need an even n")
    for attempt in range(MAX_ATTEMPTS):
        rng = Rng(5, n, seed, attempt)
        stubs = np.repeat(np.arange(n), 3)[rng.permutation(3 * n)]
        pairs = stubs.reshape(-1, 2)
        if np.any(pairs[:, 0] == pairs[:, 1]):
            continue
        es = set((min(a, b), max(a, b)) for a, b in pairs.tolist())
        if len(es) != len(pairs):
            continue
        g = Graph(n, sorted(es), name=f"reg3_{n}_s{seed}")
        if g.is_connected():
            return g
    raise RuntimeError("random_regular3: no sample")


def relabel(g: Graph, perm: Sequence[int]) -> Graph:
    """Vertex v becomes perm[v]."""
    return Graph(g.n, [(perm[u], perm[v]) for u, v in g.edges], name=g.name)


# ---------------------------------------------------------------------------
# Workload configurations (the five benchmark configurations of this project).
# ---------------------------------------------------------------------------

def config1_graph() -> Graph:
    """One connected G(n=20, p=0.25), seed 0."""
    g = gnp_connected(20, 0.25, 0)
    g.name = "C1_gnp20_p0.25_s0"
    return g


def config2_graphs() -> List[Graph]:
    """Single-graph DP at scale: 8 connected G(n, p), seeds 1..8, with
    n cycling over 28, 30, 32 and p over 0.1, 0.2, 0.3 (seed s takes
    n = (28, 30, 32)[(s-1) % 3], p = (0.1, 0.2, 0.3)[((s-1) // 3) % 3]),
    plus the 5 x 6 grid (n = 30)."""
    out = []
    for s in range(1, 9):
        n = (28, 30, 32)[(s - 1) % 3]
        p = (0.1, 0.2, 0.3)[((s - 1) // 3) % 3]
        g = gnp_connected(n, p, s)
        g.name = f"C2_gnp{n}_p{p:g}_s{s}"
        out.append(g)
    g = grid(5, 6)
    g.name = "C2_grid5x6"
    out.append(g)
    return out


def config3_graphs(count: int = 4096, seed: int = 3) -> List[Graph]:
    """Batched uneven DP: n uniform in [10, 24], three families in turn:
    G(n, p) with p uniform in [0.1, 0.5]; random tree plus k uniform in
    [0, n] extra edges; grid with 10% edge deletions."""
    rng = Rng(100, seed)
    ns = rng.randint(10, 24, count).tolist()
    out = []
    for i, n in enumerate(ns):
        fam = i % 3
        if fam == 0:
            p = 0.1 + 0.4 * float(rng.uniform(1)[0])
            g = gnp_connected(n, round(p, 6), 1000 + i)
        elif fam == 1:
            k = int(rng.randint(0, n, 1)[0])
            g = tree_plus_edges(n, k, 1000 + i)
        else:
            g = grid_deleted(n, 0.1, 1000 + i)
        out.append(g)
    return out


def config4_graphs(count: int = 256, seed: int = 4) -> List[Graph]:
    """Sparse B&B family: n uniform in [40, 64], mean degree 3-5: random
    geometric graphs (target degree uniform in [3, 5]), random 3-regular
    graphs (n rounded down to even), grids with 10% edge deletions."""
    rng = Rng(200, seed)
    ns = rng.randint(40, 64, count).tolist()
    out = []
    for i, n in enumerate(ns):
        fam = i % 3
        if fam == 0:
            d = 3.0 + 2.0 * float(rng.uniform(1)[0])
            g = random_geometric(n, d, 2000 + i)
        elif fam == 1:
            g = random_regular3(n - (n % 2), 2000 + i)
        else:
            g = grid_deleted(n, 0.1, 2000 + i)
        out.append(g)
    return out


def config5_graphs(count: int = 1024, seed: int = 5) -> List[Graph]:
    """Mixed stream: n uniform in [20, 80] over the sparse families (random
    geometric, 3-regular, deleted grids) and sparse trees plus extra edges."""
    rng = Rng(300, seed)
    ns = rng.randint(20, 80, count).tolist()
    out = []
    for i, n in enumerate(ns):
        fam = i % 4
        if fam == 0:
            d = 3.0 + 2.0 * float(rng.uniform(1)[0])
            g = random_geometric(n, d, 3000 + i)
        elif fam == 1:
            g = random_regular3(n - (n % 2), 3000 + i)
        elif fam == 2:
            g = grid_deleted(n, 0.1, 3000 + i)
        else:
            k = int(rng.randint(0, n // 2, 1)[0])
            g = tree_plus_edges(n, k, 3000 + i)
        out.append(g)
    return out
