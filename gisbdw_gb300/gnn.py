"""Learned branching order for the GPU branch and bound.

A small message-passing GNN (libgtd's gtd_gnn_* kernels: input projection,
3 mean-aggregation layers of width 64, BF16 weights, FP32 accumulation)
scores every vertex as a root of an optimal elimination tree. It is trained
on labels produced by the exact subset DP (gtd_dp_labels): for connected
induced subgraphs S of graphs with n <= 24, the set of optimal roots
R(S) = {v : td(S - v) = td(S) - 1} and td(S). The scores only ORDER the
branch and bound's candidates and seed its incumbent by greedy elimination;
they never prune, so every treedepth is still proven exactly.

Vertex features: degree, core number, eccentricity (exact BFS; "estimate" in
the sense that it is a cheap proxy of centrality), mean neighbour degree, a
pendant flag, 1/(1+degree), the graph size and a constant.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import _lib
from .graphs import Graph

IN_FEATURES = 8
HIDDEN = 64
LAYERS = 3

_vp = ctypes.c_void_p


class GnnBatch(ctypes.Structure):
    _fields_ = [("num_nodes", ctypes.c_int), ("num_graphs", ctypes.c_int), ("x", _vp),
                ("graph_start", _vp), ("nbr_start", _vp), ("nbr", _vp),
                ("root_label", _vp), ("node_mask", _vp), ("td_label", _vp)]


def _bind(L):
    if getattr(L, "_gnn_bound", False):
        return L
    L.gtd_gnn_create.argtypes = [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_uint64,
                                 ctypes.POINTER(_vp)]
    L.gtd_gnn_destroy.argtypes = [_vp]
    L.gtd_gnn_num_params.restype = ctypes.c_int64
    L.gtd_gnn_num_params.argtypes = [_vp]
    L.gtd_gnn_get_params.argtypes = [_vp, _vp]
    L.gtd_gnn_set_params.argtypes = [_vp, _vp]
    L.gtd_gnn_forward.argtypes = [_vp, ctypes.POINTER(GnnBatch), _vp, _vp]
    L.gtd_gnn_gradients.argtypes = [_vp, ctypes.POINTER(GnnBatch), ctypes.c_float, _vp, _vp]
    L.gtd_gnn_train_step.argtypes = [_vp, ctypes.POINTER(GnnBatch), ctypes.c_float, ctypes.c_float, _vp]
    L.gtd_dp_labels.argtypes = [_vp, _vp, ctypes.c_int, _vp, _vp]
    L.gtd_gnn_features.argtypes = [_vp, ctypes.c_int, _vp]
    L.gtd_gnn_pack_sizes.argtypes = [_vp, _vp, ctypes.c_int, _vp, _vp]
    L.gtd_gnn_pack.argtypes = [_vp, _vp, ctypes.c_int, _vp, _vp, _vp, _vp]
    L.gtd_gnn_make_labels.argtypes = [_vp, _vp, _vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_uint64,
                                      ctypes.c_int, _vp, _vp, _vp, _vp, _vp]
    L._gnn_bound = True
    return L


def _p(a: Optional[np.ndarray]):
    return a.ctypes.data_as(_vp) if a is not None else None


# ---------------------------------------------------------------------------
# Features and batches.
# ---------------------------------------------------------------------------

def _core_numbers(adj: List[int], n: int) -> np.ndarray:
    deg = [bin(a).count("1") for a in adj]
    core = [0] * n
    alive = (1 << n) - 1
    k = 0
    while alive:
        v = min((u for u in range(n) if alive >> u & 1), key=lambda u: deg[u])
        k = max(k, deg[v])
        core[v] = k
        alive &= ~(1 << v)
        a = adj[v] & alive
        while a:
            b = a & -a
            deg[b.bit_length() - 1] -= 1
            a ^= b
    return np.array(core, dtype=np.float32)


def _eccentricities(adj: List[int], n: int) -> np.ndarray:
    ecc = np.zeros(n, dtype=np.float32)
    for s in range(n):
        seen, frontier, d = 1 << s, 1 << s, 0
        while True:
            nb = 0
            f = frontier
            while f:
                b = f & -f
                nb |= adj[b.bit_length() - 1]
                f ^= b
            nb &= ~seen
            if not nb:
                break
            seen |= nb
            frontier = nb
            d += 1
        ecc[s] = d
    return ecc


def features(g: Graph) -> np.ndarray:
    adj = g.adjacency_masks()
    deg = np.array([bin(a).count("1") for a in adj], dtype=np.float32)
    core = _core_numbers(adj, g.n)
    ecc = _eccentricities(adj, g.n)
    nbr_deg = np.array([np.mean([deg[u] for u in range(g.n) if adj[v] >> u & 1]) if deg[v] else 0.0
                        for v in range(g.n)], dtype=np.float32)
    f = np.stack([deg / 4.0, core / 4.0, ecc / 8.0, nbr_deg / 4.0, (deg == 1).astype(np.float32),
                  1.0 / (1.0 + deg), np.full(g.n, g.n / 64.0, dtype=np.float32),
                  np.ones(g.n, dtype=np.float32)], axis=1)
    return f.astype(np.float32)


@dataclass
class Batch:
    x: np.ndarray
    graph_start: np.ndarray
    nbr_start: np.ndarray
    nbr: np.ndarray
    root_label: Optional[np.ndarray] = None
    node_mask: Optional[np.ndarray] = None
    td_label: Optional[np.ndarray] = None

    def c(self) -> GnnBatch:
        return GnnBatch(int(self.graph_start[-1]), len(self.graph_start) - 1, _p(self.x), _p(self.graph_start),
                        _p(self.nbr_start), _p(self.nbr), _p(self.root_label), _p(self.node_mask), _p(self.td_label))


def native_features(g: Graph) -> np.ndarray:
    """The library's features (gtd_gnn_features), the ones training and
    inference use; `features` above is their Python statement."""
    L = _bind(_lib.load())
    adj = g.adj128()
    x = np.zeros((g.n, IN_FEATURES), dtype=np.float32)
    st = L.gtd_gnn_features(_p(adj), g.n, _p(x))
    if st != 0:
        raise _lib._error(st, "gtd_gnn_features failed")
    return x


def _descs(ns: np.ndarray, offs: np.ndarray) -> np.ndarray:
    """gtd_graph_desc array ({int32 n, int32 offset} per graph)."""
    return np.ascontiguousarray(np.stack([np.asarray(ns), np.asarray(offs)], axis=1).astype(np.int32))


def pack(adj2: np.ndarray, ns: np.ndarray, offs: np.ndarray) -> Batch:
    """Features and CSR neighbour lists (gtd_gnn_pack) of the graphs whose
    (lo, hi) adjacency pairs start at adj2[2 * offs[i]]."""
    L = _bind(_lib.load())
    count = len(ns)
    descs = _descs(ns, offs)
    nodes, nbrs = ctypes.c_int64(), ctypes.c_int64()
    dp = _p(descs)
    st = L.gtd_gnn_pack_sizes(_p(adj2), dp, count, ctypes.byref(nodes), ctypes.byref(nbrs))
    if st != 0:
        raise _lib._error(st, "gtd_gnn_pack_sizes failed")
    b = Batch(np.zeros((nodes.value, IN_FEATURES), dtype=np.float32), np.zeros(count + 1, dtype=np.int32),
              np.zeros(nodes.value + 1, dtype=np.int32), np.zeros(max(1, nbrs.value), dtype=np.int32))
    st = L.gtd_gnn_pack(_p(adj2), dp, count, _p(b.x), _p(b.graph_start), _p(b.nbr_start), _p(b.nbr))
    if st != 0:
        raise _lib._error(st, "gtd_gnn_pack failed")
    return b


def make_batch(graphs: Sequence[Graph], roots: Optional[Sequence[np.ndarray]] = None,
               tds: Optional[Sequence[int]] = None) -> Batch:
    ns = np.array([g.n for g in graphs], dtype=np.int64)
    offs = np.concatenate([[0], np.cumsum(ns)[:-1]]).astype(np.int64)
    adj2 = np.concatenate([g.adj128() for g in graphs]).astype(np.uint64)
    b = pack(adj2, ns, offs)
    if roots is not None:
        b.root_label = np.concatenate(roots).astype(np.float32)
        b.node_mask = np.ones(int(ns.sum()), dtype=np.float32)
        b.td_label = np.array(tds, dtype=np.float32)
    return b


# ---------------------------------------------------------------------------
# The network (device) and a numpy FP64 reference of the same computation.
# ---------------------------------------------------------------------------

class GNN:
    def __init__(self, handle: _lib.Handle, seed: int = 0, in_features: int = IN_FEATURES, hidden: int = HIDDEN,
                 layers: int = LAYERS):
        self.h = handle
        self.L = _bind(handle.L)
        self.shape = (in_features, hidden, layers)
        self._g = _vp()
        handle._check(self.L.gtd_gnn_create(handle._h, in_features, hidden, layers, seed, ctypes.byref(self._g)))
        self.nparams = int(self.L.gtd_gnn_num_params(self._g))

    def close(self):
        if self._g:
            self.L.gtd_gnn_destroy(self._g)
            self._g = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self) -> np.ndarray:
        out = np.zeros(self.nparams, dtype=np.float32)
        self.h._check(self.L.gtd_gnn_get_params(self._g, _p(out)))
        return out

    def set_params(self, p: np.ndarray) -> None:
        p = np.ascontiguousarray(p, dtype=np.float32)
        self.h._check(self.L.gtd_gnn_set_params(self._g, _p(p)))

    def forward(self, b: Batch) -> Tuple[np.ndarray, np.ndarray]:
        logits = np.zeros(int(b.graph_start[-1]), dtype=np.float32)
        td = np.zeros(len(b.graph_start) - 1, dtype=np.float32)
        cb = b.c()
        self.h._check(self.L.gtd_gnn_forward(self._g, ctypes.byref(cb), _p(logits), _p(td)))
        return logits, td

    def gradients(self, b: Batch, td_weight: float = 0.05) -> Tuple[np.ndarray, float]:
        grad = np.zeros(self.nparams, dtype=np.float32)
        loss = np.zeros(1, dtype=np.float32)
        cb = b.c()
        self.h._check(self.L.gtd_gnn_gradients(self._g, ctypes.byref(cb), td_weight, _p(grad), _p(loss)))
        return grad, float(loss[0])

    def train_step(self, b: Batch, lr: float = 3e-3, td_weight: float = 0.05) -> float:
        loss = np.zeros(1, dtype=np.float32)
        cb = b.c()
        self.h._check(self.L.gtd_gnn_train_step(self._g, ctypes.byref(cb), lr, td_weight, _p(loss)))
        return float(loss[0])


def bf16_round(a: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest, ties to even), as float64."""
    u = np.ascontiguousarray(a, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def _unpack(p: np.ndarray, fin: int, H: int, L: int):
    o = 0
    W_in = p[o:o + fin * H].reshape(fin, H); o += fin * H
    b_in = p[o:o + H]; o += H
    layers = []
    for _ in range(L):
        Ws = p[o:o + H * H].reshape(H, H); o += H * H
        Wn = p[o:o + H * H].reshape(H, H); o += H * H
        bl = p[o:o + H]; o += H
        layers.append((Ws, Wn, bl))
    w_out = p[o:o + H]; o += H
    b_out = p[o]; o += 1
    w_g = p[o:o + H]; o += H
    b_g = p[o]; o += 1
    return W_in, b_in, layers, w_out, b_out, w_g, b_g


def reference_loss(params: np.ndarray, b: Batch, shape=(IN_FEATURES, HIDDEN, LAYERS), td_weight: float = 0.05,
                   want_grad: bool = True):
    """The network, loss and gradient in float64 numpy with the BF16-rounded
    weights the kernels use (the gradient is w.r.t. those weights)."""
    fin, H, L = shape
    p = bf16_round(params)
    W_in, b_in, layers, w_out, b_out, w_g, b_g = _unpack(p, fin, H, L)
    N = int(b.graph_start[-1])
    G = len(b.graph_start) - 1
    x = b.x.astype(np.float64)
    deg = np.diff(b.nbr_start).astype(np.float64)
    M = np.zeros((N, N))
    for v in range(N):
        for k in range(b.nbr_start[v], b.nbr_start[v + 1]):
            M[v, b.nbr[k]] += 1.0 / deg[v]
    gof = np.repeat(np.arange(G), np.diff(b.graph_start))
    P = np.zeros((G, N))
    for g in range(G):
        s, e = b.graph_start[g], b.graph_start[g + 1]
        P[g, s:e] = 1.0 / (e - s)
    zs, hs, as_ = [], [], []
    z = x @ W_in + b_in
    zs.append(z)
    h = np.maximum(z, 0)
    hs.append(h)
    for Ws, Wn, bl in layers:
        a = M @ h
        as_.append(a)
        z = h @ Ws + a @ Wn + bl
        zs.append(z)
        h = np.maximum(z, 0)
        hs.append(h)
    logits = h @ w_out + b_out
    pooled = P @ h
    td = pooled @ w_g + b_g
    if not want_grad:
        return logits, td
    y, m, tl = b.root_label.astype(np.float64), b.node_mask.astype(np.float64), b.td_label.astype(np.float64)
    inv = 1.0 / m.sum()
    loss = np.sum(m * (np.maximum(logits, 0) - logits * y + np.log1p(np.exp(-np.abs(logits))))) * inv
    loss += td_weight * np.mean((td - tl) ** 2)
    dl = m * (1 / (1 + np.exp(-logits)) - y) * inv
    dt = 2 * td_weight * (td - tl) / G
    g_wout = h.T @ dl
    g_bout = dl.sum()
    g_wg = pooled.T @ dt
    g_bg = dt.sum()
    dh = np.outer(dl, w_out) + P.T @ np.outer(dt, w_g)
    grads_layers = []
    for li in range(L - 1, -1, -1):
        Ws, Wn, bl = layers[li]
        dz = dh * (zs[li + 1] > 0)
        gWs = hs[li].T @ dz
        gWn = as_[li].T @ dz
        gb = dz.sum(0)
        grads_layers.append((gWs, gWn, gb))
        dh = dz @ Ws.T + M.T @ (dz @ Wn.T)
    grads_layers.reverse()
    dz = dh * (zs[0] > 0)
    gWin = x.T @ dz
    gbin = dz.sum(0)
    flat = [gWin.ravel(), gbin]
    for gWs, gWn, gb in grads_layers:
        flat += [gWs.ravel(), gWn.ravel(), gb]
    flat += [g_wout, [g_bout], g_wg, [g_bg]]
    return float(loss), np.concatenate([np.asarray(f, dtype=np.float64).ravel() for f in flat])


# ---------------------------------------------------------------------------
# Labels from the exact DP, training, and use in the branch and bound.
# ---------------------------------------------------------------------------

@dataclass
class LabelSet:
    """Samples (connected induced subgraph, optimal-root mask, td) from the
    exact DP: graph i has ns[i] vertices whose (lo, hi) adjacency pairs start
    at adj2[2 * offs[i]]."""
    adj2: np.ndarray
    ns: np.ndarray
    offs: np.ndarray
    roots: np.ndarray
    td: np.ndarray

    def __len__(self) -> int:
        return len(self.ns)

    def take(self, idx) -> "LabelSet":
        return LabelSet(self.adj2, self.ns[idx], self.offs[idx], self.roots[idx], self.td[idx])

    def split(self, frac: float) -> Tuple["LabelSet", "LabelSet"]:
        cut = int(len(self) * frac)
        return self.take(slice(0, cut)), self.take(slice(cut, len(self)))

    def packed(self) -> Batch:
        """Features and CSR lists of every sample, packed once (gtd_gnn_pack)."""
        if getattr(self, "_packed", None) is None:
            self._packed = pack(self.adj2, self.ns, self.offs)
        return self._packed

    def batch(self, idx=None) -> Batch:
        """The samples idx as one batch, gathered from the packed set."""
        P = self.packed()
        idx = np.arange(len(self)) if idx is None else np.asarray(idx)
        lens = self.ns[idx].astype(np.int64)
        starts = P.graph_start[idx].astype(np.int64)
        gs = np.zeros(len(idx) + 1, dtype=np.int64)
        np.cumsum(lens, out=gs[1:])
        total = int(gs[-1])
        shift = np.repeat(gs[:-1] - starts, lens)             # old node index -> batch index
        node = np.arange(total, dtype=np.int64) - shift       # old index of every batch node
        deg = (P.nbr_start[node + 1] - P.nbr_start[node]).astype(np.int64)
        ns_ = np.zeros(total + 1, dtype=np.int64)
        np.cumsum(deg, out=ns_[1:])
        edge = np.arange(int(ns_[-1]), dtype=np.int64) - np.repeat(ns_[:-1] - P.nbr_start[node], deg)
        nbr = P.nbr[edge] + np.repeat(shift, deg)
        b = Batch(np.ascontiguousarray(P.x[node]), gs.astype(np.int32), ns_.astype(np.int32),
                  np.ascontiguousarray(nbr.astype(np.int32)) if len(nbr) else np.zeros(1, dtype=np.int32))
        local = (np.arange(total, dtype=np.int64) - np.repeat(gs[:-1], lens)).astype(np.uint64)
        b.root_label = ((np.repeat(self.roots[idx], lens) >> local) & np.uint64(1)).astype(np.float32)
        b.node_mask = np.ones(total, dtype=np.float32)
        b.td_label = self.td[idx].astype(np.float32)
        return b

    def graph(self, i: int) -> Graph:
        n, o = int(self.ns[i]), int(self.offs[i])
        a = self.adj2[2 * o:2 * (o + n):2]
        return Graph(n, [(u, v) for u in range(n) for v in range(u + 1, n) if int(a[u]) >> v & 1])


def training_graphs(count: int, seed: int = 11) -> List[Graph]:
    """Label base graphs (n <= 24) of the config-2 and config-3 families:
    every other one a config-3 graph (G(n, p), tree plus extra edges, deleted
    grid; n in [10, 24]), the rest connected G(n, p) with n in [16, 24] and
    p in {0.1, 0.2, 0.3} like the config-2 graphs."""
    from . import graphs as G
    half = count // 2
    out = G.config3_graphs(count=count - half, seed=seed)
    for i in range(half):
        n = 16 + (i * 7 + seed) % 9
        p = (0.1, 0.2, 0.3)[i % 3]
        out.append(G.gnp_connected(n, p, 50000 + 97 * seed + i))
    return out


def family_graphs(count: int, seed: int = 13, n_min: int = 26, n_max: int = 32) -> List[Graph]:
    """Larger label base graphs of the sparse B&B families (random geometric,
    random 3-regular, deleted grids, trees plus extra edges), n in
    [n_min, n_max] — still inside the subset DP's exact range — drawn with
    seeds of their own (70000 + ...), apart from the benchmark graphs."""
    from . import graphs as G
    out = []
    for i in range(count):
        n = n_min + (i * 5 + seed) % (n_max - n_min + 1)
        s = 70000 + 31 * seed + i
        fam = i % 4
        if fam == 0:
            out.append(G.random_geometric(n, 3.0 + (i % 5) * 0.5, s))
        elif fam == 1:
            out.append(G.random_regular3(n - (n % 2), s))
        elif fam == 2:
            out.append(G.grid_deleted(n, 0.1, s))
        else:
            out.append(G.tree_plus_edges(n, (i * 3) % (n // 2 + 1), s))
    return out


def _grow_subset(g: Graph, size: int, rng: np.random.Generator) -> List[int]:
    """A connected vertex set of `size` vertices grown from a random vertex
    by random frontier vertices (fewer when its component is smaller)."""
    adj = g.adjacency_masks()
    start = int(rng.integers(g.n))
    chosen, frontier = 1 << start, adj[start] & ~(1 << start)
    while bin(chosen).count("1") < size and frontier:
        cand = [v for v in range(g.n) if frontier >> v & 1]
        v = cand[int(rng.integers(len(cand)))]
        chosen |= 1 << v
        frontier = (frontier | adj[v]) & ~chosen
    return [v for v in range(g.n) if chosen >> v & 1]


def family_label_set(handle: _lib.Handle, graphs: Sequence[Graph], per_graph: int, seed: int = 0,
                     drop: int = 12) -> "LabelSet":
    """Labels at larger sizes (n <= 36): every graph is solved exactly by the
    GPU subset DP; the graph itself and `per_graph` connected induced
    subgraphs of it (sizes uniform in [n - drop, n]) are labelled from its
    table with their treedepth and optimal-root mask (gtd_dp_labels),
    relabelled 0..k-1 in vertex order."""
    L = _bind(handle.L)
    rng = np.random.default_rng(seed)
    adj_parts, ns, roots_out, tds = [], [], [], []
    for g in graphs:
        handle.dp_solve(g.adj64(), g.n, want_order=False)
        sets = [list(range(g.n))]
        for _ in range(per_graph):
            size = int(rng.integers(max(5, g.n - drop), g.n + 1))
            sets.append(_grow_subset(g, size, rng))
        masks = np.array([sum(1 << v for v in vs) for vs in sets], dtype=np.uint64)
        td = np.zeros(len(sets), dtype=np.int32)
        roots = np.zeros(len(sets), dtype=np.uint64)
        handle._check(L.gtd_dp_labels(handle._h, _p(masks), len(sets), _p(td), _p(roots)))
        A = np.zeros((g.n, g.n), dtype=np.uint64)
        e = g.edge_array()
        if e.size:
            A[e[:, 0], e[:, 1]] = 1
            A[e[:, 1], e[:, 0]] = 1
        for vs, t, r in zip(sets, td.tolist(), roots.tolist()):
            idx = np.asarray(vs, dtype=np.int64)
            k = len(vs)
            bits = np.left_shift(np.uint64(1), np.arange(k, dtype=np.uint64))
            a2 = np.zeros(2 * k, dtype=np.uint64)
            a2[0::2] = (A[np.ix_(idx, idx)] * bits).sum(axis=1, dtype=np.uint64)  # k <= 36 < 64 bits
            rbits = (np.uint64(r) >> idx.astype(np.uint64)) & np.uint64(1)
            adj_parts.append(a2)
            ns.append(k)
            roots_out.append(int((rbits * bits).sum(dtype=np.uint64)))
            tds.append(t)
    ns = np.array(ns, dtype=np.int64)
    offs = np.concatenate([[0], np.cumsum(ns)[:-1]]).astype(np.int64)
    return LabelSet(np.concatenate(adj_parts), ns, offs, np.array(roots_out, dtype=np.uint64),
                    np.array(tds, dtype=np.int32))


def merge(a: "LabelSet", b: "LabelSet", seed: int = 0) -> "LabelSet":
    """Both label sets as one, samples shuffled (so that a later split keeps
    both kinds on each side)."""
    adj2 = np.concatenate([a.adj2, b.adj2])
    shift = len(a.adj2) // 2
    ns = np.concatenate([a.ns, b.ns])
    offs = np.concatenate([a.offs, b.offs + shift])
    roots = np.concatenate([a.roots, b.roots])
    td = np.concatenate([a.td, b.td])
    perm = np.random.default_rng(seed).permutation(len(ns))
    return LabelSet(adj2, ns[perm], offs[perm], roots[perm], td[perm])


def label_set(handle: _lib.Handle, graphs: Sequence[Graph], per_graph: int, seed: int = 0,
              min_size: int = 5) -> LabelSet:
    """Every graph (n <= 24) and `per_graph` random connected induced
    subgraphs of it, labelled from the exact DP on the GPU
    (gtd_gnn_make_labels)."""
    L = _bind(handle.L)
    ns = np.array([g.n for g in graphs], dtype=np.int64)
    offs = np.concatenate([[0], np.cumsum(ns)[:-1]]).astype(np.int64)
    adj2 = np.concatenate([g.adj128() for g in graphs]).astype(np.uint64)
    descs = _descs(ns, offs)
    cap = len(graphs) * (per_graph + 1)
    sub_adj = np.zeros(2 * 24 * cap, dtype=np.uint64)
    sub_desc = np.zeros((cap, 2), dtype=np.int32)
    roots = np.zeros(cap, dtype=np.uint64)
    td = np.zeros(cap, dtype=np.int32)
    num = ctypes.c_int()
    handle._check(L.gtd_gnn_make_labels(handle._h, _p(adj2), _p(descs), len(graphs), per_graph, min_size, seed, cap,
                                        _p(sub_adj), _p(sub_desc), _p(roots), _p(td), ctypes.byref(num)))
    k = num.value
    sns = sub_desc[:k, 0].astype(np.int64)
    soffs = sub_desc[:k, 1].astype(np.int64)
    used = int((soffs[-1] + sns[-1]) if k else 0)
    return LabelSet(sub_adj[:2 * used].copy(), sns, soffs, roots[:k].copy(), td[:k].copy())


def train(net: GNN, data: LabelSet, epochs: int = 4, batch_graphs: int = 256, lr: float = 3e-3, seed: int = 0,
          td_weight: float = 0.05) -> List[float]:
    rng = np.random.default_rng(seed)
    losses = []
    for _ in range(epochs):
        order = rng.permutation(len(data))
        for i in range(0, len(order), batch_graphs):
            losses.append(net.train_step(data.batch(order[i:i + batch_graphs]), lr=lr, td_weight=td_weight))
    return losses


def root_accuracy(net: GNN, data: LabelSet) -> dict:
    """Fraction of samples whose top-scored vertex is an optimal root, the
    same for a max-degree pick and a uniform pick, and the td estimate's mean
    absolute error."""
    hits = deg_hits = rand = 0.0
    err = []
    for i in range(0, len(data), 4096):
        idx = np.arange(i, min(len(data), i + 4096))
        b = data.batch(idx)
        logits, td = net.forward(b)
        y = b.root_label
        for k in range(len(idx)):
            s, e = b.graph_start[k], b.graph_start[k + 1]
            hits += y[s + int(np.argmax(logits[s:e]))]
            deg_hits += y[s + int(np.argmax(b.x[s:e, 0]))]
            rand += float(y[s:e].mean())
        err.append(np.abs(td - b.td_label))
    n = max(1, len(data))
    return {"top1_root": float(hits) / n, "max_degree_root": float(deg_hits) / n, "uniform_root": float(rand) / n,
            "td_mae": float(np.concatenate(err).mean()) if err else None, "samples": len(data)}


# Levels the hint sits above the rounded td estimate. Decisions above td
# succeed in a few nodes with the learned order, while those below it are
# refutations; a window that starts one level up finds the tree of td first
# and spends less on refutations below td - 1 that the proof of td - 1 makes
# unnecessary (measured: config 5, 554 proven and a median over all graphs of
# 19.0 s with offset 1 against 543 and 32.3 s with 0; config 4, 99 against 96).
HINT_OFFSET = 1


def guidance(net: GNN, graphs: Sequence[Graph], hint_offset: int = HINT_OFFSET) -> dict:
    """What the network gives the branch and bound, per graph: the branching
    order (highest score first), an incumbent (the better of the reference
    heuristic chain and a greedy elimination by score, gtd_heuristic kind 3)
    and a level hint (the rounded td estimate plus hint_offset: the decision
    level tried first). None of it prunes."""
    b = make_batch(graphs)
    logits, td_est = net.forward(b)
    scores = [logits[b.graph_start[k]:b.graph_start[k + 1]] for k in range(len(graphs))]
    orders = [np.argsort(-sc, kind="stable").astype(np.uint8) for sc in scores]
    # both incumbents of every graph in two GPU launches (gtd_heuristic_batch)
    t0, p0 = net.h.heuristic_batch(graphs, 0)
    t1, p1 = net.h.heuristic_batch(graphs, 3, scores)
    seeds = [(int(t1[k]), p1[k]) if t1[k] < t0[k] else (int(t0[k]), p0[k]) for k in range(len(graphs))]
    hints = np.clip(np.rint(td_est) + hint_offset, 1, None).astype(np.int32)
    return {"orders": orders, "seeds": seeds, "hints": hints, "td_est": td_est}


def orders_and_seeds(net: GNN, graphs: Sequence[Graph]):
    """Branching orders and incumbents only (see guidance)."""
    gd = guidance(net, graphs)
    return gd["orders"], gd["seeds"]
