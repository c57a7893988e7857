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


def make_batch(graphs: Sequence[Graph], feats: Optional[Sequence[np.ndarray]] = None,
               roots: Optional[Sequence[np.ndarray]] = None, tds: Optional[Sequence[int]] = None) -> Batch:
    xs, starts, nstart, nbr = [], [0], [0], []
    base = 0
    for i, g in enumerate(graphs):
        xs.append(feats[i] if feats is not None else features(g))
        adj = g.adjacency_masks()
        for v in range(g.n):
            us = [base + u for u in range(g.n) if adj[v] >> u & 1]
            nbr.extend(us)
            nstart.append(nstart[-1] + len(us))
        base += g.n
        starts.append(base)
    b = Batch(np.ascontiguousarray(np.concatenate(xs).astype(np.float32)), np.array(starts, dtype=np.int32),
              np.array(nstart, dtype=np.int32), np.array(nbr if nbr else [0], dtype=np.int32))
    if roots is not None:
        b.root_label = np.concatenate(roots).astype(np.float32)
        b.node_mask = np.ones(base, dtype=np.float32)
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

def _induced(g: Graph, mask: int) -> Tuple[Graph, List[int]]:
    verts = [v for v in range(g.n) if mask >> v & 1]
    idx = {v: i for i, v in enumerate(verts)}
    edges = [(idx[u], idx[v]) for u, v in g.edges if u in idx and v in idx]
    return Graph(len(verts), edges), verts


def _random_connected_subset(g: Graph, adj: List[int], size: int, rng: np.random.Generator) -> int:
    start = int(rng.integers(g.n))
    S = 1 << start
    frontier = adj[start]
    while bin(S).count("1") < size and frontier & ~S:
        cand = [u for u in range(g.n) if (frontier & ~S) >> u & 1]
        u = cand[int(rng.integers(len(cand)))]
        S |= 1 << u
        frontier |= adj[u]
    return S


def label_samples(handle: _lib.Handle, graphs: Sequence[Graph], per_graph: int, seed: int = 0,
                  min_size: int = 5):
    """(subgraph, root-label vector, td) samples: for every graph (n <= 24),
    the whole graph plus `per_graph` random connected induced subgraphs,
    labelled from the exact DP table on the GPU."""
    L = _bind(handle.L)
    rng = np.random.default_rng(seed)
    out = []
    for g in graphs:
        if g.n > 24:
            raise ValueError("label graphs must have n <= 24")
        handle.dp_solve(g.adj64(), g.n, want_order=False)
        adj = g.adjacency_masks()
        masks = {(1 << g.n) - 1}
        for _ in range(per_graph):
            size = int(rng.integers(min(min_size, g.n), g.n + 1))
            masks.add(_random_connected_subset(g, adj, size, rng))
        ms = np.array(sorted(masks), dtype=np.uint64)
        td = np.zeros(len(ms), dtype=np.int32)
        roots = np.zeros(len(ms), dtype=np.uint64)
        handle._check(L.gtd_dp_labels(handle._h, _p(ms), len(ms), _p(td), _p(roots)))
        for m, t, r in zip(ms.tolist(), td.tolist(), roots.tolist()):
            sub, verts = _induced(g, m)
            if sub.n < 2 or not sub.is_connected():
                continue
            y = np.array([(r >> v) & 1 for v in verts], dtype=np.float32)
            out.append((sub, y, t))
    return out


def train(net: GNN, samples, epochs: int = 4, batch_graphs: int = 256, lr: float = 3e-3, seed: int = 0,
          td_weight: float = 0.05) -> List[float]:
    rng = np.random.default_rng(seed)
    feats = [features(s[0]) for s in samples]
    losses = []
    for _ in range(epochs):
        order = rng.permutation(len(samples))
        for i in range(0, len(order), batch_graphs):
            idx = order[i:i + batch_graphs]
            b = make_batch([samples[j][0] for j in idx], [feats[j] for j in idx],
                           [samples[j][1] for j in idx], [samples[j][2] for j in idx])
            losses.append(net.train_step(b, lr=lr, td_weight=td_weight))
    return losses


def root_accuracy(net: GNN, samples) -> dict:
    """Fraction of samples whose top-scored vertex is an optimal root, the
    same for a max-degree pick and a uniform pick, and the td estimate's mean
    absolute error."""
    hits = deg_hits = rand = 0.0
    td_err = []
    for i in range(0, len(samples), 512):
        chunk = samples[i:i + 512]
        b = make_batch([s[0] for s in chunk])
        logits, td = net.forward(b)
        for k, (g, y, t) in enumerate(chunk):
            s, e = b.graph_start[k], b.graph_start[k + 1]
            hits += y[int(np.argmax(logits[s:e]))]
            deg_hits += y[int(np.argmax(g.degrees()))]
            rand += y.mean()
            td_err.append(abs(float(td[k]) - t))
    n = max(1, len(samples))
    return {"top1_root": float(hits) / n, "max_degree_root": float(deg_hits) / n, "uniform_root": float(rand) / n,
            "td_mae": float(np.mean(td_err)) if td_err else None, "samples": len(samples)}


def orders_and_seeds(net: GNN, graphs: Sequence[Graph]):
    """Branching order (highest score first) and incumbent for each graph:
    the better of the reference heuristic chain and a greedy elimination by
    score (gtd_heuristic kind 3)."""
    b = make_batch(graphs)
    logits, _ = net.forward(b)
    orders, seeds = [], []
    for k, g in enumerate(graphs):
        s, e = b.graph_start[k], b.graph_start[k + 1]
        sc = logits[s:e]
        orders.append(np.argsort(-sc, kind="stable").astype(np.uint8))
        t0, p0 = _lib.heuristic(g, 0)
        t1, p1 = _lib.heuristic(g, 3, sc)
        seeds.append((t1, p1) if t1 < t0 else (t0, p0))
    return orders, seeds
