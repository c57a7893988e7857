"""Reference-shaped solver classes over the gtd C ABI.

Mirrors the reference's algorithm interface (Treedepth/src): a solver object
is called on a graph and hands back the treedepth and an elimination tree.

* :class:`DynamicGPU` — ``td::DynamicGPU`` (dynamic_gpu.hpp:17-37):
  ``solver(g)`` runs the subset DP; ``GetElimination(nverts, subset_size,
  subset_code)`` returns the elimination order of the subset with that colex
  rank (dynamic_gpu.hpp:48-64); :meth:`Result` gives the
  ``EliminationTree::Result``-shaped output (elimination_tree.hpp:26-30).

Errors map to the reference's exception types: invalid input raises
``InvalidArgument`` (a ``ValueError``, the reference's
``std::invalid_argument``).
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import _lib
from .graphs import Graph


# Treedepth of a Result when a solve gave none (the reference's UINT_MAX).
NO_RESULT = 2**32 - 1


@dataclass
class Result:
    """``EliminationTree::Result`` (elimination_tree.hpp:26-30): the tree as
    a parent array (``parent[root] == -1``), its height ``treedepth`` and
    ``root``. ``td_decomp`` lists the tree edges (parent, child)."""

    treedepth: int
    root: int
    parent: np.ndarray

    @property
    def td_decomp(self) -> List[Tuple[int, int]]:
        return [(int(p), v) for v, p in enumerate(self.parent) if p >= 0]


def _masks(g: Graph) -> np.ndarray:
    return g.adj64()


def _decode(nverts: int, k: int, code: int) -> int:
    """Colex unrank (set_encoder.hpp:61-73) to a bit mask."""
    from math import comb
    mask = 0
    while k > 0:
        nverts -= 1
        c = comb(nverts, k)
        if code >= c:
            mask |= 1 << nverts
            code -= c
            k -= 1
    return mask


class DynamicGPU:
    """Exact treedepth by the GB300 subset DP (``td::DynamicGPU``)."""

    def __init__(self, device: int = 0, tile_bits: int = 0, handle: Optional[_lib.Handle] = None):
        self._h = handle or _lib.Handle(device)
        self._tile_bits = tile_bits
        self._n = 0
        self._td = None
        self._parent = None
        self._order = None
        self.stats: dict = {}

    def __call__(self, g: Graph) -> None:
        """Solves g. Running out of device memory is swallowed as the
        reference's DP functors swallow std::bad_alloc (dynamic_cpu.hpp:52-56):
        the solver then holds no result, :meth:`Result` gives treedepth
        NO_RESULT (UINT_MAX, dynamic_cpu.hpp:79-80) and GetElimination []."""
        if g.n > _lib.DP_MAX_N:
            raise _lib.InvalidArgument(1, f"subset DP supports n <= {_lib.DP_MAX_N}")
        self._n, self._td, self._parent, self._order = g.n, None, None, None
        try:
            td, parent, order, stats = self._h.dp_solve(_masks(g), g.n, tile_bits=self._tile_bits)
        except _lib.GtdError as e:
            if e.status == 3:  # GTD_OOM
                self._td = NO_RESULT
                return
            raise
        self._n, self._td, self._parent, self._order, self.stats = g.n, td, parent, order, stats

    @property
    def treedepth(self) -> int:
        if self._td is None:
            raise _lib.GtdError(7, "no solve yet")
        return self._td

    def Result(self) -> Result:
        if self._td is None:
            raise _lib.GtdError(7, "no solve yet")
        if self._td == NO_RESULT:
            return Result(NO_RESULT, -1, np.zeros(0, dtype=np.int32))
        roots = np.flatnonzero(self._parent == -1)
        return Result(self._td, int(roots[0]) if len(roots) else -1, self._parent.copy())

    def GetElimination(self, nverts: int, subset_size: int, subset_code: int) -> List[int]:
        """Elimination order of the subset of rank ``subset_code`` among the
        ``subset_size``-subsets of ``nverts`` vertices (dynamic_gpu.hpp:48-64).
        The full vertex set is (n, n, 0)."""
        if self._td == NO_RESULT:
            return []
        if subset_size == nverts == self._n and subset_code == 0 and self._order is not None:
            return self._order.tolist()
        td, order = self._h.dp_query(_decode(nverts, subset_size, subset_code))
        return order

    def GetTreedepth(self, subset_mask: int) -> int:
        td, _ = self._h.dp_query(subset_mask, want_order=False)
        return td


class BnBGPU:
    """Exact treedepth by the GB300 persistent branch and bound
    (``td::BnBGPU``, bnb_gpu.hpp:12-17: ``solver(g, heur_td) -> int``).
    Unlike the reference it also returns the elimination tree
    (:meth:`Result`). ``order`` is the branching order (vertex tried first
    at rank 0); by default ascending ids, the reference's DefaultAttemptOrder.
    ``heur_td`` below the seed tree's height is honoured as the reference's
    initial best_td (bnb_gpu.cu:275): the search decides level heur_td - 1
    first and, if that fails, heur_td (which yields the tree); it only orders
    the search, so a wrong bound cannot change the result."""

    def __init__(self, device: int = 0, handle: Optional[_lib.Handle] = None, deadline_ns: int = 0):
        self._h = handle or _lib.Handle(device)
        self._deadline = deadline_ns
        self._res = None

    def __call__(self, g: Graph, heur_td: Optional[int] = None, order=None, seed=None) -> int:
        if seed is None:
            seed = _lib.heuristic(g, 0)
        hints = None
        if heur_td is not None and 2 <= heur_td < seed[0]:
            hints = np.array([heur_td - 1], dtype=np.int32)
        res = self._h.bnb_solve_batch([g], orders=[order] if order is not None else None, seeds=[seed],
                                      deadline_ns=self._deadline, hints=hints)
        self._res = res
        return int(res["td"][0])

    def Result(self) -> Result:
        if self._res is None:
            raise _lib.GtdError(7, "no solve yet")
        par = self._res["parents"][0]
        return Result(int(self._res["td"][0]), int(np.flatnonzero(par == -1)[0]), par.copy())


def reference_chain(handle: _lib.Handle, g: Graph) -> Tuple[int, np.ndarray]:
    """The incumbent chain of the reference's bnbGPU (main.cpp:178-186):
    HighestDegree(Variance(BottomUpGPU)). Each heuristic returns its inner
    heuristic's result when that is strictly lower, else its own
    (highest_degree_heuristic.hpp:37-42); the bottom-up heuristic gives no
    result beyond n = 32 (the reference's Get returns its UINT_MAX sentinel
    when its DP cannot run to the end, bottom_up_heuristic.hpp:24-32).
    Returns (td, parent)."""
    best = (NO_RESULT, None)
    if 1 <= g.n <= _lib.BOTTOM_UP_MAX_N:
        td, par, _ = handle.bottom_up(g)
        best = (td, par)
    for kind in (2, 1):  # Variance, then HighestDegree around it
        td, par = _lib.heuristic(g, kind)
        if not best[0] < td:
            best = (td, par)
    return best


def solve_exact(handle: _lib.Handle, graphs, dp_max_n: int = 28, deadline_ns: int = 0, guidance=None,
                **bnb_kw) -> dict:
    """Exact treedepth of many connected graphs, each by the solver that suits
    its size: graphs with n <= dp_max_n by the batched subset DP (every one
    proven, in one launch), the others by the batched branch and bound
    (optionally guided: `guidance` = gnn.guidance(net, graphs)).

    Returns td, parents, status (0 proven, 4 deadline), proof_ms (per graph,
    from the start of the call; DP graphs: the DP batch's device time) and
    which solver took each graph ("dp" / "bnb")."""
    import time
    n_all = len(graphs)
    small = [i for i, g in enumerate(graphs) if g.n <= dp_max_n]
    large = [i for i, g in enumerate(graphs) if g.n > dp_max_n]
    td = np.zeros(n_all, dtype=np.int32)
    status = np.zeros(n_all, dtype=np.int32)
    proof = np.zeros(n_all, dtype=np.float32)
    parents = [None] * n_all
    solver = [""] * n_all
    t0 = time.perf_counter()
    if small:
        dtd, dpar, st = handle.dp_solve_batch([graphs[i] for i in small])
        for j, i in enumerate(small):
            td[i], parents[i], solver[i] = dtd[j], dpar[j], "dp"
            proof[i] = st["total_ms"]
    if large:
        sub = [graphs[i] for i in large]
        kw = dict(bnb_kw)
        if guidance is not None:
            kw.update(orders=[guidance["orders"][i] for i in large], seeds=[guidance["seeds"][i] for i in large],
                      hints=np.asarray(guidance["hints"])[large])
        off_ms = (time.perf_counter() - t0) * 1e3
        res = handle.bnb_solve_batch(sub, deadline_ns=deadline_ns, **kw)
        for j, i in enumerate(large):
            td[i], parents[i], status[i], solver[i] = res["td"][j], res["parents"][j], res["status"][j], "bnb"
            proof[i] = res["proof_ms"][j] + off_ms if res["status"][j] == 0 else -1.0
    return {"td": td, "parents": parents, "status": status, "proof_ms": proof, "solver": solver}
