"""ctypes binding of libgtd.so (the C ABI declared in include/gtd.h).

The library is built in-tree by gisbdw_gb300/build.py. There is no CPU
fallback: if the library is missing or cannot load, every entry point raises.
"""
from __future__ import annotations

import ctypes
import os
import threading
from collections.abc import Sequence
from typing import Optional, Tuple

import numpy as np

from . import build as _build

_vp = ctypes.c_void_p
_i = ctypes.c_int
_i32p = ctypes.POINTER(ctypes.c_int32)
_u64 = ctypes.c_uint64

STATUS = {
    0: "GTD_OK", 1: "GTD_INVALID_ARG", 2: "GTD_NOT_CONNECTED", 3: "GTD_OOM",
    4: "GTD_TIMEOUT", 5: "GTD_ABORTED", 6: "GTD_CUDA_ERROR", 7: "GTD_NO_RESULT",
}
DP_MAX_N = 36


class GtdError(RuntimeError):
    """A gtd call returned a status other than GTD_OK."""

    def __init__(self, status: int, message: str):
        self.status = status
        self.status_name = STATUS.get(status, f"status {status}")
        super().__init__(f"{self.status_name}: {message}")


class InvalidArgument(GtdError, ValueError):
    """GTD_INVALID_ARG / GTD_NOT_CONNECTED (the reference throws
    std::invalid_argument: elimination_tree.hpp:171-179)."""


class DeadlineExceeded(GtdError, TimeoutError):
    """GTD_TIMEOUT."""


def _error(status: int, message: str) -> GtdError:
    if status in (1, 2):
        return InvalidArgument(status, message)
    if status == 4:
        return DeadlineExceeded(status, message)
    return GtdError(status, message)


class DpOpts(ctypes.Structure):
    _fields_ = [("tile_bits", ctypes.c_int), ("ctas_per_sm", ctypes.c_int),
                ("timeout_ns", ctypes.c_uint64)]


class DpStats(ctypes.Structure):
    _fields_ = [("dp_ms", ctypes.c_float), ("tree_ms", ctypes.c_float),
                ("total_ms", ctypes.c_float), ("table_bytes", ctypes.c_uint64),
                ("alg_bytes", ctypes.c_uint64), ("tile_bits", ctypes.c_int),
                ("tiles", ctypes.c_int), ("ctas", ctypes.c_int)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class GraphDesc(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int32), ("offset", ctypes.c_int32)]


class BatchOpts(ctypes.Structure):
    _fields_ = [("tile_bits", ctypes.c_int), ("ctas_per_sm", ctypes.c_int),
                ("timeout_ns", ctypes.c_uint64), ("use_cuda_graph", ctypes.c_int)]


class BatchStats(ctypes.Structure):
    _fields_ = [("dp_ms", ctypes.c_float), ("total_ms", ctypes.c_float),
                ("subsets", ctypes.c_uint64), ("alg_bytes", ctypes.c_uint64),
                ("table_bytes", ctypes.c_uint64), ("tile_bits", ctypes.c_int),
                ("tiles", ctypes.c_int), ("ctas", ctypes.c_int), ("graph_replayed", ctypes.c_int),
                ("tile_bits_by_n", ctypes.c_int * (DP_MAX_N + 1))]

    def as_dict(self) -> dict:
        d = {k: getattr(self, k) for k, _ in self._fields_}
        d["tile_bits_by_n"] = {n: b for n, b in enumerate(self.tile_bits_by_n) if b}
        return d


_LIB = None
_LOCK = threading.Lock()


def library_path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Loads libgtd.so, building it first when it is missing or stale."""
    global _LIB
    with _LOCK:
        if _LIB is not None:
            return _LIB
        if build_if_missing and not _build.up_to_date():
            _build.build()
        if not os.path.exists(_build.LIB):
            raise RuntimeError(f"gtd native library not found at {_build.LIB}; run gisbdw_gb300.build.build()")
        L = ctypes.CDLL(_build.LIB)
        L.gtd_create.argtypes = [ctypes.POINTER(_vp), _i, _vp]
        L.gtd_destroy.argtypes = [_vp]
        L.gtd_status_string.restype = ctypes.c_char_p
        L.gtd_status_string.argtypes = [_i]
        L.gtd_last_error.restype = ctypes.c_char_p
        L.gtd_last_error.argtypes = [_vp]
        L.gtd_dp_solve.argtypes = [_vp, _vp, _i, _vp, _vp, _vp, ctypes.POINTER(DpOpts), ctypes.POINTER(DpStats)]
        L.gtd_dp_solve_device.argtypes = [_vp, _vp, _i, _vp, _vp, _vp, ctypes.POINTER(DpOpts)]
        L.gtd_sync.argtypes = [_vp, ctypes.POINTER(DpStats)]
        L.gtd_dp_query.argtypes = [_vp, _u64, _vp, _vp]
        L.gtd_dp_table.argtypes = [_vp, ctypes.POINTER(_vp), ctypes.POINTER(_u64),
                                   ctypes.POINTER(_i), ctypes.POINTER(_i)]
        L.gtd_dp_table_index.restype = _u64
        L.gtd_dp_table_index.argtypes = [_i, _i, _u64]
        L.gtd_dp_read_table.argtypes = [_vp, _vp, _u64]
        L.gtd_dp_solve_batch.argtypes = [_vp, _vp, _i, _vp, ctypes.c_int64, _vp, _vp,
                                         ctypes.POINTER(BatchOpts), ctypes.POINTER(BatchStats)]
        L.gtd_dp_solve_batch_device.argtypes = [_vp, _vp, _i, _vp, ctypes.c_int64, _vp, _vp,
                                                ctypes.POINTER(BatchOpts)]
        L.gtd_dp_batch_sync.argtypes = [_vp, ctypes.POINTER(BatchStats)]
        L.gtd_dp_autotune.argtypes = [_vp, _i, _i, _vp, _vp]
        L.gtd_dp_set_rates.argtypes = [_vp, _i, _i, _vp, _vp]
        L.gtd_abort.argtypes = [_vp]
        L.gtd_inject_fault.argtypes = [_i, _i]
        _LIB = L
        return L


def _ptr(a: np.ndarray) -> ctypes.c_void_p:
    return a.ctypes.data_as(_vp)


FAULT_NONE, FAULT_ALLOC, FAULT_STALL, FAULT_POISON = 0, 1, 2, 3


def inject_fault(kind: int, count: int = 1) -> None:
    """gtd_inject_fault (tests of the error paths): FAULT_ALLOC makes the
    count-th device allocation from now fail (GTD_OOM); FAULT_STALL makes the
    next count single-graph DP solves wait on a tile nothing computes
    (GTD_TIMEOUT); FAULT_POISON fills the next count DP solves' tables with
    0xFF first (results unchanged unless a tile is read before it is
    visible); FAULT_NONE clears all."""
    st = load().gtd_inject_fault(kind, count)
    if st != 0:
        raise _error(st, "gtd_inject_fault")


class Handle:
    """One gtd handle: a CUDA device, a stream and the device buffers."""

    def __init__(self, device: int = 0, stream: Optional[int] = None):
        self.L = load()
        self._h = _vp()
        st = self.L.gtd_create(ctypes.byref(self._h), device, _vp(stream) if stream else None)
        if st != 0:
            raise _error(st, f"gtd_create(device={device}) failed")

    def _check(self, st: int) -> None:
        if st != 0:
            raise _error(st, self.L.gtd_last_error(self._h).decode())

    def abort(self) -> None:
        """gtd_abort: stops the call running on this handle (from another
        thread); that call raises GtdError with GTD_ABORTED."""
        self._check(self.L.gtd_abort(self._h))

    def close(self) -> None:
        if self._h:
            self.L.gtd_destroy(self._h)
            self._h = _vp()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- subset DP --------------------------------------------------------
    def dp_solve(self, adj: np.ndarray, n: int, tile_bits: int = 0, ctas_per_sm: int = 0,
                 timeout_ns: int = 0, want_order: bool = True):
        """Returns (td, parent[n], order[n] or None, stats dict)."""
        adj = np.ascontiguousarray(adj, dtype=np.uint64)
        if adj.size < n:
            raise ValueError("adjacency shorter than n")
        td = ctypes.c_int32()
        parent = np.zeros(n, dtype=np.int32)
        order = np.zeros(n, dtype=np.int32) if want_order else None
        opts = DpOpts(tile_bits, ctas_per_sm, timeout_ns)
        stats = DpStats()
        self._check(self.L.gtd_dp_solve(self._h, _ptr(adj), n, ctypes.byref(td), _ptr(parent),
                                        _ptr(order) if want_order else None, ctypes.byref(opts),
                                        ctypes.byref(stats)))
        return td.value, parent, order, stats.as_dict()

    def dp_solve_device(self, d_adj: int, n: int, d_td: int, d_parent: int, d_order: int = 0,
                        tile_bits: int = 0, ctas_per_sm: int = 0, timeout_ns: int = 0) -> None:
        opts = DpOpts(tile_bits, ctas_per_sm, timeout_ns)
        self._check(self.L.gtd_dp_solve_device(self._h, _vp(d_adj), n, _vp(d_td), _vp(d_parent),
                                               _vp(d_order) if d_order else None, ctypes.byref(opts)))

    def sync(self) -> dict:
        stats = DpStats()
        self._check(self.L.gtd_sync(self._h, ctypes.byref(stats)))
        return stats.as_dict()

    def dp_query(self, subset_mask: int, want_order: bool = True):
        td = ctypes.c_int32()
        k = bin(subset_mask).count("1")
        order = np.zeros(max(k, 1), dtype=np.int32)
        self._check(self.L.gtd_dp_query(self._h, subset_mask, ctypes.byref(td),
                                        _ptr(order) if want_order else None))
        return td.value, (order[:k].tolist() if want_order else None)

    # -- batched subset DP -------------------------------------------------
    def dp_solve_batch(self, graphs, tile_bits: int = 0, ctas_per_sm: int = 0, timeout_ns: int = 0,
                       use_cuda_graph: bool = True, packed=None):
        """Solves every graph; returns (td[count], [parent arrays], stats)."""
        descs, pool = packed if packed is not None else pack_batch(graphs)
        count = len(descs)
        td = np.zeros(count, dtype=np.int32)
        parent = np.zeros(max(1, pool.size), dtype=np.int32)
        opts = BatchOpts(tile_bits, ctas_per_sm, timeout_ns, int(use_cuda_graph))
        stats = BatchStats()
        self._check(self.L.gtd_dp_solve_batch(self._h, ctypes.cast(descs, _vp), count, _ptr(pool), pool.size,
                                              _ptr(td), _ptr(parent), ctypes.byref(opts), ctypes.byref(stats)))
        return td, PerGraph(parent, descs), stats.as_dict()

    def dp_solve_batch_device(self, descs, count: int, d_pool: int, pool_len: int, d_td: int, d_parent: int,
                              tile_bits: int = 0, ctas_per_sm: int = 0, timeout_ns: int = 0,
                              use_cuda_graph: bool = True) -> None:
        opts = BatchOpts(tile_bits, ctas_per_sm, timeout_ns, int(use_cuda_graph))
        self._check(self.L.gtd_dp_solve_batch_device(self._h, ctypes.cast(descs, _vp), count, _vp(d_pool),
                                                     pool_len, _vp(d_td), _vp(d_parent), ctypes.byref(opts)))

    def dp_batch_sync(self) -> dict:
        stats = BatchStats()
        self._check(self.L.gtd_dp_batch_sync(self._h, ctypes.byref(stats)))
        return stats.as_dict()

    def dp_autotune(self, n_min: int, n_max: int, with_mixed: bool = False):
        """Rates (subsets per microsecond), rows n_min..n_max, columns tile
        bits 8..12; with_mixed: also the mixed-size kernel's efficiency per
        largest tile size 8..12 (returns (rates, eff))."""
        rates = np.zeros((n_max - n_min + 1, 5), dtype=np.float32)
        eff = np.zeros(5, dtype=np.float32)
        self._check(self.L.gtd_dp_autotune(self._h, n_min, n_max, _ptr(rates), _ptr(eff)))
        return (rates, eff) if with_mixed else rates

    def dp_set_rates(self, n_min: int, rates: np.ndarray, mixed_eff=None) -> None:
        """gtd_dp_set_rates: rates rows n_min.., columns tile bits 8..12;
        mixed_eff: 5 efficiencies of the mixed-size kernel (None: never mix)."""
        r = np.ascontiguousarray(rates, dtype=np.float32)
        e = np.ascontiguousarray(mixed_eff, dtype=np.float32) if mixed_eff is not None else None
        self._check(self.L.gtd_dp_set_rates(self._h, n_min, n_min + r.shape[0] - 1, _ptr(r),
                                            _ptr(e) if e is not None else None))

    def dp_table_info(self) -> Tuple[int, int, int, int]:
        ptr, nbytes, n, lb = _vp(), _u64(), _i(), _i()
        self._check(self.L.gtd_dp_table(self._h, ctypes.byref(ptr), ctypes.byref(nbytes),
                                        ctypes.byref(n), ctypes.byref(lb)))
        return ptr.value or 0, nbytes.value, n.value, lb.value

    def dp_read_table(self) -> Tuple[np.ndarray, int, int]:
        """Raw table bytes (tiled layout), n and tile bits of the last solve."""
        _, nbytes, n, lb = self.dp_table_info()
        out = np.empty(nbytes, dtype=np.uint8)
        self._check(self.L.gtd_dp_read_table(self._h, _ptr(out), nbytes))
        return out, n, lb


class PerGraph(Sequence):
    """Per-graph views into one flat result array (parents of a batch), made
    on access: the batch call returns without building thousands of views.
    Indexing gives an array view; a slice gives a list of views."""
    __slots__ = ("_flat", "_off", "_n")

    def __init__(self, flat, descs):
        self._flat = flat
        if len(descs):
            arr = np.ctypeslib.as_array(descs)
            self._off, self._n = arr["offset"].tolist(), arr["n"].tolist()
        else:
            self._off, self._n = [], []

    def __len__(self):
        return len(self._off)

    def __getitem__(self, i):
        if isinstance(i, slice):
            return [self[k] for k in range(*i.indices(len(self)))]
        o = self._off[i]
        return self._flat[o:o + self._n[i]]


def pack_batch(graphs):
    """Adjacency pool and descriptors for a list of graphs (offsets = running
    sum of n)."""
    descs = (GraphDesc * len(graphs))()
    off = 0
    pool = np.zeros(sum(g.n for g in graphs), dtype=np.uint64)
    for i, g in enumerate(graphs):
        descs[i].n = g.n
        descs[i].offset = off
        pool[off:off + g.n] = g.adj64()
        off += g.n
    return descs, pool


def table_index(n: int, tile_bits: int, subset_mask: int) -> int:
    return int(load().gtd_dp_table_index(n, tile_bits, subset_mask))


# ---------------------------------------------------------------------------
# Branch and bound and heuristics.
# ---------------------------------------------------------------------------

BNB_MAX_N = 104


class BnbOpts(ctypes.Structure):
    _fields_ = [("memo_log2", ctypes.c_int), ("deadline_ns", ctypes.c_uint64), ("ctas_per_sm", ctypes.c_int),
                ("level_hint", ctypes.c_void_p), ("first_budget", ctypes.c_uint32), ("window", ctypes.c_int)]


class BnbStats(ctypes.Structure):
    _fields_ = [("ms", ctypes.c_float), ("total_ms", ctypes.c_float), ("nodes", ctypes.c_uint64),
                ("passes", ctypes.c_int32)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


def _bind_bnb(L):
    if getattr(L, "_bnb_bound", False):
        return L
    L.gtd_bnb_solve_batch.argtypes = [_vp, _vp, _i, _vp, ctypes.c_int64, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                      ctypes.POINTER(BnbOpts), ctypes.POINTER(BnbStats)]
    L.gtd_heuristic.argtypes = [_vp, _i, _i, _vp, _vp, _vp]
    L._bnb_bound = True
    return L


def _heuristic_batch(self, graphs, kind: int = 0, scores=None):
    """gtd_heuristic on the GPU for every graph (gtd_heuristic_batch):
    returns (td[count], [parent arrays])."""
    L = _bind_bnb(self.L)
    if not getattr(L, "_hb_bound", False):
        L.gtd_heuristic_batch.argtypes = [_vp, _vp, _i, _vp, ctypes.c_int64, _i, _vp, _vp, _vp]
        L._hb_bound = True
    ns = np.array([g.n for g in graphs], dtype=np.int32)
    offs = np.concatenate([[0], np.cumsum(ns)[:-1]]).astype(np.int32)
    descs = np.ascontiguousarray(np.stack([ns, offs], axis=1))
    adj = np.ascontiguousarray(np.concatenate([g.adj128() for g in graphs]).astype(np.uint64))
    total = int(ns.sum())
    sc = np.ascontiguousarray(np.concatenate(scores), dtype=np.float32) if scores is not None else None
    td = np.zeros(len(graphs), dtype=np.int32)
    par = np.zeros(total, dtype=np.int32)
    self._check(L.gtd_heuristic_batch(self._h, _ptr(descs), len(graphs), _ptr(adj), total, kind,
                                      _ptr(sc) if sc is not None else None, _ptr(td), _ptr(par)))
    return td, [par[o:o + n].copy() for o, n in zip(offs, ns)]


Handle.heuristic_batch = _heuristic_batch


BOTTOM_UP_MAX_N = 32


def _bottom_up(self, g):
    """gtd_bottom_up: the reference's bottom-up union-find heuristic DP on
    the GPU (n <= 32). Returns (td, parent, order)."""
    L = self.L
    if not getattr(L, "_bu_bound", False):
        L.gtd_bottom_up.argtypes = [_vp, _vp, _i, _vp, _vp, _vp]
        L._bu_bound = True
    adj = np.ascontiguousarray(g.adj64(), dtype=np.uint64)
    td = ctypes.c_int32()
    par = np.zeros(g.n, dtype=np.int32)
    order = np.zeros(g.n, dtype=np.int32)
    self._check(L.gtd_bottom_up(self._h, _ptr(adj), g.n, ctypes.byref(td), _ptr(par), _ptr(order)))
    return td.value, par, order


Handle.bottom_up = _bottom_up


def heuristic(g, kind: int = 0, scores=None):
    """Greedy incumbent (gtd_heuristic): kind 0 HighestDegree(Variance),
    1 HighestDegree, 2 Variance, 3 highest score first. Host only."""
    L = _bind_bnb(load())
    adj = g.adj128()
    td = ctypes.c_int32()
    par = np.zeros(g.n, dtype=np.int32)
    sc = np.ascontiguousarray(scores, dtype=np.float32) if scores is not None else None
    st = L.gtd_heuristic(_ptr(adj), g.n, kind, _ptr(sc) if sc is not None else None, ctypes.byref(td), _ptr(par))
    if st != 0:
        raise _error(st, "gtd_heuristic failed")
    return td.value, par


def pack_bnb(graphs, orders=None, seeds=None, seed_kind: int = 0):
    """Descriptors, 128-bit adjacency pool, order pool and seeds."""
    descs = (GraphDesc * len(graphs))()
    total = sum(g.n for g in graphs)
    adj = np.zeros(2 * max(total, 1), dtype=np.uint64)
    order = np.zeros(max(total, 1), dtype=np.uint8)
    seed_td = np.zeros(len(graphs), dtype=np.int32)
    seed_par = np.zeros(max(total, 1), dtype=np.int32)
    off = 0
    for i, g in enumerate(graphs):
        descs[i].n = g.n
        descs[i].offset = off
        adj[2 * off:2 * (off + g.n)] = g.adj128()
        order[off:off + g.n] = orders[i] if orders is not None else np.arange(g.n)
        if seeds is not None:
            t, p = seeds[i]
        else:
            t, p = heuristic(g, seed_kind)
        seed_td[i] = t
        seed_par[off:off + g.n] = p
        off += g.n
    return descs, adj, order, seed_td, seed_par, total


def _bnb_method(self, graphs, orders=None, seeds=None, memo_log2: int = 0, deadline_ns: int = 0,
                ctas_per_sm: int = 0, packed=None, hints=None, first_budget: int = 0, window: int = 0):
    """Exact treedepth of every graph by the persistent B&B kernel.
    Returns dict: td, parents, status, proof_ms, nodes, stats."""
    L = _bind_bnb(self.L)
    if packed is None and seeds is None:
        # the reference heuristic chain's incumbents, all graphs in one GPU launch
        std, spar = self.heuristic_batch(graphs, 0)
        seeds = list(zip(std.tolist(), spar))
    descs, adj, order, seed_td, seed_par, total = packed if packed is not None else pack_bnb(graphs, orders, seeds)
    count = len(descs)
    td = np.zeros(count, dtype=np.int32)
    par = np.zeros(max(total, 1), dtype=np.int32)
    status = np.zeros(count, dtype=np.int32)
    proof = np.zeros(count, dtype=np.float32)
    nodes = np.zeros(count, dtype=np.uint64)
    hint_arr = np.ascontiguousarray(hints, dtype=np.int32) if hints is not None else None
    if hint_arr is not None and hint_arr.size != count:
        raise ValueError("one level hint per graph")
    opts = BnbOpts(memo_log2, deadline_ns, ctas_per_sm, _ptr(hint_arr) if hint_arr is not None else None,
                   first_budget, window)
    stats = BnbStats()
    self._check(L.gtd_bnb_solve_batch(self._h, ctypes.cast(descs, _vp), count, _ptr(adj), total,
                                      _ptr(order), _ptr(seed_td), _ptr(seed_par), _ptr(td), _ptr(par),
                                      _ptr(status), _ptr(proof), _ptr(nodes), ctypes.byref(opts),
                                      ctypes.byref(stats)))
    parents = [par[d.offset:d.offset + d.n].copy() for d in descs]
    lbs = np.zeros(count, dtype=np.int32)
    if not getattr(L, "_lbs_bound", False):
        L.gtd_bnb_lower_bounds.argtypes = [_vp, _vp, _i]
        L._lbs_bound = True
    self._check(L.gtd_bnb_lower_bounds(self._h, _ptr(lbs), count))
    return {"td": td, "parents": parents, "status": status, "proof_ms": proof, "nodes": nodes,
            "stats": stats.as_dict(), "seed_td": seed_td, "lower_bound": lbs}


Handle.bnb_solve_batch = _bnb_method
