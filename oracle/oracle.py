"""ORACLE — TEST INFRASTRUCTURE ONLY.

ctypes bindings for the CPU checker:

* ``Port``: the C restatement in oracle/gtd_oracle.c (built into
  oracle/_build/libgtd_oracle.so), available wherever gcc is.
* ``Ref``: the reference's own CPU solvers compiled unchanged from their
  sources against the Boost-API shim (oracle/_ref/libgtdref.so, built by
  oracle/Makefile where the reference sources exist).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline/reference
legs may import this module; the product never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from typing import List, Optional, Tuple

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_SO = os.path.join(HERE, "_build", "libgtd_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libgtdref.so")
# The reference's Treedepth/ sources: $GTD_REFERENCE_TREEDEPTH, else a
# checkout named `reference` beside this repository.
REF_SRC = os.environ.get("GTD_REFERENCE_TREEDEPTH",
                         os.path.normpath(os.path.join(HERE, "..", "..", "reference", "Treedepth")))

_vp = ctypes.c_void_p
_i = ctypes.c_int
_ip = ctypes.POINTER(ctypes.c_int)
_i64 = ctypes.c_int64
_u64 = ctypes.c_uint64


def build(ref: bool = False) -> None:
    """Builds the port (and, if asked and the sources exist, the reference)."""
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    if ref and os.path.isdir(REF_SRC):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={REF_SRC}"], check=True)


def _ptr(a: np.ndarray) -> ctypes.c_void_p:
    return a.ctypes.data_as(_vp)


class Port:
    """The C restatement (gtd_oracle.c)."""

    def __init__(self, path: str = PORT_SO):
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        L.gtdo_nchoosek.restype = _u64
        L.gtdo_nchoosek.argtypes = [_u64, _u64]
        L.gtdo_encode.restype = _u64
        L.gtdo_encode.argtypes = [_vp, _i]
        L.gtdo_decode.argtypes = [_i, _i, _u64, _vp]
        L.gtdo_edge_lower_bound.argtypes = [_i, _i]
        L.gtdo_dp_table.argtypes = [_i, _vp, _vp, _i]
        L.gtdo_tree_from_table.argtypes = [_i, _vp, _vp, _ip, _vp]
        L.gtdo_get_elimination.argtypes = [_i, _vp, _vp, _u64, _vp]
        L.gtdo_dp_solve.argtypes = [_i, _vp, _i, _ip, _vp]
        L.gtdo_dp_improv.argtypes = [_i, _vp, _ip, _vp, ctypes.POINTER(_i64)]
        L.gtdo_elimination_tree.argtypes = [_i, _vp, _vp, _ip, _vp]
        L.gtdo_bottom_up.argtypes = [_i, _vp, _vp]
        L.gtdo_check_valid.argtypes = [_i, _vp, _i, _vp, _i]
        L.gtdo_heuristic.argtypes = [_i, _vp, _i, _ip, _vp]
        L.gtdo_bnb.argtypes = [_i, _vp, _i, _i, _i64, _ip, _vp, ctypes.POINTER(_i64)]
        self.L = L

    def nchoosek(self, n: int, k: int) -> int:
        return int(self.L.gtdo_nchoosek(n, k))

    def encode(self, s) -> int:
        a = np.ascontiguousarray(s, dtype=np.int32)
        return int(self.L.gtdo_encode(_ptr(a), len(a)))

    def decode(self, n: int, k: int, code: int) -> List[int]:
        out = np.zeros(max(k, 1), dtype=np.int32)
        self.L.gtdo_decode(n, k, code, _ptr(out))
        return out[:k].tolist()

    def edge_lower_bound(self, n: int, e: int) -> int:
        return int(self.L.gtdo_edge_lower_bound(n, e))

    def dp_table(self, g, nthreads: int = 1) -> np.ndarray:
        adj = g.adj64()
        T = np.empty(1 << g.n, dtype=np.uint8)  # gtdo_dp_table writes every entry
        rc = self.L.gtdo_dp_table(g.n, _ptr(adj), _ptr(T), nthreads)
        if rc:
            raise ValueError(f"gtdo_dp_table rc={rc}")
        return T

    def tree_from_table(self, g, T: np.ndarray) -> Tuple[int, np.ndarray]:
        adj = g.adj64()
        par = np.zeros(g.n, dtype=np.int32)
        td = ctypes.c_int()
        rc = self.L.gtdo_tree_from_table(g.n, _ptr(adj), _ptr(T), ctypes.byref(td), _ptr(par))
        if rc:
            raise ValueError(f"gtdo_tree_from_table rc={rc}")
        return td.value, par

    def get_elimination(self, g, T: np.ndarray, subset: int) -> List[int]:
        adj = g.adj64()
        out = np.zeros(max(1, bin(subset).count("1")), dtype=np.int32)
        rc = self.L.gtdo_get_elimination(g.n, _ptr(adj), _ptr(T), subset, _ptr(out))
        if rc:
            raise ValueError(f"gtdo_get_elimination rc={rc}")
        return out[:bin(subset).count("1")].tolist()

    def dp_solve(self, g, nthreads: int = 1) -> Tuple[int, np.ndarray]:
        adj = g.adj64()
        par = np.zeros(g.n, dtype=np.int32)
        td = ctypes.c_int()
        rc = self.L.gtdo_dp_solve(g.n, _ptr(adj), nthreads, ctypes.byref(td), _ptr(par))
        if rc:
            raise ValueError(f"gtdo_dp_solve rc={rc}")
        return td.value, par

    def dp_improv(self, g) -> Tuple[int, np.ndarray]:
        adj = g.adj64()
        par = np.zeros(g.n, dtype=np.int32)
        td = ctypes.c_int()
        memo = _i64()
        rc = self.L.gtdo_dp_improv(g.n, _ptr(adj), ctypes.byref(td), _ptr(par), ctypes.byref(memo))
        if rc:
            raise ValueError(f"gtdo_dp_improv rc={rc}")
        return td.value, par

    def elimination_tree(self, g, order) -> Tuple[int, np.ndarray]:
        adj = g.adj64()
        o = np.ascontiguousarray(order, dtype=np.int32)
        par = np.zeros(g.n, dtype=np.int32)
        td = ctypes.c_int()
        rc = self.L.gtdo_elimination_tree(g.n, _ptr(adj), _ptr(o), ctypes.byref(td), _ptr(par))
        if rc:
            raise ValueError(f"gtdo_elimination_tree rc={rc}")
        return td.value, par

    def bottom_up(self, g) -> Tuple[int, np.ndarray, List[int]]:
        """BottomUpHeuristicGPU::Get (bottom_up_heuristic.hpp:18-33): the
        bottom-up DP's elimination order and its EliminationTree replay:
        (td, parent, order)."""
        adj = g.adj64()
        order = np.zeros(g.n, dtype=np.int32)
        rc = self.L.gtdo_bottom_up(g.n, _ptr(adj), _ptr(order))
        if rc:
            raise ValueError(f"gtdo_bottom_up rc={rc}")
        td, par = self.elimination_tree(g, order)
        return td, par, order.tolist()

    def check_valid(self, g, td: int, parent, allow_forest: bool = False) -> bool:
        adj = g.adj64()
        p = np.ascontiguousarray(parent, dtype=np.int32)
        return bool(self.L.gtdo_check_valid(g.n, _ptr(adj), int(td), _ptr(p), int(allow_forest)))

    def heuristic(self, g, kind: int = 0) -> Tuple[int, np.ndarray]:
        adj = g.adj128()
        par = np.zeros(g.n, dtype=np.int32)
        td = ctypes.c_int()
        rc = self.L.gtdo_heuristic(g.n, _ptr(adj), kind, ctypes.byref(td), _ptr(par))
        if rc:
            raise ValueError(f"gtdo_heuristic rc={rc}")
        return td.value, par

    def bnb(self, g, lb_kind: int = 0, heur_kind: int = 0, node_limit: int = 0):
        """Returns (status, td, parent, nodes); status 0 solved, 1 limit hit."""
        adj = g.adj128()
        par = np.zeros(g.n, dtype=np.int32)
        td = ctypes.c_int()
        nodes = _i64()
        rc = self.L.gtdo_bnb(g.n, _ptr(adj), lb_kind, heur_kind, node_limit,
                             ctypes.byref(td), _ptr(par), ctypes.byref(nodes))
        if rc < 0:
            raise ValueError(f"gtdo_bnb rc={rc}")
        return rc, td.value, par, nodes.value


class Ref:
    """The reference's own CPU solvers (oracle/_ref/libgtdref.so)."""

    def __init__(self, path: str = REF_SO):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        L = ctypes.CDLL(path)
        L.ref_dp_cpu.argtypes = [_i, _i, _vp, _ip, _ip, _vp]
        L.ref_dp_cpu_improv.argtypes = [_i, _i, _vp, _ip, _ip, _vp]
        L.ref_bnb_cpu.argtypes = [_i, _i, _vp, _i, _i, _ip, _ip, _vp]
        L.ref_heuristic.argtypes = [_i, _i, _vp, _i, _ip, _ip, _vp]
        L.ref_elimination_tree.argtypes = [_i, _i, _vp, _vp, _ip, _ip, _vp]
        L.ref_check_valid.argtypes = [_i, _i, _vp, _i, _i, _vp]
        L.ref_edge_lower_bound.restype = ctypes.c_uint
        L.ref_edge_lower_bound.argtypes = [_i, _i]
        L.ref_nchoosek.restype = _u64
        L.ref_nchoosek.argtypes = [_u64, _u64]
        L.ref_encode.restype = _u64
        L.ref_encode.argtypes = [_vp, _u64]
        L.ref_encode_excluded.restype = _u64
        L.ref_encode_excluded.argtypes = [_vp, _u64, _u64]
        L.ref_decode.argtypes = [_u64, _u64, _u64, _vp]
        self.L = L

    @staticmethod
    def available(path: str = REF_SO) -> bool:
        return os.path.exists(path)

    def _call(self, fn, g, *extra):
        e = g.edge_array().ravel().astype(np.int32)
        if e.size == 0:
            e = np.zeros(2, dtype=np.int32)
        td, root = ctypes.c_int(), ctypes.c_int()
        par = np.zeros(g.n, dtype=np.int32)
        rc = fn(g.n, g.m, _ptr(e), *extra, ctypes.byref(td), ctypes.byref(root), _ptr(par))
        return rc, td.value, root.value, par

    def dp_cpu(self, g):
        return self._call(self.L.ref_dp_cpu, g)

    def dp_cpu_improv(self, g):
        return self._call(self.L.ref_dp_cpu_improv, g)

    def bnb_cpu(self, g, lb_kind: int = 0, heur_kind: int = 0):
        return self._call(self.L.ref_bnb_cpu, g, lb_kind, heur_kind)

    def heuristic(self, g, kind: int):
        return self._call(self.L.ref_heuristic, g, kind)

    def elimination_tree(self, g, order):
        o = np.ascontiguousarray(order, dtype=np.int32)
        return self._call(self.L.ref_elimination_tree, g, _ptr(o))

    def check_valid(self, g, td: int, root: int, parent) -> int:
        e = g.edge_array().ravel().astype(np.int32)
        if e.size == 0:
            e = np.zeros(2, dtype=np.int32)
        p = np.ascontiguousarray(parent, dtype=np.int32)
        return int(self.L.ref_check_valid(g.n, g.m, _ptr(e), td, root, _ptr(p)))

    def edge_lower_bound(self, n: int, e: int) -> int:
        return int(self.L.ref_edge_lower_bound(n, e))

    def nchoosek(self, n: int, k: int) -> int:
        return int(self.L.ref_nchoosek(n, k))

    def encode(self, s) -> int:
        a = np.ascontiguousarray(s, dtype=np.int32)
        return int(self.L.ref_encode(_ptr(a), len(a)))

    def decode(self, n: int, k: int, code: int) -> List[int]:
        out = np.zeros(max(k, 1), dtype=np.int32)
        self.L.ref_decode(n, k, code, _ptr(out))
        return out[:k].tolist()
