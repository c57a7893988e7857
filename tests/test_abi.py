"""The C ABI library: it builds, loads, exports every symbol include/gtd.h
declares, and its host-only helpers behave. No compute calls (no GPU here)."""
import ctypes
import os
import re

import numpy as np

from gisbdw_gb300 import _lib, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            text = open(os.path.join(ROOT, "include", fn)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names |= set(re.findall(r"\b(gtd_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    L = _lib.load()
    names = declared_functions()
    assert "gtd_dp_solve" in names and "gtd_create" in names
    for name in names:
        assert hasattr(L, name), name


def test_status_strings():
    L = _lib.load()
    for code, name in _lib.STATUS.items():
        assert L.gtd_status_string(code).decode() == name


def _index_py(n, lb, S):
    from math import comb
    lb = min(lb, n)
    H = S >> lb
    j = bin(H).count("1")
    off = sum(comb(n - lb, i) for i in range(j))
    r, q = 0, 0
    for b in range(n - lb):
        if H >> b & 1:
            q += 1
            r += comb(b, q)
    return ((off + r) << lb) | (S & ((1 << lb) - 1))


def test_table_index_is_a_level_major_bijection():
    for n, lb in ((9, 8), (12, 8), (12, 10), (13, 12), (14, 10)):
        idx = np.array([_lib.table_index(n, lb, S) for S in range(1 << n)], dtype=np.int64)
        assert sorted(idx.tolist()) == list(range(1 << n))
        for S in range(0, 1 << n, 37):
            assert idx[S] == _index_py(n, lb, S)
        # tiles ordered by popcount of the high part
        hp = np.array([bin(S >> lb).count("1") for S in range(1 << n)])
        assert np.all(np.diff(hp[np.argsort(idx)]) >= 0)


def test_create_without_gpu_fails_cleanly():
    import torch
    if torch.cuda.is_available():
        return
    L = _lib.load()
    h = ctypes.c_void_p()
    st = L.gtd_create(ctypes.byref(h), 0, None)
    assert st in (1, 6) and not h.value


def test_batch_parents_are_per_graph_views():
    """dp_solve_batch hands back the flat parent pool as per-graph views made
    on access: indexing, negative indices, slices and iteration agree with
    the descriptors' offsets, and an empty batch is an empty sequence."""
    from gisbdw_gb300 import graphs as G
    gs = [G.path(5), G.cycle(7), G.complete(3), G.grid(2, 3)]
    descs, pool = _lib.pack_batch(gs)
    flat = np.arange(pool.size, dtype=np.int32)
    pg = _lib.PerGraph(flat, descs)
    want = [flat[d.offset:d.offset + d.n] for d in descs]
    assert len(pg) == len(gs)
    assert all(np.array_equal(a, b) for a, b in zip(pg, want))
    assert np.array_equal(pg[-1], want[-1])
    assert [x.tolist() for x in pg[1::2]] == [x.tolist() for x in want[1::2]]
    assert np.shares_memory(pg[0], flat)
    assert len(_lib.PerGraph(flat, (_lib.GraphDesc * 0)())) == 0


def test_noalloc_source_allocates_nothing():
    """The no-allocation entry point's translation unit calls no allocator."""
    src = open(os.path.join(ROOT, "gisbdw_gb300", "csrc", "gtd_noalloc.cu")).read()
    code = re.sub(r"//[^\n]*", "", re.sub(r"/\*.*?\*/", "", src, flags=re.S))
    for name in ("cudaMalloc", "cudaFree", "cudaMallocAsync", "cudaMallocManaged", "cudaHostAlloc", "malloc(",
                 "new "):
        assert name not in code, name


def test_noalloc_epoch_wraps_and_clears(tmp_path):
    """The shared flags' epoch: first call clears, then 2, 3, ...; after the
    last epoch the next call is 1 again and clears every flag."""
    import subprocess
    prog = tmp_path / "epoch.cpp"
    prog.write_text("""
#include <cstdio>
#include "gtd_noalloc_epoch.h"
int main() {
  bool c = false;
  unsigned e = gtd::noalloc_next_epoch(0, &c);
  std::printf("%u %d\\n", e, (int)c);
  e = gtd::noalloc_next_epoch(e, &c);
  std::printf("%u %d\\n", e, (int)c);
  e = gtd::noalloc_next_epoch(gtd::kNoallocLastEpoch - 1, &c);
  std::printf("%u %d\\n", e, (int)c);
  e = gtd::noalloc_next_epoch(e, &c);
  std::printf("%u %d\\n", e, (int)c);
  return 0;
}
""")
    exe = str(tmp_path / "epoch")
    subprocess.run(["g++", "-std=c++17", "-I" + os.path.join(ROOT, "gisbdw_gb300", "csrc"), str(prog), "-o", exe],
                   check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split()
    assert out == ["1", "1", "2", "0", str(0xFFFFFFFE), "0", "1", "1"]
