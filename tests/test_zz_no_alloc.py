"""gtd_dp_solve_noalloc: the subset DP for callers that cannot allocate
device memory (its scratch is a fixed __device__ array inside the library).

Called through the C ABI with device buffers this test owns, and checked
against the allocating entry point gtd_dp_solve on two calls in a row (the
second call reuses the scratch the first one left behind). This file is
collected last so that a run stopping at its first failure has already run
every other test."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(L, d_adj, n, d_td, d_par, d_order, stream):
    return L.gtd_dp_solve_noalloc(ctypes.c_void_p(d_adj), n, ctypes.c_void_p(d_td),
                                  ctypes.c_void_p(d_par), ctypes.c_void_p(d_order),
                                  ctypes.c_void_p(stream))


def test_noalloc_matches_allocating_entry_point():
    import torch

    from gisbdw_gb300 import Handle, _lib
    from gisbdw_gb300 import graphs as G

    L = _lib.load()
    L.gtd_dp_solve_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    torch.cuda.init()
    stream = torch.cuda.Stream()
    h = Handle(0)
    graphs = [G.gnp_connected(22, 0.2, 11), G.sparse_connected(24, 4)]
    for g in graphs:  # two calls in a row on the shared scratch
        td_ref, par_ref, order_ref, _ = h.dp_solve(g.adj64(), g.n)
        d_adj = torch.from_numpy(g.adj64().view(np.int64)).cuda()
        d_td = torch.full((1,), -7, dtype=torch.int32, device="cuda")
        d_par = torch.full((g.n,), -7, dtype=torch.int32, device="cuda")
        d_order = torch.full((g.n,), -7, dtype=torch.int32, device="cuda")
        torch.cuda.synchronize()
        st = _noalloc(L, d_adj.data_ptr(), g.n, d_td.data_ptr(), d_par.data_ptr(),
                      d_order.data_ptr(), stream.cuda_stream)
        assert st == 0, _lib.STATUS.get(st, st)
        assert int(d_td.item()) == td_ref, g.name
        assert d_par.cpu().numpy().tolist() == par_ref.tolist(), g.name
        assert d_order.cpu().numpy().tolist() == order_ref.tolist(), g.name
    # sizes beyond the fixed scratch are rejected, and nothing else breaks
    big = G.path(25)
    d_adj = torch.from_numpy(big.adj64().view(np.int64)).cuda()
    d_buf = torch.zeros(64, dtype=torch.int32, device="cuda")
    st = _noalloc(L, d_adj.data_ptr(), 25, d_buf.data_ptr(), d_buf.data_ptr(), 0, stream.cuda_stream)
    assert st == 1  # GTD_INVALID_ARG
    h.close()


def test_noalloc_allocates_nothing_and_reports_bad_input():
    """Across repeated calls the device's free memory and torch's allocation
    stay the same; an asymmetric adjacency is rejected on the device
    (GTD_INVALID_ARG, no hang); d_order may be NULL."""
    import torch

    from gisbdw_gb300 import Handle, _lib
    from gisbdw_gb300 import graphs as G

    L = _lib.load()
    L.gtd_dp_solve_noalloc.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    stream = torch.cuda.Stream()
    g = G.gnp_connected(23, 0.2, 5)
    d_adj = torch.from_numpy(g.adj64().view(np.int64)).cuda()
    d_td = torch.zeros(1, dtype=torch.int32, device="cuda")
    d_par = torch.zeros(g.n, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    assert _noalloc(L, d_adj.data_ptr(), g.n, d_td.data_ptr(), d_par.data_ptr(), 0, stream.cuda_stream) == 0
    free0, _ = torch.cuda.mem_get_info()
    alloc0 = torch.cuda.memory_allocated()
    for _ in range(3):
        assert _noalloc(L, d_adj.data_ptr(), g.n, d_td.data_ptr(), d_par.data_ptr(), 0, stream.cuda_stream) == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert torch.cuda.memory_allocated() == alloc0
    h = Handle(0)
    td_ref, par_ref, _, _ = h.dp_solve(g.adj64(), g.n, want_order=False)
    h.close()
    assert int(d_td.item()) == td_ref and d_par.cpu().numpy().tolist() == par_ref.tolist()
    bad = g.adj64().copy()
    u = int(np.flatnonzero([(int(bad[0]) >> v) & 1 for v in range(g.n)])[0])
    bad[u] &= ~np.uint64(1)  # edge 0-u kept only in 0's mask
    d_bad = torch.from_numpy(bad.view(np.int64)).cuda()
    st = _noalloc(L, d_bad.data_ptr(), g.n, d_td.data_ptr(), d_par.data_ptr(), 0, stream.cuda_stream)
    assert st == 1  # GTD_INVALID_ARG from the device-side check
    assert _noalloc(L, d_adj.data_ptr(), g.n, d_td.data_ptr(), d_par.data_ptr(), 0, stream.cuda_stream) == 0
    assert int(d_td.item()) == td_ref
