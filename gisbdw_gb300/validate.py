"""Elimination-tree validity, as the reference's CheckIfTdDecompIsValid
(Treedepth/common/utils/utils.hpp:50-86): every edge joins an ancestor and a
descendant of the tree, and the tree height (in vertices) equals td."""
from __future__ import annotations

import numpy as np

from .graphs import Graph


def check_tree(g: Graph, td: int, parent, allow_forest: bool = False) -> bool:
    par = np.asarray(parent, dtype=np.int64)
    n = g.n
    if par.shape != (n,) or np.any(par < -1) or np.any(par >= n) or np.any(par == np.arange(n)):
        return False
    depth = np.zeros(n, dtype=np.int64)
    for v in range(n):
        d, u = 0, v
        while u >= 0 and d <= n:
            d += 1
            u = int(par[u])
        if d > n:
            return False
        depth[v] = d
    roots = int(np.sum(par == -1))
    if roots < 1 or (roots != 1 and not allow_forest):
        return False
    for a, b in g.edges:
        if depth[a] < depth[b]:
            a, b = b, a
        while depth[a] > depth[b]:
            a = int(par[a])
        if a != b:
            return False
    return int(depth.max()) == int(td)
