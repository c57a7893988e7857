"""CPU checks of the invariants the subset-DP kernel (gtd_dp.cu) relies on.

* The bitwise recurrence: the children S - v of S have treedepth td(S) - 1
  or td(S), so with s = OR(td) + AND(td) over the children,
  td(S) = (s >> 1) + ((s & 1) | connected(S)); a third accumulator tracks
  "at least two connected children". Restated here at the kernel's word
  level (4 subsets per 32-bit word, byte = td << 1 | connected): the
  cross-tile summary kept as two virtual children (children reduced two
  or three at a time), the in-tile children addressed as the unrolled
  classes address them, the in-word order 00 -> 01, 10 -> 11 with byte
  permutes, the byte-at-a-time path for |S| <= 2 and the level-0 tile. Checked against the oracle's tables
  (DynamicCPU's values, dynamic_cpu.hpp / dynamic_gpu.cu:68-111).
* The colex rank of H - v from per-bit terms (prefix and suffix sums), and
  the warp-parallel tile decode (level by running totals, unranking one
  element at a time), against the serial definitions (set_encoder.hpp:40-46).
"""
from math import comb

import numpy as np
import pytest

from gisbdw_gb300 import graphs as G

M32 = 0xFFFFFFFF


def byte_perm(x, y, sel):
    b = [(x >> (8 * i)) & 0xFF for i in range(4)] + [(y >> (8 * i)) & 0xFF for i in range(4)]
    return sum(b[(sel >> (4 * i)) & 7] << (8 * i) for i in range(4))


class Acc:
    def __init__(self):
        self.o, self.a, self.d = 0, M32, 0

    def add2(self, x, y):
        self.d |= (self.o & (x | y)) | (x & y)
        self.o |= x | y
        self.a &= x & y

    def add1(self, x):
        self.d |= self.o & x
        self.o |= x
        self.a &= x

    def add3(self, x, y, z):
        any_ = x | y | z
        self.d |= (self.o & any_) | (x & y) | (x & z) | (y & z)
        self.o |= any_
        self.a &= x & y & z


def resolve4(g):
    """The kernel's form: half = 2 (s >> 1) | connected, plus (s & 1 | connected) << 1."""
    s = ((g.o & 0xFEFEFEFE) + (g.a & 0xFEFEFEFE)) >> 1
    half = (s & 0xFEFEFEFE) | (g.d & 0x01010101)
    return (half + (((s | g.d) & 0x01010101) << 1)) & M32


def resolve4_reference_form(g):
    s = ((g.o & 0xFEFEFEFE) + (g.a & 0xFEFEFEFE)) >> 1
    cn = g.d & 0x01010101
    return (((s & 0xFEFEFEFE) + (((s | cn) & 0x01010101) << 1)) | cn) & M32


def child_words(w, tbase=0x4A0):
    """In-tile children of word w as the kernel addresses them: A = T + 4w,
    bits taken lowest first with r4 & (r4 - 4), child at A + n1 - r4 (pairs),
    then A - r4 for an odd last one; returned as word indices."""
    A = tbase + 4 * w
    r4, out = w << 2, []
    for _ in range(bin(w).count("1") // 2):
        n1 = r4 & (r4 - 4)
        n2 = n1 & (n1 - 4)
        out += [(A + n1 - r4 - tbase) >> 2, (A + n2 - n1 - tbase) >> 2]
        r4 = n2
    if bin(w).count("1") & 1:
        out.append((A - r4 - tbase) >> 2)
    return out


def resolve1(o, a, d, k, adjacent):
    if k == 0:
        return 0
    cn = 1 if k == 1 else (int(adjacent) if k == 2 else d & 1)
    s = ((o & 0xFE) + (a & 0xFE)) >> 1
    return ((s & 0xFE) + (((s | cn) & 1) << 1)) | cn


def second_child(g):
    return (g.a & 0xFEFEFEFE) | (g.d & 0x01010101)


def word_dp(g, lb, triples=False):
    """The kernel's schedule on one graph with tiles of 2^lb subsets (cross-
    tile children three at a time with `triples`, as from 10-bit tiles up);
    returns the table indexed by subset mask (byte = td << 1 | connected)."""
    n = g.n
    adj = g.adjacency_masks()
    nh = n - lb
    words = 1 << (lb - 2)
    tab = np.zeros(1 << n, dtype=np.int64)

    def word_of(H, w):
        base = (H << lb) | (w << 2)
        return int(sum(int(tab[base + b]) << (8 * b) for b in range(4)))

    for H in sorted(range(1 << nh), key=lambda h: (bin(h).count("1"), h)):
        j = bin(H).count("1")
        kids = [H & ~(1 << h) for h in range(nh) if H >> h & 1]
        T, U = [0] * words, [0] * words
        for w in range(words):
            acc = Acc()
            m = 0
            while triples and m + 3 <= len(kids):
                acc.add3(word_of(kids[m], w), word_of(kids[m + 1], w), word_of(kids[m + 2], w))
                m += 3
            while m + 2 <= len(kids):
                acc.add2(word_of(kids[m], w), word_of(kids[m + 1], w))
                m += 2
            if m < len(kids):
                acc.add1(word_of(kids[m], w))
            T[w], U[w] = acc.o, second_child(acc)
        for s in range(lb - 1):
            for w in (x for x in range(words) if bin(x).count("1") == s):
                acc = Acc()
                if j > 0:
                    acc.add2(T[w], U[w])
                cw = child_words(w)
                for i in range(0, len(cw) - 1, 2):
                    acc.add2(T[cw[i]], T[cw[i + 1]])
                if len(cw) & 1:
                    acc.add1(T[cw[-1]])
                k = j + s
                if k >= 3:
                    v = resolve4(acc)
                    x = byte_perm(v, 0, 0x4004)
                    acc.d |= acc.o & x
                    acc.o |= x
                    acc.a &= x | 0xFF0000FF
                    v = resolve4(acc)
                    y1, y2 = byte_perm(v, 0, 0x1444), byte_perm(v, 0, 0x2444)
                    acc.d |= (acc.o & (y1 | y2)) | (y1 & y2)
                    acc.o |= y1 | y2
                    acc.a &= (y1 & y2) | 0x00FFFFFF
                    T[w] = resolve4(acc)
                else:
                    S0 = (H << lb) | (w << 2)
                    o = [(acc.o >> (8 * q)) & 0xFF for q in range(4)]
                    a = [(acc.a >> (8 * q)) & 0xFF for q in range(4)]
                    d = [(acc.d >> (8 * q)) & 0xFF for q in range(4)]

                    def edge(S):
                        u = (S & -S).bit_length() - 1
                        v = S.bit_length() - 1
                        return bool(adj[u] >> v & 1)

                    def fold(q, val):
                        d[q] |= o[q] & val
                        o[q] |= val
                        a[q] &= val
                    v0 = resolve1(o[0], a[0], d[0], k, k == 2 and edge(S0))
                    fold(1, v0)
                    fold(2, v0)
                    v1 = resolve1(o[1], a[1], d[1], k + 1, k + 1 == 2 and edge(S0 | 1))
                    v2 = resolve1(o[2], a[2], d[2], k + 1, k + 1 == 2 and edge(S0 | 2))
                    fold(3, v1)
                    fold(3, v2)
                    v3 = resolve1(o[3], a[3], d[3], k + 2, k + 2 == 2 and edge(S0 | 3))
                    T[w] = v0 | (v1 << 8) | (v2 << 16) | (v3 << 24)
        for w in range(words):
            for b in range(4):
                tab[(H << lb) | (w << 2) | b] = (T[w] >> (8 * b)) & 0xFF
    return tab


def connected_flags(g):
    adj = g.adjacency_masks()
    out = np.zeros(1 << g.n, dtype=np.int64)
    for S in range(1, 1 << g.n):
        reach = frontier = S & -S
        while frontier:
            nb = 0
            f = frontier
            while f:
                b = f & -f
                nb |= adj[b.bit_length() - 1]
                f ^= b
            frontier = nb & S & ~reach
            reach |= frontier
        out[S] = int(reach == S)
    return out


GRAPHS = [G.gnp_connected(9, 0.3, 1), G.gnp_connected(10, 0.5, 2), G.sparse_connected(10, 3), G.grid(2, 5),
          G.complete(8), G.path(9), G.cycle(10), G.star(9),
          G.Graph(10, [(0, 1), (2, 3), (3, 4), (6, 7), (7, 8), (8, 6)], name="forest10"),
          G.Graph(8, [], name="empty8")]


@pytest.mark.parametrize("lb,triples", [(4, False), (6, False), (6, True)])
def test_word_level_recurrence_matches_oracle(port, lb, triples):
    for g in GRAPHS:
        tab = word_dp(g, lb, triples)
        assert np.array_equal(tab >> 1, port.dp_table(g)), (g.name, lb)
        conn = connected_flags(g)
        assert np.array_equal(tab[1:] & 1, conn[1:]), (g.name, lb)


def test_in_tile_child_addresses():
    """Every word of a 12-bit tile (10 word bits): the kernel's address steps
    visit exactly the words w - b, b a bit of w, lowest bit first."""
    for w in range(1 << 10):
        assert child_words(w) == [w ^ (1 << b) for b in range(10) if w >> b & 1], w


def test_resolve4_forms_agree():
    """The kernel's resolve4 equals the longer reference form on every word
    whose bytes hold treedepths < 64 (per-byte sums below 256: no carries)."""
    rng = np.random.default_rng(5)
    for _ in range(20000):
        acc = Acc()
        acc.o, acc.a, acc.d = (int(x) for x in rng.integers(0, 1 << 32, 3, dtype=np.uint64))
        acc.o &= 0x7F7F7F7F | 0x01010101
        acc.a &= 0x7F7F7F7F | 0x01010101
        assert resolve4(acc) == resolve4_reference_form(acc)


def test_two_virtual_children_reproduce_the_summary():
    rng = np.random.default_rng(0)
    for _ in range(2000):
        count = int(rng.integers(1, 9))
        kids = [int(x) for x in rng.integers(0, 1 << 32, size=count, dtype=np.uint64)]
        acc = Acc()
        for x in kids:
            acc.add1(x)
        pair = Acc()
        pair.add2(acc.o, second_child(acc))
        assert pair.o == acc.o
        assert pair.a & 0xFEFEFEFE == acc.a & 0xFEFEFEFE
        assert pair.d & 0x01010101 == acc.d & 0x01010101


def rank_colex(H):
    r, q = 0, 0
    while H:
        b = (H & -H).bit_length() - 1
        q += 1
        r += comb(b, q)
        H &= H - 1
    return r


def test_child_ranks_by_prefix_and_suffix_sums():
    for nh in range(0, 11):
        for H in range(1 << nh):
            t1, t0 = [0] * 32, [0] * 32
            for v in range(nh):
                if H >> v & 1:
                    q = bin(H & ((1 << v) - 1)).count("1")
                    t1[v], t0[v] = comb(v, q + 1), comb(v, q)
            for v in range(nh):
                if H >> v & 1:
                    assert sum(t1[:v]) + sum(t0[v + 1:]) == rank_colex(H & ~(1 << v))


def test_warp_tile_decode_matches_serial():
    def serial(nh, t):
        off = prev = j = 0
        while off + comb(nh, j) <= t:
            prev, off, j = off, off + comb(nh, j), j + 1
        r, H, k, a = t - off, 0, j, nh - 1
        while k > 0:
            if r >= comb(a, k):
                H |= 1 << a
                r -= comb(a, k)
                k -= 1
            a -= 1
        return j, H, prev

    def warp(nh, t):
        cum = np.cumsum([comb(nh, i) if i <= nh else 0 for i in range(32)])
        j = sum(1 for i in range(32) if i <= nh and cum[i] <= t)
        off, prev = int(cum[(j + 31) & 31]), int(cum[(j + 30) & 31])
        r, H = t - (off if j >= 1 else 0), 0
        for k in range(j, 0, -1):
            a = max(x for x in range(32) if (comb(x, k) if x < nh else M32) <= r)
            H |= 1 << a
            r -= comb(a, k)
        return j, H, prev if j >= 2 else 0

    for nh in range(0, 11):
        for t in range(1 << nh):
            assert serial(nh, t) == warp(nh, t), (nh, t)


def _canonical_tree(g, T, S):
    """The canonical elimination forest of the vertex set S from a DP table
    (every component rooted at its first v with T[C - v] = T[C] - 1):
    parent and depth per vertex of S."""
    adj = g.adjacency_masks()

    def comp(R, v):
        reach, frontier = 1 << v, 1 << v
        while frontier:
            nb = 0
            for u in range(g.n):
                if frontier >> u & 1:
                    nb |= adj[u]
            nb &= R & ~reach
            reach |= nb
            frontier = nb
        return reach

    parent, depth = {}, {}
    stack = []
    rest = S
    while rest:
        c = comp(rest, (rest & -rest).bit_length() - 1)
        rest &= ~c
        stack.append((c, -1, 1))
    while stack:
        C, owner, d = stack.pop()
        if C & (C - 1) == 0:
            r = C.bit_length() - 1
        else:
            r = min((v for v in range(g.n) if C >> v & 1), key=lambda v: (int(T[C & ~(1 << v)]), v))
        parent[r], depth[r] = owner, d
        rest = C & ~(1 << r)
        while rest:
            c = comp(rest, (rest & -rest).bit_length() - 1)
            rest &= ~c
            stack.append((c, r, d + 1))
    return parent, depth


def _order_from_tree(parent):
    """GetElimination read off the canonical forest (the DP's tree kernel):
    repeatedly take the active subtree of greatest height, ties to the one
    with the lowest vertex, emit its root and activate its children."""
    kids = {v: [] for v in parent}
    for v, p in parent.items():
        if p >= 0:
            kids[p].append(v)

    def hl(v):
        hs = [hl(c) for c in kids[v]]
        return (1 + max((h for h, _ in hs), default=0), min([v] + [m for _, m in hs]))

    info = {v: hl(v) for v in parent}
    active = [v for v, p in parent.items() if p < 0]
    order = []
    while active:
        a = max(active, key=lambda v: (info[v][0], -info[v][1]))
        order.append(a)
        active.remove(a)
        active += kids[a]
    return order


def test_elimination_order_is_read_off_the_canonical_tree(port):
    """The GetElimination order (dynamic_gpu.hpp:48-64: the root of the first
    deepest component of the remaining set, repeatedly) equals the traversal
    of the canonical tree by subtree height, ties to the lowest vertex — the
    form the GPU tree kernel computes — on full vertex sets and random
    subsets, connected or not."""
    rng = np.random.default_rng(7)
    gs = [G.gnp(n, p, s) for n in (6, 9, 12) for p in (0.2, 0.4) for s in range(3)]
    gs += [G.grid(3, 4), G.cycle(9), G.Graph(8, [(0, 1), (2, 3), (3, 4), (6, 7)])]
    for g in gs:
        T = port.dp_table(g)
        full = (1 << g.n) - 1
        for S in [full] + [int(x) for x in rng.integers(1, full + 1, 6)]:
            parent, _ = _canonical_tree(g, T, S)
            assert _order_from_tree(parent) == port.get_elimination(g, T, S), (g.name, S)
