// K2: exact treedepth by branch and bound, persistent GPU kernel (sm_103a).
//
// Reference: BranchAndBound::Algorithm (Treedepth/src/branch_and_bound/
// branch_and_bound.cpp:51-114) searches elimination orders depth first on an
// EliminationTree, branching on the vertices of the first component and
// pruning when depth + EdgeLowerBound >= incumbent; BnBGPU (bnb_gpu.cu:107-380)
// keeps elimination prefixes on a global stack and replays them per thread.
// This kernel searches the same space — which vertex of a connected
// component is eliminated first — as the decision recursion
//     td(C) <= k  <=>  some v in C has td(D) <= k - 1 for every component D
//                     of C - v,
// and returns the treedepth AND an elimination tree:
//
//  * decide(C, k), depth first with an explicit frame stack per warp in
//    shared memory: |C| <= k accepts at once, lower bounds reject, else
//    candidates v are tried in a priority order (ascending ids = the
//    reference's DefaultAttemptOrder, branch_and_bound.cpp:9-16; or a learned
//    score order) and the components of C - v are decided largest first with
//    k - 1 (one failing component rejects v; the first v whose components
//    all pass accepts C).
//  * Bounds: the reference's edge bound in exact integer form
//    (edge_lower_bound.hpp:13-20: smallest d with (d-1)(2n-d) >= 2e), a
//    minor-min-width treewidth bound (td >= tw + 1), a longest-path bound
//    (td >= ceil(log2(L + 1)) for a greedy path of L vertices, one walk per
//    lane, tried when 2^k <= |C|), root domination (u is not tried as a
//    root when N(u) lies in N[v] for a v of larger degree or equal degree
//    and smaller id: v is at least as good), and a per-graph memo in HBM of
//    a lower and an upper bound (with a root achieving it) per component,
//    keyed by the component's vertex mask in 128-bit slots updated by
//    atomic CAS and shared by every warp working on that graph. Components
//    of 6-10 vertices are decided exactly by the subset-DP recurrence in a
//    per-warp table (their exact td goes to the memo); the memo bounds of
//    the vertex-deleted subsets C - v refute (td(C) >= td(C - v)) or accept
//    (root v) a component before any root is tried.
//  * Schedule: one persistent cooperative launch over a global atomic queue
//    of items (graph, level k, root candidate), issued for k descending from
//    the incumbent minus one, candidates in priority order, graphs
//    interleaved. Passes: an item may spend a node budget per pass; an item
//    that spends it stops and is issued again in the next pass with twice
//    its own budget (the memo keeps every subproblem it settled, so the
//    rerun resumes cheaply). The last warp to finish a pass counts the open
//    graphs and starts the next pass (next_pass: a bounded grid-wide wait;
//    every CTA is resident). Only a window of W levels per graph runs at a time:
//    k in (top - W, top], top = best - 1, or a caller's level hint clamped
//    into [proven lower bound, best - 1] (the learned td estimate: it orders
//    which decisions run first and never prunes; a wrong hint only moves the
//    window). Easy graphs finish in the first passes instead of waiting
//    behind the long items of hard graphs. A pass that started at least one
//    item per warp drains once half of its warps found no ticket left: the
//    items still running yield as if their budget were spent.
//    Split items: when a batch has fewer first-root items than the GPU has
//    warps, an item is a pair (first root v, second root u) deciding C - v
//    under root u at depth k - 1 (C - v connected; else the u = 0 item
//    decides all of v), so a single graph uses n^2 warps.
//    A success at level k improves the graph's best (atomicMin) and
//    cancels every remaining item at levels >= k; when every candidate at
//    level k has failed, the graph's proven lower bound becomes k + 1 and
//    every item below is cancelled. A graph is proven when the lower bound
//    meets the best. Running items re-check this (and a per-graph deadline
//    on %globaltimer) every 64 nodes and stop early.
//  * Trees: the first success of a level builds its elimination tree at
//    once (re-deciding each component at the depth it needs: memo hits)
//    into a per-level buffer, and only then publishes the level; the final
//    kernel copies the best level's tree (or the seed's) out.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <string>
#include <vector>

#include "gtd_handle.h"

namespace gtd {

constexpr int kBnbMaxN = GTD_BNB_MAX_N;  // 104: memo keys hold 104 vertex bits
constexpr int kBnbWarps = 4;
constexpr int kMaxComps = 40;            // components with >= 3 vertices: <= 104 / 3
constexpr int kMemoProbes = 8;
constexpr int kMmdMin = 10;              // minor-min-width bound for |C| >= this
constexpr int kSubsetMin = 16;           // memo bounds of the C - v for |C| >= this
constexpr int kMiniMin = 6, kMiniMax = 10;  // components decided exactly by a subset DP
constexpr uint32_t kSeedRoot = 0xFFu;

// The subsets of kMiniMax vertices grouped by size, increasing bit masks
// inside a group. Increasing masks are colex order, so for a component of
// m <= kMiniMax vertices the first C(m, l) masks of group l are exactly its
// l-subsets: the small-component DP walks each level without skipping.
struct MiniOrder {
  uint16_t subset[1 << kMiniMax];
  uint16_t start[kMiniMax + 2];
  uint16_t count[kMiniMax + 1][kMiniMax + 1];  // count[m][l] = C(m, l)
};

constexpr MiniOrder make_mini_order() {
  MiniOrder o{};
  int pos = 0;
  for (int l = 0; l <= kMiniMax; ++l) {
    o.start[l] = static_cast<uint16_t>(pos);
    for (int S = 0; S < (1 << kMiniMax); ++S) {
      int c = 0;
      for (int x = S; x; x &= x - 1)
        ++c;
      if (c == l)
        o.subset[pos++] = static_cast<uint16_t>(S);
    }
  }
  o.start[kMiniMax + 1] = static_cast<uint16_t>(pos);
  for (int m = 0; m <= kMiniMax; ++m) {
    o.count[m][0] = 1;
    for (int l = 1; l <= kMiniMax; ++l)
      o.count[m][l] = m == 0 ? 0 : static_cast<uint16_t>(o.count[m - 1][l - 1] + o.count[m - 1][l]);
  }
  return o;
}

static __device__ const MiniOrder kMiniOrder = make_mini_order();
constexpr int kUnknownUb = 127;
constexpr int kIoUnfinished = 3;         // d_io word: items that spent their budget this round
constexpr int kIoExited = 200;           // d_io words: warps that left the current pass, items started in it
constexpr int kIoPassDone = 202;         // d_io word: warps that finished the current pass
constexpr int kIoPassGen = 203;          // d_io word: passes completed (released by the pass's last warp)
constexpr int kIoPassStop = 204;         // d_io word: 1 when no further pass is needed
constexpr uint64_t kFirstBudget = 1024;  // search nodes of an item's first run
constexpr uint32_t kMaxDoublings = 30;   // an item's budget grows to at most 2^30 times the first
constexpr uint32_t kItemDone = 0xFF;
constexpr int kRoundWindow = 3;          // levels run at a time per graph
constexpr int kMaxRounds = 4096;

enum BnbStatus : int32_t { kBnbRunning = 0, kBnbTimeout = 2 };

struct BnbGraph {
  uint32_t adj_off;    // first vertex's (lo, hi) pair: adj[2 * (adj_off + v)]
  uint32_t out_idx;    // position in the caller's arrays
  uint64_t memo_off;   // first memo slot of the graph
  int32_t n;
  int32_t lb0;         // lower bound of the whole graph
  int32_t ub0;         // incumbent (seed) treedepth
  int32_t hint;        // level to try first (0 = none: top-down from the incumbent)
};

struct BnbParams {
  const BnbGraph* graphs = nullptr;
  int num_graphs = 0;
  int max_n = 0;
  int levels = 0;                  // max over graphs of ub0 - lb0
  const uint64_t* adj = nullptr;   // (lo, hi) per vertex
  const uint8_t* order = nullptr;  // order[adj_off + r] = vertex of rank r
  uint4* memo = nullptr;
  uint32_t memo_mask = 0;
  uint32_t* best = nullptr;        // per graph: k << 8 | root (kSeedRoot = seed tree)
  uint32_t* lbp = nullptr;         // per graph: proven lower bound
  uint32_t* fails = nullptr;       // per graph x level: failed candidates
  uint32_t* claim = nullptr;       // per graph x level: tree buffer taken
  uint8_t* item_state = nullptr;   // per graph x level x rank: kItemDone, or the item's budget doublings so far
  uint64_t budget = 0;             // an item's first budget in search nodes (0 = unlimited)
  int window = 0;                  // levels run at a time below a graph's top level (0 = all)
  int split = 0;                   // 1: an item is a pair (first root, second root)
  uint32_t* unfinished = nullptr;  // items that used up their budget this round
  uint8_t* mini = nullptr;         // per warp: 2^kMiniMax-byte small-component DP table
  uint32_t* exited = nullptr;      // [0] warps that found no ticket left, [1] items started (this pass)
  uint32_t drain_at = 0;           // running items yield once this many warps have left
  uint32_t full_at = 0;            // ... and at least this many items have started
  uint32_t* pass_done = nullptr;   // warps that finished the current pass
  uint32_t* pass_gen = nullptr;    // passes completed
  uint32_t* pass_stop = nullptr;   // set by the last warp of a pass: the search is over
  uint64_t pass_wait_ns = 0;       // bound on a warp's wait for the rest of its pass
  int8_t* lvl_parent = nullptr;    // per graph x level: tree (max_n entries, -1 root)
  int32_t* status = nullptr;       // per graph BnbStatus
  uint64_t* t_begin = nullptr;     // per graph: first item start (globaltimer ns)
  unsigned long long* t_end = nullptr;  // per graph: proof time
  unsigned long long* t0 = nullptr;     // launch start (min over items)
  unsigned long long* nodes = nullptr;  // per graph search nodes
  uint32_t* ticket = nullptr;
  int32_t* error = nullptr;
  uint64_t deadline_ns = 0;        // per-graph cap on time to proof
  // reconstruction
  const int32_t* seed_parent = nullptr;  // pool, per graph at adj_off
  int32_t* td_out = nullptr;
  int32_t* parent_out = nullptr;   // pool, per graph at adj_off
};

struct Frame {
  uint64_t lo, hi;     // component C
  uint8_t k, nxt, v, ci;        // depth bound, next rank, candidate, component index
  uint8_t m, state, single, pad;
};
enum FrameState : uint8_t { kEnter = 0, kNextV = 1, kNextComp = 2, kWaitChild = 3, kFail = 4, kAccept = 5 };

struct WarpMem {
  uint64_t alo[kBnbMaxN], ahi[kBnbMaxN];   // graph adjacency
  uint64_t wlo[kBnbMaxN], whi[kBnbMaxN];   // contraction work copy (minor-min-width)
  uint64_t slo[kMaxComps], shi[kMaxComps]; // components of C - v with >= 3 vertices
  Frame fr[kBnbMaxN + 2];
  uint64_t qlo[kBnbMaxN], qhi[kBnbMaxN];   // tree building: components still to root
  uint8_t qown[kBnbMaxN], qk[kBnbMaxN], qdep[kBnbMaxN];
  uint8_t ssz[kMaxComps];
  uint8_t order[kBnbMaxN];
  uint8_t mvert[kMiniMax];   // small-component DP: vertex of each local id
  uint16_t madj[kMiniMax];   // ... and its local adjacency
};

__device__ __forceinline__ bool has(uint64_t lo, uint64_t hi, int v) {
  return v < 64 ? ((lo >> v) & 1ull) : ((hi >> (v - 64)) & 1ull);
}
__device__ __forceinline__ void bit_clear(uint64_t& lo, uint64_t& hi, int v) {
  if (v < 64)
    lo &= ~(1ull << v);
  else
    hi &= ~(1ull << (v - 64));
}
__device__ __forceinline__ void bit_set(uint64_t& lo, uint64_t& hi, int v) {
  if (v < 64)
    lo |= 1ull << v;
  else
    hi |= 1ull << (v - 64);
}
__device__ __forceinline__ int popc128(uint64_t lo, uint64_t hi) { return __popcll(lo) + __popcll(hi); }
__device__ __forceinline__ int first128(uint64_t lo, uint64_t hi) {
  return lo ? __ffsll(static_cast<long long>(lo)) - 1 : 63 + __ffsll(static_cast<long long>(hi));
}

__device__ __forceinline__ void warp_or128(uint64_t& lo, uint64_t& hi) {
  const uint32_t a = __reduce_or_sync(0xffffffffu, static_cast<uint32_t>(lo));
  const uint32_t b = __reduce_or_sync(0xffffffffu, static_cast<uint32_t>(lo >> 32));
  const uint32_t c = __reduce_or_sync(0xffffffffu, static_cast<uint32_t>(hi));
  const uint32_t d = __reduce_or_sync(0xffffffffu, static_cast<uint32_t>(hi >> 32));
  lo = (static_cast<uint64_t>(b) << 32) | a;
  hi = (static_cast<uint64_t>(d) << 32) | c;
}

// 128-bit atomic compare-and-swap on one memo slot; returns the old value.
__device__ __forceinline__ void cas128(uint4* addr, uint64_t clo, uint64_t chi, uint64_t slo, uint64_t shi,
                                       uint64_t& olo, uint64_t& ohi) {
  asm volatile(
      "{\n\t.reg .b128 d, c, s;\n\tmov.b128 c, {%2, %3};\n\tmov.b128 s, {%4, %5};\n\t"
      "atom.global.cas.b128 d, [%6], c, s;\n\tmov.b128 {%0, %1}, d;\n\t}"
      : "=l"(olo), "=l"(ohi)
      : "l"(clo), "l"(chi), "l"(slo), "l"(shi), "l"(addr)
      : "memory");
}

// Memo slot: lo = mask bits 0..63; hi = mask bits 64..103 (bits 0..39) |
// lb << 40 | ub << 47 | root << 54. An all-zero slot is empty (the empty set
// is never stored).
constexpr uint64_t kKeyHiMask = (1ull << 40) - 1;

__device__ __forceinline__ uint64_t memo_hash(uint64_t lo, uint64_t hi) {
  uint64_t x = lo * 0x9E3779B97F4A7C15ull ^ (hi + 0x632BE59BD9B4E019ull) * 0xC2B2AE3D27D4EB4Full;
  x ^= x >> 31;
  x *= 0xBF58476D1CE4E5B9ull;
  return x ^ (x >> 29);
}

struct MemoHit {
  int lb, ub, root;  // lb 0 / ub 127 when unknown
};

__device__ __forceinline__ MemoHit unpack(uint64_t chi) {
  return MemoHit{static_cast<int>((chi >> 40) & 0x7F), static_cast<int>((chi >> 47) & 0x7F),
                 static_cast<int>((chi >> 54) & 0x7F)};
}

// Lookup (lane 0). Reads are atomic: a CAS that can only write back the
// value it found.
__device__ MemoHit memo_get(uint4* table, uint32_t mask, uint64_t lo, uint64_t hi) {
  const uint64_t h = memo_hash(lo, hi);
  for (int p = 0; p < kMemoProbes; ++p) {
    uint4* slot = table + ((h + p) & mask);
    uint64_t clo, chi;
    cas128(slot, 0, 0, 0, 0, clo, chi);
    if (clo == 0 && chi == 0)
      break;
    if (clo == lo && (chi & kKeyHiMask) == hi)
      return unpack(chi);
  }
  return MemoHit{0, kUnknownUb, 0};
}

// Merges bounds into the memo (lane 0): lb = max, ub = min (with its root).
__device__ void memo_put(uint4* table, uint32_t mask, uint64_t lo, uint64_t hi, int lb, int ub, int root) {
  const uint64_t h = memo_hash(lo, hi);
  auto merged = [&](uint64_t chi, bool empty) {
    MemoHit c = empty ? MemoHit{0, kUnknownUb, 0} : unpack(chi);
    const int nlb = max(c.lb, lb);
    int nub = c.ub, nroot = c.root;
    if (ub < nub) {
      nub = ub;
      nroot = root;
    }
    return hi | (static_cast<uint64_t>(nlb & 0x7F) << 40) | (static_cast<uint64_t>(nub & 0x7F) << 47) |
           (static_cast<uint64_t>(nroot & 0x7F) << 54);
  };
  int victim = 0, victim_size = 1 << 30;
  for (int p = 0; p < kMemoProbes; ++p) {
    uint4* slot = table + ((h + p) & mask);
    uint64_t clo = 0, chi = 0;
    cas128(slot, 0, 0, 0, 0, clo, chi);
    for (int tries = 0; tries < 64; ++tries) {
      const bool empty = clo == 0 && chi == 0;
      if (!empty && !(clo == lo && (chi & kKeyHiMask) == hi)) {
        const int sz = __popcll(clo) + __popcll(chi & kKeyHiMask);
        if (sz < victim_size) {
          victim_size = sz;
          victim = p;
        }
        break;  // another key: next probe
      }
      const uint64_t nhi = merged(chi, empty);
      if (!empty && nhi == chi)
        return;
      uint64_t olo, ohi;
      cas128(slot, clo, chi, lo, nhi, olo, ohi);
      if (olo == clo && ohi == chi)
        return;
      clo = olo;
      chi = ohi;
    }
  }
  // every probe holds another key: the memo is a cache, so overwrite the
  // entry of the smallest component (the cheapest to decide again)
  uint4* slot = table + ((h + victim) & mask);
  uint64_t clo = 0, chi = 0;
  cas128(slot, 0, 0, 0, 0, clo, chi);
  for (int tries = 0; tries < 64; ++tries) {
    uint64_t olo, ohi;
    cas128(slot, clo, chi, lo, merged(0, true), olo, ohi);
    if (olo == clo && ohi == chi)
      return;
    clo = olo;
    chi = ohi;
  }
}

// Why a running search should stop early.
struct StopCheck {
  const uint32_t* best = nullptr;  // stop when best k <= item_k
  const uint32_t* lbp = nullptr;   // stop when proven lb > item_k
  int item_k = 0;
  uint64_t deadline = 0;           // absolute ns, 0 = none
  uint64_t budget = 0;             // nodes before the item yields, 0 = none
  const uint32_t* exited = nullptr; // warps that left this pass, items started in it:
  uint32_t drain_at = 0;            // a pass that started at least one item per warp
  uint32_t full_at = 0;             // drains once half of its warps have left
  const int32_t* error = nullptr;   // the launch's error word: an abort or an error elsewhere
};

struct Search {
  WarpMem* w;
  int lane, n;
  uint4* memo;
  uint32_t memo_mask;
  StopCheck stop;
  unsigned long long nodes;
  bool timed_out, cancelled;
  bool yielded = false;
  uint8_t* mini = nullptr;  // this warp's 2^kMiniMax-byte table in global memory (L1-resident)

  // Exact treedepth of a component of m <= kMiniMax vertices by the subset
  // DP of the single-graph kernel (the reference's TreedepthInfo bound,
  // branch_and_bound.hpp:27-28, computed rather than looked up): byte of S =
  // td << 1 | connected; |S| >= 3 is connected iff two children S - v are;
  // td = 1 + min over children if connected, else the max. Subsets are
  // resolved level by level, lanes across each level. *root_out = the first
  // local vertex v with td(C - v) = td(C) - 1, as a global vertex.
  __device__ int mini_dp(uint64_t Clo, uint64_t Chi, int m, int* root_out) {
    if (lane == 0) {
      int i = 0;
      for (uint64_t xlo = Clo, xhi = Chi; xlo | xhi; ++i) {
        const int v = first128(xlo, xhi);
        bit_clear(xlo, xhi, v);
        w->mvert[i] = static_cast<uint8_t>(v);
      }
    }
    __syncwarp();
    if (lane < m) {
      const int v = w->mvert[lane];
      uint16_t a = 0;
      for (int j = 0; j < m; ++j)
        if (has(w->alo[v], w->ahi[v], w->mvert[j]))
          a |= static_cast<uint16_t>(1u << j);
      w->madj[lane] = a;
    }
    __syncwarp();
    uint8_t* T = mini;
    const uint32_t full = (1u << m) - 1u;
    for (int l = 1; l <= m; ++l) {
      const int level_size = kMiniOrder.count[m][l], base = kMiniOrder.start[l];
      for (int e = lane; e < level_size; e += 32) {
        const uint32_t S = kMiniOrder.subset[base + e];
        uint32_t b;
        if (l == 1) {
          b = 3u;  // td 1, connected
        } else if (l == 2) {
          const int u = __ffs(S) - 1, v = 31 - __clz(S);
          b = ((w->madj[u] >> v) & 1u) ? 5u : 2u;  // td 2 connected, or td 1 disconnected
        } else {
          uint32_t mn = 255u, mx = 0u, cnt = 0u;
          for (uint32_t x = S; x; x &= x - 1) {
            const uint32_t c = T[S & ~(x & (0u - x))];
            mn = min(mn, c);
            mx = max(mx, c);
            cnt += c & 1u;
          }
          b = cnt >= 2u ? ((mn & ~1u) + 3u) : (mx & ~1u);
        }
        T[S] = static_cast<uint8_t>(b);
      }
      __syncwarp();
    }
    const int td = T[full] >> 1;
    const bool is_root = lane < m && (T[full & ~(1u << lane)] >> 1) == static_cast<uint32_t>(td - 1);
    const uint32_t roots = __ballot_sync(0xffffffffu, is_root);
    *root_out = roots ? w->mvert[__ffs(roots) - 1] : w->mvert[0];
    __syncwarp();
    return td;
  }

  __device__ void component(uint64_t Slo, uint64_t Shi, int v, uint64_t& rlo, uint64_t& rhi) const {
    rlo = v < 64 ? (1ull << v) : 0ull;
    rhi = v >= 64 ? (1ull << (v - 64)) : 0ull;
    uint64_t flo = rlo, fhi = rhi;
    while (flo | fhi) {
      uint64_t nlo = 0, nhi = 0;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int u = lane + 32 * k;
        if (u < n && has(flo, fhi, u)) {
          nlo |= w->alo[u];
          nhi |= w->ahi[u];
        }
      }
      warp_or128(nlo, nhi);
      nlo &= Slo & ~rlo;
      nhi &= Shi & ~rhi;
      rlo |= nlo;
      rhi |= nhi;
      flo = nlo;
      fhi = nhi;
    }
  }

  __device__ int edges(uint64_t lo, uint64_t hi) const {
    int e = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int u = lane + 32 * k;
      if (u < n && has(lo, hi, u))
        e += __popcll(w->alo[u] & lo) + __popcll(w->ahi[u] & hi);
    }
    return __reduce_add_sync(0xffffffffu, e) / 2;
  }

  // EdgeLowerBound: smallest d in [1, nv] with (d - 1)(2 nv - d) >= 2e.
  __device__ static int edge_lb(int nv, int e) {
    int lo = 1, hi = nv;
    while (lo < hi) {
      const int d = (lo + hi) >> 1;
      if (static_cast<long long>(d - 1) * (2 * nv - d) >= 2ll * e)
        hi = d;
      else
        lo = d + 1;
    }
    return lo;
  }

  __device__ int deg_in(int v, uint64_t lo, uint64_t hi) const {
    return __popcll(w->alo[v] & lo) + __popcll(w->ahi[v] & hi);
  }

  // Path and cycle bound: td(C) >= ceil(log2(L + 1)) for a path of L
  // vertices in C, and td(C) >= 1 + ceil(log2(m)) for a cycle of m >= 3
  // vertices (treedepth is monotone under subgraphs; td(P_L) =
  // ceil(log2(L + 1)), and C_m minus any vertex is P_(m-1)). Each lane grows
  // one path greedily from its own start vertex, extending one end by the
  // neighbour with the fewest unvisited neighbours (Warnsdorff's rule) until
  // it is stuck, then the other end, and stops once the path has `need`
  // vertices; every chord between path vertices i < j positions apart
  // closes a cycle of j - i + 1 vertices. The bound is the best over lanes.
  __device__ int path_lb(uint64_t Clo, uint64_t Chi, int need) const {
    int start = -1;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int u = lane + 32 * k;
      if (start < 0 && u < n && has(Clo, Chi, u))
        start = u;
    }
    uint32_t len = 0, cyc = 0;
    if (start >= 0) {
      int8_t pos[kBnbMaxN];  // position on the path: front >= 0, back < 0
      uint64_t plo = 0, phi = 0;
      bit_set(plo, phi, start);
      pos[start] = 0;
      int e0 = start, e1 = start, side = 0, stuck = 0, front = 0, back = 0;
      len = 1;
      while (static_cast<int>(len) < need && stuck < 2) {
        const int e = side ? e1 : e0;
        uint64_t xlo = w->alo[e] & Clo & ~plo, xhi = w->ahi[e] & Chi & ~phi;
        if (!(xlo | xhi)) {
          ++stuck;
          side ^= 1;
          continue;
        }
        int best = -1, bd = 1 << 30;
        while (xlo | xhi) {
          const int x = first128(xlo, xhi);
          bit_clear(xlo, xhi, x);
          const int d = __popcll(w->alo[x] & Clo & ~plo) + __popcll(w->ahi[x] & Chi & ~phi);
          if (d < bd) {
            bd = d;
            best = x;
          }
        }
        bit_set(plo, phi, best);
        if (side) {
          e1 = best;
          pos[best] = static_cast<int8_t>(-(++back));
        } else {
          e0 = best;
          pos[best] = static_cast<int8_t>(++front);
        }
        ++len;
      }
      // the path alone does not refute; a cycle on it can (it has at most len
      // vertices and needs more than need / 2)
      if (static_cast<int>(len) < need && static_cast<int>(len) > (need >> 1)) {
        for (uint64_t xlo = plo, xhi = phi; xlo | xhi;) {
          const int v = first128(xlo, xhi);
          bit_clear(xlo, xhi, v);
          for (uint64_t ylo = w->alo[v] & plo, yhi = w->ahi[v] & phi; ylo | yhi;) {
            const int u = first128(ylo, yhi);
            bit_clear(ylo, yhi, u);
            const int d = pos[u] - pos[v];
            if (d >= 2)
              cyc = max(cyc, static_cast<uint32_t>(d + 1));
          }
        }
      }
    }
    const int lb_path = 32 - __clz(static_cast<int>(len));
    const int lb_cyc = cyc >= 3 ? 1 + (32 - __clz(static_cast<int>(cyc - 1))) : 0;
    return static_cast<int>(__reduce_max_sync(0xffffffffu, static_cast<uint32_t>(max(lb_path, lb_cyc))));
  }

  // Memo bounds of the vertex-deleted subsets C - v (one lookup per vertex,
  // lanes in parallel): the largest lower bound (0 where nothing is known)
  // and, in *ub_root, (smallest upper bound << 8 | its v). Memo keys are
  // components, so a hit on C - v means C - v is connected.
  __device__ int subset_bounds(uint64_t Clo, uint64_t Chi, uint32_t* ub_root) const {
    int best = 0;
    uint32_t ubr = 0xFFFFFFFFu;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int v = lane + 32 * k;
      if (v < n && has(Clo, Chi, v)) {
        uint64_t lo = Clo, hi = Chi;
        bit_clear(lo, hi, v);
        const MemoHit m = memo_get(memo, memo_mask, lo, hi);
        best = max(best, m.lb);
        if (m.ub < kUnknownUb)
          ubr = min(ubr, (static_cast<uint32_t>(m.ub) << 8) | static_cast<uint32_t>(v));
      }
    }
    *ub_root = __reduce_min_sync(0xffffffffu, ubr);
    return static_cast<int>(__reduce_max_sync(0xffffffffu, static_cast<uint32_t>(best)));
  }

  // Root domination (per lane, no warp collectives). If N_C(u) is contained
  // in N_C[v] for some v != u in C, swapping u and v in any elimination tree
  // of C rooted at u gives a valid tree of the same height rooted at v (v's
  // edges reach everything from the root; each neighbour of u other than v
  // is a neighbour of v, so it stays comparable with v's old position). So u
  // need not be tried as a root. Such v have deg_C(v) >= deg_C(u); skipping
  // u only for a v with a larger (degree, -id) keeps the chain of skips
  // acyclic, so a non-skipped root at least as good always remains. The
  // dominators of u are the intersection of N_C[w] over w in N_C(u).
  __device__ bool dominated(int u, uint64_t Clo, uint64_t Chi) const {
    uint64_t nlo = w->alo[u] & Clo, nhi = w->ahi[u] & Chi;
    const int du = __popcll(nlo) + __popcll(nhi);
    if (du == 0)
      return false;
    uint64_t ilo = Clo, ihi = Chi;
    for (uint64_t m = nlo; m && (ilo | ihi); m &= m - 1) {
      const int x = __ffsll(static_cast<long long>(m)) - 1;
      ilo &= w->alo[x] | (1ull << x);
      ihi &= w->ahi[x];
    }
    for (uint64_t m = nhi; m && (ilo | ihi); m &= m - 1) {
      const int x = 64 + __ffsll(static_cast<long long>(m)) - 1;
      ilo &= w->alo[x];
      ihi &= w->ahi[x] | (1ull << (x - 64));
    }
    bit_clear(ilo, ihi, u);
    while (ilo | ihi) {
      const int v = first128(ilo, ihi);
      bit_clear(ilo, ihi, v);
      const int dv = deg_in(v, Clo, Chi);
      if (dv > du || (dv == du && v < u))
        return true;
    }
    return false;
  }

  // Minor-min-width: repeatedly contract a minimum-degree vertex into its
  // minimum-degree neighbour; the largest minimum degree seen is a treewidth
  // lower bound, so td(C) >= it + 1.
  __device__ int mmd_lb(uint64_t Clo, uint64_t Chi) {
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      const int u = lane + 32 * k;
      if (u < n) {
        const bool in = has(Clo, Chi, u);
        w->wlo[u] = in ? (w->alo[u] & Clo) : 0ull;
        w->whi[u] = in ? (w->ahi[u] & Chi) : 0ull;
      }
    }
    __syncwarp();
    uint64_t Rlo = Clo, Rhi = Chi;
    int lb = 0;
    for (int remaining = popc128(Clo, Chi); remaining > 1; --remaining) {
      uint32_t best = 0xFFFFFFFFu;
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int u = lane + 32 * k;
        if (u < n && has(Rlo, Rhi, u))
          best = min(best, (static_cast<uint32_t>(__popcll(w->wlo[u]) + __popcll(w->whi[u])) << 8) | u);
      }
      best = __reduce_min_sync(0xffffffffu, best);
      const int d = static_cast<int>(best >> 8), v = static_cast<int>(best & 0xFF);
      lb = max(lb, d);
      const uint64_t vlo = w->wlo[v], vhi = w->whi[v];
      int u = -1;
      if (d > 0) {
        uint32_t bu = 0xFFFFFFFFu;
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const int x = lane + 32 * k;
          if (x < n && has(vlo, vhi, x))
            bu = min(bu, (static_cast<uint32_t>(__popcll(w->wlo[x]) + __popcll(w->whi[x])) << 8) | x);
        }
        bu = __reduce_min_sync(0xffffffffu, bu);
        u = static_cast<int>(bu & 0xFF);
      }
      __syncwarp();
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int x = lane + 32 * k;
        if (x < n && has(Rlo, Rhi, x) && x != v) {
          uint64_t xlo = w->wlo[x], xhi = w->whi[x];
          if (x == u) {
            xlo |= vlo;
            xhi |= vhi;
            bit_clear(xlo, xhi, u);
            bit_clear(xlo, xhi, v);
          } else if (has(vlo, vhi, x)) {
            bit_clear(xlo, xhi, v);
            if (u >= 0)
              bit_set(xlo, xhi, u);
          }
          w->wlo[x] = xlo;
          w->whi[x] = xhi;
        }
      }
      bit_clear(Rlo, Rhi, v);
      __syncwarp();
    }
    return lb + 1;
  }

  // Components of C - v with >= 3 vertices into w->slo/shi/ssz, largest
  // first (ties: smallest vertex first); returns their count and the size of
  // the largest component with <= 2 vertices.
  __device__ int split(uint64_t Clo, uint64_t Chi, int v, int& small_max) {
    uint64_t rlo = Clo, rhi = Chi;
    bit_clear(rlo, rhi, v);
    int m = 0;
    small_max = 0;
    while (rlo | rhi) {
      uint64_t clo, chi;
      component(rlo, rhi, first128(rlo, rhi), clo, chi);
      rlo &= ~clo;
      rhi &= ~chi;
      const int sz = popc128(clo, chi);
      if (sz <= 2) {
        small_max = max(small_max, sz);
        continue;
      }
      if (lane == 0 && m < kMaxComps) {
        int pos = m;
        while (pos > 0 && w->ssz[pos - 1] < sz) {
          w->slo[pos] = w->slo[pos - 1];
          w->shi[pos] = w->shi[pos - 1];
          w->ssz[pos] = w->ssz[pos - 1];
          --pos;
        }
        w->slo[pos] = clo;
        w->shi[pos] = chi;
        w->ssz[pos] = static_cast<uint8_t>(sz);
      }
      ++m;
      __syncwarp();
    }
    return m < kMaxComps ? m : kMaxComps;
  }

  // Next candidate of frame f: smallest rank >= f.nxt whose vertex is in C
  // and is not dominated as a root (a pendant vertex of a component with
  // >= 3 vertices is dominated by its neighbour).
  __device__ int next_candidate(Frame& f, int csize) {
    for (int base = f.nxt; base < n; base += 32) {
      const int r = base + lane;
      bool ok = false;
      if (r < n) {
        const int v = w->order[r];
        ok = has(f.lo, f.hi, v) && (csize < 3 || !dominated(v, f.lo, f.hi));
      }
      const uint32_t b = __ballot_sync(0xffffffffu, ok);
      if (b) {
        const int r0 = base + __ffs(b) - 1;
        __syncwarp();
        if (lane == 0)
          f.nxt = static_cast<uint8_t>(r0 + 1);
        __syncwarp();
        return w->order[r0];
      }
    }
    __syncwarp();
    if (lane == 0)
      f.nxt = static_cast<uint8_t>(n);
    __syncwarp();
    return -1;
  }

  // Every 64 nodes: deadline, the item became useless, or its node budget
  // for this round is spent.
  __device__ bool should_stop() {
    if (nodes & 63)
      return false;
    int flag = 0;
    if (lane == 0) {
      if (stop.deadline && global_ns() > stop.deadline)
        flag = 1;
      else if (stop.budget && (nodes >= stop.budget ||
                               (stop.exited && ld_acquire_u32(stop.exited) >= stop.drain_at &&
                                ld_acquire_u32(stop.exited + 1) >= stop.full_at)))
        flag = 3;  // budget spent, or the pass is draining: back next pass with twice the budget
      else if ((stop.best && static_cast<int>(ld_acquire_u32(stop.best) >> 8) <= stop.item_k) ||
               (stop.lbp && static_cast<int>(ld_acquire_u32(stop.lbp)) > stop.item_k) ||
               (stop.error && ld_relaxed_s32(stop.error) != 0))
        flag = 2;
    }
    flag = __shfl_sync(0xffffffffu, flag, 0);
    if (flag == 1)
      timed_out = true;
    if (flag == 2)
      cancelled = true;
    if (flag == 3)
      yielded = true;
    return flag != 0;
  }

  // decide(C, k): is td(G[C]) <= k? With single >= 0 only that root is tried
  // (the root items of the persistent kernel) and nothing is memoised for C.
  // On acceptance *root_out is the accepted root.
  __device__ bool decide(uint64_t Clo, uint64_t Chi, int k, int single, int* root_out) {
    int depth = 1;
    if (lane == 0) {
      Frame& f = w->fr[0];
      f.lo = Clo;
      f.hi = Chi;
      f.k = static_cast<uint8_t>(k);
      f.state = kEnter;
      f.single = single >= 0 ? 1 : 0;
      f.v = static_cast<uint8_t>(single >= 0 ? single : 0);
    }
    __syncwarp();
    bool ret = false;
    int ret_root = -1;
    while (depth > 0) {
      Frame& f = w->fr[depth - 1];
      __syncwarp();
      const uint8_t state = f.state;
      const int fk = f.k;
      __syncwarp();
      if (state == kEnter) {
        ++nodes;
        if (should_stop()) {
          ret = false;
          ret_root = -1;
          break;
        }
        const int csize = popc128(f.lo, f.hi);
        int decision = -1;  // 0 reject, 1 accept
        int vroot = -1;
        if (!f.single) {
          if (csize <= fk) {
            decision = 1;
            vroot = first128(f.lo, f.hi);
          } else if (fk <= 0 || csize <= 2) {
            decision = 0;
          } else {
            MemoHit hit{0, kUnknownUb, 0};
            if (lane == 0)
              hit = memo_get(memo, memo_mask, f.lo, f.hi);
            hit.lb = __shfl_sync(0xffffffffu, hit.lb, 0);
            hit.ub = __shfl_sync(0xffffffffu, hit.ub, 0);
            hit.root = __shfl_sync(0xffffffffu, hit.root, 0);
            if (hit.ub <= fk) {
              decision = 1;
              vroot = hit.root;
            } else if (hit.lb > fk) {
              decision = 0;
            } else if (mini && csize >= kMiniMin && csize <= kMiniMax) {
              int r = 0;
              const int td = mini_dp(f.lo, f.hi, csize, &r);
              if (lane == 0)
                memo_put(memo, memo_mask, f.lo, f.hi, td, td, r);
              decision = td <= fk ? 1 : 0;
              vroot = r;
            } else {
              const int ecount = edges(f.lo, f.hi);
              int lb = max(hit.lb, edge_lb(csize, ecount));
              if (lb <= fk && hit.lb == 0 && csize >= kMmdMin) {
                lb = max(lb, mmd_lb(f.lo, f.hi));
                if (lane == 0)
                  memo_put(memo, memo_mask, f.lo, f.hi, lb, kUnknownUb, 0);
              }
              // a path of 2^fk vertices, or a cycle of 2^(fk-1) + 1, would
              // refute td <= fk (a tree, with fewer edges than vertices, has
              // no cycle)
              if (lb <= fk && fk < 8 && ((1 << fk) <= csize || (ecount >= csize && (1 << (fk - 1)) < csize))) {
                const int pl = path_lb(f.lo, f.hi, 1 << fk);
                if (pl > fk) {
                  lb = pl;
                  if (lane == 0)
                    memo_put(memo, memo_mask, f.lo, f.hi, lb, kUnknownUb, 0);
                }
              }
              // td is monotone under vertex deletion: a memo entry proving
              // td(C - v) > fk for any v refutes td(C) <= fk at once; one
              // proving td(C - v) <= fk - 1 (C - v connected) accepts root v
              uint32_t ubr = 0xFFFFFFFFu;
              if (lb <= fk && csize >= kSubsetMin) {
                const int sl = subset_bounds(f.lo, f.hi, &ubr);
                if (sl > fk) {
                  lb = sl;
                  if (lane == 0)
                    memo_put(memo, memo_mask, f.lo, f.hi, lb, kUnknownUb, 0);
                }
              }
              if (lb > fk) {
                decision = 0;
              } else if (ubr != 0xFFFFFFFFu && static_cast<int>(ubr >> 8) <= fk - 1) {
                decision = 1;
                vroot = static_cast<int>(ubr & 0xFF);
                if (lane == 0)
                  memo_put(memo, memo_mask, f.lo, f.hi, 0, fk, vroot);
              }
            }
          }
        }
        if (decision >= 0) {
          ret = decision == 1;
          ret_root = vroot;
          --depth;
          continue;
        }
        __syncwarp();
        if (lane == 0) {
          f.nxt = 0;
          f.state = kNextV;
        }
        __syncwarp();
        continue;
      }
      if (state == kNextV) {
        const int csize = popc128(f.lo, f.hi);
        int v;
        if (f.single) {
          v = f.nxt == 0 ? f.v : -1;
          __syncwarp();
          if (lane == 0)
            f.nxt = 1;
        } else {
          v = next_candidate(f, csize);
        }
        __syncwarp();
        if (v < 0) {
          if (lane == 0)
            f.state = kFail;
          __syncwarp();
          continue;
        }
        int small_max = 0;
        const int m = split(f.lo, f.hi, v, small_max);
        // quick rejections: components too big for depth k - 1
        bool reject = small_max > fk - 1;
        for (int i = 0; i < m && !reject; ++i)
          reject = w->ssz[i] > fk - 1 && edge_lb(w->ssz[i], edges(w->slo[i], w->shi[i])) > fk - 1;
        __syncwarp();
        if (lane == 0) {
          f.v = static_cast<uint8_t>(v);
          f.ci = 0;
          f.m = static_cast<uint8_t>(m);
          f.state = reject ? kNextV : kNextComp;
        }
        __syncwarp();
        continue;
      }
      if (state == kNextComp) {
        if (f.ci == f.m) {
          __syncwarp();
          if (lane == 0)
            f.state = kAccept;
          __syncwarp();
          continue;
        }
        // recompute the sorted components of C - v (a deeper frame may have
        // replaced the list) and descend into the ci-th
        int small_max = 0;
        split(f.lo, f.hi, f.v, small_max);
        const int ci = f.ci;
        __syncwarp();
        if (lane == 0) {
          Frame& c = w->fr[depth];
          c.lo = w->slo[ci];
          c.hi = w->shi[ci];
          c.k = static_cast<uint8_t>(fk - 1);
          c.state = kEnter;
          c.single = 0;
          f.state = kWaitChild;
        }
        __syncwarp();
        ++depth;
        continue;
      }
      if (state == kWaitChild) {
        if (lane == 0) {
          if (!ret) {
            f.state = kNextV;
          } else {
            ++f.ci;
            f.state = kNextComp;
          }
        }
        __syncwarp();
        continue;
      }
      // kAccept / kFail
      const bool ok = state == kAccept;
      const int fv = f.v;
      if (!f.single && lane == 0) {
        if (ok)
          memo_put(memo, memo_mask, f.lo, f.hi, 0, fk, fv);
        else
          memo_put(memo, memo_mask, f.lo, f.hi, fk + 1, kUnknownUb, 0);
      }
      ret = ok;
      ret_root = ok ? fv : -1;
      __syncwarp();
      --depth;
    }
    if (root_out)
      *root_out = ret_root;
    return ret && !timed_out && !cancelled && !yielded;
  }

  // Elimination tree of C (depth <= k) below the accepted root: every
  // component left is decided again at the depth it needs, which the memo
  // entries written by the accepting search answer at once (a search only
  // where an entry has been evicted). parent_out[u] (int8, -1 at the root)
  // for u in C. With root2 >= 0 (C - root connected), root2 is fixed as
  // root's only child. False if a component fails (an error), or on a stop.
  __device__ bool build_tree(uint64_t Clo, uint64_t Chi, int k, int root, int8_t* parent_out, int root2 = -1) {
    if (lane == 0) {
      parent_out[root] = -1;
      if (root2 >= 0)
        parent_out[root2] = static_cast<int8_t>(root);
    }
    int top = 0;
    uint64_t rlo = Clo, rhi = Chi;
    bit_clear(rlo, rhi, root);
    const int owner0 = root2 >= 0 ? root2 : root;
    const int k0 = root2 >= 0 ? k - 2 : k - 1;
    if (root2 >= 0)
      bit_clear(rlo, rhi, root2);
    while (rlo | rhi) {
      uint64_t clo, chi;
      component(rlo, rhi, first128(rlo, rhi), clo, chi);
      rlo &= ~clo;
      rhi &= ~chi;
      if (lane == 0) {
        w->qlo[top] = clo;
        w->qhi[top] = chi;
        w->qown[top] = static_cast<uint8_t>(owner0);
        w->qk[top] = static_cast<uint8_t>(k0);
        w->qdep[top] = static_cast<uint8_t>(root2 >= 0 ? 3 : 2);
      }
      ++top;
    }
    __syncwarp();
    while (top > 0) {
      --top;
      const uint64_t clo = w->qlo[top], chi = w->qhi[top];
      const int owner = w->qown[top], kk = w->qk[top], depth = w->qdep[top];
      __syncwarp();
      int r = -1;
      if (depth > k || !decide(clo, chi, kk, -1, &r) || r < 0)
        return false;
      if (lane == 0)
        parent_out[r] = static_cast<int8_t>(owner);
      uint64_t xlo = clo, xhi = chi;
      bit_clear(xlo, xhi, r);
      while (xlo | xhi) {
        uint64_t dlo, dhi;
        component(xlo, xhi, first128(xlo, xhi), dlo, dhi);
        xlo &= ~dlo;
        xhi &= ~dhi;
        if (lane == 0) {
          w->qlo[top] = dlo;
          w->qhi[top] = dhi;
          w->qown[top] = static_cast<uint8_t>(r);
          w->qk[top] = static_cast<uint8_t>(kk - 1);
          w->qdep[top] = static_cast<uint8_t>(depth + 1);
        }
        ++top;
      }
      __syncwarp();
    }
    return true;
  }
};

__device__ void load_graph(WarpMem* w, const BnbParams& p, const BnbGraph& G, int lane) {
  for (int v = lane; v < G.n; v += 32) {
    w->alo[v] = p.adj[2 * (size_t(G.adj_off) + v)];
    w->ahi[v] = p.adj[2 * (size_t(G.adj_off) + v) + 1];
    w->order[v] = p.order[G.adj_off + v];
  }
  __syncwarp();
}

__device__ __forceinline__ void full_set(int n, uint64_t& lo, uint64_t& hi) {
  lo = n >= 64 ? ~0ull : ((1ull << n) - 1);
  hi = n > 64 ? ((1ull << (n - 64)) - 1) : 0ull;
}

// Records the proof time once the proven lower bound meets the best.
__device__ __forceinline__ void check_proved(const BnbParams& p, int g) {
  const uint32_t b = ld_acquire_u32(p.best + g) >> 8;
  const uint32_t l = ld_acquire_u32(p.lbp + g);
  if (l >= b)
    atomicCAS(p.t_end + g, 0ull, static_cast<unsigned long long>(global_ns()));
}

// End of a pass for one warp. Every warp arrives; the last one (all items of
// the pass are then finished) counts the graphs still open, resets the pass
// counters, decides whether another pass is needed and releases the next
// pass; the others wait for that release, bounded by p.pass_wait_ns (on
// expiry the kernel records a timeout and every warp leaves). Returns true
// when the warp should run another pass. The launch is cooperative, so every
// CTA is resident and the wait always ends.
__device__ bool next_pass(const BnbParams& p, uint32_t pass) {
  const int lane = threadIdx.x & 31;
  int last = 0;
  if (lane == 0) {
    __threadfence();  // this warp's item results before its arrival
    const uint32_t arrived = atomicAdd(p.pass_done, 1u) + 1u;
    last = arrived == gridDim.x * static_cast<uint32_t>(kBnbWarps);
    if (last)
      __threadfence();  // every arrival (and what preceded it) before the bookkeeping
  }
  last = __shfl_sync(0xffffffffu, last, 0);
  if (last) {
    uint32_t open = 0;
    for (int g = lane; g < p.num_graphs; g += 32)
      open += ld_relaxed_s32(p.status + g) != kBnbTimeout &&
              ld_acquire_u32(p.lbp + g) < (ld_acquire_u32(p.best + g) >> 8);
    open = __reduce_add_sync(0xffffffffu, open);
    if (lane == 0) {
      const bool stop = open == 0 || ld_relaxed_s32(p.error) != 0 || pass + 1 >= static_cast<uint32_t>(kMaxRounds);
      *reinterpret_cast<volatile uint32_t*>(p.ticket) = 0u;
      *reinterpret_cast<volatile uint32_t*>(p.unfinished) = 0u;
      reinterpret_cast<volatile uint32_t*>(p.exited)[0] = 0u;
      reinterpret_cast<volatile uint32_t*>(p.exited)[1] = 0u;
      *reinterpret_cast<volatile uint32_t*>(p.pass_done) = 0u;
      *reinterpret_cast<volatile uint32_t*>(p.pass_stop) = stop ? 1u : 0u;
      __threadfence();
      st_release_u32(p.pass_gen, pass + 1u);
    }
  } else if (lane == 0) {
    const uint64_t deadline = global_ns() + p.pass_wait_ns;
    unsigned sleep_ns = 64;
    while (ld_acquire_u32(p.pass_gen) <= pass) {
      if (global_ns() > deadline) {
        raise_error(p.error, kDevWaitTimeout, static_cast<int32_t>(pass));
        break;
      }
      __nanosleep(sleep_ns);
      if (sleep_ns < 4096)
        sleep_ns *= 2;
    }
  }
  uint32_t go = 0;
  if (lane == 0)
    go = ld_acquire_u32(p.pass_gen) > pass && ld_acquire_u32(p.pass_stop) == 0u && ld_relaxed_s32(p.error) == 0;
  return __shfl_sync(0xffffffffu, go, 0) != 0;
}

__global__ void __launch_bounds__(32 * kBnbWarps, 6) bnb_kernel(const __grid_constant__ BnbParams p) {
  extern __shared__ __align__(16) uint8_t smem[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  WarpMem* w = reinterpret_cast<WarpMem*>(smem) + warp;
  int cur_g = -1;
  const uint32_t S = p.split ? static_cast<uint32_t>(p.max_n) : 1u;  // second roots per first root
  const uint32_t per_level = static_cast<uint32_t>(p.max_n) * S * static_cast<uint32_t>(p.num_graphs);
  const uint32_t total = per_level * static_cast<uint32_t>(p.levels);
  for (uint32_t pass = 0;; ++pass) {
  for (;;) {
    uint32_t item = 0;
    if (lane == 0)
      item = ld_relaxed_s32(p.error) != 0 ? 0xffffffffu : atomicAdd(p.ticket, 1u);
    item = __shfl_sync(0xffffffffu, item, 0);
    if (item >= total) {
      if (lane == 0 && p.exited)
        atomicAdd(p.exited, 1u);
      break;
    }
    const int li = static_cast<int>(item / per_level);
    const uint32_t rem = item % per_level;
    const uint32_t rr = rem / p.num_graphs;
    const int g = static_cast<int>(rem % p.num_graphs);
    const int r = static_cast<int>(rr / S), r2 = static_cast<int>(rr % S);
    const BnbGraph G = p.graphs[g];
    const int k = G.ub0 - 1 - li;
    if (r >= G.n || r2 >= (p.split ? G.n : 1) || k < G.lb0)
      continue;
    const size_t item_idx = ((size_t(g) * p.levels + li) * p.max_n + r) * S + r2;
    const uint32_t istate = p.item_state[item_idx];
    if (istate == kItemDone)
      continue;  // finished in an earlier round
    int useful = 0;
    if (lane == 0) {
      const unsigned long long now = global_ns();
      atomicMin(p.t0, now);
      atomicCAS(reinterpret_cast<unsigned long long*>(p.t_begin + g), 0ull, now);
      const int bk = static_cast<int>(ld_acquire_u32(p.best + g) >> 8);
      const int lk = static_cast<int>(ld_acquire_u32(p.lbp + g));
      useful = bk > k && lk <= k && ld_relaxed_s32(p.status + g) != kBnbTimeout;
      // window: the top level is best - 1, or the hint clamped into [lbp, best - 1]
      const int top = G.hint > 0 ? min(bk - 1, max(G.hint, lk)) : bk - 1;
      if (useful && p.window && (k > top || k <= top - p.window))
        useful = 2;  // outside the window: a later pass
    }
    useful = __shfl_sync(0xffffffffu, useful, 0);
    if (useful == 2)
      continue;
    if (!useful) {
      // best only falls, the proven bound only rises and a timeout is final:
      // a useless item stays useless
      if (lane == 0)
        p.item_state[item_idx] = kItemDone;
      continue;
    }
    if (g != cur_g) {
      load_graph(w, p, G, lane);
      cur_g = g;
    }
    const int v = w->order[r];
    uint64_t fl, fh;
    full_set(G.n, fl, fh);
    Search s{w, lane, G.n, p.memo + G.memo_off, p.memo_mask, StopCheck{}, 0ull, false, false};
    s.mini = p.mini ? p.mini + (size_t(blockIdx.x) * kBnbWarps + warp) * (1u << kMiniMax) : nullptr;
    s.stop.best = p.best + g;
    s.stop.lbp = p.lbp + g;
    s.stop.item_k = k;
    s.stop.budget = p.budget ? (p.budget << istate) : 0;
    s.stop.exited = p.exited;
    s.stop.drain_at = p.drain_at;
    s.stop.full_at = p.full_at;
    s.stop.error = p.error;
    if (lane == 0 && p.exited)
      atomicAdd(p.exited + 1, 1u);
    if (p.deadline_ns) {
      uint64_t b = 0;
      if (lane == 0)
        b = *reinterpret_cast<volatile uint64_t*>(p.t_begin + g);
      s.stop.deadline = __shfl_sync(0xffffffffu, b, 0) + p.deadline_ns;
    }
    bool ok = false;
    int u = -1;  // fixed second root (split items)
    const bool skip = G.n >= 3 && s.dominated(v, fl, fh);  // another root is at least as good
    if (!skip && !p.split) {
      ok = s.decide(fl, fh, k, v, nullptr);
    } else if (!skip) {
      // Split item (v, order[r2]): when C - v is connected, decide C - v under
      // root u at depth k - 1; else item r2 = 0 decides all of v and the
      // others have nothing to do (they count as failed).
      uint64_t cl = fl, ch = fh;
      bit_clear(cl, ch, v);
      bool conn = false;
      if (G.n >= 3) {
        uint64_t dl, dh;
        s.component(cl, ch, first128(cl, ch), dl, dh);
        conn = dl == cl && dh == ch;
      }
      if (!conn) {
        if (r2 == 0)
          ok = s.decide(fl, fh, k, v, nullptr);
      } else {
        const int cand = w->order[r2];
        // u = v, or u dominated as a root of C - v: another second root is at least as good
        if (cand != v && !(G.n - 1 >= 3 && s.dominated(cand, cl, ch))) {
          ok = s.decide(cl, ch, k - 1, cand, nullptr);
          u = cand;
        }
      }
    }
    // A success is published only with its tree: the first success of a
    // level claims the level's parent buffer and builds the tree while the
    // memo entries of its search are fresh; later successes of the level
    // are redundant.
    bool publish = false;
    if (ok) {
      int claimed = 0;
      if (lane == 0)
        claimed = atomicCAS(p.claim + size_t(g) * p.levels + li, 0u, 1u) == 0u;
      claimed = __shfl_sync(0xffffffffu, claimed, 0);
      if (claimed) {
        int8_t* tree = p.lvl_parent + (size_t(g) * p.levels + li) * p.max_n;
        s.stop.budget = 0;  // the tree is mostly memo hits: no yield half way (nor a drain)
        publish = s.build_tree(fl, fh, k, v, tree, ok ? u : -1);
        if (!publish && !s.timed_out && !s.cancelled && lane == 0)
          raise_error(p.error, kDevNoRoot, g);
        __threadfence();
      }
    }
    if (lane == 0) {
      atomicAdd(p.nodes + g, s.nodes);
      if (s.yielded && !s.timed_out && !s.cancelled) {
        atomicAdd(p.unfinished, 1u);  // run again next pass with twice the budget
        p.item_state[item_idx] = static_cast<uint8_t>(min(istate + 1, kMaxDoublings));
      } else {
        p.item_state[item_idx] = kItemDone;
      }
      if (s.timed_out) {
        atomicExch(p.status + g, kBnbTimeout);
      } else if (!s.cancelled && !s.yielded) {
        if (ok) {
          if (publish)
            atomicMin(p.best + g, (static_cast<uint32_t>(k) << 8) | static_cast<uint32_t>(v));
        } else if (atomicAdd(p.fails + size_t(g) * p.levels + li, 1u) + 1 ==
                   static_cast<uint32_t>(p.split ? G.n * G.n : G.n)) {
          atomicMax(p.lbp + g, static_cast<uint32_t>(k + 1));  // every root failed: td > k
        }
        check_proved(p, g);
      }
    }
    __syncwarp();
  }
  if (!next_pass(p, pass))
    break;
  }
}

// One warp per graph: td and tree of the best level (or the seed's).
__global__ void bnb_tree_kernel(const __grid_constant__ BnbParams p) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int g = blockIdx.x * kBnbWarps + warp; g < p.num_graphs; g += gridDim.x * kBnbWarps) {
    const BnbGraph G = p.graphs[g];
    int32_t* parent = p.parent_out + G.adj_off;
    const uint32_t b = p.best[g];
    const int td = static_cast<int>(b >> 8), root = static_cast<int>(b & 0xFF);
    if (lane == 0)
      p.td_out[G.out_idx] = td;
    if (root == static_cast<int>(kSeedRoot)) {
      for (int v = lane; v < G.n; v += 32)
        parent[v] = p.seed_parent[G.adj_off + v];
      continue;
    }
    const int li = G.ub0 - 1 - td;
    const int8_t* tree = p.lvl_parent + (size_t(g) * p.levels + li) * p.max_n;
    for (int v = lane; v < G.n; v += 32)
      parent[v] = tree[v];
  }
}

}  // namespace gtd

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------

using namespace gtd;

namespace {

using u128 = unsigned __int128;

u128 mask_of(const uint64_t* adj2, int v) { return (u128(adj2[2 * v + 1]) << 64) | adj2[2 * v]; }

bool connected128(const uint64_t* adj2, int n) {
  u128 seen = 1, frontier = 1;
  const u128 all = n == 128 ? ~u128(0) : ((u128(1) << n) - 1);
  while (frontier) {
    u128 nb = 0;
    for (int v = 0; v < n; ++v)
      if ((frontier >> v) & 1)
        nb |= mask_of(adj2, v);
    nb &= all & ~seen;
    seen |= nb;
    frontier = nb;
  }
  return seen == all;
}

gtd_status check_graph128(gtd_handle h, const uint64_t* adj2, int n, int idx) {
  const std::string pre = "graph " + std::to_string(idx) + ": ";
  if (n < 1 || n > GTD_BNB_MAX_N)
    return fail(h, GTD_INVALID_ARG, pre + "n out of range [1, " + std::to_string(GTD_BNB_MAX_N) + "]");
  const u128 all = (u128(1) << n) - 1;
  for (int v = 0; v < n; ++v) {
    const u128 a = mask_of(adj2, v);
    if ((a >> v) & 1)
      return fail(h, GTD_INVALID_ARG, pre + "Self loops are not allowed");
    if (a & ~all)
      return fail(h, GTD_INVALID_ARG, pre + "adjacency bit >= n");
    for (int u = 0; u < n; ++u)
      if (((a >> u) & 1) != ((mask_of(adj2, u) >> v) & 1))
        return fail(h, GTD_INVALID_ARG, pre + "adjacency is not symmetric");
  }
  if (!connected128(adj2, n))
    return fail(h, GTD_NOT_CONNECTED, pre + "EliminationTree works only on connected graphs");
  return GTD_OK;
}

int edge_lb_host(int nv, int e) {
  for (int d = 1; d <= nv; ++d)
    if (static_cast<long long>(d - 1) * (2 * nv - d) >= 2ll * e)
      return d;
  return nv;
}

// Minor-min-width bound of the whole graph (host), td >= tw bound + 1.
int mmd_host(const uint64_t* adj2, int n) {
  std::vector<u128> a(n);
  for (int v = 0; v < n; ++v)
    a[v] = mask_of(adj2, v);
  u128 R = (u128(1) << n) - 1;
  auto popc = [](u128 x) {
    return __builtin_popcountll(static_cast<uint64_t>(x)) + __builtin_popcountll(static_cast<uint64_t>(x >> 64));
  };
  int lb = 0;
  for (int remaining = n; remaining > 1; --remaining) {
    int v = -1, d = 1 << 30;
    for (int x = 0; x < n; ++x)
      if (((R >> x) & 1) && popc(a[x]) < d) {
        d = popc(a[x]);
        v = x;
      }
    lb = std::max(lb, d);
    int u = -1, du = 1 << 30;
    for (int x = 0; x < n; ++x)
      if (((a[v] >> x) & 1) && popc(a[x]) < du) {
        du = popc(a[x]);
        u = x;
      }
    const u128 nv = a[v];
    for (int x = 0; x < n; ++x) {
      if (!((R >> x) & 1) || x == v)
        continue;
      if (x == u)
        a[x] = (a[x] | nv) & ~(u128(1) << u) & ~(u128(1) << v);
      else if ((nv >> x) & 1)
        a[x] = (a[x] & ~(u128(1) << v)) | (u >= 0 ? (u128(1) << u) : 0);
    }
    a[v] = 0;
    R &= ~(u128(1) << v);
  }
  return lb + 1;
}

template <typename T>
gtd_status grow(gtd_handle h, T** p, size_t* cap, size_t count) {
  GTD_CUDA(h, ensure_field(p, cap, count));
  return GTD_OK;
}

}  // namespace

// Branch-and-bound buffers of a handle.
struct gtd_bnb_state {
  BnbGraph* graphs = nullptr;
  size_t graphs_cap = 0;
  uint64_t* adj = nullptr;
  size_t adj_cap = 0;
  uint8_t* order = nullptr;
  size_t order_cap = 0;
  uint4* memo = nullptr;
  size_t memo_cap = 0;
  int32_t* i32 = nullptr;  // seed parents, parents, td, status
  size_t i32_cap = 0;
  uint32_t* u32 = nullptr; // best, lbp, fails
  size_t u32_cap = 0;
  uint64_t* u64 = nullptr; // t_begin, t_end, nodes, t0
  size_t u64_cap = 0;
  int8_t* i8 = nullptr;    // per-level trees
  size_t i8_cap = 0;
  uint8_t* mini = nullptr; // per-warp small-component DP tables
  size_t mini_cap = 0;
  std::vector<int32_t> last_lb;  // proven lower bound per graph of the last solve
};

void gtd_bnb_release(gtd_handle h) {
  if (!h->bnb)
    return;
  gtd_bnb_state* b = h->bnb;
  cudaFree(b->graphs);
  cudaFree(b->adj);
  cudaFree(b->order);
  cudaFree(b->memo);
  cudaFree(b->i32);
  cudaFree(b->u32);
  cudaFree(b->u64);
  cudaFree(b->i8);
  cudaFree(b->mini);
  delete b;
  h->bnb = nullptr;
}

extern "C" gtd_status gtd_bnb_solve_batch(gtd_handle h, const gtd_graph_desc* descs, int count,
                                          const uint64_t* adj2_pool, int64_t pool_len, const uint8_t* order_pool,
                                          const int32_t* seed_td, const int32_t* seed_parent, int32_t* td_out,
                                          int32_t* parent_out, int32_t* status_out, float* proof_ms_out,
                                          uint64_t* nodes_out, const gtd_bnb_opts* opts, gtd_bnb_stats* stats) {
  if (!h)
    return GTD_INVALID_ARG;
  if (!descs || count < 1 || !adj2_pool || !seed_td || !seed_parent || !td_out || !parent_out || !status_out)
    return fail(h, GTD_INVALID_ARG, "null pointer argument or empty batch");
  int max_n = 0;
  for (int i = 0; i < count; ++i) {
    const gtd_graph_desc& d = descs[i];
    if (d.offset < 0 || int64_t(d.offset) + d.n > pool_len)
      return fail(h, GTD_INVALID_ARG, "graph " + std::to_string(i) + ": offset outside the pool");
    gtd_status s = check_graph128(h, adj2_pool + 2 * size_t(d.offset), d.n, i);
    if (s != GTD_OK)
      return s;
    if (seed_td[i] < 1 || seed_td[i] > d.n)
      return fail(h, GTD_INVALID_ARG, "graph " + std::to_string(i) + ": seed treedepth out of range");
    max_n = std::max(max_n, d.n);
  }
  const auto t_call = std::chrono::steady_clock::now();
  DeviceGuard guard(h->device);
  if (!h->bnb)
    h->bnb = new gtd_bnb_state();
  gtd_bnb_state& B = *h->bnb;
  int memo_log2 = (opts && opts->memo_log2 > 0) ? std::min(opts->memo_log2, 26) : 0;
  if (memo_log2 == 0) {
    // HBM is the memo: up to a quarter of the free memory (at most 32 GiB),
    // 2^16 .. 2^24 slots of 16 bytes per graph
    size_t free_b = 0, total_b = 0;
    GTD_CUDA(h, cudaMemGetInfo(&free_b, &total_b));
    const size_t budget = std::min(free_b / 4 + B.memo_cap * sizeof(uint4), size_t(32) << 30);
    const size_t per_graph = budget / sizeof(uint4) / size_t(count);
    memo_log2 = 16;
    while (memo_log2 < 24 && (size_t(1) << (memo_log2 + 1)) <= per_graph)
      ++memo_log2;
  }
  const size_t slots = size_t(1) << memo_log2;

  std::vector<BnbGraph> graphs(count);
  std::vector<uint8_t> order(static_cast<size_t>(pool_len) + 1);
  std::vector<uint32_t> best(count), lbp(count);
  int levels = 1;
  for (int i = 0; i < count; ++i) {
    const gtd_graph_desc& d = descs[i];
    const uint64_t* a = adj2_pool + 2 * size_t(d.offset);
    BnbGraph& G = graphs[i];
    G.adj_off = static_cast<uint32_t>(d.offset);
    G.out_idx = static_cast<uint32_t>(i);
    G.memo_off = slots * i;
    G.n = d.n;
    int e = 0;
    for (int v = 0; v < d.n; ++v)
      e += __builtin_popcountll(a[2 * v]) + __builtin_popcountll(a[2 * v + 1]);
    G.lb0 = std::max(edge_lb_host(d.n, e / 2), d.n >= 2 ? mmd_host(a, d.n) : 1);
    G.ub0 = seed_td[i];
    G.hint = (opts && opts->level_hint) ? std::max(0, std::min(opts->level_hint[i], d.n)) : 0;
    if (G.lb0 > G.ub0)
      return fail(h, GTD_INVALID_ARG, "graph " + std::to_string(i) + ": seed treedepth below a lower bound");
    levels = std::max(levels, G.ub0 - G.lb0);
    for (int r = 0; r < d.n; ++r)
      order[d.offset + r] = order_pool ? order_pool[d.offset + r] : static_cast<uint8_t>(r);
    if (order_pool) {
      std::vector<char> seen(d.n, 0);
      for (int r = 0; r < d.n; ++r) {
        const int v = order[d.offset + r];
        if (v >= d.n || seen[v])
          return fail(h, GTD_INVALID_ARG, "graph " + std::to_string(i) + ": order is not a permutation");
        seen[v] = 1;
      }
    }
    best[i] = (static_cast<uint32_t>(G.ub0) << 8) | kSeedRoot;
    lbp[i] = static_cast<uint32_t>(G.lb0);
  }

  gtd_status s;
  if ((s = grow(h, &B.graphs, &B.graphs_cap, count)) != GTD_OK) return s;
  if ((s = grow(h, &B.adj, &B.adj_cap, 2 * size_t(pool_len))) != GTD_OK) return s;
  if ((s = grow(h, &B.order, &B.order_cap, size_t(pool_len) + 16)) != GTD_OK) return s;
  if ((s = grow(h, &B.memo, &B.memo_cap, slots * count)) != GTD_OK) return s;
  if ((s = grow(h, &B.i32, &B.i32_cap, 2 * size_t(pool_len) + 2 * size_t(count))) != GTD_OK) return s;
  if ((s = grow(h, &B.u32, &B.u32_cap, size_t(count) * (2 + 2 * size_t(levels)))) != GTD_OK) return s;
  // Split items (first root x second root) when the batch is too small to
  // give every warp a first-root item: a single graph then uses n^2 warps.
  size_t first_items = 0;
  for (int i = 0; i < count; ++i)
    first_items += size_t(descs[i].n) * std::min(levels, kRoundWindow);
  const int split = (first_items < size_t(h->num_sms) * 16 &&
                     size_t(count) * levels * max_n * max_n < (size_t(1) << 31)) ? 1 : 0;
  const size_t S = split ? size_t(max_n) : 1;
  if ((s = grow(h, &B.i8, &B.i8_cap, size_t(count) * levels * max_n * (1 + S))) != GTD_OK) return s;
  if ((s = grow(h, &B.u64, &B.u64_cap, 3 * size_t(count) + 1)) != GTD_OK) return s;
  int32_t* d_seed_parent = B.i32;
  int32_t* d_parent = B.i32 + pool_len;
  int32_t* d_td = B.i32 + 2 * pool_len;
  int32_t* d_status = d_td + count;
  uint32_t* d_best = B.u32;
  uint32_t* d_lbp = B.u32 + count;
  uint32_t* d_fails = B.u32 + 2 * count;
  uint32_t* d_claim = d_fails + size_t(count) * levels;
  uint64_t* d_tbeg = B.u64;
  uint64_t* d_tend = B.u64 + count;
  uint64_t* d_nodes = B.u64 + 2 * count;
  uint64_t* d_t0 = B.u64 + 3 * count;

  // plain (pageable) copies: this entry point is host-synchronous anyway
  GTD_CUDA(h, cudaMemcpyAsync(B.graphs, graphs.data(), count * sizeof(BnbGraph), cudaMemcpyHostToDevice, h->stream));
  GTD_CUDA(h, cudaMemcpyAsync(B.adj, adj2_pool, 2 * size_t(pool_len) * sizeof(uint64_t), cudaMemcpyHostToDevice,
                              h->stream));
  GTD_CUDA(h, cudaMemcpyAsync(B.order, order.data(), size_t(pool_len), cudaMemcpyHostToDevice, h->stream));
  GTD_CUDA(h, cudaMemcpyAsync(d_seed_parent, seed_parent, size_t(pool_len) * sizeof(int32_t), cudaMemcpyHostToDevice,
                              h->stream));
  GTD_CUDA(h, cudaMemcpyAsync(d_best, best.data(), count * sizeof(uint32_t), cudaMemcpyHostToDevice, h->stream));
  GTD_CUDA(h, cudaMemcpyAsync(d_lbp, lbp.data(), count * sizeof(uint32_t), cudaMemcpyHostToDevice, h->stream));
  GTD_CUDA(h, cudaMemsetAsync(d_fails, 0, 2 * size_t(count) * levels * sizeof(uint32_t), h->stream));
  GTD_CUDA(h, cudaMemsetAsync(B.i8 + size_t(count) * levels * max_n, 0, size_t(count) * levels * max_n * S,
                              h->stream));
  GTD_CUDA(h, cudaMemsetAsync(B.memo, 0, slots * count * sizeof(uint4), h->stream));
  GTD_CUDA(h, cudaMemsetAsync(d_status, 0, count * sizeof(int32_t), h->stream));
  GTD_CUDA(h, cudaMemsetAsync(B.u64, 0, 3 * size_t(count) * sizeof(uint64_t), h->stream));
  GTD_CUDA(h, cudaMemsetAsync(d_t0, 0xFF, sizeof(uint64_t), h->stream));
  GTD_CUDA(h, cudaMemsetAsync(h->d_io, 0, 4 * sizeof(int32_t), h->stream));

  BnbParams p;
  p.graphs = B.graphs;
  p.num_graphs = count;
  p.max_n = max_n;
  p.levels = levels;
  p.adj = B.adj;
  p.order = B.order;
  p.memo = B.memo;
  p.memo_mask = static_cast<uint32_t>(slots - 1);
  p.best = d_best;
  p.lbp = d_lbp;
  p.fails = d_fails;
  p.claim = d_claim;
  p.lvl_parent = B.i8;
  p.item_state = reinterpret_cast<uint8_t*>(B.i8 + size_t(count) * levels * max_n);
  p.split = split;
  p.unfinished = reinterpret_cast<uint32_t*>(h->d_io + kIoUnfinished);
  p.exited = reinterpret_cast<uint32_t*>(h->d_io + kIoExited);
  p.window = (opts && opts->window > 0) ? opts->window : kRoundWindow;
  p.status = d_status;
  p.t_begin = d_tbeg;
  p.t_end = reinterpret_cast<unsigned long long*>(d_tend);
  p.t0 = reinterpret_cast<unsigned long long*>(d_t0);
  p.nodes = reinterpret_cast<unsigned long long*>(d_nodes);
  p.ticket = reinterpret_cast<uint32_t*>(h->d_io + kIoTicket);
  p.error = h->d_io + kIoError;
  p.deadline_ns = (opts && opts->deadline_ns) ? opts->deadline_ns : 120ull * 1000 * 1000 * 1000;
  p.seed_parent = d_seed_parent;
  p.td_out = d_td;
  p.parent_out = d_parent;

  const size_t smem = sizeof(WarpMem) * kBnbWarps;
  GTD_CUDA(h, cudaFuncSetAttribute(bnb_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
  int occ = 0;
  GTD_CUDA(h, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, bnb_kernel, 32 * kBnbWarps, smem));
  if (opts && opts->ctas_per_sm > 0 && opts->ctas_per_sm < occ)
    occ = opts->ctas_per_sm;
  if (occ < 1)
    occ = 1;
  const long long items = static_cast<long long>(count) * max_n * levels * static_cast<long long>(S);
  const long long ctas =
      std::max(1ll, std::min<long long>(static_cast<long long>(h->num_sms) * occ, (items + kBnbWarps - 1) / kBnbWarps));
  p.drain_at = static_cast<uint32_t>(std::max(1ll, ctas * kBnbWarps / 2));
  if ((s = grow(h, &B.mini, &B.mini_cap, size_t(ctas) * kBnbWarps * (size_t(1) << kMiniMax))) != GTD_OK) return s;
  p.mini = B.mini;
  p.full_at = static_cast<uint32_t>(ctas * kBnbWarps);
  // One cooperative launch runs every pass: each item may spend its node
  // budget per pass (twice its last one after a yield), and the last warp of
  // a pass starts the next one until every graph is proven or past its
  // deadline (next_pass). Cooperative: every CTA is resident, so the warps
  // waiting at the end of a pass never wait on a CTA that cannot run.
  p.budget = (opts && opts->first_budget) ? opts->first_budget : kFirstBudget;
  p.pass_done = reinterpret_cast<uint32_t*>(h->d_io + kIoPassDone);
  p.pass_gen = reinterpret_cast<uint32_t*>(h->d_io + kIoPassGen);
  p.pass_stop = reinterpret_cast<uint32_t*>(h->d_io + kIoPassStop);
  p.pass_wait_ns = p.deadline_ns + 30ull * 1000 * 1000 * 1000;
  GTD_CUDA(h, cudaMemsetAsync(h->d_io + kIoExited, 0, 5 * sizeof(int32_t), h->stream));
  GTD_CUDA(h, cudaEventRecord(h->ev[0], h->stream));
  {
    void* args[] = {&p};
    GTD_CUDA(h, cudaLaunchCooperativeKernel(reinterpret_cast<void*>(bnb_kernel), dim3(static_cast<unsigned>(ctas)),
                                            dim3(32 * kBnbWarps), args, smem, h->stream));
  }
  const int tree_ctas = std::min(4096, (count + kBnbWarps - 1) / kBnbWarps);
  bnb_tree_kernel<<<tree_ctas, 32 * kBnbWarps, 0, h->stream>>>(p);
  GTD_CUDA(h, cudaGetLastError());
  GTD_CUDA(h, cudaEventRecord(h->ev[1], h->stream));

  std::vector<int32_t> st(count);
  std::vector<uint32_t> bst(count), lb(count);
  std::vector<uint64_t> te(count), nd(count);
  uint64_t t_first = 0;
  int32_t io[4] = {0, 0, 0, 0};
  std::vector<int32_t> par(static_cast<size_t>(pool_len));
  GTD_CUDA(h, cudaMemcpyAsync(td_out, d_td, count * sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
  GTD_CUDA(h, cudaMemcpyAsync(st.data(), d_status, count * sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
  GTD_CUDA(h, cudaMemcpyAsync(bst.data(), d_best, count * sizeof(uint32_t), cudaMemcpyDeviceToHost, h->stream));
  GTD_CUDA(h, cudaMemcpyAsync(lb.data(), d_lbp, count * sizeof(uint32_t), cudaMemcpyDeviceToHost, h->stream));
  GTD_CUDA(h, cudaMemcpyAsync(te.data(), d_tend, count * sizeof(uint64_t), cudaMemcpyDeviceToHost, h->stream));
  GTD_CUDA(h, cudaMemcpyAsync(nd.data(), d_nodes, count * sizeof(uint64_t), cudaMemcpyDeviceToHost, h->stream));
  GTD_CUDA(h, cudaMemcpyAsync(&t_first, d_t0, sizeof(uint64_t), cudaMemcpyDeviceToHost, h->stream));
  GTD_CUDA(h, cudaMemcpyAsync(io, h->d_io, 4 * sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
  uint32_t passes = 0;
  GTD_CUDA(h, cudaMemcpyAsync(&passes, h->d_io + kIoPassGen, sizeof(uint32_t), cudaMemcpyDeviceToHost, h->stream));
  GTD_CUDA(h, cudaMemcpyAsync(par.data(), d_parent, size_t(pool_len) * sizeof(int32_t), cudaMemcpyDeviceToHost,
                              h->stream));
  GTD_CUDA(h, cudaStreamSynchronize(h->stream));
  gtd_status es = map_device_error(h, io[1], io[2]);
  if (es != GTD_OK)
    return es;
  uint64_t total_nodes = 0;
  B.last_lb.assign(count, 0);
  for (int i = 0; i < count; ++i) {
    const gtd_graph_desc& d = descs[i];
    B.last_lb[i] = static_cast<int32_t>(std::min(lb[i], bst[i] >> 8));
    std::memcpy(parent_out + d.offset, par.data() + d.offset, d.n * sizeof(int32_t));
    const bool proved = lb[i] >= (bst[i] >> 8);
    status_out[i] = proved ? GTD_OK : GTD_TIMEOUT;
    if (proof_ms_out)
      proof_ms_out[i] = (proved && te[i] > t_first) ? float(double(te[i] - t_first) * 1e-6) : (proved ? 0.f : -1.f);
    if (nodes_out)
      nodes_out[i] = nd[i];
    total_nodes += nd[i];
  }
  if (stats) {
    float ms = 0;
    cudaEventElapsedTime(&ms, h->ev[0], h->ev[1]);
    stats->ms = ms;
    stats->nodes = total_nodes;
    stats->passes = static_cast<int32_t>(passes);
    stats->total_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t_call).count();
  }
  return GTD_OK;
}

extern "C" gtd_status gtd_bnb_lower_bounds(gtd_handle h, int32_t* lb_out, int count) {
  if (!h)
    return GTD_INVALID_ARG;
  if (!h->bnb || h->bnb->last_lb.empty())
    return fail(h, GTD_NO_RESULT, "no branch-and-bound solve yet");
  if (!lb_out || count != static_cast<int>(h->bnb->last_lb.size()))
    return fail(h, GTD_INVALID_ARG, "count must be the last solve's batch size");
  std::memcpy(lb_out, h->bnb->last_lb.data(), sizeof(int32_t) * count);
  return GTD_OK;
}
