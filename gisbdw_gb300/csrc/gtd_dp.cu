// K1: the level-by-level subset DP for exact treedepth on sm_103a.
//
// Reference: DynamicGPU (Treedepth/src/dynamic_gpu/dynamic_gpu.cu:40-201),
// which runs one thread per k-subset per level, labels components by repeated
// CSR sweeps, re-encodes S - v with 64-bit divides and gathers 8-byte
// {td, root} entries at random. This kernel computes the same table values
// with a different schedule and layout:
//
//  * Recurrence. For |S| >= 3, S is connected iff at least two v in S leave
//    S - v connected (a connected graph has >= 2 non-cut vertices, and if
//    S - u and S - v are connected, u has a neighbour in S - v). For a
//    disconnected S, td(S) = max_v td(S - v) (treedepth is monotone under
//    vertex deletion, and deleting a vertex outside a deepest component keeps
//    it). So every subset is resolved from its |S| children S - v alone:
//      T[S] = 1 + min_v T[S - v]   (connected; dynamic_gpu.cu:68-89)
//      T[S] = max_v T[S - v]       (disconnected; = max over components,
//                                   dynamic_gpu.cu:90-111)
//    with each table byte holding td << 1 | connected. No per-subset BFS, no
//    ranking per child.
//  * Reduction. Deleting a vertex lowers treedepth by at most one, so the
//    children's treedepths are td(S) - 1 or td(S): two consecutive values at
//    most. Their OR plus their AND is then 2a + 1 when both a and a + 1
//    occur (td(S) = a + 1, connected or not) and 2v when all equal v
//    (td(S) = v + connected(S)), so with s = OR + AND,
//      td(S) = (s >> 1) + ((s & 1) | connected(S)).
//    OR and AND of the raw bytes are plain 32-bit logic over 4 subsets at
//    once; a third word collects "at least two connected children" in bit 0.
//  * Layout (gtd_dp_layout.h). Tiles of 2^lb subsets share a high part H;
//    a tile's cross-tile children are the whole tiles H - h one level down,
//    read as contiguous 2^lb-byte blocks (16-byte vector loads through L2);
//    the in-tile children are resolved in shared memory, 4 subsets per
//    32-bit word, words in popcount order of the word index, one unrolled
//    pass per popcount class (its size and child count compile-time).
//  * Schedule. One persistent launch; every warp is an independent tile
//    worker (no CTA barriers in the loop). A warp takes a tile by ticket
//    (atomicAdd) in level-major order and decodes it with ballots over a
//    shared-memory binomial table; lane v in H ranks child tile H - v by a
//    prefix and a suffix sum and waits on its ready flag (each wait bounded
//    by a deadline). The warp reduces the cross-tile children with OR / AND /
//    majority logic on 16-byte loads, keeps that summary as two virtual
//    children in shared memory, resolves the tile there, stores it and
//    publishes its flag with a release store. A tile only waits on tiles
//    with smaller tickets, and a ticket is only taken by a running warp, so
//    the smallest unfinished ticket can always proceed.
//
// Reconstruction (dp_tree_kernel): one warp, one lane per vertex, rebuilds
// the reference's tree (first-argmin root per component, dynamic_gpu.cu:84-87,
// dynamic_cpu.hpp:59-81) and GetElimination order (dynamic_gpu.hpp:48-64).
#include <cuda_runtime.h>

#include <cstdint>

#include "gtd_device.cuh"
#include "gtd_dp_kernels.h"

namespace gtd {

// One warp resolves one tile; a CTA holds kDpWarps independent tile workers
// that share only the adjacency and the word order table.
constexpr int kDpWarps = 4;

template <int LB>
struct TileShape {
  static constexpr int kEntries = 1 << LB;
  static constexpr int kWords = kEntries / 4;   // 4 subsets per 32-bit word
  static constexpr int kWordBits = LB - 2;
  // dynamic shared memory: per warp T and U (kWords words each), then, for
  // the CTA, the word order (kWords uint16) and a copy of the binomial
  // table, then per warp the child-tile list (32 words). Between the two
  // phases T and U hold the cross-tile children's summary as two virtual
  // children (see the in-tile loop); T then receives the tile.
  static constexpr size_t kPerWarp = size_t(2) * kWords * 4;
  static constexpr size_t kOrderOff = size_t(kDpWarps) * kPerWarp;
  static constexpr size_t kBinomOff = (kOrderOff + kWords * 2 + 15) & ~size_t(15);
  static constexpr size_t kKidsOff = (kBinomOff + sizeof(uint32_t) * (kDpMaxHigh + 1) * (kDpMaxHigh + 1) + 15) &
                                     ~size_t(15);
  static constexpr size_t kSmem = kKidsOff + size_t(kDpWarps) * 32 * 4;
};

using Binom = uint32_t[kDpMaxHigh + 1][kDpMaxHigh + 1];

// Per word (4 subsets, one per byte): o = OR and a = AND of the children's
// bytes, d = "at least two connected children" in bit 0 of each byte.
struct Acc {
  uint32_t o, a, d;
};

__device__ __forceinline__ void acc_init(Acc& c) {
  c.o = 0u;
  c.a = 0xFFFFFFFFu;
  c.d = 0u;
}

__device__ __forceinline__ void acc_add2(Acc& c, uint32_t x, uint32_t y) {
  c.d |= (c.o & (x | y)) | (x & y);  // majority of (any before, x, y)
  c.o |= x | y;
  c.a &= x & y;
}

__device__ __forceinline__ void acc_add3(Acc& c, uint32_t x, uint32_t y, uint32_t z) {
  const uint32_t any = x | y | z;
  c.d |= (c.o & any) | (x & y) | (x & z) | (y & z);  // at least two of (any before, x, y, z)
  c.o |= any;
  c.a &= x & y & z;
}

__device__ __forceinline__ void acc_add1(Acc& c, uint32_t x) {
  c.d |= c.o & x;
  c.o |= x;
  c.a &= x;
}

// Four subsets with |S| >= 3 (connected <=> >= 2 connected children) and at
// least one child each: per byte s = OR(td) + AND(td) <= 126, so no carries;
// td = (s >> 1) + ((s & 1) | connected), stored as td << 1 | connected.
__device__ __forceinline__ uint32_t resolve4(uint32_t o, uint32_t a, uint32_t d) {
  const uint32_t s = ((o & 0xFEFEFEFEu) + (a & 0xFEFEFEFEu)) >> 1;
  const uint32_t half = (s & 0xFEFEFEFEu) | (d & 0x01010101u);  // 2 (s >> 1) | connected
  return half + (((s | d) & 0x01010101u) << 1);
}

__device__ __forceinline__ bool adjacent_in(const uint64_t* adj, int n, uint64_t s2) {
  const int u = __ffsll(static_cast<long long>(s2)) - 1;
  const int v = 63 - __clzll(static_cast<long long>(s2));
  return u < n && v < n && ((__ldg(adj + u) >> v) & 1ull);
}

// One subset of size k from its children's OR o, AND a and count flag d;
// `adjacent` gives connectivity when k == 2.
__device__ __forceinline__ uint32_t resolve1(uint32_t o, uint32_t a, uint32_t d, int k, bool adjacent) {
  if (k == 0)
    return 0u;  // empty set: td 0
  const uint32_t cn = k == 1 ? 1u : k == 2 ? (adjacent ? 1u : 0u) : (d & 1u);
  const uint32_t s = ((o & 0xFEu) + (a & 0xFEu)) >> 1;
  return ((s & 0xFEu) + (((s | cn) & 1u) << 1)) | cn;
}

__device__ __forceinline__ void fold1(uint32_t& o, uint32_t& a, uint32_t& d, uint32_t v) {
  d |= o & v;
  o |= v;
  a &= v;
}

__device__ __forceinline__ void fold2(uint32_t& o, uint32_t& a, uint32_t& d, uint32_t x, uint32_t y) {
  d |= (o & (x | y)) | (x & y);  // majority of (any before, x, y)
  o |= x | y;
  a &= x & y;
}

// The word's four subsets (low bits 00, 01, 10, 11), all of size >= 3, from
// the summary (o, a, d) of their children outside the word: subset 00 is
// final first and is folded into 01 and 10, which are then final and are
// folded into 11.
__device__ __forceinline__ uint32_t resolve_word(uint32_t o, uint32_t a, uint32_t d) {
  uint32_t v = resolve4(o, a, d);
  const uint32_t x = __byte_perm(v, 0u, 0x4004u);  // byte 0 into bytes 1 and 2
  d |= o & x;
  o |= x;
  a &= x | 0xFF0000FFu;
  v = resolve4(o, a, d);
  const uint32_t y1 = __byte_perm(v, 0u, 0x1444u), y2 = __byte_perm(v, 0u, 0x2444u);  // bytes 1, 2 into 3
  d |= (o & (y1 | y2)) | (y1 & y2);
  o |= y1 | y2;
  a &= (y1 & y2) | 0x00FFFFFFu;
  return resolve4(o, a, d);
}

// The same for a word that may hold subsets of size <= 2 (k = |S| of its
// subset 00; S0 the subset 00 itself): one byte at a time, connectivity of a
// pair from the adjacency.
__device__ __forceinline__ uint32_t resolve_word_small(uint32_t go, uint32_t ga, uint32_t gd, int k,
                                                       const uint64_t* adj, int n, uint64_t S0) {
  uint32_t o[4], a[4], d[4];
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    o[q] = (go >> (8 * q)) & 0xFFu;
    a[q] = (ga >> (8 * q)) & 0xFFu;
    d[q] = (gd >> (8 * q)) & 0xFFu;
  }
  const uint32_t v0 = resolve1(o[0], a[0], d[0], k, k == 2 && adjacent_in(adj, n, S0));
  fold1(o[1], a[1], d[1], v0);
  fold1(o[2], a[2], d[2], v0);
  const uint32_t v1 = resolve1(o[1], a[1], d[1], k + 1, k + 1 == 2 && adjacent_in(adj, n, S0 | 1u));
  const uint32_t v2 = resolve1(o[2], a[2], d[2], k + 1, k + 1 == 2 && adjacent_in(adj, n, S0 | 2u));
  fold1(o[3], a[3], d[3], v1);
  fold1(o[3], a[3], d[3], v2);
  const uint32_t v3 = resolve1(o[3], a[3], d[3], k + 2, k + 2 == 2 && adjacent_in(adj, n, S0 | 3u));
  return v0 | (v1 << 8) | (v2 << 16) | (v3 << 24);
}

// A word's summary (o, a, d) of at least one child is reproduced by two
// virtual children: o itself and a with bit 0 replaced by d. Their OR is o
// (a's bits lie inside o's, d implies o's bit 0), their AND carries a's
// treedepth bits, and both have bit 0 set exactly when d is: at least two
// connected children.
__device__ __forceinline__ uint32_t second_child(const Acc& c) {
  return (c.a & 0xFEFEFEFEu) | (c.d & 0x01010101u);
}

// Level j, high part H and start of level j - 1 of local tile t of a graph
// with nh high vertices (level-major order, colex rank inside a level),
// computed by the whole warp: lane i <= nh holds the running level total
// sum_{k <= i} C(nh, k) and a ballot counts the levels that end at or before
// t; each element of H is then the largest a < nh with C(a, k) <= r (colex
// unranking, one ballot per element, k = j .. 1).
__device__ __forceinline__ void decode_tile(const Binom& binom, int nh, uint32_t t, int& j, uint32_t& H,
                                                 uint32_t& off_prev) {
  const int lane = threadIdx.x & 31;
  uint32_t cum = lane <= nh ? binom[nh][lane] : 0u;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t x = __shfl_up_sync(0xffffffffu, cum, d);
    if (lane >= d)
      cum += x;
  }
  j = __popc(__ballot_sync(0xffffffffu, lane <= nh && cum <= t));
  const uint32_t off = __shfl_sync(0xffffffffu, cum, (j + 31) & 31);       // lane j - 1
  const uint32_t prev = __shfl_sync(0xffffffffu, cum, (j + 30) & 31);      // lane j - 2
  off_prev = j >= 2 ? prev : 0u;
  uint32_t r = t - (j >= 1 ? off : 0u);
  H = 0;
  for (int k = j; k > 0; --k) {
    const uint32_t c = lane < nh ? binom[lane][k] : 0xFFFFFFFFu;
    const int a = 31 - __clz(__ballot_sync(0xffffffffu, c <= r));
    H |= 1u << a;
    r -= binom[a][k];
  }
}

__device__ __forceinline__ uint32_t rank_colex(const Binom& binom, uint32_t H) {
  uint32_t r = 0;
  int q = 0;
  for (; H; H &= H - 1)
    r += binom[__ffs(H) - 1][++q];
  return r;
}

// Checks each graph's adjacency masks — no self loop, no bit >= n,
// symmetric — one warp per graph, lane v checking vertex v (and v + 32).
__global__ void dp_validate_kernel(const __grid_constant__ DpBatchParams p) {
  const int lane = threadIdx.x & 31;
  const int g = static_cast<int>((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  if (g >= p.num_graphs)
    return;  // the whole warp
  const DpGraph G = p.graphs ? p.graphs[g] : p.single;
  const uint64_t* adj = p.adj + G.adj_off;
  const int n = G.n;
  const uint64_t allowed = n >= 64 ? ~0ull : ((1ull << n) - 1);
  bool ok = true;
  for (int v = lane; v < n && ok; v += 32) {
    const uint64_t a = adj[v];
    if (((a >> v) & 1ull) || (a & ~allowed))
      ok = false;
    for (uint64_t s = a; s && ok; s &= s - 1)
      if (!((adj[__ffsll(static_cast<long long>(s)) - 1] >> v) & 1ull))
        ok = false;
  }
  if (__any_sync(0xffffffffu, !ok) && lane == 0)
    raise_error(p.error, kDevInvalidInput, g);
}

// Batches issue tickets level-major across graphs (every graph's level-0
// tiles, then every level-1 tile, ...), so that a tile's children lie far
// back in the ticket stream; tables and flags stay graph-major.
__global__ void dp_fill_tile_map_kernel(const __grid_constant__ DpBatchParams p) {
  for (int g = blockIdx.x; g < p.num_graphs; g += gridDim.x) {
    const DpGraph G = p.graphs[g];
    uint32_t local = 0;
    for (int j = 0; j <= G.nh; ++j) {
      const uint32_t count = p.binom[G.nh][j];
      const uint32_t base = p.level_base[size_t(g) * (kDpMaxHigh + 2) + j];
      for (uint32_t i = threadIdx.x; i < count; i += blockDim.x)
        p.tile_map[base + i] = make_uint2(static_cast<uint32_t>(g), local + i);
      local += count;
    }
  }
}

// Word indices of `bits` bits ordered by popcount, colex rank inside each
// popcount class. For a tile of fewer word bits the words of class s are the
// first C(wb, s) entries of the class (colex order lists the subsets of the
// lower positions first), so one table serves every smaller tile size.
__device__ void build_word_order(uint16_t* sOrder, const Binom& binom, int bits) {
  for (int w = threadIdx.x; w < (1 << bits); w += blockDim.x) {
    const int i = __popc(w);
    uint32_t pos = 0;
    for (int q = 0; q < i; ++q)
      pos += binom[bits][q];
    pos += rank_colex(binom, static_cast<uint32_t>(w));
    sOrder[pos] = static_cast<uint16_t>(w);
  }
}

__device__ __forceinline__ uint32_t smem_u32(const void* ptr) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(ptr));
}

__device__ __forceinline__ uint32_t lds_u32(uint32_t addr) {
  uint32_t v;
  asm volatile("ld.shared.u32 %0, [%1];" : "=r"(v) : "r"(addr));
  return v;
}

__device__ __forceinline__ void sts_u32(uint32_t addr, uint32_t v) {
  asm volatile("st.shared.u32 [%0], %1;" ::"r"(addr), "r"(v) : "memory");
}

__host__ __device__ constexpr uint32_t cbinom(int n, int k) {
  if (k < 0 || k > n)
    return 0u;
  uint64_t r = 1;
  for (int i = 1; i <= k; ++i)
    r = r * static_cast<uint64_t>(n - k + i) / static_cast<uint64_t>(i);
  return static_cast<uint32_t>(r);
}

// In-tile phase, popcount class S of the word index and every class above
// it: each lane resolves whole words of the class (listed in sOrder), whose
// in-tile children are the S words w - b (b a bit of w) of class S - 1,
// already final in T (shared address tbase); T and U (u_off bytes further)
// at w hold the cross-tile children's summary as two virtual children. The
// class size and the number of children are compile-time, so the child loop
// is unrolled and child w - b is read at A - 4b, A = tbase + 4w, the bits
// taken lowest first (r4 & (r4 - 4) drops the lowest).
template <int LB, int S>
__device__ __forceinline__ void intile_class(const DpBatchParams& p, const DpGraph& G, uint64_t Hfull, int j,
                                             uint32_t tbase, uint32_t u_off, const uint16_t* sOrder,
                                             int order_bits) {
  constexpr int kWordBits = LB - 2;
  constexpr uint32_t kCount = cbinom(kWordBits, S);
  const int lane = threadIdx.x & 31;
#pragma unroll 1
  for (uint32_t e = lane; e < kCount; e += 32) {
    const uint32_t w = sOrder[e];
    const uint32_t A = tbase + (w << 2);
    uint32_t o = 0u, a = 0xFFFFFFFFu, d = 0u;
    if (j > 0) {  // the level-0 tile has no cross-tile children
      const uint32_t x = lds_u32(A), y = lds_u32(A + u_off);
      o = x | y;
      a = x & y;
      d = a;
    }
    uint32_t r4 = w << 2;
#pragma unroll
    for (int i = 0; i + 2 <= S; i += 2) {
      const uint32_t n1 = r4 & (r4 - 4u), n2 = n1 & (n1 - 4u);
      fold2(o, a, d, lds_u32(A + n1 - r4), lds_u32(A + n2 - n1));
      r4 = n2;
    }
    if constexpr ((S & 1) != 0)
      fold1(o, a, d, lds_u32(A - r4));
    uint32_t out;
    if constexpr (S >= 3) {
      out = resolve_word(o, a, d);
    } else {
      if (j + S >= 3)
        out = resolve_word(o, a, d);
      else
        out = resolve_word_small(o, a, d, j + S, p.adj + G.adj_off, G.n, Hfull | (uint64_t(w) << 2));
    }
    sts_u32(A, out);
  }
  __syncwarp();
  if constexpr (S < kWordBits)  // the order table's class sizes (order_bits >= kWordBits)
    intile_class<LB, S + 1>(p, G, Hfull, j, tbase, u_off, sOrder + p.binom[order_bits][S], order_bits);
}

constexpr uint32_t kNoPending = 0xFFFFFFFFu;

// Publishes the ready flag p.flags[pending] of the tile this warp stored
// last. The tile's stores are warp-wide instructions of every lane; the
// warp barrier orders them before lane 0's store, and that store is a
// gpu-scope release, which is cumulative: a reader that acquires the flag
// sees every byte of the tile. (No separate fence: the release is the
// fence.) The tile loops call this right after tile_work returns, before
// the next ticket, so the flag is not delayed; keeping the release out of
// tile_work's body lets the one-size kernel fit in 43 registers, 10 CTAs
// per SM, against 55 with it inside.
__device__ __forceinline__ void publish_pending(const DpBatchParams& p, uint32_t& pending) {
  if (pending == kNoPending)
    return;
  __syncwarp();
  if ((threadIdx.x & 31) == 0)
    st_release_u32(p.flags + pending, p.epoch);
  pending = kNoPending;
}

// One warp resolves local tile tl of graph G (tiles of LB bits): waits for
// its child tiles, reduces them, resolves the tile in T / U (shared memory,
// 2^LB / 4 words each) and stores it; `pending` then names its flag for
// publish_pending. sOrder is a word order table of order_bits >= LB - 2
// bits. False if a wait gave up.
template <int LB>
__device__ __forceinline__ bool tile_work(const DpBatchParams& p, const DpGraph& G, uint32_t tl, uint32_t* T,
                                          uint32_t* U, const uint16_t* sOrder, int order_bits, const Binom& sBinom,
                                          uint32_t* kids, uint32_t& pending) {
  constexpr int kWords = TileShape<LB>::kWords;
  const int lane = threadIdx.x & 31;
  uint8_t* const table = p.table + G.table_off;
  uint32_t* const flags = p.flags + G.tile_base;

  int j;
  uint32_t H, off_prev;
  decode_tile(sBinom, G.nh, tl, j, H, off_prev);

  // Lane v (a high vertex, v < nh <= 26) with v in H owns child tile
  // H - v. Its colex rank keeps the terms C(u, i + 1) of the bits u < v and
  // shifts the bits u > v down one place, C(u, i): a prefix sum and a
  // suffix sum over the lanes. The child goes to kids[index of v in H].
  const bool inH = (H >> lane) & 1u;
  const uint32_t q = __popc(H & ((1u << lane) - 1u));
  const uint32_t t1 = inH ? sBinom[lane][q + 1] : 0u, t0 = inH ? sBinom[lane][q] : 0u;
  uint32_t pre = t1, suf = t0;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t x = __shfl_up_sync(0xffffffffu, pre, d);
    const uint32_t y = __shfl_down_sync(0xffffffffu, suf, d);
    if (lane >= d)
      pre += x;
    if (lane + d < 32)
      suf += y;
  }
  bool ok = true;
  if (inH) {
    const uint32_t child = off_prev + (pre - t1) + (suf - t0);
    kids[q] = child;
    ok = wait_flag(flags + child, p.epoch, p.timeout_ns, p.error);
  }
  if (__any_sync(0xffffffffu, !ok))
    return false;
  __syncwarp();  // kids[] written above, read by every lane below

  // Cross-tile children: j whole tiles, 4 subsets per word, children three
  // at a time from 10-bit tiles up (three 16-byte loads in flight per
  // lane), else two at a time.
  if constexpr (kWords >= 128) {
#pragma unroll 1
    for (int c0 = 0; c0 < kWords; c0 += 128) {
      Acc g[4];
#pragma unroll
      for (int q = 0; q < 4; ++q)
        acc_init(g[q]);
      int m = 0;
      for (; LB >= 10 && m + 3 <= j; m += 3) {  // three loads in flight
        const uint4 a = __ldcg(reinterpret_cast<const uint4*>(table + (size_t(kids[m]) << LB)) + (c0 >> 2) + lane);
        const uint4 b =
            __ldcg(reinterpret_cast<const uint4*>(table + (size_t(kids[m + 1]) << LB)) + (c0 >> 2) + lane);
        const uint4 c =
            __ldcg(reinterpret_cast<const uint4*>(table + (size_t(kids[m + 2]) << LB)) + (c0 >> 2) + lane);
        acc_add3(g[0], a.x, b.x, c.x);
        acc_add3(g[1], a.y, b.y, c.y);
        acc_add3(g[2], a.z, b.z, c.z);
        acc_add3(g[3], a.w, b.w, c.w);
      }
      for (; m + 2 <= j; m += 2) {  // pairs: the remainder, or every child below 10 bits
        const uint32_t c_a = kids[m];
        const uint32_t c_b = kids[m + 1];
        const uint4 a = __ldcg(reinterpret_cast<const uint4*>(table + (size_t(c_a) << LB)) + (c0 >> 2) + lane);
        const uint4 b = __ldcg(reinterpret_cast<const uint4*>(table + (size_t(c_b) << LB)) + (c0 >> 2) + lane);
        acc_add2(g[0], a.x, b.x);
        acc_add2(g[1], a.y, b.y);
        acc_add2(g[2], a.z, b.z);
        acc_add2(g[3], a.w, b.w);
      }
      if (m < j) {
        const uint32_t c_a = kids[m];
        const uint4 a = __ldcg(reinterpret_cast<const uint4*>(table + (size_t(c_a) << LB)) + (c0 >> 2) + lane);
        acc_add1(g[0], a.x);
        acc_add1(g[1], a.y);
        acc_add1(g[2], a.z);
        acc_add1(g[3], a.w);
      }
      reinterpret_cast<uint4*>(T + c0)[lane] = make_uint4(g[0].o, g[1].o, g[2].o, g[3].o);
      reinterpret_cast<uint4*>(U + c0)[lane] =
          make_uint4(second_child(g[0]), second_child(g[1]), second_child(g[2]), second_child(g[3]));
    }
  } else {
    for (int w = lane; w < kWords; w += 32) {
      Acc g;
      acc_init(g);
      for (int m = 0; m < j; ++m) {
        const uint32_t c_a = kids[m];
        acc_add1(g, __ldcg(reinterpret_cast<const uint32_t*>(table + (size_t(c_a) << LB)) + w));
      }
      T[w] = g.o;
      U[w] = second_child(g);
    }
  }
  __syncwarp();

  // In-tile children: words in popcount order of the word index, one
  // unrolled pass per popcount class; inside a word the subsets with low
  // bits 00, then 01 and 10, then 11.
  // U lies u_off bytes after T: 2^LB in the one-size kernel, the largest
  // tile's 2^lb in the mixed one.
  const uint32_t u_off =
      static_cast<uint32_t>(reinterpret_cast<const uint8_t*>(U) - reinterpret_cast<const uint8_t*>(T));
  intile_class<LB, 0>(p, G, static_cast<uint64_t>(H) << LB, j, smem_u32(T), u_off, sOrder, order_bits);

  // Store the tile; the caller publishes it (publish_pending).
  uint32_t* dst = reinterpret_cast<uint32_t*>(table + (size_t(tl) << LB));
  if constexpr (kWords >= 128) {
    for (int w4 = lane; w4 < kWords / 4; w4 += 32)
      reinterpret_cast<uint4*>(dst)[w4] = reinterpret_cast<const uint4*>(T)[w4];
  } else {
    for (int w = lane; w < kWords; w += 32)
      dst[w] = T[w];
  }
  pending = G.tile_base + tl;
  return true;
}

// Takes the next ticket (lane 0) and maps it to (graph, local tile);
// false when the tickets are used up or an error was raised.
__device__ __forceinline__ bool next_tile(const DpBatchParams& p, uint32_t& gi, uint32_t& tl) {
  const int lane = threadIdx.x & 31;
  uint32_t t = 0;
  gi = 0;
  tl = 0;
  if (lane == 0) {
    t = ld_relaxed_s32(p.error) != 0 ? 0xffffffffu : atomicAdd(p.ticket, 1u);
    tl = t;
    if (t < p.total_tiles && p.graphs) {
      const uint2 m = __ldg(p.tile_map + t);
      gi = m.x;
      tl = m.y;
    }
  }
  t = __shfl_sync(0xffffffffu, t, 0);
  gi = __shfl_sync(0xffffffffu, gi, 0);
  tl = __shfl_sync(0xffffffffu, tl, 0);
  return t < p.total_tiles;
}

// Every tile of the launch has LB bits (single-graph solves, and batches
// that use one tile size).
template <int LB>
__device__ __forceinline__ void dp_tile_body(const DpBatchParams& p) {
  using Shape = TileShape<LB>;
  extern __shared__ __align__(16) uint8_t smem[];
  const int warp = threadIdx.x >> 5;
  uint32_t* T = reinterpret_cast<uint32_t*>(smem + size_t(warp) * Shape::kPerWarp);
  uint32_t* U = T + Shape::kWords;
  uint16_t* sOrder = reinterpret_cast<uint16_t*>(smem + Shape::kOrderOff);
  Binom& sBinom = *reinterpret_cast<Binom*>(smem + Shape::kBinomOff);
  uint32_t* kids = reinterpret_cast<uint32_t*>(smem + Shape::kKidsOff) + warp * 32;

  for (int i = threadIdx.x; i < (kDpMaxHigh + 1) * (kDpMaxHigh + 1); i += blockDim.x)
    (&sBinom[0][0])[i] = (&p.binom[0][0])[i];
  build_word_order(sOrder, p.binom, Shape::kWordBits);
  __syncthreads();

  uint32_t gi, tl, pending = kNoPending;
  while (publish_pending(p, pending), next_tile(p, gi, tl)) {
    const DpGraph G = p.graphs ? p.graphs[gi] : p.single;
    if (!tile_work<LB>(p, G, tl, T, U, sOrder, Shape::kWordBits, sBinom, kids, pending))
      break;
  }
  publish_pending(p, pending);
}

// Tiles of 10 to 12 bits (three cross-tile loads in flight): the launch
// bound holds the registers to the CTAs per SM that shared memory allows, 10
// at 10 and 11 bits, 6 at 12.
template <int LB>
constexpr int kDpMinCtas = LB >= 12 ? 6 : 10;

template <int LB>
__global__ void __launch_bounds__(32 * kDpWarps, kDpMinCtas<LB>)
    dp_tile_kernel(const __grid_constant__ DpBatchParams p) {
  dp_tile_body<LB>(p);
}

// Smaller tiles (pairs of cross-tile loads): registers left to the compiler.
template <int LB>
__global__ void __launch_bounds__(32 * kDpWarps) dp_tile_kernel_small(const __grid_constant__ DpBatchParams p) {
  dp_tile_body<LB>(p);
}

template <int LB>
constexpr auto tile_kernel_for() {
  if constexpr (LB >= 10)
    return &dp_tile_kernel<LB>;
  else
    return &dp_tile_kernel_small<LB>;
}

// Batches whose graphs use different tile sizes (DpGraph::lb, 8 .. p.lb):
// shared memory is laid out for the largest (p.lb, a runtime value, so the
// launch's occupancy follows it) and each tile dispatches on its graph's lb.
// The five inlined tile sizes raise the register count (64 against 47 for
// one size), so this kernel holds fewer CTAs than the one-size kernel; the
// autotuner measures that cost and the planner only mixes sizes when the
// per-size gains outweigh it.
__global__ void __launch_bounds__(32 * kDpWarps)
    dp_tile_kernel_mixed(const __grid_constant__ DpBatchParams p) {
  extern __shared__ __align__(16) uint8_t smem[];
  const int warp = threadIdx.x >> 5;
  const int words = (1 << p.lb) / 4, bits = p.lb - 2;
  const size_t per_warp = size_t(2) * words * 4;
  const size_t order_off = kDpWarps * per_warp;
  const size_t binom_off = (order_off + size_t(words) * 2 + 15) & ~size_t(15);
  const size_t kids_off = (binom_off + sizeof(Binom) + 15) & ~size_t(15);
  uint32_t* T = reinterpret_cast<uint32_t*>(smem + size_t(warp) * per_warp);
  uint32_t* U = T + words;
  uint16_t* sOrder = reinterpret_cast<uint16_t*>(smem + order_off);
  Binom& sBinom = *reinterpret_cast<Binom*>(smem + binom_off);
  uint32_t* kids = reinterpret_cast<uint32_t*>(smem + kids_off) + warp * 32;

  for (int i = threadIdx.x; i < (kDpMaxHigh + 1) * (kDpMaxHigh + 1); i += blockDim.x)
    (&sBinom[0][0])[i] = (&p.binom[0][0])[i];
  build_word_order(sOrder, p.binom, bits);
  __syncthreads();

  uint32_t gi, tl, pending = kNoPending;
  while (publish_pending(p, pending), next_tile(p, gi, tl)) {
    const DpGraph G = p.graphs[gi];
    bool ok = false;
    if (G.lb > p.lb) {  // the planner never does this: the tile would not fit
      raise_error(p.error, kDevInvalidInput, static_cast<int32_t>(gi));
      break;
    }
    switch (G.lb) {
      case 8: ok = tile_work<8>(p, G, tl, T, U, sOrder, bits, sBinom, kids, pending); break;
      case 9: ok = tile_work<9>(p, G, tl, T, U, sOrder, bits, sBinom, kids, pending); break;
      case 10: ok = tile_work<10>(p, G, tl, T, U, sOrder, bits, sBinom, kids, pending); break;
      case 11: ok = tile_work<11>(p, G, tl, T, U, sOrder, bits, sBinom, kids, pending); break;
      case 12: ok = tile_work<12>(p, G, tl, T, U, sOrder, bits, sBinom, kids, pending); break;
      default: raise_error(p.error, kDevInvalidInput, static_cast<int32_t>(gi)); break;
    }
    if (!ok)
      break;
  }
  publish_pending(p, pending);
}

// Dynamic shared memory of the mixed kernel for tiles of up to lb bits.
size_t dp_mixed_smem(int lb) {
  const size_t words = (size_t(1) << lb) / 4;
  const size_t order_off = kDpWarps * 2 * words * 4;
  const size_t binom_off = (order_off + words * 2 + 15) & ~size_t(15);
  const size_t kids_off = (binom_off + sizeof(Binom) + 15) & ~size_t(15);
  return kids_off + size_t(kDpWarps) * 32 * 4;
}

// ---------------------------------------------------------------------------
// Reconstruction: one warp per graph; lanes cover vertices lane, lane + 32.
// ---------------------------------------------------------------------------

constexpr int kTreeWarps = 4;

__device__ __forceinline__ uint64_t ballot64(bool lo, bool hi) {
  const uint32_t a = __ballot_sync(0xffffffffu, lo);
  const uint32_t b = __ballot_sync(0xffffffffu, hi);
  return (static_cast<uint64_t>(b) << 32) | a;
}

__device__ __forceinline__ uint64_t warp_or64(uint64_t x) {
  const uint32_t lo = __reduce_or_sync(0xffffffffu, static_cast<uint32_t>(x));
  const uint32_t hi = __reduce_or_sync(0xffffffffu, static_cast<uint32_t>(x >> 32));
  return (static_cast<uint64_t>(hi) << 32) | lo;
}

__device__ uint64_t warp_component(uint64_t S, int v, const uint64_t* adj, int n) {
  const int lane = threadIdx.x & 31;
  uint64_t reach = 1ull << v, frontier = reach;
  while (frontier) {
    uint64_t nb = 0;
    for (int u = lane; u < n; u += 32)
      if ((frontier >> u) & 1ull)
        nb |= adj[u];
    nb = warp_or64(nb) & S & ~reach;
    reach |= nb;
    frontier = nb;
  }
  return reach;
}

struct TreeCtx {
  const Binom& binom;
  const uint8_t* table;
  int lb, nh, n;
  __device__ uint32_t td_of(uint64_t S) const {
    const uint32_t H = static_cast<uint32_t>(S >> lb);
    const int j = __popc(H);
    uint32_t off = 0;
    for (int i = 0; i < j; ++i)
      off += binom[nh][i];
    const uint64_t tile = off + rank_colex(binom, H);
    return table[(tile << lb) | (S & ((1ull << lb) - 1))] >> 1;
  }
  // First vertex v of the connected set C with td(C - v) = td(C) - 1, i.e.
  // the first argmin of td(C - v) (td(C) = 1 + min_v td(C - v) for a
  // connected C): one round of table reads, no read of td(C) itself.
  __device__ int root(uint64_t C) const {
    if (__popcll(C) == 1)
      return __ffsll(static_cast<long long>(C)) - 1;
    const int lane = threadIdx.x & 31;
    const bool in_lo = (C >> lane) & 1ull;
    const bool in_hi = lane + 32 < n && ((C >> (lane + 32)) & 1ull);
    const uint32_t t_lo = in_lo ? td_of(C & ~(1ull << lane)) : 0xFFFFFFFFu;
    const uint32_t t_hi = in_hi ? td_of(C & ~(1ull << (lane + 32))) : 0xFFFFFFFFu;
    const uint32_t m = __reduce_min_sync(0xffffffffu, min(t_lo, t_hi));
    const uint64_t hits = ballot64(in_lo && t_lo == m, in_hi && t_hi == m);
    return hits ? __ffsll(static_cast<long long>(hits)) - 1 : -1;
  }
};

__global__ void __launch_bounds__(32 * kTreeWarps)
    dp_tree_kernel(const __grid_constant__ DpBatchParams p) {
  __shared__ uint64_t sAdjAll[kTreeWarps][kDpMaxN];
  __shared__ uint64_t stMaskAll[kTreeWarps][kDpMaxN];
  __shared__ int32_t stOwnerAll[kTreeWarps][kDpMaxN];
  __shared__ int32_t stDepthAll[kTreeWarps][kDpMaxN];
  __shared__ int32_t sParAll[kTreeWarps][kDpMaxN];     // the canonical tree
  __shared__ int32_t sDepAll[kTreeWarps][kDpMaxN];     // depth of each vertex in it
  __shared__ uint32_t sHgtAll[kTreeWarps][kDpMaxN];    // subtree height (in vertices)
  __shared__ uint32_t sLowAll[kTreeWarps][kDpMaxN];    // 255 - the subtree's lowest vertex
  __shared__ unsigned long long sKidsAll[kTreeWarps][kDpMaxN];  // children of each vertex
  // The binomial table in shared memory: every lane ranks a different subset,
  // which the parameter bank would serve one address at a time.
  __shared__ Binom sBinom;
  for (int i = threadIdx.x; i < (kDpMaxHigh + 1) * (kDpMaxHigh + 1); i += blockDim.x)
    (&sBinom[0][0])[i] = (&p.binom[0][0])[i];
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint64_t* sAdj = sAdjAll[warp];
  uint64_t* stMask = stMaskAll[warp];
  int32_t* stOwner = stOwnerAll[warp];
  int32_t* stDepth = stDepthAll[warp];
  if (ld_relaxed_s32(p.error) != 0)
    return;

  for (int g = blockIdx.x * kTreeWarps + warp; g < p.num_graphs; g += gridDim.x * kTreeWarps) {
    const DpGraph G = p.graphs ? p.graphs[g] : p.single;
    const int n = G.n;
    for (int v = lane; v < n; v += 32)
      sAdj[v] = p.adj[G.adj_off + v];
    __syncwarp();
    const TreeCtx ctx{sBinom, p.table + G.table_off, G.lb, G.nh, n};
    const uint64_t query = p.query ? p.query : (n == 64 ? ~0ull : ((1ull << n) - 1));
    const uint32_t td = query ? ctx.td_of(query) : 0u;
    if (lane == 0 && p.td_out)
      p.td_out[G.out_idx] = static_cast<int32_t>(td);

    // Canonical tree of the query set: every component is rooted at
    // ctx.root and its sub-components hang below that root
    // (dynamic_cpu.hpp:59-81); kept in shared memory for the order below.
    int32_t* sPar = sParAll[warp];
    int32_t* sDep = sDepAll[warp];
    int top = 0, height = 0;
    for (uint64_t rest = query; rest;) {
      const uint64_t c = warp_component(rest, __ffsll(static_cast<long long>(rest)) - 1, sAdj, n);
      rest &= ~c;
      if (lane == 0) {
        stMask[top] = c;
        stOwner[top] = -1;
        stDepth[top] = 1;
      }
      ++top;
    }
    __syncwarp();
    while (top > 0) {
      --top;
      const uint64_t C = stMask[top];
      const int owner = stOwner[top], depth = stDepth[top];
      __syncwarp();
      const int r = ctx.root(C);
      if (r < 0) {
        if (lane == 0)
          raise_error(p.error, kDevNoRoot, g);
        return;
      }
      if (lane == 0) {
        sPar[r] = owner;
        sDep[r] = depth;
      }
      height = max(height, depth);
      for (uint64_t rest = C & ~(1ull << r); rest;) {
        const uint64_t c = warp_component(rest, __ffsll(static_cast<long long>(rest)) - 1, sAdj, n);
        rest &= ~c;
        if (lane == 0) {
          stMask[top] = c;
          stOwner[top] = r;
          stDepth[top] = depth + 1;
        }
        ++top;
      }
      __syncwarp();
    }
    if (static_cast<uint32_t>(height) != td) {
      if (lane == 0)
        raise_error(p.error, kDevNoRoot, g);
      return;
    }
    if (p.parent_out) {
      int32_t* parent = p.parent_out + G.adj_off;
      for (int v = lane; v < n; v += 32)
        if ((query >> v) & 1ull)
          parent[v] = sPar[v];
    }

    if (p.order_out) {
      // GetElimination (dynamic_gpu.hpp:58-63): repeatedly remove the stored
      // root of the remaining set; for a disconnected set that is the root of
      // its first deepest component, components taken in order of their
      // lowest vertex (dynamic_gpu.cu:92-103). The components of the
      // remaining set are subtrees of the canonical tree and a component's
      // treedepth is its subtree's height, so the order is read off the tree:
      // the active subtree of greatest height, ties to the lowest vertex,
      // gives its root and is replaced by its children's subtrees.
      uint32_t* sHgt = sHgtAll[warp];
      uint32_t* sLow = sLowAll[warp];
      unsigned long long* sKids = sKidsAll[warp];
      for (int v = lane; v < n; v += 32) {
        sHgt[v] = 0u;  // the tallest child so far
        sLow[v] = 255u - static_cast<uint32_t>(v);
        sKids[v] = 0ull;
      }
      __syncwarp();
      for (int d = height; d >= 1; --d) {  // deepest first: children before parents
        for (int v = lane; v < n; v += 32) {
          if (((query >> v) & 1ull) && sDep[v] == d) {
            const uint32_t h = sHgt[v] + 1u;  // own height = tallest child + 1
            sHgt[v] = h;
            const int pv = sPar[v];
            if (pv >= 0) {
              atomicMax(&sHgt[pv], h);
              atomicMax(&sLow[pv], sLow[v]);
              atomicOr(&sKids[pv], 1ull << v);
            }
          }
        }
        __syncwarp();
      }
      int32_t* order = p.order_out + G.adj_off;
      uint64_t active = 0;
      for (int v = lane; v < n; v += 32)
        if (((query >> v) & 1ull) && sPar[v] < 0)
          active |= 1ull << v;
      active = warp_or64(active);
      for (int step = 0; active; ++step) {
        // key: height << 8 | 255 - lowest vertex (unique: the subtrees are disjoint)
        const uint32_t k_lo = ((active >> lane) & 1ull) ? (sHgt[lane] << 8 | sLow[lane]) : 0u;
        const uint32_t k_hi = (lane + 32 < n && ((active >> (lane + 32)) & 1ull))
                                  ? (sHgt[lane + 32] << 8 | sLow[lane + 32]) : 0u;
        const uint32_t m = __reduce_max_sync(0xffffffffu, max(k_lo, k_hi));
        const uint64_t hit = ballot64(k_lo == m && k_lo != 0u, k_hi == m && k_hi != 0u);
        const int a = __ffsll(static_cast<long long>(hit)) - 1;
        if (lane == 0)
          order[step] = a;
        active = (active & ~(1ull << a)) | sKids[a];
      }
    }
    __syncwarp();
  }
}

// ---------------------------------------------------------------------------
// Host-side launch helpers.
// ---------------------------------------------------------------------------

void dp_fill_binom(DpBatchParams& p) {
  for (int a = 0; a <= kDpMaxHigh; ++a) {
    for (int b = 0; b <= kDpMaxHigh; ++b)
      p.binom[a][b] = 0;
    p.binom[a][0] = 1;
    for (int b = 1; b <= a; ++b)
      p.binom[a][b] = p.binom[a - 1][b - 1] + (b <= a - 1 ? p.binom[a - 1][b] : 0u);
  }
}

template <int LB>
static cudaError_t launch_tiles(const DpBatchParams& p, int ctas, cudaStream_t s) {
  tile_kernel_for<LB>()<<<ctas, 32 * kDpWarps, TileShape<LB>::kSmem, s>>>(p);
  return cudaGetLastError();
}

template <int LB>
static int occupancy_tiles() {
  if (cudaFuncSetAttribute(tile_kernel_for<LB>(), cudaFuncAttributeMaxDynamicSharedMemorySize,
                           static_cast<int>(TileShape<LB>::kSmem)) != cudaSuccess)
    return 0;
  int blocks = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, tile_kernel_for<LB>(), 32 * kDpWarps,
                                                TileShape<LB>::kSmem);
  return blocks;
}

int dp_tile_occupancy(int lb) {
  switch (lb) {
#define GTD_CASE(X) \
  case X:           \
    return occupancy_tiles<X>();
    GTD_CASE(2) GTD_CASE(3) GTD_CASE(4) GTD_CASE(5) GTD_CASE(6)
    GTD_CASE(7) GTD_CASE(8) GTD_CASE(9) GTD_CASE(10) GTD_CASE(11) GTD_CASE(12)
#undef GTD_CASE
    default:
      return 0;
  }
}

cudaError_t dp_launch_validate(const DpBatchParams& p, cudaStream_t s) {
  dp_validate_kernel<<<(p.num_graphs + 3) / 4, 128, 0, s>>>(p);  // one warp per graph
  return cudaGetLastError();
}

cudaError_t dp_launch_fill_tile_map(const DpBatchParams& p, cudaStream_t s) {
  const int blocks = p.num_graphs < 4096 ? p.num_graphs : 4096;
  dp_fill_tile_map_kernel<<<blocks, 256, 0, s>>>(p);
  return cudaGetLastError();
}

int dp_mixed_occupancy(int lb) {
  const size_t smem = dp_mixed_smem(lb);
  if (cudaFuncSetAttribute(dp_tile_kernel_mixed, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           static_cast<int>(dp_mixed_smem(kDpMaxTileBits))) != cudaSuccess)
    return 0;
  int blocks = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, dp_tile_kernel_mixed, 32 * kDpWarps, smem);
  return blocks;
}

cudaError_t dp_launch_tiles(const DpBatchParams& p, int ctas, cudaStream_t s) {
  if (p.mixed) {
    if (p.lb < kDpMinTileBits || p.lb > kDpMaxTileBits)
      return cudaErrorInvalidValue;
    dp_tile_kernel_mixed<<<ctas, 32 * kDpWarps, dp_mixed_smem(p.lb), s>>>(p);
    return cudaGetLastError();
  }
  switch (p.lb) {
#define GTD_CASE(X) \
  case X:           \
    return launch_tiles<X>(p, ctas, s);
    GTD_CASE(2) GTD_CASE(3) GTD_CASE(4) GTD_CASE(5) GTD_CASE(6)
    GTD_CASE(7) GTD_CASE(8) GTD_CASE(9) GTD_CASE(10) GTD_CASE(11) GTD_CASE(12)
#undef GTD_CASE
    default:
      return cudaErrorInvalidValue;
  }
}

cudaError_t dp_launch_tree(const DpBatchParams& p, cudaStream_t s) {
  int blocks = (p.num_graphs + kTreeWarps - 1) / kTreeWarps;
  if (blocks > 4096)
    blocks = 4096;
  dp_tree_kernel<<<blocks, 32 * kTreeWarps, 0, s>>>(p);
  return cudaGetLastError();
}

// Training labels from a solved table (single graph): for each subset S,
// td(S) and, when S is connected, its optimal-root set
// R(S) = {v in S : td(S - v) = td(S) - 1} (one warp per subset).
__global__ void __launch_bounds__(32 * kTreeWarps)
    dp_labels_kernel(const __grid_constant__ DpBatchParams p, const uint64_t* subsets, int count, int32_t* td_out,
                     uint64_t* roots_out) {
  __shared__ Binom sBinom;  // lanes rank different subsets: shared memory, not the parameter bank
  for (int i = threadIdx.x; i < (kDpMaxHigh + 1) * (kDpMaxHigh + 1); i += blockDim.x)
    (&sBinom[0][0])[i] = (&p.binom[0][0])[i];
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const DpGraph G = p.single;
  const TreeCtx ctx{sBinom, p.table + G.table_off, G.lb, G.nh, G.n};
  for (int i = blockIdx.x * kTreeWarps + warp; i < count; i += gridDim.x * kTreeWarps) {
    const uint64_t S = subsets[i];
    if (S == 0) {
      if (lane == 0) {
        td_out[i] = 0;
        roots_out[i] = 0;
      }
      continue;
    }
    const uint32_t td = ctx.td_of(S);
    bool lo = false, hi = false;
    if ((S >> lane) & 1ull)
      lo = ctx.td_of(S & ~(1ull << lane)) + 1u == td;
    if (lane + 32 < G.n && ((S >> (lane + 32)) & 1ull))
      hi = ctx.td_of(S & ~(1ull << (lane + 32))) + 1u == td;
    const uint64_t roots = ballot64(lo, hi);
    if (lane == 0) {
      td_out[i] = static_cast<int32_t>(td);
      roots_out[i] = roots;
    }
  }
}

cudaError_t dp_launch_labels(const DpBatchParams& p, const uint64_t* subsets, int count, int32_t* td_out,
                             uint64_t* roots_out, cudaStream_t s) {
  int blocks = (count + kTreeWarps - 1) / kTreeWarps;
  if (blocks > 8192)
    blocks = 8192;
  if (blocks < 1)
    blocks = 1;
  dp_labels_kernel<<<blocks, 32 * kTreeWarps, 0, s>>>(p, subsets, count, td_out, roots_out);
  return cudaGetLastError();
}

}  // namespace gtd
