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
//    with the connected flag kept in bit 7 of each table byte. No per-subset
//    BFS, no ranking per child.
//  * Layout (gtd_dp_layout.h). Tiles of 2^lb subsets share a high part H;
//    a tile's cross-tile children are the whole tiles H - h one level down,
//    read as contiguous 2^lb-byte blocks; the in-tile children are resolved
//    in shared memory in popcount order of the low part.
//  * Schedule. One persistent launch: CTAs take tiles by ticket (atomicAdd)
//    in level-major order, wait on per-tile ready flags of the |H| child
//    tiles (each wait bounded by a deadline), reduce the children with 4-way
//    SIMD byte min/max, resolve the tile, store it, publish its flag. A tile
//    only waits on tiles with smaller tickets, and a ticket is only taken by
//    a running CTA, so the smallest unfinished ticket can always proceed.
//
// Reconstruction (dp_tree_kernel): one warp, one lane per vertex, rebuilds
// the reference's tree (first-argmin root per component, dynamic_gpu.cu:84-87,
// dynamic_cpu.hpp:59-81) and GetElimination order (dynamic_gpu.hpp:48-64).
#include <cuda_runtime.h>

#include <cstdint>

#include "gtd_device.cuh"
#include "gtd_dp_kernels.h"

namespace gtd {

template <int LB>
struct TileShape {
  static constexpr int kEntries = 1 << LB;
  static constexpr int kWords = kEntries / 4;
  static constexpr int kThreads = kWords < 32 ? 32 : kWords;
};

// Checks the adjacency masks: no self loop, no bit >= n, symmetric.
__device__ __forceinline__ bool adjacency_ok(const uint64_t* adj, int n) {
  const uint64_t allowed = n >= 64 ? ~0ull : ((1ull << n) - 1);
  for (int v = 0; v < n; ++v) {
    uint64_t a = adj[v];
    if ((a >> v) & 1ull)
      return false;
    if (a & ~allowed)
      return false;
    for (uint64_t s = a; s; s &= s - 1) {
      int u = __ffsll(static_cast<long long>(s)) - 1;
      if (!((adj[u] >> v) & 1ull))
        return false;
    }
  }
  return true;
}

template <int LB>
__global__ void __launch_bounds__(TileShape<LB>::kThreads)
    dp_tile_kernel(const DpKernelParams p) {
  using Shape = TileShape<LB>;
  constexpr int kEntries = Shape::kEntries;
  constexpr int kWords = Shape::kWords;
  constexpr int kThreads = Shape::kThreads;

  __shared__ uint32_t sT[kWords];
  __shared__ uint32_t sMin[kWords];
  __shared__ uint32_t sMax[kWords];
  __shared__ uint32_t sCnt[kWords];
  __shared__ uint16_t sOrder[kEntries];
  __shared__ uint64_t sAdj[kDpMaxN];
  __shared__ uint32_t sChild[kDpMaxHigh];
  __shared__ uint32_t sTile;
  __shared__ int sBadInput;

  const int tid = threadIdx.x;
  const DpLayout& lay = p.lay;
  const int n = lay.n;

  for (int v = tid; v < n; v += kThreads)
    sAdj[v] = p.adj[v];
  // Low parts ordered by popcount, colex rank inside each popcount class.
  for (int L = tid; L < kEntries; L += kThreads) {
    const int i = __popc(L);
    uint32_t pos = 0;
    for (int q = 0; q < i; ++q)
      pos += lay.binom[LB][q];
    int m = 0;
    for (uint32_t r = static_cast<uint32_t>(L); r; r &= r - 1)
      pos += lay.binom[__ffs(r) - 1][++m];
    sOrder[pos] = static_cast<uint16_t>(L);
  }
  __syncthreads();
  if (tid == 0) {
    sBadInput = adjacency_ok(sAdj, n) ? 0 : 1;
    if (sBadInput)
      raise_error(p.error, kDevInvalidInput, 0);
  }
  __syncthreads();
  if (sBadInput)
    return;

  const uint8_t* bMin = reinterpret_cast<const uint8_t*>(sMin);
  const uint8_t* bMax = reinterpret_cast<const uint8_t*>(sMax);
  const uint8_t* bCnt = reinterpret_cast<const uint8_t*>(sCnt);
  uint8_t* bT = reinterpret_cast<uint8_t*>(sT);
  const uint32_t* gT = reinterpret_cast<const uint32_t*>(p.table);

  for (;;) {
    if (tid == 0)
      sTile = ld_relaxed_s32(p.error) != 0 ? 0xffffffffu : atomicAdd(p.ticket, 1u);
    __syncthreads();
    const uint32_t t = sTile;
    if (t >= lay.ntiles)
      break;

    // Level j and high part H of tile t.
    int j = 0;
    while (lay.level_off[j + 1] <= t)
      ++j;
    uint32_t H = 0;
    {
      uint32_t r = t - lay.level_off[j];
      int k = j;
      for (int a = lay.nh - 1; k > 0; --a) {
        const uint32_t c = lay.binom[a][k];
        if (r >= c) {
          H |= 1u << a;
          r -= c;
          --k;
        }
      }
    }

    // Child tiles H - h, one per thread; wait until each is published.
    bool ok = true;
    if (tid < j) {
      uint32_t rest = H;
      for (int q = 0; q < tid; ++q)
        rest &= rest - 1;
      const uint32_t hc = H & ~(rest & (0u - rest));
      const uint32_t child = lay.level_off[j - 1] + lay.rank_high(hc);
      sChild[tid] = child;
      ok = wait_flag(p.flags + child, p.epoch, p.timeout_ns, p.error);
    }
    if (__syncthreads_or(!ok))
      break;

    // Cross-tile children: whole tiles, 4 subsets per 32-bit word.
    if (tid < kWords) {
      uint32_t mn = 0x3F3F3F3Fu, mx = 0u, cnt = 0u;
      int m = 0;
      for (; m + 4 <= j; m += 4) {
        const uint32_t x0 = __ldcg(gT + static_cast<size_t>(sChild[m]) * kWords + tid);
        const uint32_t x1 = __ldcg(gT + static_cast<size_t>(sChild[m + 1]) * kWords + tid);
        const uint32_t x2 = __ldcg(gT + static_cast<size_t>(sChild[m + 2]) * kWords + tid);
        const uint32_t x3 = __ldcg(gT + static_cast<size_t>(sChild[m + 3]) * kWords + tid);
        const uint32_t y0 = x0 & 0x3F3F3F3Fu, y1 = x1 & 0x3F3F3F3Fu;
        const uint32_t y2 = x2 & 0x3F3F3F3Fu, y3 = x3 & 0x3F3F3F3Fu;
        mn = __vminu4(mn, __vminu4(__vminu4(y0, y1), __vminu4(y2, y3)));
        mx = __vmaxu4(mx, __vmaxu4(__vmaxu4(y0, y1), __vmaxu4(y2, y3)));
        cnt += ((x0 >> 7) & 0x01010101u) + ((x1 >> 7) & 0x01010101u) +
               ((x2 >> 7) & 0x01010101u) + ((x3 >> 7) & 0x01010101u);
      }
      for (; m < j; ++m) {
        const uint32_t x = __ldcg(gT + static_cast<size_t>(sChild[m]) * kWords + tid);
        const uint32_t y = x & 0x3F3F3F3Fu;
        mn = __vminu4(mn, y);
        mx = __vmaxu4(mx, y);
        cnt += (x >> 7) & 0x01010101u;
      }
      sMin[tid] = mn;
      sMax[tid] = mx;
      sCnt[tid] = cnt;
    }
    __syncthreads();

    // In-tile children, resolved in popcount order of the low part.
    const uint64_t Hfull = static_cast<uint64_t>(H) << LB;
    uint32_t start = 0;
#pragma unroll 1
    for (int i = 0; i <= LB; ++i) {
      const uint32_t count = lay.binom[LB][i];
      for (uint32_t e = tid; e < count; e += kThreads) {
        const int L = sOrder[start + e];
        uint32_t mn = bMin[L], mx = bMax[L], c = bCnt[L];
        for (uint32_t s = static_cast<uint32_t>(L); s; s &= s - 1) {
          const uint32_t x = bT[L ^ (s & (0u - s))];
          mn = min(mn, x & 63u);
          mx = max(mx, x & 63u);
          c += x >> 7;
        }
        const int k = j + i;
        uint32_t val;
        if (k == 0) {
          val = 0u;
        } else if (k == 1) {
          val = 0x81u;
        } else {
          bool conn;
          if (k == 2) {
            const uint64_t S = Hfull | static_cast<uint64_t>(L);
            const int u = __ffsll(static_cast<long long>(S)) - 1;
            const int v = 63 - __clzll(static_cast<long long>(S));
            conn = (sAdj[u] >> v) & 1ull;
          } else {
            conn = c >= 2u;
          }
          val = conn ? ((mn + 1u) | 0x80u) : mx;
        }
        bT[L] = static_cast<uint8_t>(val);
      }
      start += count;
      __syncthreads();
    }

    // Store the tile, then publish it.
    if (tid < kWords)
      reinterpret_cast<uint32_t*>(p.table)[static_cast<size_t>(t) * kWords + tid] = sT[tid];
    __threadfence();
    __syncthreads();
    if (tid == 0)
      st_release_u32(p.flags + t, p.epoch);
  }
}

// ---------------------------------------------------------------------------
// Reconstruction: one warp; lanes cover vertices lane and lane + 32.
// ---------------------------------------------------------------------------

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

__device__ __forceinline__ uint32_t td_of(const DpKernelParams& p, uint64_t S) {
  return p.table[p.lay.index(S)] & 63u;
}

// First vertex v of the connected set C with td(C - v) = td(C) - 1.
__device__ int warp_root(const DpKernelParams& p, uint64_t C) {
  if (__popcll(C) == 1)
    return __ffsll(static_cast<long long>(C)) - 1;
  const int lane = threadIdx.x & 31;
  const uint32_t want = td_of(p, C) - 1u;
  bool hit_lo = false, hit_hi = false;
  if ((C >> lane) & 1ull)
    hit_lo = td_of(p, C & ~(1ull << lane)) == want;
  if (lane + 32 < p.lay.n && ((C >> (lane + 32)) & 1ull))
    hit_hi = td_of(p, C & ~(1ull << (lane + 32))) == want;
  const uint64_t hits = ballot64(hit_lo, hit_hi);
  return hits ? __ffsll(static_cast<long long>(hits)) - 1 : -1;
}

__global__ void __launch_bounds__(32)
    dp_tree_kernel(const DpKernelParams p, uint64_t query, int32_t* td_out,
                   int32_t* parent_out, int32_t* order_out) {
  __shared__ uint64_t sAdj[kDpMaxN];
  __shared__ uint64_t stMask[kDpMaxN];
  __shared__ int32_t stOwner[kDpMaxN];
  __shared__ int32_t stDepth[kDpMaxN];
  const int lane = threadIdx.x;
  const int n = p.lay.n;
  for (int v = lane; v < n; v += 32)
    sAdj[v] = p.adj[v];
  __syncwarp();
  if (ld_relaxed_s32(p.error) != 0)
    return;

  const uint32_t td = query ? td_of(p, query) : 0u;
  if (lane == 0 && td_out)
    *td_out = static_cast<int32_t>(td);

  if (parent_out) {
    // Canonical tree: every component is rooted at warp_root and its
    // sub-components hang below that root (dynamic_cpu.hpp:59-81).
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
      const int r = warp_root(p, C);
      if (r < 0) {
        if (lane == 0)
          raise_error(p.error, kDevNoRoot, static_cast<int32_t>(__popcll(C)));
        return;
      }
      if (lane == 0)
        parent_out[r] = owner;
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
    if (static_cast<uint32_t>(height) != td && lane == 0)
      raise_error(p.error, kDevNoRoot, -1);
  }

  if (order_out) {
    // GetElimination (dynamic_gpu.hpp:58-63): repeatedly remove the stored
    // root of the remaining set; for a disconnected set that is the root of
    // its first deepest component (dynamic_gpu.cu:92-103).
    uint64_t R = query;
    for (int step = 0; R; ++step) {
      uint64_t best = 0;
      uint32_t best_td = 0;
      for (uint64_t rest = R; rest;) {
        const uint64_t c = warp_component(rest, __ffsll(static_cast<long long>(rest)) - 1, sAdj, n);
        rest &= ~c;
        const uint32_t t = td_of(p, c);
        if (best == 0 || t > best_td) {
          best = c;
          best_td = t;
        }
      }
      const int r = warp_root(p, best);
      if (r < 0) {
        if (lane == 0)
          raise_error(p.error, kDevNoRoot, -2);
        return;
      }
      if (lane == 0)
        order_out[step] = r;
      R &= ~(1ull << r);
    }
  }
}

// ---------------------------------------------------------------------------
// Host-side launch helpers.
// ---------------------------------------------------------------------------

template <int LB>
static cudaError_t launch_tiles(const DpKernelParams& p, int ctas, cudaStream_t s) {
  dp_tile_kernel<LB><<<ctas, TileShape<LB>::kThreads, 0, s>>>(p);
  return cudaGetLastError();
}

template <int LB>
static int occupancy_tiles() {
  int blocks = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, dp_tile_kernel<LB>,
                                                TileShape<LB>::kThreads, 0);
  return blocks;
}

int dp_tile_threads(int lb) { return lb <= 7 ? 32 : (1 << (lb - 2)); }

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

cudaError_t dp_launch_tiles(const DpKernelParams& p, int ctas, cudaStream_t s) {
  switch (p.lay.lb) {
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

cudaError_t dp_launch_tree(const DpKernelParams& p, uint64_t query, int32_t* td,
                           int32_t* parent, int32_t* order, cudaStream_t s) {
  dp_tree_kernel<<<1, 32, 0, s>>>(p, query, td, parent, order);
  return cudaGetLastError();
}

}  // namespace gtd
