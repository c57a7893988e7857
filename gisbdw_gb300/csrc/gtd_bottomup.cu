// The bottom-up union-find heuristic DP on sm_103a.
//
// Reference: BottomUpHeuristicGPU (Treedepth/src/branch_and_bound/heuristics/
// bottom_up_heuristic.hpp:18-33) over BottomUpHeuristicGPUAlgorithm
// (bottom_up_heuristic_gpu_algorithm.cu:57-258). Level by level over subset
// sizes, every subset S keeps ONE elimination forest: the forest of a child
// S - v with v added as the root over the trees of its neighbours in S,
// for the first v (ascending) giving the least forest height. The last
// vertex added to each subset is kept for every level; GetElimination reads
// the last vertex of V, of V minus it, and so on, and the heuristic's tree is
// the elimination-tree replay of that order. It is the innermost heuristic of
// the reference's bnbGPU / bnbCPU incumbent chains (main.cpp:170-186).
//
// The reference runs one thread per subset with a union-find array per
// thread in shared memory (int8, n + 2 entries) and path-compressed Find.
// Here one warp handles one subset and lane u owns vertex u:
//  * Forests are stored fully compressed, one 32-byte row per subset (n <=
//    32): byte u is the root of u's tree, or 0x80 | height for a root. Only
//    roots and their heights matter to the recurrence (Find's compression in
//    the reference never changes a root or a height), so the results are the
//    reference's. A warp reads a child's row with one coalesced 32-byte load.
//  * Adding v: the roots adjacent to v are a warp OR of (1 << root(u)) over
//    v's neighbours u in S, v's height is 1 + a warp max over those roots'
//    heights, and every lane whose root is among them re-points to v.
//  * Subsets of a level are ranked in colex order (the reference's
//    set_encoder); a warp unranks its subset with ballots over a binomial
//    table and lane v ranks the child S - v by a prefix and a suffix sum.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "gtd_handle.h"

namespace gtd {
namespace {

constexpr int kBuMaxN = GTD_BOTTOM_UP_MAX_N;  // 32: one 32-byte row, lane = vertex
constexpr int kBuWarps = 8;
constexpr int kBuChunk = 16;  // consecutive subsets per warp between unrankings
constexpr uint8_t kFreshRoot = 0x81;  // a root of height 1 (a vertex not yet added)

struct BuParams {
  uint32_t binom[kBuMaxN + 1][kBuMaxN + 1];  // C(a, b)
  uint64_t adj[kBuMaxN];                     // adjacency masks
  int n = 0;
  int level = 0;                             // subset size i
  uint32_t count = 0;                        // C(n, i)
  uint64_t last_off = 0;                     // first history entry of level i
  const uint8_t* prev = nullptr;             // level i - 1 rows (32 B)
  const uint8_t* prev_h = nullptr;           // level i - 1 forest heights
  uint8_t* next = nullptr;                   // level i rows
  uint8_t* next_h = nullptr;
  uint8_t* last = nullptr;                   // history: last vertex of every subset, level-major
};

__global__ void __launch_bounds__(32 * kBuWarps) bu_level_kernel(const __grid_constant__ BuParams p) {
  // The binomial table in shared memory: lanes read different entries
  // (C(lane, k)), which the parameter bank would serve one address at a time.
  __shared__ uint32_t binom[kBuMaxN + 1][kBuMaxN + 1];
  for (int i = threadIdx.x; i < (kBuMaxN + 1) * (kBuMaxN + 1); i += blockDim.x)
    (&binom[0][0])[i] = (&p.binom[0][0])[i];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const uint32_t full = 0xffffffffu;
  // lane u's neighbours (n <= 32); u is a neighbour of v iff v is one of u's
  const uint32_t my_adj = lane < p.n ? static_cast<uint32_t>(p.adj[lane]) : 0u;
  const uint32_t warps = gridDim.x * kBuWarps;
  // Each warp takes kBuChunk consecutive ranks: it unranks the first and
  // steps to the next subset of the level in colex order (the next larger
  // mask of the same popcount) for the others.
  uint32_t S = 0;
  for (uint64_t r = uint64_t(blockIdx.x * kBuWarps + (threadIdx.x >> 5)) * kBuChunk, first = r, cend = 0;
       r < p.count; ++r) {
    if (r == first) {
      cend = first + kBuChunk;
      // unrank r among the i-subsets (colex): the largest a with C(a, k) <= rest
      uint32_t rest = static_cast<uint32_t>(r);
      S = 0;
      for (int k = p.level; k > 0; --k) {
        const uint32_t c = lane < p.n ? binom[lane][k] : 0xffffffffu;
        const int a = 31 - __clz(__ballot_sync(full, c <= rest));
        S |= 1u << a;
        rest -= binom[a][k];
      }
    } else {
      const uint64_t low = S & (0u - S), up = uint64_t(S) + low;  // warp-uniform
      S = static_cast<uint32_t>(((up ^ S) >> (__ffs(static_cast<int>(S)) + 1)) | up);
    }
    // lane v in S: colex rank of S - v (bits below v keep their term
    // C(u, q + 1), bits above shift down to C(u, q))
    const bool inS = (S >> lane) & 1u;
    const uint32_t q = __popc(S & ((1u << lane) - 1u));
    const uint32_t t1 = inS ? binom[lane][q + 1] : 0u, t0 = inS ? binom[lane][q] : 0u;
    uint32_t pre = t1, suf = t0;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t x = __shfl_up_sync(full, pre, d);
      const uint32_t y = __shfl_down_sync(full, suf, d);
      if (lane >= d)
        pre += x;
      if (lane + d < 32)
        suf += y;
    }
    const uint32_t child = (pre - t1) + (suf - t0);

    uint32_t best = 0xffu, best_v = 0xffu;
    uint32_t best_ent = kFreshRoot;
    // candidates in ascending order; the next candidate's child row is loaded
    // while the current one is evaluated
    uint32_t todo = S;
    int v = __ffs(todo) - 1;
    uint32_t c = __shfl_sync(full, child, v);
    uint32_t ent = p.prev[size_t(c) * 32 + lane];  // rows are whole: lanes >= n hold fresh roots
    uint32_t hc = p.prev_h[c];
    for (;;) {
      const uint32_t todo_next = todo & (todo - 1);
      int v_next = 0;
      uint32_t ent_next = kFreshRoot, hc_next = 0;
      if (todo_next) {  // warp-uniform
        v_next = __ffs(todo_next) - 1;
        const uint32_t c_next = __shfl_sync(full, child, v_next);
        ent_next = p.prev[size_t(c_next) * 32 + lane];
        hc_next = p.prev_h[c_next];
      }
      const bool is_root = ent & 0x80u;
      const uint32_t root = is_root ? static_cast<uint32_t>(lane) : ent;
      const bool nbr = inS && ((my_adj >> v) & 1u);  // lane is a neighbour of v inside S
      const uint32_t R = __reduce_or_sync(full, nbr ? (1u << root) : 0u);
      const uint32_t m = __reduce_max_sync(full, ((R >> lane) & 1u) ? (ent & 0x7Fu) : 0u);
      const uint32_t h = max(hc, m + 1);
      if (h < best) {  // strict: the first v with the least height
        best = h;
        best_v = static_cast<uint32_t>(v);
        best_ent = lane == v ? (0x80u | (m + 1)) : (((R >> root) & 1u) ? static_cast<uint32_t>(v) : ent);
      }
      if (!todo_next)
        break;
      todo = todo_next;
      v = v_next;
      ent = ent_next;
      hc = hc_next;
    }
    p.next[size_t(r) * 32 + lane] = static_cast<uint8_t>(best_ent);
    if (lane == 0) {
      p.next_h[r] = static_cast<uint8_t>(best);
      p.last[p.last_off + r] = static_cast<uint8_t>(best_v);
    }
    if (r + 1 == cend) {  // chunk done: jump to this warp's next chunk
      first = r + 1 + uint64_t(warps - 1) * kBuChunk;
      r = first - 1;
    }
  }
}

// GetElimination(n, n, 0) (bottom_up_heuristic_gpu_algorithm.hpp:104-120):
// the last vertex of the remaining set, level by level down from V.
__global__ void bu_order_kernel(const __grid_constant__ BuParams p, const uint64_t* level_off, int32_t* order) {
  if (threadIdx.x != 0 || blockIdx.x != 0)
    return;
  uint32_t S = p.n == 32 ? 0xffffffffu : ((1u << p.n) - 1u);
  for (int step = 0; step < p.n; ++step) {
    const int k = __popc(S);
    uint32_t rank = 0;
    int qq = 0;
    for (uint32_t t = S; t; t &= t - 1)
      rank += p.binom[__ffs(t) - 1][++qq];
    const int v = p.last[level_off[k] + rank];
    order[step] = v;
    S &= ~(1u << (v & 31));
  }
}

uint64_t binom64(int a, int b) {
  if (b < 0 || b > a)
    return 0;
  uint64_t r = 1;
  for (int i = 1; i <= b; ++i)
    r = r * uint64_t(a - b + i) / uint64_t(i);
  return r;
}

// The elimination-tree replay of an order (elimination_tree.cpp:24-70, as
// BottomUpHeuristicGPU::Get eliminates its order): each vertex's parent is
// the last eliminated vertex whose component contained it.
int replay_order(const uint64_t* adj, int n, const int32_t* order, int32_t* parent) {
  uint64_t remaining = n == 64 ? ~0ull : ((1ull << n) - 1);
  std::vector<int> owner(n, -1), depth(n, 0);
  int height = 0;
  for (int i = 0; i < n; ++i) {
    const int v = order[i];
    if (v < 0 || v >= n || !((remaining >> v) & 1ull))
      return -1;
    parent[v] = owner[v];
    height = std::max(height, depth[v] + 1);
    uint64_t reach = 1ull << v, frontier = reach;
    while (frontier) {
      uint64_t nb = 0;
      for (uint64_t f = frontier; f; f &= f - 1)
        nb |= adj[__builtin_ctzll(f)];
      nb &= remaining & ~reach;
      reach |= nb;
      frontier = nb;
    }
    remaining &= ~(1ull << v);
    for (uint64_t s = reach & ~(1ull << v); s; s &= s - 1) {
      const int u = __builtin_ctzll(s);
      owner[u] = v;
      depth[u] = depth[v] + 1;
    }
  }
  return height;
}

}  // namespace
}  // namespace gtd

using namespace gtd;

extern "C" gtd_status gtd_bottom_up(gtd_handle h, const uint64_t* adj, int n, int32_t* td_out, int32_t* parent_out,
                                    int32_t* order_out) {
  if (!h)
    return GTD_INVALID_ARG;
  if (!adj || !td_out || !parent_out)
    return fail(h, GTD_INVALID_ARG, "null pointer argument");
  if (n < 1)
    return fail(h, GTD_INVALID_ARG, "n must be at least 1");
  if (n > kBuMaxN)
    return fail(h, GTD_NO_RESULT, "the bottom-up heuristic keeps one 32-byte forest per subset: n <= " +
                                      std::to_string(kBuMaxN));
  gtd_status s = check_adjacency(h, adj, n);
  if (s != GTD_OK)
    return s;
  DeviceGuard guard(h->device);
  uint64_t max_c = 0;
  std::vector<uint64_t> level_off(n + 2, 0);
  for (int k = 0; k <= n; ++k) {
    max_c = std::max(max_c, binom64(n, k));
    level_off[k + 1] = level_off[k] + binom64(n, k);
  }
  // [prev rows][next rows][prev heights][next heights][history][level offsets][order]
  const size_t rows = max_c * 32, heights = max_c, hist = size_t(1) << n;
  const size_t off_next = rows, off_ph = 2 * rows, off_nh = off_ph + heights, off_hist = off_nh + heights;
  const size_t off_lvl = (off_hist + hist + 15) & ~size_t(15);
  const size_t off_order = off_lvl + level_off.size() * sizeof(uint64_t);
  const size_t bytes = off_order + 64 * sizeof(int32_t);
  GTD_CUDA(h, ensure_field(&h->d_bu, &h->bu_cap, bytes));
  uint8_t* base = h->d_bu;

  BuParams p;
  for (int a = 0; a <= kBuMaxN; ++a)
    for (int b = 0; b <= kBuMaxN; ++b)
      p.binom[a][b] = static_cast<uint32_t>(binom64(a, b));
  for (int v = 0; v < kBuMaxN; ++v)
    p.adj[v] = v < n ? adj[v] : 0ull;
  p.n = n;
  p.last = base + off_hist;
  uint8_t* rows_a = base;
  uint8_t* rows_b = base + off_next;
  uint8_t* h_a = base + off_ph;
  uint8_t* h_b = base + off_nh;
  // level 0: the empty set's forest (every vertex a fresh root), height 1
  GTD_CUDA(h, cudaMemsetAsync(rows_a, kFreshRoot, 32, h->stream));
  GTD_CUDA(h, cudaMemsetAsync(h_a, 1, 1, h->stream));
  GTD_CUDA(h, cudaMemsetAsync(p.last, 0xFF, 1, h->stream));
  GTD_CUDA(h, cudaMemcpyAsync(base + off_lvl, level_off.data(), level_off.size() * sizeof(uint64_t),
                              cudaMemcpyHostToDevice, h->stream));
  int occ = 0;
  GTD_CUDA(h, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, bu_level_kernel, 32 * kBuWarps, 0));
  const uint64_t max_ctas = uint64_t(h->num_sms) * std::max(1, occ);
  GTD_CUDA(h, cudaEventRecord(h->ev[0], h->stream));
  for (int i = 1; i <= n; ++i) {
    p.level = i;
    p.count = static_cast<uint32_t>(binom64(n, i));
    p.last_off = level_off[i];
    p.prev = rows_a;
    p.prev_h = h_a;
    p.next = rows_b;
    p.next_h = h_b;
    const uint64_t ctas = std::min<uint64_t>(max_ctas, (p.count + kBuWarps * kBuChunk - 1) / (kBuWarps * kBuChunk));
    bu_level_kernel<<<static_cast<unsigned>(ctas), 32 * kBuWarps, 0, h->stream>>>(p);
    GTD_CUDA(h, cudaGetLastError());
    std::swap(rows_a, rows_b);
    std::swap(h_a, h_b);
  }
  int32_t* d_order = reinterpret_cast<int32_t*>(base + off_order);
  bu_order_kernel<<<1, 32, 0, h->stream>>>(p, reinterpret_cast<const uint64_t*>(base + off_lvl), d_order);
  GTD_CUDA(h, cudaGetLastError());
  GTD_CUDA(h, cudaEventRecord(h->ev[1], h->stream));
  std::vector<int32_t> order(n);
  GTD_CUDA(h, cudaMemcpyAsync(order.data(), d_order, n * sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
  GTD_CUDA(h, cudaStreamSynchronize(h->stream));
  const int height = replay_order(adj, n, order.data(), parent_out);
  if (height < 0)
    return fail(h, GTD_ABORTED, "the bottom-up order is not a permutation");
  *td_out = height;
  if (order_out)
    std::memcpy(order_out, order.data(), n * sizeof(int32_t));
  return GTD_OK;
}
