// The greedy elimination heuristics of gtd_heuristics.cu as one batched GPU
// launch: one warp per graph, the same picks in the same order, so the trees
// are identical to the host's (and so to the reference's heuristic chain,
// Treedepth/src/branch_and_bound/heuristics/).
//
// Every step takes the component of the smallest remaining vertex
// (ComponentCmp, elimination_tree.hpp:67-72), picks a vertex of it and
// eliminates it: its parent is the vertex eliminated last in its component.
//   kind 1  highest degree inside the component, ties to the smallest id
//           (highest_degree_heuristic.hpp:18-44)
//   kind 2  variance score D / sqrt(gamma + A) + E * #components of C - v,
//           ties to the higher degree, then the smallest id
//           (variance_heuristic.hpp:24-78; A, D, E = 1.0, 0.2, 0.8), in
//           double with the host's operation order
//   kind 0  the better of kinds 1 and 2 (benchmark.cpp:50-55)
//   kind 3  the highest caller score, ties to the smallest id
#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "gtd_handle.h"

namespace gtd {
namespace {

constexpr int kHWarps = 4;
constexpr int kHMaxN = 128;

struct HeurGraph {
  int32_t n;
  int32_t off;  // first vertex's (lo, hi) pair in the pool, parent pool offset
};

struct HeurWarp {
  uint64_t alo[kHMaxN], ahi[kHMaxN];
  int16_t owner[kHMaxN];
  uint8_t cdepth[kHMaxN];
};

__device__ __forceinline__ bool hhas(uint64_t lo, uint64_t hi, int v) {
  return v < 64 ? ((lo >> v) & 1ull) : ((hi >> (v - 64)) & 1ull);
}
__device__ __forceinline__ void hclear(uint64_t& lo, uint64_t& hi, int v) {
  if (v < 64)
    lo &= ~(1ull << v);
  else
    hi &= ~(1ull << (v - 64));
}
__device__ __forceinline__ int hfirst(uint64_t lo, uint64_t hi) {
  return lo ? __ffsll(static_cast<long long>(lo)) - 1 : 63 + __ffsll(static_cast<long long>(hi));
}
__device__ __forceinline__ int hpopc(uint64_t lo, uint64_t hi) { return __popcll(lo) + __popcll(hi); }

// Component of S holding v, by one lane (serial BFS).
__device__ void lane_component(const HeurWarp* w, uint64_t Slo, uint64_t Shi, int v, uint64_t& rlo, uint64_t& rhi) {
  rlo = v < 64 ? (1ull << v) : 0ull;
  rhi = v >= 64 ? (1ull << (v - 64)) : 0ull;
  uint64_t flo = rlo, fhi = rhi;
  while (flo | fhi) {
    uint64_t nlo = 0, nhi = 0;
    while (flo | fhi) {
      const int u = hfirst(flo, fhi);
      hclear(flo, fhi, u);
      nlo |= w->alo[u];
      nhi |= w->ahi[u];
    }
    nlo &= Slo & ~rlo;
    nhi &= Shi & ~rhi;
    rlo |= nlo;
    rhi |= nhi;
    flo = nlo;
    fhi = nhi;
  }
}

// Variance score of removing v from C (variance_heuristic.hpp:40-56 as
// restated on the host, same order of operations).
__device__ double variance_coef(const HeurWarp* w, uint64_t Clo, uint64_t Chi, int v) {
  const float A = 1.0f, D = 0.2f, E = 0.8f;
  uint8_t sizes[kHMaxN];
  int nc = 0;
  uint64_t rlo = Clo, rhi = Chi;
  hclear(rlo, rhi, v);
  while (rlo | rhi) {
    uint64_t clo, chi;
    lane_component(w, rlo, rhi, hfirst(rlo, rhi), clo, chi);
    rlo &= ~clo;
    rhi &= ~chi;
    sizes[nc++] = static_cast<uint8_t>(hpopc(clo, chi));
  }
  // explicit round-to-nearest operations: no contraction into FMAs, so the
  // result is bit-identical to the host's
  double acc = 0.0;
  for (int i = 0; i < nc; ++i)
    acc = __dadd_rn(acc, static_cast<double>(sizes[i]));
  const double avg = __ddiv_rn(acc, static_cast<double>(nc));
  double gamma = 0.0;
  for (int i = 0; i < nc; ++i) {
    const double d = __dsub_rn(static_cast<double>(sizes[i]), avg);
    gamma = __dadd_rn(gamma, __dmul_rn(d, d));
  }
  const float enc = __fmul_rn(E, static_cast<float>(nc));
  return __dadd_rn(__ddiv_rn(static_cast<double>(D), __dsqrt_rn(__dadd_rn(gamma, static_cast<double>(A)))),
                   static_cast<double>(enc));
}

struct Pick {
  double coef;
  int deg, v;
};
// The host's scan order: higher coef, then higher degree, then smaller id.
__device__ __forceinline__ bool better(const Pick& a, const Pick& b) {
  if (a.v < 0)
    return false;
  if (b.v < 0)
    return true;
  if (a.coef != b.coef)
    return a.coef > b.coef;
  if (a.deg != b.deg)
    return a.deg > b.deg;
  return a.v < b.v;
}

// One greedy elimination of the warp's graph; returns the tree height.
__device__ int greedy(HeurWarp* w, int n, int kind, const float* scores, int32_t* parent) {
  const int lane = threadIdx.x & 31;
  for (int u = lane; u < n; u += 32) {
    w->owner[u] = -1;
    w->cdepth[u] = 0;
  }
  __syncwarp();
  uint64_t rem_lo = n >= 64 ? ~0ull : ((1ull << n) - 1);
  uint64_t rem_hi = n > 64 ? (n == 128 ? ~0ull : ((1ull << (n - 64)) - 1)) : 0ull;
  int height = 0;
  while (rem_lo | rem_hi) {
    // component of the smallest remaining vertex (every lane computes it)
    uint64_t Clo, Chi;
    lane_component(w, rem_lo, rem_hi, hfirst(rem_lo, rem_hi), Clo, Chi);
    Pick best{0.0, -1, -1};
    for (int k = 0; k < kHMaxN / 32; ++k) {
      const int u = lane + 32 * k;
      if (u >= n || !hhas(Clo, Chi, u))
        continue;
      Pick c{0.0, hpopc(w->alo[u] & Clo, w->ahi[u] & Chi), u};
      if (kind == 2)
        c.coef = variance_coef(w, Clo, Chi, u);
      else if (kind == 3)
        c = Pick{static_cast<double>(scores[u]), 0, u};
      else
        c.coef = static_cast<double>(c.deg);
      if (better(c, best))
        best = c;
    }
    for (int off = 16; off > 0; off >>= 1) {
      Pick o;
      o.coef = __shfl_xor_sync(0xffffffffu, best.coef, off);
      o.deg = __shfl_xor_sync(0xffffffffu, best.deg, off);
      o.v = __shfl_xor_sync(0xffffffffu, best.v, off);
      if (better(o, best))
        best = o;
    }
    const int v = best.v;
    const int dv = w->cdepth[v];
    if (lane == 0)
      parent[v] = w->owner[v];
    height = max(height, dv + 1);
    __syncwarp();
    for (int k = 0; k < kHMaxN / 32; ++k) {
      const int u = lane + 32 * k;
      if (u < n && u != v && hhas(Clo, Chi, u)) {
        w->owner[u] = static_cast<int16_t>(v);
        w->cdepth[u] = static_cast<uint8_t>(dv + 1);
      }
    }
    hclear(rem_lo, rem_hi, v);
    __syncwarp();
  }
  return height;
}

__global__ void __launch_bounds__(32 * kHWarps) heuristic_kernel(const HeurGraph* graphs, int count,
                                                                 const uint64_t* adj2, int kind, const float* scores,
                                                                 int32_t* td_out, int32_t* parent_out,
                                                                 int32_t* tmp_parent) {
  __shared__ HeurWarp wm[kHWarps];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  HeurWarp* w = &wm[warp];
  for (int g = blockIdx.x * kHWarps + warp; g < count; g += gridDim.x * kHWarps) {
    const HeurGraph G = graphs[g];
    for (int u = lane; u < G.n; u += 32) {
      w->alo[u] = adj2[2 * (size_t(G.off) + u)];
      w->ahi[u] = adj2[2 * (size_t(G.off) + u) + 1];
    }
    __syncwarp();
    int32_t* par = parent_out + G.off;
    const float* sc = scores ? scores + G.off : nullptr;
    int td;
    if (kind == 0) {
      td = greedy(w, G.n, 1, nullptr, par);
      int32_t* alt = tmp_parent + G.off;
      const int va = greedy(w, G.n, 2, nullptr, alt);
      __syncwarp();
      if (va < td) {  // the variance tree only when strictly lower, as on the host
        for (int u = lane; u < G.n; u += 32)
          par[u] = alt[u];
        td = va;
      }
    } else {
      td = greedy(w, G.n, kind, sc, par);
    }
    if (lane == 0)
      td_out[g] = td;
    __syncwarp();
  }
}

}  // namespace
}  // namespace gtd

using gtd::DeviceGuard;
using gtd::ensure_device;
using gtd::fail;

extern "C" gtd_status gtd_heuristic_batch(gtd_handle h, const gtd_graph_desc* descs, int count,
                                          const uint64_t* adj2_pool, int64_t pool_len, int kind,
                                          const float* scores_pool, int32_t* td_out, int32_t* parent_out) {
  if (!h)
    return GTD_INVALID_ARG;
  if (!descs || count < 1 || !adj2_pool || pool_len < 1 || !td_out || !parent_out || kind < 0 || kind > 3 ||
      (kind == 3 && !scores_pool))
    return fail(h, GTD_INVALID_ARG, "null pointer argument, empty batch, or kind outside 0..3 (3 needs scores)");
  std::vector<gtd::HeurGraph> graphs(count);
  for (int i = 0; i < count; ++i) {
    const gtd_graph_desc& d = descs[i];
    if (d.n < 1 || d.n > gtd::kHMaxN || d.offset < 0 || int64_t(d.offset) + d.n > pool_len)
      return fail(h, GTD_INVALID_ARG, "graph " + std::to_string(i) + ": n outside [1, 128] or outside the pool");
    const uint64_t* a = adj2_pool + 2 * size_t(d.offset);
    const uint64_t lo_ok = d.n >= 64 ? ~0ull : ((1ull << d.n) - 1);
    const uint64_t hi_ok = d.n <= 64 ? 0ull : (d.n >= 128 ? ~0ull : ((1ull << (d.n - 64)) - 1));
    for (int v = 0; v < d.n; ++v) {
      const bool self = v < 64 ? ((a[2 * v] >> v) & 1ull) : ((a[2 * v + 1] >> (v - 64)) & 1ull);
      const bool beyond = (a[2 * v] & ~lo_ok) != 0 || (a[2 * v + 1] & ~hi_ok) != 0;
      if (self || beyond)
        return fail(h, GTD_INVALID_ARG, "graph " + std::to_string(i) + ": self loop or adjacency bit >= n");
    }
    graphs[i] = gtd::HeurGraph{d.n, d.offset};
  }
  DeviceGuard guard(h->device);
  const size_t n_pool = static_cast<size_t>(pool_len);
  const size_t bytes = 256 + count * sizeof(gtd::HeurGraph) + 2 * n_pool * sizeof(uint64_t) +
                       (scores_pool ? n_pool * sizeof(float) : 0) + size_t(count) * 4 + 2 * n_pool * 4 + 1024;
  GTD_CUDA(h, ensure_device(&h->d_scratch, &h->scratch_cap, bytes));
  char* base = static_cast<char*>(h->d_scratch);
  auto carve = [&](size_t b) {
    char* p = base;
    base += (b + 255) & ~size_t(255);
    return p;
  };
  auto* d_graphs = reinterpret_cast<gtd::HeurGraph*>(carve(count * sizeof(gtd::HeurGraph)));
  auto* d_adj = reinterpret_cast<uint64_t*>(carve(2 * n_pool * sizeof(uint64_t)));
  auto* d_scores = scores_pool ? reinterpret_cast<float*>(carve(n_pool * sizeof(float))) : nullptr;
  auto* d_td = reinterpret_cast<int32_t*>(carve(size_t(count) * 4));
  auto* d_par = reinterpret_cast<int32_t*>(carve(n_pool * 4));
  auto* d_tmp = reinterpret_cast<int32_t*>(carve(n_pool * 4));
  cudaStream_t s = h->stream;
  GTD_CUDA(h, cudaMemcpyAsync(d_graphs, graphs.data(), count * sizeof(gtd::HeurGraph), cudaMemcpyHostToDevice, s));
  GTD_CUDA(h, cudaMemcpyAsync(d_adj, adj2_pool, 2 * n_pool * sizeof(uint64_t), cudaMemcpyHostToDevice, s));
  if (d_scores)
    GTD_CUDA(h, cudaMemcpyAsync(d_scores, scores_pool, n_pool * sizeof(float), cudaMemcpyHostToDevice, s));
  const int blocks = std::min(4096, (count + gtd::kHWarps - 1) / gtd::kHWarps);
  gtd::heuristic_kernel<<<blocks, 32 * gtd::kHWarps, 0, s>>>(d_graphs, count, d_adj, kind, d_scores, d_td, d_par,
                                                              d_tmp);
  GTD_CUDA(h, cudaGetLastError());
  GTD_CUDA(h, cudaMemcpyAsync(td_out, d_td, size_t(count) * 4, cudaMemcpyDeviceToHost, s));
  GTD_CUDA(h, cudaMemcpyAsync(parent_out, d_par, n_pool * 4, cudaMemcpyDeviceToHost, s));
  GTD_CUDA(h, cudaStreamSynchronize(s));
  return GTD_OK;
}
