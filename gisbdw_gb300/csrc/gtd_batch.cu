// Batched subset DP: many graphs of uneven size in one persistent launch.
//
// Planning (host): graphs are put in descending n, each gets a table region,
// a flag range and a descriptor. Tickets run level-major across graphs
// (level 0 of every graph, then level 1, ...), so the children a tile waits
// for were issued long before it; the ticket -> (graph, tile) map is filled
// on the device. The launch sequence (zero the flags and
// control words, validate, DP, tree) is captured once in a CUDA graph and
// replayed while the batch keeps its shape and buffers.
//
// The autotuner times the DP kernel per (n, tile bits) on seeded random
// graphs; the planner then gives each vertex count its own tile size
// (pick_tile_bits) and, when the sizes differ, launches the mixed-size
// kernel, whose tiles dispatch on their graph's size.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "gtd_handle.h"

namespace gtd {
namespace {

struct Plan {
  int lb = 10;                  // the launch's (largest) tile bits
  bool mixed = false;           // graphs carry their own tile bits
  int lb_by_n[GTD_DP_MAX_N + 1] = {};
  std::vector<DpGraph> graphs;  // processing order
  uint64_t table_bytes = 0;
  uint32_t total_tiles = 0;
  uint64_t subsets = 0;
  uint64_t alg_bytes = 0;
  std::vector<uint32_t> level_base;  // [graph][level]: first ticket of that level
};

constexpr int kLevelSlots = kDpMaxHigh + 2;

// Tile bits per vertex count. An explicit opts->tile_bits gives every graph
// that size. Otherwise, when the autotuner has rates (subsets per us of the
// one-size kernel at its own occupancy) for every n of the batch, the
// candidates are
//  * one size lb for all graphs: predicted time sum 2^max(n, lb) / rate(n, lb);
//  * per cap c = 8..12, each n at its own best size lb <= c in the mixed-size
//    kernel, whose shared memory is laid out for c: a size-lb tile then runs
//    at the mixed kernel's occupancy at c instead of the one-size kernel's at
//    lb (time x occ_one(lb) / occ_mixed(c) when that is above 1), divided by
//    the autotuner's measured mixed-kernel efficiency at c with its own
//    occupancy share taken out (what is left: the dispatch's extra work);
// and the least predicted time wins. No rates: 10 bits. force_cap > 0 (the
// autotuner's own measurement) plans a mixed launch at that cap.
void pick_tile_bits(gtd_handle h, const gtd_graph_desc* descs, int count, const gtd_dp_batch_opts* opts, Plan& P,
                    int force_cap = 0) {
  std::vector<int> count_by_n(GTD_DP_MAX_N + 1, 0);
  for (int i = 0; i < count; ++i)
    ++count_by_n[descs[i].n];
  auto uniform = [&](int lb) {
    P.lb = lb;
    P.mixed = false;
    for (int n = 0; n <= GTD_DP_MAX_N; ++n)
      P.lb_by_n[n] = count_by_n[n] ? lb : 0;
  };
  if (force_cap > 0) {
    uniform(force_cap);
    P.mixed = true;
    return;
  }
  if (opts && opts->tile_bits > 0) {
    uniform(std::min(std::max(opts->tile_bits, kTuneLbMin), kTuneLbMax));
    return;
  }
  for (int n = 0; n <= GTD_DP_MAX_N; ++n)
    for (int lb = kTuneLbMin; lb <= kTuneLbMax && count_by_n[n]; ++lb)
      if (h->tune[n][lb] <= 0) {
        uniform(10);
        return;
      }
  auto t_of = [&](int n, int lb) { return double(uint64_t(1) << std::max(n, lb)) / h->tune[n][lb]; };
  double best_cost = -1;
  for (int lb = kTuneLbMin; lb <= kTuneLbMax; ++lb) {
    double cost = 0;
    for (int n = 0; n <= GTD_DP_MAX_N; ++n)
      if (count_by_n[n])
        cost += t_of(n, lb) * count_by_n[n];
    if (best_cost < 0 || cost < best_cost) {
      best_cost = cost;
      uniform(lb);
    }
  }
  int occ_one[kTuneLbMax + 1] = {};
  for (int lb = kTuneLbMin; lb <= kTuneLbMax; ++lb)
    occ_one[lb] = std::max(1, dp_tile_occupancy(lb));
  for (int c = kTuneLbMin; c <= kTuneLbMax; ++c) {
    const int occ_mixed = dp_mixed_occupancy(c);
    const float eff = h->tune_mixed_eff[c];
    if (eff <= 0 || occ_mixed < 1)
      continue;  // unmeasured: never mix at this cap
    const double slow_c = std::max(1.0, double(occ_one[c]) / occ_mixed);
    const double residual = std::min(1.0, eff * slow_c);  // efficiency beyond the occupancy effect
    int choice[GTD_DP_MAX_N + 1] = {};
    double cost = 0;
    int lo = kTuneLbMax, hi = kTuneLbMin;
    for (int n = 0; n <= GTD_DP_MAX_N; ++n) {
      if (!count_by_n[n])
        continue;
      double best_t = -1;
      for (int lb = kTuneLbMin; lb <= c; ++lb) {
        const double t = t_of(n, lb) * std::max(1.0, double(occ_one[lb]) / occ_mixed);
        if (best_t < 0 || t < best_t) {
          best_t = t;
          choice[n] = lb;
        }
      }
      cost += best_t * count_by_n[n];
      lo = std::min(lo, choice[n]);
      hi = std::max(hi, choice[n]);
    }
    cost /= residual;
    if (lo != hi && hi == c && cost < best_cost) {
      best_cost = cost;
      P.lb = c;
      P.mixed = true;
      for (int n = 0; n <= GTD_DP_MAX_N; ++n)
        P.lb_by_n[n] = choice[n];
    }
  }
}

void make_plan(Plan& P, const gtd_graph_desc* descs, int count) {
  std::vector<int> order(count);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return descs[a].n > descs[b].n; });
  P.graphs.resize(count);
  uint64_t off = 0;
  uint32_t tile = 0;
  for (int k = 0; k < count; ++k) {
    const gtd_graph_desc& d = descs[order[k]];
    DpGraph& G = P.graphs[k];
    const int lb = P.lb_by_n[d.n];
    G.n = d.n;
    G.lb = lb;
    G.nh = d.n > lb ? d.n - lb : 0;
    G.ntiles = 1u << G.nh;
    G.table_off = off;
    G.tile_base = tile;
    G.adj_off = static_cast<uint32_t>(d.offset);
    G.out_idx = order[k];
    off += uint64_t(G.ntiles) << lb;
    tile += G.ntiles;
    const uint64_t sub = uint64_t(1) << d.n;
    P.subsets += sub;
    P.alg_bytes += sub + uint64_t(d.n) * (sub / 2);
  }
  P.table_bytes = off;
  P.total_tiles = tile;
  // Tickets level-major across graphs: level 0 of every graph, then level 1...
  P.level_base.assign(size_t(count) * kLevelSlots, 0);
  uint32_t binom[kDpMaxHigh + 1][kDpMaxHigh + 1] = {};
  for (int a = 0; a <= kDpMaxHigh; ++a) {
    binom[a][0] = 1;
    for (int b = 1; b <= a; ++b)
      binom[a][b] = binom[a - 1][b - 1] + (b <= a - 1 ? binom[a - 1][b] : 0u);
  }
  uint32_t ticket = 0;
  for (int j = 0; j <= kDpMaxHigh; ++j)
    for (int k = 0; k < count; ++k) {
      const DpGraph& G = P.graphs[k];
      if (j <= G.nh) {
        P.level_base[size_t(k) * kLevelSlots + j] = ticket;
        ticket += binom[G.nh][j];
      }
    }
}

uint64_t fingerprint(const Plan& P, const void* adj, const void* td, const void* par, int ctas,
                     uint64_t timeout) {
  uint64_t x = 1469598103934665603ull;
  auto mix = [&](uint64_t v) {
    x ^= v + 0x9e3779b97f4a7c15ull + (x << 6) + (x >> 2);
  };
  mix(P.lb);
  mix(P.mixed);
  mix(P.graphs.size());
  for (const DpGraph& G : P.graphs) {
    mix(G.n);
    mix(G.lb);
    mix(G.adj_off);
    mix(G.out_idx);
  }
  mix(reinterpret_cast<uintptr_t>(adj));
  mix(reinterpret_cast<uintptr_t>(td));
  mix(reinterpret_cast<uintptr_t>(par));
  mix(ctas);
  mix(timeout);
  return x;
}

gtd_status check_descs(gtd_handle h, const gtd_graph_desc* descs, int count, int64_t pool_len) {
  if (!descs || count < 1)
    return fail(h, GTD_INVALID_ARG, "empty batch");
  for (int i = 0; i < count; ++i) {
    const gtd_graph_desc& d = descs[i];
    if (d.n < 1 || d.n > GTD_DP_MAX_N)
      return fail(h, GTD_INVALID_ARG, "graph " + std::to_string(i) + ": n out of range");
    if (d.offset < 0 || int64_t(d.offset) + d.n > pool_len)
      return fail(h, GTD_INVALID_ARG, "graph " + std::to_string(i) + ": offset outside the pool");
  }
  return GTD_OK;
}

// Plans the batch, (re)builds device state when the shape changed and
// enqueues the launch (graph replay or direct). Device pointers in/out.
gtd_status batch_enqueue(gtd_handle h, const gtd_graph_desc* descs, int count, const uint64_t* d_adj,
                         int32_t* d_td, int32_t* d_parent, const gtd_dp_batch_opts* opts, int force_cap = 0) {
  Plan P;
  pick_tile_bits(h, descs, count, opts, P, force_cap);
  make_plan(P, descs, count);
  const int lb = P.lb;
  const uint64_t timeout = (opts && opts->timeout_ns) ? opts->timeout_ns : 10ull * 1000 * 1000 * 1000;
  int occ = P.mixed ? dp_mixed_occupancy(lb) : dp_tile_occupancy(lb);
  if (opts && opts->ctas_per_sm > 0 && opts->ctas_per_sm < occ)
    occ = opts->ctas_per_sm;
  if (occ < 1)
    occ = 1;
  long long ctas = static_cast<long long>(h->num_sms) * occ;
  if (ctas > P.total_tiles)
    ctas = P.total_tiles;
  const bool use_graph = !opts || opts->use_cuda_graph;
  const uint64_t key = fingerprint(P, d_adj, d_td, d_parent, static_cast<int>(ctas), timeout);

  gtd_dp_batch_stats& st = h->bstats;
  st = gtd_dp_batch_stats{};
  st.subsets = P.subsets;
  st.alg_bytes = P.alg_bytes;
  st.table_bytes = P.table_bytes;
  st.tile_bits = lb;
  st.tiles = static_cast<int>(P.total_tiles);
  st.ctas = static_cast<int>(ctas);
  for (int n = 0; n <= GTD_DP_MAX_N; ++n)
    st.tile_bits_by_n[n] = P.lb_by_n[n];

  // The captured graph holds the handle's buffer addresses: replay only while
  // no other call has reallocated them (a larger single solve grows the table).
  const DpBatchParams& cap = h->bparams;
  const bool same_buffers = cap.table == h->d_table && cap.flags == h->d_flags && cap.tile_map == h->d_tile_map &&
                            cap.level_base == h->d_level_base && cap.graphs == h->d_bgraphs;
  const bool poison = take_poison_fault();  // test injection (gtd_inject_fault)
  if (use_graph && h->bgraph_valid && h->bgraph_key == key && same_buffers) {
    st.graph_replayed = 1;
    if (poison)
      GTD_CUDA(h, cudaMemsetAsync(h->d_table, 0xFF, P.table_bytes, h->stream));
    GTD_CUDA(h, cudaEventRecord(h->ev[0], h->stream));
    GTD_CUDA(h, cudaGraphLaunch(h->bgraph, h->stream));
    GTD_CUDA(h, cudaEventRecord(h->ev[1], h->stream));
    h->have_table = false;
    return GTD_OK;
  }

  // Device state for this shape.
  h->have_table = false;
  h->bgraph_valid = false;
  GTD_CUDA(h, ensure_field(&h->d_table, &h->table_cap, P.table_bytes));
  gtd_status s = ensure_flags(h, P.total_tiles);
  if (s != GTD_OK)
    return s;
  GTD_CUDA(h, ensure_field(&h->d_tile_map, &h->tile_map_cap, P.total_tiles));
  GTD_CUDA(h, ensure_field(&h->d_level_base, &h->level_base_cap, P.level_base.size()));
  GTD_CUDA(h, ensure_field(&h->d_bgraphs, &h->bgraphs_cap, size_t(count)));
  // Descriptors and level bases go up through pinned staging (synchronised
  // below, so the staging is released right after).
  const size_t gbytes = count * sizeof(DpGraph), lbytes = P.level_base.size() * sizeof(uint32_t);
  void* stage = nullptr;
  GTD_CUDA(h, cudaMallocHost(&stage, gbytes + lbytes));
  std::memcpy(stage, P.graphs.data(), gbytes);
  std::memcpy(static_cast<char*>(stage) + gbytes, P.level_base.data(), lbytes);
  cudaError_t e = cudaMemcpyAsync(h->d_bgraphs, stage, gbytes, cudaMemcpyHostToDevice, h->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(h->d_level_base, static_cast<char*>(stage) + gbytes, lbytes, cudaMemcpyHostToDevice,
                        h->stream);
  if (e == cudaSuccess)
    e = cudaStreamSynchronize(h->stream);
  cudaFreeHost(stage);
  GTD_CUDA(h, e);

  DpBatchParams& bp = h->bparams;
  bp = DpBatchParams{};
  dp_fill_binom(bp);
  bp.graphs = h->d_bgraphs;
  bp.tile_map = h->d_tile_map;
  bp.level_base = h->d_level_base;
  bp.num_graphs = count;
  bp.lb = lb;
  bp.mixed = P.mixed ? 1 : 0;
  bp.total_tiles = P.total_tiles;
  bp.table = h->d_table;
  bp.flags = h->d_flags;
  bp.ticket = reinterpret_cast<uint32_t*>(h->d_io + kIoTicket);
  bp.error = h->d_io + kIoError;
  bp.adj = d_adj;
  bp.timeout_ns = timeout;
  bp.td_out = d_td;
  bp.parent_out = d_parent;
  GTD_CUDA(h, dp_launch_fill_tile_map(bp, h->stream));
  if (poison)
    GTD_CUDA(h, cudaMemsetAsync(h->d_table, 0xFF, P.table_bytes, h->stream));

  if (use_graph) {
    if (h->bgraph) {
      cudaGraphExecDestroy(h->bgraph);
      h->bgraph = nullptr;
    }
    bp.epoch = kGraphEpoch;
    cudaGraph_t graph = nullptr;
    GTD_CUDA(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t ce = cudaMemsetAsync(h->d_flags, 0, size_t(P.total_tiles) * sizeof(uint32_t), h->stream);
    if (ce == cudaSuccess)
      ce = cudaMemsetAsync(h->d_io, 0, 4 * sizeof(int32_t), h->stream);
    if (ce == cudaSuccess)
      ce = dp_launch_validate(bp, h->stream);
    if (ce == cudaSuccess)
      ce = dp_launch_tiles(bp, static_cast<int>(ctas), h->stream);
    if (ce == cudaSuccess)
      ce = dp_launch_tree(bp, h->stream);
    cudaError_t ee = cudaStreamEndCapture(h->stream, &graph);
    if (ce == cudaSuccess)
      ce = ee;
    if (ce == cudaSuccess)
      ce = cudaGraphInstantiate(&h->bgraph, graph, 0);
    if (graph)
      cudaGraphDestroy(graph);
    GTD_CUDA(h, ce);
    h->bgraph_key = key;
    h->bgraph_valid = true;
    GTD_CUDA(h, cudaEventRecord(h->ev[0], h->stream));
    GTD_CUDA(h, cudaGraphLaunch(h->bgraph, h->stream));
    GTD_CUDA(h, cudaEventRecord(h->ev[1], h->stream));
  } else {
    s = next_epoch(h, &bp.epoch);
    if (s != GTD_OK)
      return s;
    GTD_CUDA(h, cudaMemsetAsync(h->d_io, 0, 4 * sizeof(int32_t), h->stream));
    GTD_CUDA(h, cudaEventRecord(h->ev[0], h->stream));
    GTD_CUDA(h, dp_launch_validate(bp, h->stream));
    GTD_CUDA(h, dp_launch_tiles(bp, static_cast<int>(ctas), h->stream));
    GTD_CUDA(h, dp_launch_tree(bp, h->stream));
    GTD_CUDA(h, cudaEventRecord(h->ev[1], h->stream));
  }
  return GTD_OK;
}

gtd_status batch_finish(gtd_handle h, gtd_dp_batch_stats* stats) {
  int32_t* h_io = reinterpret_cast<int32_t*>(static_cast<char*>(h->h_pinned) + 1024);
  GTD_CUDA(h, cudaMemcpyAsync(h_io, h->d_io, 4 * sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
  GTD_CUDA(h, cudaStreamSynchronize(h->stream));
  float ms = 0;
  if (cudaEventElapsedTime(&ms, h->ev[0], h->ev[1]) == cudaSuccess)
    h->bstats.dp_ms = ms;
  if (stats)
    *stats = h->bstats;
  return map_device_error(h, h_io[kIoError], h_io[kIoError + 1]);
}

gtd_status grow_pinned(gtd_handle h, size_t bytes) {
  if (h->bstage_cap >= bytes)
    return GTD_OK;
  if (h->h_bstage)
    cudaFreeHost(h->h_bstage);
  h->h_bstage = nullptr;
  h->bstage_cap = 0;
  GTD_CUDA(h, cudaMallocHost(&h->h_bstage, bytes));
  h->bstage_cap = bytes;
  return GTD_OK;
}

// Seeded random G(n, 0.3) graphs for the autotuner (splitmix64 draws).
void random_graph(int n, uint64_t seed, uint64_t* adj) {
  uint64_t s = seed * 0x9E3779B97F4A7C15ull + 0x243F6A8885A308D3ull;
  for (int v = 0; v < n; ++v)
    adj[v] = 0;
  for (int u = 0; u < n; ++u)
    for (int v = u + 1; v < n; ++v) {
      s += 0x9E3779B97F4A7C15ull;
      uint64_t z = s;
      z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
      z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
      z ^= z >> 31;
      if ((z >> 11) * (1.0 / 9007199254740992.0) < 0.3) {
        adj[u] |= 1ull << v;
        adj[v] |= 1ull << u;
      }
    }
}

}  // namespace
}  // namespace gtd

namespace gtd {
namespace {
gtd_status solve_batch_host(gtd_handle h, const gtd_graph_desc* descs, int count, const uint64_t* adj_pool,
                            int64_t pool_len, int32_t* td_out, int32_t* parent_out, const gtd_dp_batch_opts* opts,
                            gtd_dp_batch_stats* stats, int force_cap);
}  // namespace
}  // namespace gtd

using namespace gtd;

extern "C" {

gtd_status gtd_dp_solve_batch_device(gtd_handle h, const gtd_graph_desc* descs, int count,
                                     const uint64_t* d_adj_pool, int64_t pool_len, int32_t* d_td,
                                     int32_t* d_parent, const gtd_dp_batch_opts* opts) {
  if (!h)
    return GTD_INVALID_ARG;
  gtd_status s = check_descs(h, descs, count, pool_len);
  if (s != GTD_OK)
    return s;
  if (!d_adj_pool || !d_td || !d_parent)
    return fail(h, GTD_INVALID_ARG, "null pointer argument");
  DeviceGuard g(h->device);
  return batch_enqueue(h, descs, count, d_adj_pool, d_td, d_parent, opts);
}

gtd_status gtd_dp_batch_sync(gtd_handle h, gtd_dp_batch_stats* stats) {
  if (!h)
    return GTD_INVALID_ARG;
  DeviceGuard g(h->device);
  return batch_finish(h, stats);
}

gtd_status gtd_dp_solve_batch(gtd_handle h, const gtd_graph_desc* descs, int count, const uint64_t* adj_pool,
                              int64_t pool_len, int32_t* td_out, int32_t* parent_out,
                              const gtd_dp_batch_opts* opts, gtd_dp_batch_stats* stats) {
  return solve_batch_host(h, descs, count, adj_pool, pool_len, td_out, parent_out, opts, stats, 0);
}

}  // extern "C"

namespace gtd {
namespace {

gtd_status solve_batch_host(gtd_handle h, const gtd_graph_desc* descs, int count, const uint64_t* adj_pool,
                            int64_t pool_len, int32_t* td_out, int32_t* parent_out, const gtd_dp_batch_opts* opts,
                            gtd_dp_batch_stats* stats, int force_cap) {
  if (!h)
    return GTD_INVALID_ARG;
  gtd_status s = check_descs(h, descs, count, pool_len);
  if (s != GTD_OK)
    return s;
  if (!adj_pool || !td_out || !parent_out)
    return fail(h, GTD_INVALID_ARG, "null pointer argument");
  for (int i = 0; i < count; ++i) {
    s = check_adjacency(h, adj_pool + descs[i].offset, descs[i].n);
    if (s != GTD_OK)
      return fail(h, s, "graph " + std::to_string(i) + ": " + h->last_error);
  }
  const auto t0 = std::chrono::steady_clock::now();
  DeviceGuard g(h->device);
  const size_t adj_bytes = size_t(pool_len) * sizeof(uint64_t);
  const size_t out_bytes = size_t(count) * sizeof(int32_t) + size_t(pool_len) * sizeof(int32_t);
  s = grow_pinned(h, adj_bytes + out_bytes);
  if (s != GTD_OK)
    return s;
  GTD_CUDA(h, ensure_field(&h->d_badj, &h->badj_cap, size_t(pool_len)));
  GTD_CUDA(h, ensure_field(&h->d_btd, &h->btd_cap, size_t(count)));
  GTD_CUDA(h, ensure_field(&h->d_bparent, &h->bparent_cap, size_t(pool_len)));

  char* stage = static_cast<char*>(h->h_bstage);
  std::memcpy(stage, adj_pool, adj_bytes);
  GTD_CUDA(h, cudaMemcpyAsync(h->d_badj, stage, adj_bytes, cudaMemcpyHostToDevice, h->stream));
  s = batch_enqueue(h, descs, count, h->d_badj, h->d_btd, h->d_bparent, opts, force_cap);
  if (s != GTD_OK)
    return s;
  int32_t* h_td = reinterpret_cast<int32_t*>(stage + adj_bytes);
  int32_t* h_par = h_td + count;
  GTD_CUDA(h, cudaMemcpyAsync(h_td, h->d_btd, count * sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
  GTD_CUDA(h, cudaMemcpyAsync(h_par, h->d_bparent, size_t(pool_len) * sizeof(int32_t), cudaMemcpyDeviceToHost,
                              h->stream));
  s = batch_finish(h, nullptr);
  if (s != GTD_OK)
    return s;
  std::memcpy(td_out, h_td, count * sizeof(int32_t));
  for (int i = 0; i < count; ++i)
    std::memcpy(parent_out + descs[i].offset, h_par + descs[i].offset, descs[i].n * sizeof(int32_t));
  h->bstats.total_ms =
      std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (stats)
    *stats = h->bstats;
  return GTD_OK;
}

}  // namespace
}  // namespace gtd

extern "C" {

gtd_status gtd_dp_set_rates(gtd_handle h, int n_min, int n_max, const float* rates, const float* mixed_eff) {
  if (!h)
    return GTD_INVALID_ARG;
  if (!rates || n_min < 2 || n_max > GTD_DP_MAX_N || n_min > n_max)
    return fail(h, GTD_INVALID_ARG, "rates must cover a range inside [2, " + std::to_string(GTD_DP_MAX_N) + "]");
  for (int n = n_min; n <= n_max; ++n)
    for (int lb = kTuneLbMin; lb <= kTuneLbMax; ++lb) {
      const float r = rates[(n - n_min) * (kTuneLbMax - kTuneLbMin + 1) + (lb - kTuneLbMin)];
      h->tune[n][lb] = r > 0 ? r : 0.f;
    }
  for (int c = kTuneLbMin; c <= kTuneLbMax; ++c)
    h->tune_mixed_eff[c] = (mixed_eff && mixed_eff[c - kTuneLbMin] > 0) ? mixed_eff[c - kTuneLbMin] : 0.f;
  h->bgraph_valid = false;  // a plan may change
  return GTD_OK;
}

gtd_status gtd_dp_autotune(gtd_handle h, int n_min, int n_max, float* rates_out, float* mixed_eff_out) {
  if (!h)
    return GTD_INVALID_ARG;
  if (n_min < 2 || n_max > 30 || n_min > n_max)
    return fail(h, GTD_INVALID_ARG, "autotune range must lie in [2, 30]");
  DeviceGuard g(h->device);
  for (int n = n_min; n <= n_max; ++n) {
    const int count = n >= 20 ? 64 : (1 << (26 - n));
    std::vector<uint64_t> adj(size_t(count) * n);
    std::vector<gtd_graph_desc> descs(count);
    for (int i = 0; i < count; ++i) {
      random_graph(n, uint64_t(n) * 1000003ull + i, adj.data() + size_t(i) * n);
      descs[i].n = n;
      descs[i].offset = i * n;
    }
    const int64_t pool = int64_t(count) * n;
    std::vector<int32_t> td(count), par(pool);
    // the one-size kernel at every tile size; at n_max also the mixed-size
    // kernel at every cap (all graphs at that size), for its efficiency
    for (int pass = 0; pass < (n == n_max ? 2 : 1); ++pass)
      for (int lb = kTuneLbMin; lb <= kTuneLbMax; ++lb) {
        gtd_dp_batch_opts o{lb, 0, 0, 1};
        gtd_dp_batch_stats st{};
        float best = 0;
        for (int rep = 0; rep < 3; ++rep) {
          gtd_status s = solve_batch_host(h, descs.data(), count, adj.data(), pool, td.data(), par.data(),
                                          pass ? nullptr : &o, &st, pass ? lb : 0);
          if (s != GTD_OK)
            return s;
          if (rep > 0 && (best == 0 || st.dp_ms < best))
            best = st.dp_ms;
        }
        const float rate = best > 0 ? float(double(st.subsets) / (best * 1000.0)) : 0.f;  // per microsecond
        if (pass == 0) {
          h->tune[n][lb] = rate;
          if (rates_out)
            rates_out[(n - n_min) * (kTuneLbMax - kTuneLbMin + 1) + (lb - kTuneLbMin)] = rate;
        } else {
          h->tune_mixed_eff[lb] = h->tune[n][lb] > 0 ? rate / h->tune[n][lb] : 0.f;
          if (mixed_eff_out)
            mixed_eff_out[lb - kTuneLbMin] = h->tune_mixed_eff[lb];
        }
      }
  }
  return GTD_OK;
}

}  // extern "C"
