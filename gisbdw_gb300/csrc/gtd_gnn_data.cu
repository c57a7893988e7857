// Host-side data pipeline of the learned branching order: vertex features,
// CSR batch packing, and training labels sampled from the exact DP.
//
// Labels: for a base graph (n <= 24) the DP table is solved on the GPU
// (gtd_dp_solve), connected induced subgraphs are sampled on the host (grown
// from a random vertex by random frontier vertices), and gtd_dp_labels reads
// td(S) and the optimal-root mask {v : td(S - v) = td(S) - 1} of each one.
// Every sample is written relabelled 0..|S|-1 in increasing vertex order.
//
// Features per vertex (8): degree / 4, core number / 4, eccentricity / 8,
// mean neighbour degree / 4, pendant flag, 1 / (1 + degree), n / 64, 1.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "gtd_handle.h"

namespace {

using u128 = unsigned __int128;

constexpr int kFeatures = 8;

inline int popc128(u128 x) {
  return __builtin_popcountll(static_cast<uint64_t>(x)) + __builtin_popcountll(static_cast<uint64_t>(x >> 64));
}
inline int ctz128(u128 x) {
  const uint64_t lo = static_cast<uint64_t>(x);
  return lo ? __builtin_ctzll(lo) : 64 + __builtin_ctzll(static_cast<uint64_t>(x >> 64));
}
inline u128 bit(int v) { return u128(1) << v; }

inline uint64_t splitmix(uint64_t& s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

void features(const u128* adj, int n, float* x) {
  std::vector<int> deg(n), core(n), ecc(n);
  for (int v = 0; v < n; ++v)
    deg[v] = popc128(adj[v]);
  // core numbers: repeatedly remove a minimum-degree vertex (smallest id)
  {
    std::vector<int> d(deg);
    std::vector<char> alive(n, 1);
    int k = 0;
    for (int it = 0; it < n; ++it) {
      int v = -1;
      for (int u = 0; u < n; ++u)
        if (alive[u] && (v < 0 || d[u] < d[v]))
          v = u;
      k = std::max(k, d[v]);
      core[v] = k;
      alive[v] = 0;
      for (u128 a = adj[v]; a; a &= a - 1) {
        const int u = ctz128(a);
        if (alive[u])
          --d[u];
      }
    }
  }
  // eccentricity within the vertex's component (BFS layers)
  for (int s = 0; s < n; ++s) {
    u128 seen = bit(s), frontier = bit(s);
    int dist = 0;
    for (;;) {
      u128 nb = 0;
      for (u128 f = frontier; f; f &= f - 1)
        nb |= adj[ctz128(f)];
      nb &= ~seen;
      if (!nb)
        break;
      seen |= nb;
      frontier = nb;
      ++dist;
    }
    ecc[s] = dist;
  }
  for (int v = 0; v < n; ++v) {
    float nd = 0.f;
    if (deg[v]) {
      float sum = 0.f;
      for (u128 a = adj[v]; a; a &= a - 1)
        sum += static_cast<float>(deg[ctz128(a)]);
      nd = sum / static_cast<float>(deg[v]);
    }
    float* o = x + size_t(v) * kFeatures;
    o[0] = static_cast<float>(deg[v]) / 4.0f;
    o[1] = static_cast<float>(core[v]) / 4.0f;
    o[2] = static_cast<float>(ecc[v]) / 8.0f;
    o[3] = nd / 4.0f;
    o[4] = deg[v] == 1 ? 1.0f : 0.0f;
    o[5] = 1.0f / (1.0f + static_cast<float>(deg[v]));
    o[6] = static_cast<float>(n) / 64.0f;
    o[7] = 1.0f;
  }
}

bool load_graph(const uint64_t* adj2, int n, std::vector<u128>& adj) {
  adj.assign(n, 0);
  const u128 all = n == 128 ? ~u128(0) : (bit(n) - 1);
  for (int v = 0; v < n; ++v) {
    adj[v] = (u128(adj2[2 * v + 1]) << 64) | adj2[2 * v];
    if ((adj[v] >> v) & 1 || (adj[v] & ~all))
      return false;
  }
  for (int v = 0; v < n; ++v)
    for (u128 a = adj[v]; a; a &= a - 1)
      if (!((adj[ctz128(a)] >> v) & 1))
        return false;
  return true;
}

}  // namespace

using gtd::fail;

extern "C" {

gtd_status gtd_gnn_features(const uint64_t* adj2, int n, float* x_out) {
  if (!adj2 || !x_out || n < 1 || n > 128)
    return GTD_INVALID_ARG;
  std::vector<u128> adj;
  if (!load_graph(adj2, n, adj))
    return GTD_INVALID_ARG;
  features(adj.data(), n, x_out);
  return GTD_OK;
}

gtd_status gtd_gnn_pack_sizes(const uint64_t* adj2_pool, const gtd_graph_desc* descs, int count,
                              int64_t* nodes_out, int64_t* nbrs_out) {
  if (!adj2_pool || !descs || count < 1 || !nodes_out || !nbrs_out)
    return GTD_INVALID_ARG;
  int64_t nodes = 0, nbrs = 0;
  for (int i = 0; i < count; ++i) {
    if (descs[i].n < 1 || descs[i].n > 128 || descs[i].offset < 0)
      return GTD_INVALID_ARG;
    nodes += descs[i].n;
    const uint64_t* a = adj2_pool + 2 * size_t(descs[i].offset);
    for (int v = 0; v < 2 * descs[i].n; ++v)
      nbrs += __builtin_popcountll(a[v]);
  }
  *nodes_out = nodes;
  *nbrs_out = nbrs;
  return GTD_OK;
}

gtd_status gtd_gnn_pack(const uint64_t* adj2_pool, const gtd_graph_desc* descs, int count, float* x_out,
                        int32_t* graph_start_out, int32_t* nbr_start_out, int32_t* nbr_out) {
  if (!adj2_pool || !descs || count < 1 || !x_out || !graph_start_out || !nbr_start_out || !nbr_out)
    return GTD_INVALID_ARG;
  std::vector<u128> adj;
  int32_t base = 0, e = 0;
  graph_start_out[0] = 0;
  nbr_start_out[0] = 0;
  for (int i = 0; i < count; ++i) {
    const int n = descs[i].n;
    if (n < 1 || n > 128 || descs[i].offset < 0 || !load_graph(adj2_pool + 2 * size_t(descs[i].offset), n, adj))
      return GTD_INVALID_ARG;
    features(adj.data(), n, x_out + size_t(base) * kFeatures);
    for (int v = 0; v < n; ++v) {
      for (u128 a = adj[v]; a; a &= a - 1)
        nbr_out[e++] = base + ctz128(a);
      nbr_start_out[base + v + 1] = e;
    }
    base += n;
    graph_start_out[i + 1] = base;
  }
  return GTD_OK;
}

gtd_status gtd_gnn_make_labels(gtd_handle h, const uint64_t* adj2_pool, const gtd_graph_desc* descs, int count,
                               int per_graph, int min_size, uint64_t seed, int capacity, uint64_t* sub_adj2_out,
                               gtd_graph_desc* sub_desc_out, uint64_t* root_out, int32_t* td_out, int* num_out) {
  if (!h)
    return GTD_INVALID_ARG;
  if (!adj2_pool || !descs || count < 1 || per_graph < 0 || capacity < 1 || !sub_adj2_out || !sub_desc_out ||
      !root_out || !td_out || !num_out)
    return fail(h, GTD_INVALID_ARG, "null pointer argument or empty input");
  *num_out = 0;
  uint64_t rng = seed * 0xD1B54A32D192ED03ull + 0x8CB92BA72F3D8DD7ull;
  std::vector<u128> adj;
  std::vector<uint64_t> adj64, masks;
  std::vector<int32_t> parent, tds;
  std::vector<uint64_t> roots;
  int out = 0, off = 0;
  for (int b = 0; b < count && out < capacity; ++b) {
    const int n = descs[b].n;
    if (n < 2 || n > 24 || descs[b].offset < 0 || !load_graph(adj2_pool + 2 * size_t(descs[b].offset), n, adj))
      return fail(h, GTD_INVALID_ARG, "label graph " + std::to_string(b) + ": needs 2 <= n <= 24 and a simple graph");
    adj64.assign(n, 0);
    for (int v = 0; v < n; ++v)
      adj64[v] = static_cast<uint64_t>(adj[v]);
    parent.assign(n, 0);
    int32_t td = 0;
    gtd_status s = gtd_dp_solve(h, adj64.data(), n, &td, parent.data(), nullptr, nullptr, nullptr);
    if (s != GTD_OK)
      return s;
    masks.clear();
    masks.push_back((uint64_t(1) << n) - 1);
    const int lo = std::min(min_size, n);
    for (int i = 0; i < per_graph; ++i) {
      const int size = lo + static_cast<int>(splitmix(rng) % uint64_t(n - lo + 1));
      const int start = static_cast<int>(splitmix(rng) % uint64_t(n));
      uint64_t S = uint64_t(1) << start, frontier = adj64[start];
      while (__builtin_popcountll(S) < size && (frontier & ~S)) {
        uint64_t cand = frontier & ~S;
        int k = static_cast<int>(splitmix(rng) % uint64_t(__builtin_popcountll(cand)));
        while (k-- > 0)
          cand &= cand - 1;
        const int u = __builtin_ctzll(cand);
        S |= uint64_t(1) << u;
        frontier |= adj64[u];
      }
      masks.push_back(S);
    }
    std::sort(masks.begin(), masks.end());
    masks.erase(std::unique(masks.begin(), masks.end()), masks.end());
    tds.assign(masks.size(), 0);
    roots.assign(masks.size(), 0);
    s = gtd_dp_labels(h, masks.data(), static_cast<int>(masks.size()), tds.data(), roots.data());
    if (s != GTD_OK)
      return s;
    for (size_t i = 0; i < masks.size() && out < capacity; ++i) {
      const uint64_t S = masks[i];
      const int k = __builtin_popcountll(S);
      if (k < 2 || roots[i] == 0)  // single vertices, disconnected sets
        continue;
      int idx[24];
      int j = 0;
      for (uint64_t m = S; m; m &= m - 1)
        idx[__builtin_ctzll(m)] = j++;
      uint64_t r = 0;
      for (uint64_t m = S; m; m &= m - 1) {
        const int v = __builtin_ctzll(m);
        uint64_t a = 0;
        for (uint64_t x = adj64[v] & S; x; x &= x - 1)
          a |= uint64_t(1) << idx[__builtin_ctzll(x)];
        sub_adj2_out[2 * size_t(off + idx[v])] = a;
        sub_adj2_out[2 * size_t(off + idx[v]) + 1] = 0;
        if ((roots[i] >> v) & 1)
          r |= uint64_t(1) << idx[v];
      }
      sub_desc_out[out].n = k;
      sub_desc_out[out].offset = off;
      root_out[out] = r;
      td_out[out] = tds[i];
      off += k;
      ++out;
    }
  }
  *num_out = out;
  return GTD_OK;
}

}  // extern "C"
