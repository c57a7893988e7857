// Greedy elimination heuristics that seed the branch and bound's incumbent
// (host code). They restate the reference's heuristic chain
// (Treedepth/src/branch_and_bound/heuristics/): every step eliminates one
// vertex of the first component (the one holding the smallest remaining
// vertex, ComponentCmp elimination_tree.hpp:67-72) and the tree is the
// resulting elimination tree.
//   kind 0  HighestDegree(Variance(nullptr, 1.0, 0.2, 0.8)): the better of
//           the two (benchmark.cpp:50-55)
//   kind 1  HighestDegreeHeuristic (highest_degree_heuristic.hpp:18-44)
//   kind 2  VarianceHeuristic (variance_heuristic.hpp:24-78)
//   kind 3  score greedy: the vertex with the highest score (ties: smallest
//           id), for scores from a learned model
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/gtd.h"

namespace {

using u128 = unsigned __int128;

inline bool has(u128 s, int v) { return (s >> v) & 1; }
inline int popc(u128 s) {
  return __builtin_popcountll(static_cast<uint64_t>(s)) + __builtin_popcountll(static_cast<uint64_t>(s >> 64));
}
inline int first(u128 s) {
  const uint64_t lo = static_cast<uint64_t>(s);
  return lo ? __builtin_ctzll(lo) : 64 + __builtin_ctzll(static_cast<uint64_t>(s >> 64));
}

struct G128 {
  int n;
  std::vector<u128> adj;
  u128 component(u128 S, int v) const {
    u128 reach = u128(1) << v, frontier = reach;
    while (frontier) {
      u128 nb = 0;
      for (u128 f = frontier; f; f &= f - 1)
        nb |= adj[first(f)];
      nb &= S & ~reach;
      reach |= nb;
      frontier = nb;
    }
    return reach;
  }
};

template <typename Pick>
int greedy(const G128& g, Pick pick, int32_t* parent) {
  u128 remaining = g.n == 128 ? ~u128(0) : ((u128(1) << g.n) - 1);
  std::vector<int> owner(g.n, -1), cdepth(g.n, 0);
  int height = 0;
  while (remaining) {
    const u128 C = g.component(remaining, first(remaining));
    const int v = pick(C);
    parent[v] = owner[v];
    height = std::max(height, cdepth[v] + 1);
    remaining &= ~(u128(1) << v);
    for (u128 s = C & ~(u128(1) << v); s; s &= s - 1) {
      const int u = first(s);
      owner[u] = v;
      cdepth[u] = cdepth[v] + 1;
    }
  }
  return height;
}

int highest_degree(const G128& g, int32_t* parent) {
  return greedy(g, [&](u128 C) {
    int best = -1, bd = -1;
    for (u128 s = C; s; s &= s - 1) {
      const int v = first(s);
      const int d = popc(g.adj[v] & C);
      if (d > bd) {
        bd = d;
        best = v;
      }
    }
    return best;
  }, parent);
}

int variance(const G128& g, int32_t* parent) {
  const float A = 1.0f, D = 0.2f, E = 0.8f;
  return greedy(g, [&](u128 C) {
    double best_coef = -1;
    int best_deg = -1, best = 0;
    for (u128 s = C; s; s &= s - 1) {
      const int v = first(s);
      const int deg = popc(g.adj[v] & C);
      std::vector<int> sizes;
      for (u128 rest = C & ~(u128(1) << v); rest;) {
        const u128 comp = g.component(rest, first(rest));
        rest &= ~comp;
        sizes.push_back(popc(comp));
      }
      const int nc = static_cast<int>(sizes.size());
      double acc = 0.0;
      for (int x : sizes)
        acc = acc + x;
      const double avg = acc / nc;
      double gamma = 0.0;
      for (int x : sizes)
        gamma = gamma + (x - avg) * (x - avg);
      const double coef = D / std::sqrt(gamma + A) + E * static_cast<float>(nc);
      if (coef > best_coef || (coef == best_coef && deg > best_deg)) {
        best_coef = coef;
        best_deg = deg;
        best = v;
      }
    }
    return best;
  }, parent);
}

int score_greedy(const G128& g, const float* scores, int32_t* parent) {
  return greedy(g, [&](u128 C) {
    int best = -1;
    for (u128 s = C; s; s &= s - 1) {
      const int v = first(s);
      if (best < 0 || scores[v] > scores[best])
        best = v;
    }
    return best;
  }, parent);
}

}  // namespace

extern "C" gtd_status gtd_heuristic(const uint64_t* adj2, int n, int kind, const float* scores, int32_t* td_out,
                                    int32_t* parent_out) {
  if (!adj2 || !td_out || !parent_out || n < 1 || n > 128)
    return GTD_INVALID_ARG;
  G128 g{n, std::vector<u128>(n)};
  for (int v = 0; v < n; ++v) {
    g.adj[v] = (u128(adj2[2 * v + 1]) << 64) | adj2[2 * v];
    if (has(g.adj[v], v))
      return GTD_INVALID_ARG;
  }
  switch (kind) {
    case 0: {
      std::vector<int32_t> tmp(n);
      int hd = highest_degree(g, parent_out);
      const int va = variance(g, tmp.data());
      if (va < hd) {
        std::memcpy(parent_out, tmp.data(), sizeof(int32_t) * n);
        hd = va;
      }
      *td_out = hd;
      return GTD_OK;
    }
    case 1:
      *td_out = highest_degree(g, parent_out);
      return GTD_OK;
    case 2:
      *td_out = variance(g, parent_out);
      return GTD_OK;
    case 3:
      if (!scores)
        return GTD_INVALID_ARG;
      *td_out = score_greedy(g, scores, parent_out);
      return GTD_OK;
    default:
      return GTD_INVALID_ARG;
  }
}
