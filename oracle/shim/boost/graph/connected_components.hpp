// Boost-API shim (test infrastructure for oracle/_ref): connected_components.
#pragma once
#include <vector>

#include "boost/graph/adjacency_list.hpp"

namespace boost {
// Labels every vertex with its component id (0-based, in order of the
// smallest vertex of each component) and returns the number of components.
template <typename G, typename Out>
int connected_components(G const& g, Out comp) {
  std::size_t n = num_vertices(g);
  std::vector<int> label(n, -1);
  int ncomp = 0;
  std::vector<std::size_t> stack;
  for (std::size_t s = 0; s < n; ++s) {
    if (label[s] >= 0)
      continue;
    label[s] = ncomp;
    stack.push_back(s);
    while (!stack.empty()) {
      std::size_t u = stack.back();
      stack.pop_back();
      for (auto v : g.adj_[u])
        if (label[v] < 0) {
          label[v] = ncomp;
          stack.push_back(v);
        }
    }
    ++ncomp;
  }
  for (std::size_t i = 0; i < n; ++i)
    comp[i] = label[i];
  return ncomp;
}
}  // namespace boost
