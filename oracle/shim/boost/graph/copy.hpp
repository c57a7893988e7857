// Boost-API shim (test infrastructure for oracle/_ref): copy_graph.
#pragma once
#include "boost/graph/adjacency_list.hpp"

namespace boost {
// Copies vertex count and every edge of src into dst (dst is overwritten).
template <typename G1, typename G2>
void copy_graph(G1 const& src, G2& dst) {
  dst = G2(num_vertices(src));
  for (std::size_t u = 0; u < num_vertices(src); ++u)
    for (auto v : src.adj_[u])
      if (u <= v)
        add_edge(u, v, dst);
}
}  // namespace boost
