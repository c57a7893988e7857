// Boost-API shim (test infrastructure for oracle/_ref): BGL_FORALL_ADJ_T.
#pragma once
#include "boost/graph/adjacency_list.hpp"

// Loops V over the vertices adjacent to U in graph G of type GT, ascending.
#define BGL_FORALL_ADJ_T(U, V, G, GT)                                \
  for (typename ::boost::graph_traits<GT>::vertex_descriptor V :     \
       ::boost::shim_detail::adj_range((U), (G)))
#define BGL_FORALL_ADJ(U, V, G, GT) BGL_FORALL_ADJ_T(U, V, G, GT)
