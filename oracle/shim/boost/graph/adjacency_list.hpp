// Minimal Boost.Graph-compatible adjacency list, written for this project so
// that the reference's CPU treedepth solvers compile without Boost.
//
// TEST INFRASTRUCTURE ONLY: used by oracle/Makefile to build the reference's
// own sources into oracle/_ref/. Nothing in the product links it.
//
// Only the surface the reference's CPU solvers use is provided:
//   adjacency_list<OutEdgeList, VertexList, undirectedS, ...>, graph_traits,
//   add_edge, edge, num_vertices, num_edges, out_edges, target, source,
//   adjacent_vertices, out_degree, tie.
// Semantics follow Boost for an undirected graph whose out-edge container is a
// set (mapS/setS): no parallel edges, add_edge on an existing edge is a no-op,
// add_edge grows the vertex set (vecS) to cover both endpoints, adjacent
// vertices are visited in ascending order, num_edges counts each undirected
// edge once.
#pragma once

#include <cstddef>
#include <iostream>
#include <iterator>
#include <set>
#include <tuple>
#include <utility>
#include <vector>

namespace boost {

struct mapS {};
struct setS {};
struct vecS {};
struct listS {};
struct undirectedS {};
struct no_property {};

using std::tie;

template <typename Graph>
struct graph_traits;

namespace shim_detail {
struct Edge {
  std::size_t u = 0;
  std::size_t v = 0;
  bool operator==(Edge const& o) const { return u == o.u && v == o.v; }
  bool operator!=(Edge const& o) const { return !(*this == o); }
};

// Iterates the out-edges of one vertex as Edge{source, target}.
class OutEdgeIterator {
 public:
  using iterator_category = std::forward_iterator_tag;
  using value_type = Edge;
  using difference_type = std::ptrdiff_t;
  using pointer = Edge const*;
  using reference = Edge;
  OutEdgeIterator() = default;
  OutEdgeIterator(std::size_t src, std::set<std::size_t>::const_iterator it)
      : src_(src), it_(it) {}
  Edge operator*() const { return Edge{src_, *it_}; }
  OutEdgeIterator& operator++() {
    ++it_;
    return *this;
  }
  OutEdgeIterator operator++(int) {
    auto t = *this;
    ++it_;
    return t;
  }
  bool operator==(OutEdgeIterator const& o) const { return it_ == o.it_; }
  bool operator!=(OutEdgeIterator const& o) const { return it_ != o.it_; }

 private:
  std::size_t src_ = 0;
  std::set<std::size_t>::const_iterator it_{};
};
}  // namespace shim_detail

template <typename OutEdgeList = vecS,
          typename VertexList = vecS,
          typename Directed = undirectedS,
          typename... Rest>
class adjacency_list {
 public:
  using vertex_descriptor = std::size_t;
  using edge_descriptor = shim_detail::Edge;

  adjacency_list() = default;
  explicit adjacency_list(std::size_t n) : adj_(n) {}
  // Builds from a range of (u, v) pairs, like Boost's edge-iterator ctor.
  template <typename EdgeIter>
  adjacency_list(EdgeIter first, EdgeIter last, std::size_t n) : adj_(n) {
    for (; first != last; ++first)
      add((*first).first, (*first).second);
  }

  std::pair<edge_descriptor, bool> add(std::size_t u, std::size_t v) {
    std::size_t need = (u > v ? u : v) + 1;
    if (adj_.size() < need)
      adj_.resize(need);
    bool inserted = adj_[u].insert(v).second;
    if (u != v)
      adj_[v].insert(u);
    if (inserted)
      ++nedges_;
    return {edge_descriptor{u, v}, inserted};
  }

  std::vector<std::set<std::size_t>> adj_;
  std::size_t nedges_ = 0;
};

template <typename... A>
struct graph_traits<adjacency_list<A...>> {
  using vertex_descriptor = std::size_t;
  using edge_descriptor = shim_detail::Edge;
  using out_edge_iterator = shim_detail::OutEdgeIterator;
  using adjacency_iterator = std::set<std::size_t>::const_iterator;
  using vertices_size_type = std::size_t;
  using edges_size_type = std::size_t;
  using degree_size_type = std::size_t;
};

template <typename G>
struct graph_traits<const G> : graph_traits<G> {};

template <typename... A>
std::size_t num_vertices(adjacency_list<A...> const& g) {
  return g.adj_.size();
}

template <typename... A>
std::size_t num_edges(adjacency_list<A...> const& g) {
  return g.nedges_;
}

template <typename... A>
std::pair<shim_detail::Edge, bool> add_edge(std::size_t u,
                                            std::size_t v,
                                            adjacency_list<A...>& g) {
  return g.add(u, v);
}

template <typename... A>
std::pair<shim_detail::Edge, bool> edge(std::size_t u,
                                        std::size_t v,
                                        adjacency_list<A...> const& g) {
  if (u >= g.adj_.size())
    return {shim_detail::Edge{u, v}, false};
  return {shim_detail::Edge{u, v}, g.adj_[u].count(v) != 0};
}

template <typename... A>
std::pair<shim_detail::OutEdgeIterator, shim_detail::OutEdgeIterator>
out_edges(std::size_t u, adjacency_list<A...> const& g) {
  return {shim_detail::OutEdgeIterator(u, g.adj_[u].begin()),
          shim_detail::OutEdgeIterator(u, g.adj_[u].end())};
}

template <typename... A>
std::pair<std::set<std::size_t>::const_iterator,
          std::set<std::size_t>::const_iterator>
adjacent_vertices(std::size_t u, adjacency_list<A...> const& g) {
  return {g.adj_[u].begin(), g.adj_[u].end()};
}

template <typename... A>
std::size_t out_degree(std::size_t u, adjacency_list<A...> const& g) {
  return g.adj_[u].size();
}

template <typename G>
std::size_t target(shim_detail::Edge const& e, G const&) {
  return e.v;
}

template <typename G>
std::size_t source(shim_detail::Edge const& e, G const&) {
  return e.u;
}

namespace shim_detail {
template <typename... A>
std::set<std::size_t> const& adj_range(std::size_t u,
                                       adjacency_list<A...> const& g) {
  return g.adj_[u];
}
}  // namespace shim_detail
}  // namespace boost
