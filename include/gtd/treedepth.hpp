// Header-only C++ layer over the gtd C ABI with the reference's class names
// and call shapes (Zackere/GiSBDW, Treedepth/src):
//
//   td::DynamicGPU dp;            // dynamic_gpu.hpp:17-37
//   dp(g);                        // any graph with Boost's free functions
//   auto order = dp.GetElimination<std::size_t>(n, n, 0);   // hpp:48-64
//   td::gtd::Result r = dp.Decompose();   // treedepth, root, parent, edges
//
//   td::BnBGPU bnb;               // bnb_gpu.hpp:12-31
//   int t = bnb(g, heur_td);      // exact treedepth by the persistent B&B
//   td::gtd::Result r2 = bnb.Decompose();
//
// `g` is read through the Boost.Graph free functions num_vertices(g) and
// adjacent_vertices(v, g) found by argument-dependent lookup, so a
// boost::adjacency_list (what the reference's callers hold) is accepted
// unchanged; the graph is copied into adjacency masks and the caller keeps
// ownership, as in the reference (dynamic_gpu.hpp:37-46).
//
// gtd_status codes become the reference's exception types:
//   GTD_INVALID_ARG, GTD_NOT_CONNECTED -> std::invalid_argument
//   GTD_OOM                           -> std::bad_alloc
//   anything else                     -> std::runtime_error
// except that td::DynamicGPU swallows running out of device memory the way
// the reference's DP functors swallow std::bad_alloc (dynamic_cpu.hpp:52-56,
// dynamic_cpu_improv.hpp:58-72): the call returns with no result,
// GetElimination then gives an empty list and Decompose() the reference's
// "no result" sentinel, treedepth = UINT_MAX (dynamic_cpu.hpp:79-80).
#pragma once

#include <cstdint>
#include <limits>
#include <list>
#include <new>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "../gtd.h"

namespace td {
namespace gtd {

inline void check(gtd_status s, gtd_handle h) {
  if (s == GTD_OK)
    return;
  std::string msg = std::string(gtd_status_string(s)) + ": " + (h ? gtd_last_error(h) : "");
  if (s == GTD_INVALID_ARG || s == GTD_NOT_CONNECTED)
    throw std::invalid_argument(msg);
  if (s == GTD_OOM)
    throw std::bad_alloc();
  throw std::runtime_error(msg);
}

// EliminationTree::Result (elimination_tree.hpp:26-30) as a parent array.
struct Result {
  std::vector<int32_t> parent;  // parent[root] == -1
  unsigned treedepth = 0;
  std::size_t root = 0;
  // Tree edges (parent, child), the td_decomp graph of the reference.
  std::vector<std::pair<std::size_t, std::size_t>> Edges() const {
    std::vector<std::pair<std::size_t, std::size_t>> e;
    for (std::size_t v = 0; v < parent.size(); ++v)
      if (parent[v] >= 0)
        e.emplace_back(static_cast<std::size_t>(parent[v]), v);
    return e;
  }
};

// RAII handle.
class Handle {
 public:
  explicit Handle(int device = 0, void* stream = nullptr) { check(gtd_create(&h_, device, stream), nullptr); }
  ~Handle() {
    if (h_)
      gtd_destroy(h_);
  }
  Handle(const Handle&) = delete;
  Handle& operator=(const Handle&) = delete;
  gtd_handle get() const { return h_; }

 private:
  gtd_handle h_ = nullptr;
};

template <typename Graph>
std::vector<uint64_t> AdjacencyMasks(Graph const& g) {
  const std::size_t n = num_vertices(g);
  if (n > 64)
    throw std::invalid_argument("adjacency masks need n <= 64");
  std::vector<uint64_t> adj(n, 0);
  for (std::size_t v = 0; v < n; ++v) {
    auto range = adjacent_vertices(v, g);
    for (auto it = range.first; it != range.second; ++it)
      adj[v] |= uint64_t(1) << static_cast<std::size_t>(*it);
  }
  return adj;
}

// (lo, hi) 64-bit words per vertex for the B&B (n <= GTD_BNB_MAX_N).
template <typename Graph>
std::vector<uint64_t> AdjacencyMasks128(Graph const& g) {
  const std::size_t n = num_vertices(g);
  if (n > GTD_BNB_MAX_N)
    throw std::invalid_argument("the branch and bound takes n <= " + std::to_string(GTD_BNB_MAX_N));
  std::vector<uint64_t> adj(2 * n, 0);
  for (std::size_t v = 0; v < n; ++v) {
    auto range = adjacent_vertices(v, g);
    for (auto it = range.first; it != range.second; ++it) {
      const std::size_t u = static_cast<std::size_t>(*it);
      adj[2 * v + (u >> 6)] |= uint64_t(1) << (u & 63);
    }
  }
  return adj;
}

}  // namespace gtd

// Exact treedepth by the GB300 subset DP.
class DynamicGPU {
 public:
  explicit DynamicGPU(int device = 0) : handle_(device) {}

  template <typename Graph>
  void operator()(Graph const& g) {
    adj_ = gtd::AdjacencyMasks(g);
    n_ = static_cast<int>(adj_.size());
    parent_.assign(n_, -1);
    order_.assign(n_, 0);
    int32_t td = 0;
    have_ = false;
    const gtd_status s = gtd_dp_solve(handle_.get(), adj_.data(), n_, &td, parent_.data(), order_.data(),
                                      nullptr, &stats_);
    if (s == GTD_OOM) {  // the reference's catch (std::bad_alloc const&) { return; }
      parent_.clear();
      order_.clear();
      return;
    }
    gtd::check(s, handle_.get());
    td_ = td;
    have_ = true;
  }

  // Elimination order of the subset with colex rank subset_code among the
  // subset_size-subsets of nverts vertices (dynamic_gpu.hpp:48-64);
  // (n, n, 0) is the whole graph. Empty when the last call gave no result.
  template <typename VertexType>
  std::list<VertexType> GetElimination(std::size_t nverts, std::size_t subset_size, std::size_t subset_code) {
    if (!have_)
      return {};
    if (nverts == static_cast<std::size_t>(n_) && subset_size == nverts && subset_code == 0)
      return std::list<VertexType>(order_.begin(), order_.end());
    uint64_t mask = Decode(nverts, subset_size, subset_code);
    std::vector<int32_t> order(subset_size);
    int32_t td = 0;
    gtd::check(gtd_dp_query(handle_.get(), mask, &td, order.data()), handle_.get());
    return std::list<VertexType>(order.begin(), order.end());
  }

  // The tree the reference's main builds from GetElimination
  // (main.cpp:187-195): parent array, height and root; with no result, an
  // empty tree of height UINT_MAX (the reference's sentinel).
  gtd::Result Decompose() const {
    gtd::Result r;
    if (!have_) {
      r.treedepth = std::numeric_limits<unsigned>::max();
      return r;
    }
    r.parent = parent_;
    r.treedepth = static_cast<unsigned>(td_);
    for (int v = 0; v < n_; ++v)
      if (parent_[v] < 0) {
        r.root = static_cast<std::size_t>(v);
        break;
      }
    return r;
  }

  unsigned Treedepth() const { return have_ ? static_cast<unsigned>(td_) : std::numeric_limits<unsigned>::max(); }
  bool HasResult() const { return have_; }
  const gtd_dp_stats& Stats() const { return stats_; }

 private:
  // Colex unrank (set_encoder.hpp:61-73) to a bit mask.
  static uint64_t Decode(std::size_t nverts, std::size_t k, std::size_t code) {
    uint64_t mask = 0;
    while (k > 0) {
      --nverts;
      std::size_t c = Binom(nverts, k);
      if (code >= c) {
        mask |= uint64_t(1) << nverts;
        code -= c;
        --k;
      }
    }
    return mask;
  }
  static std::size_t Binom(std::size_t n, std::size_t k) {
    if (k > n)
      return 0;
    std::size_t r = 1;
    for (std::size_t i = 1; i <= k; ++i)
      r = r * (n - k + i) / i;
    return r;
  }

  gtd::Handle handle_;
  std::vector<uint64_t> adj_;
  std::vector<int32_t> parent_, order_;
  int n_ = 0;
  int td_ = 0;
  bool have_ = false;
  gtd_dp_stats stats_{};
};

// Exact treedepth by the GB300 branch and bound (persistent kernel), the
// call shape of BnBGPU (bnb_gpu.hpp:12-17): operator()(g, heur_td) returns
// the treedepth. The incumbent tree comes from the library's reference
// heuristic chain (HighestDegree(Variance), gtd_heuristic kind 0). A caller's
// heur_td below that chain's height is honoured as the reference's initial
// best_td (bnb_gpu.cu:275) is: the search starts at level heur_td - 1, and if
// no tree of that height exists it decides level heur_td next, which also
// yields the tree (a bound without a tree cannot be returned as one). The
// bound only orders the search, so a wrong heur_td cannot change the result.
// n <= GTD_BNB_MAX_N (104; the reference's BnBGPU takes n <= 127, int8
// vertices, bnb_gpu.cu:107-165, and BranchAndBound n <= 128): larger graphs
// throw std::invalid_argument. Unlike the reference, the result also carries
// a tree (Decompose). A disconnected graph throws std::invalid_argument, as
// BranchAndBound does (branch_and_bound.hpp:67-75).
class BnBGPU {
 public:
  explicit BnBGPU(int device = 0, uint64_t deadline_ns = 0) : handle_(device), deadline_ns_(deadline_ns) {}

  template <typename Graph>
  int operator()(Graph const& g, std::size_t heur_td = 0) {
    std::vector<uint64_t> adj = gtd::AdjacencyMasks128(g);
    const int n = static_cast<int>(num_vertices(g));
    if (n == 0)
      throw std::invalid_argument("empty graph");
    std::vector<int32_t> seed_parent(n);
    int32_t seed_td = 0;
    gtd::check(gtd_heuristic(adj.data(), n, 0, nullptr, &seed_td, seed_parent.data()), handle_.get());
    // heur_td < seed: decide level heur_td - 1 first (then heur_td if that fails)
    int32_t hint = (heur_td >= 2 && static_cast<int32_t>(heur_td) < seed_td) ? static_cast<int32_t>(heur_td) - 1 : 0;
    gtd_graph_desc desc{n, 0};
    int32_t td = 0, status = 0;
    float proof_ms = 0;
    uint64_t nodes = 0;
    parent_.assign(n, -1);
    gtd_bnb_opts opts{0, deadline_ns_, 0, hint > 0 ? &hint : nullptr, 0, 0};
    gtd::check(gtd_bnb_solve_batch(handle_.get(), &desc, 1, adj.data(), n, nullptr, &seed_td, seed_parent.data(),
                                   &td, parent_.data(), &status, &proof_ms, &nodes, &opts, &stats_),
               handle_.get());
    gtd::check(static_cast<gtd_status>(status), handle_.get());
    td_ = td;
    return td;
  }

  gtd::Result Decompose() const {
    gtd::Result r;
    r.parent = parent_;
    r.treedepth = static_cast<unsigned>(td_);
    for (std::size_t v = 0; v < parent_.size(); ++v)
      if (parent_[v] < 0) {
        r.root = v;
        break;
      }
    return r;
  }

  const gtd_bnb_stats& Stats() const { return stats_; }

 private:
  gtd::Handle handle_;
  uint64_t deadline_ns_ = 0;
  std::vector<int32_t> parent_;
  int td_ = 0;
  gtd_bnb_stats stats_{};
};

}  // namespace td
