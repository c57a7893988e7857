// ORACLE TEST INFRASTRUCTURE — not product code.
//
// A C-ABI harness around the reference's OWN CPU treedepth solvers, compiled
// unchanged from the reference sources (see oracle/Makefile) against the
// Boost-API shim in oracle/shim/. It is used only to pin the C restatement in
// oracle/gtd_oracle.c and to generate the golden fixtures in tests/golden/.
// It is never linked into, called by, or shipped with the product library.
//
// Graph convention for every entry point: n vertices 0..n-1 and m undirected
// edges given as 2*m ints (u0, v0, u1, v1, ...). Trees come back as a parent
// array (parent[root] = -1) derived from the reference's Result::td_decomp.
// Return codes: 0 ok, -1 std::invalid_argument, -2 std::runtime_error,
// -3 other exception, -4 solver produced no result (UINT_MAX sentinel).
#include <cstdint>
#include <cstring>
#include <memory>
#include <queue>
#include <stdexcept>
#include <vector>

#include "common/utils/utils.hpp"
#include "src/branch_and_bound/branch_and_bound.hpp"
#include "src/branch_and_bound/heuristics/highest_degree_heuristic.hpp"
#include "src/branch_and_bound/heuristics/spanning_tree_heuristic.hpp"
#include "src/branch_and_bound/heuristics/variance_heuristic.hpp"
#include "src/branch_and_bound/lower_bound/basic_lower_bound.hpp"
#include "src/branch_and_bound/lower_bound/edge_lower_bound.hpp"
#include "src/dynamic_cpu/dynamic_cpu.hpp"
#include "src/dynamic_cpu/dynamic_cpu_improv.hpp"
#include "src/elimination_tree/elimination_tree.hpp"
#include "src/set_encoder/set_encoder.hpp"

// The reference declares this name a friend of EliminationTree::Component
// (elimination_tree.hpp:46) for its unit tests; the harness defines it to
// build a Component with a given vertex and edge count.
class ParametrizedEliminationTreeFixture {
 public:
  static td::EliminationTree::Component MakeComponent(int nverts, int nedges) {
    td::EliminationTree::Component c;
    for (int i = 0; i < nverts; ++i)
      c.neighbours_[i];
    c.nedges_ = static_cast<unsigned>(nedges);
    return c;
  }
};

namespace {
using Graph = boost::adjacency_list<boost::mapS, boost::vecS, boost::undirectedS>;

Graph MakeGraph(int n, int m, int const* edges) {
  Graph g(n);
  for (int i = 0; i < m; ++i)
    boost::add_edge(edges[2 * i], edges[2 * i + 1], g);
  return g;
}

// Walks Result::td_decomp from its root and writes parent[] (root -> -1).
int ResultToParents(td::EliminationTree::Result const& r, int n, int* td,
                    int* root, int* parent) {
  if (r.treedepth == std::numeric_limits<unsigned>::max())
    return -4;
  *td = static_cast<int>(r.treedepth);
  *root = static_cast<int>(r.root);
  if (!parent)
    return 0;
  for (int i = 0; i < n; ++i)
    parent[i] = -2;
  if (static_cast<int>(boost::num_vertices(r.td_decomp)) < n)
    return -4;
  std::queue<std::size_t> q;
  parent[r.root] = -1;
  q.push(r.root);
  while (!q.empty()) {
    auto u = q.front();
    q.pop();
    for (auto [ai, ae] = boost::adjacent_vertices(u, r.td_decomp); ai != ae;
         ++ai) {
      if (parent[*ai] == -2) {
        parent[*ai] = static_cast<int>(u);
        q.push(*ai);
      }
    }
  }
  return 0;
}

td::EliminationTree::Result ParentsToResult(int n, int td, int root,
                                            int const* parent) {
  td::EliminationTree::Result r{td::EliminationTree::BoostGraph(n),
                                static_cast<unsigned>(td),
                                static_cast<std::size_t>(root)};
  for (int v = 0; v < n; ++v)
    if (parent[v] >= 0)
      boost::add_edge(v, parent[v], r.td_decomp);
  return r;
}

template <typename F>
int Guard(F&& f) {
  try {
    return f();
  } catch (std::invalid_argument const&) {
    return -1;
  } catch (std::runtime_error const&) {
    return -2;
  } catch (...) {
    return -3;
  }
}

std::unique_ptr<td::BranchAndBound::Heuristic> MakeHeuristic(int kind) {
  switch (kind) {
    case 0:  // benchmark.cpp:50-55 pure-CPU chain
      return std::make_unique<td::HighestDegreeHeuristic>(
          std::make_unique<td::VarianceHeuristic>(nullptr, 1.0, 0.2, 0.8));
    case 1:  // main.cpp:172-177 chain without the GPU bottom-up heuristic
      return std::make_unique<td::HighestDegreeHeuristic>(
          std::make_unique<td::SpanningTreeHeuristic>(
              std::make_unique<td::VarianceHeuristic>(nullptr, 1.0, 0.2,
                                                      0.8)));
    case 2:
      return std::make_unique<td::HighestDegreeHeuristic>(nullptr);
    case 3:
      return std::make_unique<td::VarianceHeuristic>(nullptr, 1.0, 0.2, 0.8);
    case 4:
      return std::make_unique<td::SpanningTreeHeuristic>(nullptr);
    default:
      return nullptr;
  }
}
}  // namespace

extern "C" {

// td::DynamicCPU (dynamic_cpu.cpp:41-107) + GetTDDecomp(0, g) as main.cpp:159-162.
int ref_dp_cpu(int n, int m, int const* edges, int* td, int* root,
               int* parent) {
  return Guard([&] {
    Graph g = MakeGraph(n, m, edges);
    td::DynamicCPU d;
    d(g);
    return ResultToParents(d.GetTDDecomp(0, g), n, td, root, parent);
  });
}

// td::DynamicCPUImprov (dynamic_cpu_improv.cpp:21-65) as main.cpp:163-168.
int ref_dp_cpu_improv(int n, int m, int const* edges, int* td, int* root,
                      int* parent) {
  return Guard([&] {
    Graph g = MakeGraph(n, m, edges);
    td::DynamicCPUImprov d;
    d(g);
    td::DynamicCPUImprov::CodeType code = 1;
    code <<= n;
    return ResultToParents(d.GetTDDecomp(--code, g), n, td, root, parent);
  });
}

// td::BranchAndBound (branch_and_bound.cpp:51-114) with EdgeLowerBound
// (lb_kind 0) or BasicLowerBound (lb_kind 1) and heuristic chain heur_kind.
int ref_bnb_cpu(int n, int m, int const* edges, int lb_kind, int heur_kind,
                int* td, int* root, int* parent) {
  return Guard([&] {
    Graph g = MakeGraph(n, m, edges);
    td::BranchAndBound bnb;
    std::unique_ptr<td::BranchAndBound::LowerBound> lb;
    if (lb_kind == 0)
      lb = std::make_unique<td::EdgeLowerBound>();
    else
      lb = std::make_unique<td::BasicLowerBound>();
    auto res = bnb(g, std::move(lb), MakeHeuristic(heur_kind));
    return ResultToParents(res, n, td, root, parent);
  });
}

// One heuristic of the chain alone (kind as MakeHeuristic).
int ref_heuristic(int n, int m, int const* edges, int kind, int* td, int* root,
                  int* parent) {
  return Guard([&] {
    Graph g = MakeGraph(n, m, edges);
    auto h = MakeHeuristic(kind);
    if (!h)
      return -3;
    return ResultToParents(h->Get(g), n, td, root, parent);
  });
}

// EliminationTree (elimination_tree.cpp:24-70) replay of a full order, then
// Decompose (elimination_tree.hpp:193-215).
int ref_elimination_tree(int n, int m, int const* edges, int const* order,
                         int* td, int* root, int* parent) {
  return Guard([&] {
    Graph g = MakeGraph(n, m, edges);
    td::EliminationTree et(g);
    for (int i = 0; i < n; ++i)
      et.Eliminate(order[i]);
    return ResultToParents(et.Decompose(), n, td, root, parent);
  });
}

// CheckIfTdDecompIsValid (common/utils/utils.hpp:50-86). 1 valid, 0 invalid.
int ref_check_valid(int n, int m, int const* edges, int td, int root,
                    int const* parent) {
  return Guard([&] {
    Graph g = MakeGraph(n, m, edges);
    return CheckIfTdDecompIsValid(g, ParentsToResult(n, td, root, parent)) ? 1
                                                                            : 0;
  });
}

// EdgeLowerBound::Get (edge_lower_bound.hpp:13-20) evaluated by the
// reference class itself on a component with nverts vertices and nedges edges.
unsigned ref_edge_lower_bound(int nverts, int nedges) {
  auto c = ParametrizedEliminationTreeFixture::MakeComponent(nverts, nedges);
  auto r = td::EdgeLowerBound().Get(c);
  return std::get<td::BranchAndBound::LowerBound::LowerBoundInfo>(r)
      .lower_bound;
}

uint64_t ref_nchoosek(uint64_t n, uint64_t k) {
  return td::set_encoder::NChooseK(n, k);
}

uint64_t ref_encode(int const* sorted_set, uint64_t k) {
  return td::set_encoder::Encode(sorted_set, k);
}

uint64_t ref_encode_excluded(int const* sorted_set, uint64_t k,
                             uint64_t exclude) {
  return td::set_encoder::Encode(sorted_set, k, exclude);
}

void ref_decode(uint64_t nverts, uint64_t k, uint64_t code, int* out) {
  td::set_encoder::Decode(nverts, k, code, out);
}
}
