// C++ drop-in check: the reference's calling pattern (main.cpp:187-195) with
// a Boost-style adjacency_list (the Boost-API shim from oracle/shim) through
// include/gtd/treedepth.hpp. Prints "td root order..." per graph; the pytest
// driver compares with the oracle. Exit code 0 on success.
#include <boost/graph/adjacency_list.hpp>
#include <cstdio>
#include <stdexcept>

#include "gtd/treedepth.hpp"

using Graph = boost::adjacency_list<boost::mapS, boost::vecS, boost::undirectedS>;

int main() {
  // P7 (elimination_tree_unittest.cpp:188-270): td 3
  Graph p7(7);
  for (int i = 0; i < 6; ++i)
    boost::add_edge(i, i + 1, p7);
  // C5: td 4
  Graph c5(5);
  for (int i = 0; i < 5; ++i)
    boost::add_edge(i, (i + 1) % 5, c5);
  td::DynamicGPU dyngpu;
  for (Graph* g : {&p7, &c5}) {
    dyngpu(*g);
    auto el = dyngpu.GetElimination<std::size_t>(boost::num_vertices(*g), boost::num_vertices(*g), 0);
    auto r = dyngpu.Decompose();
    std::printf("%u %zu", r.treedepth, r.root);
    for (auto v : el)
      std::printf(" %zu", v);
    std::printf("\n");
  }
  // a self loop is rejected with std::invalid_argument, as the reference does
  Graph bad(3);
  boost::add_edge(0, 1, bad);
  boost::add_edge(1, 1, bad);
  try {
    dyngpu(bad);
    std::printf("no-throw\n");
    return 1;
  } catch (std::invalid_argument const&) {
    std::printf("invalid_argument\n");
  }
  // the branch and bound through the reference's BnBGPU call shape
  td::BnBGPU bnb;
  for (Graph* g : {&p7, &c5}) {
    const int t = bnb(*g, 0);
    auto r = bnb.Decompose();
    std::printf("bnb %d %u %zu\n", t, r.treedepth, r.root);
  }
  Graph two(4);
  boost::add_edge(0, 1, two);
  boost::add_edge(2, 3, two);
  try {
    bnb(two, 0);
    std::printf("no-throw\n");
    return 1;
  } catch (std::invalid_argument const&) {
    std::printf("invalid_argument\n");
  }
  // a caller's bound only orders the search: a correct one (3 for P7) and a
  // wrong one (3 for C5, whose treedepth is 4) give the exact treedepth
  std::printf("heur %d %d\n", bnb(p7, 3), bnb(c5, 3));
  // out of device memory: no result and the reference's sentinel
  // (dynamic_cpu.hpp:52-56, 79-80), then the next call succeeds
  Graph p20(20);
  for (int i = 0; i < 19; ++i)
    boost::add_edge(i, i + 1, p20);
  gtd_inject_fault(GTD_FAULT_ALLOC, 1);
  dyngpu(p20);
  std::printf("oom %d %u %zu\n", dyngpu.HasResult() ? 1 : 0, dyngpu.Decompose().treedepth,
              dyngpu.GetElimination<std::size_t>(20, 20, 0).size());
  dyngpu(p20);
  std::printf("after %d %u\n", dyngpu.HasResult() ? 1 : 0, dyngpu.Decompose().treedepth);
  return 0;
}
