/* ORACLE — TEST INFRASTRUCTURE ONLY.
 *
 * CPU restatement of the reference's (Zackere/GiSBDW) exact treedepth
 * algorithms, used as the checker for the GPU product and as the timed CPU
 * baseline ("port"). Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline / reference legs may load it; the product never does.
 *
 * Parity pinning: every function here is checked against the reference's own
 * sources compiled unchanged (oracle/_ref, built by oracle/Makefile against
 * the shim in oracle/shim) on the golden fixtures in tests/golden/, and
 * against the reference unit tests' known answers.
 *
 * Graphs: n vertices 0..n-1, adjacency as bit masks (adj[v] bit u set iff
 * edge uv). DP functions take 64-bit masks (n <= 64, tables need n <= 34);
 * branch and bound takes 128-bit masks as (lo, hi) word pairs (n <= 128).
 * Trees are parent arrays, parent[root] = -1.
 */
#ifndef GTD_ORACLE_H_
#define GTD_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Reference-style binomial coefficient (set_encoder.cu:6-17). */
uint64_t gtdo_nchoosek(uint64_t n, uint64_t k);
/* rank_k(S) = sum_i C(s_i, i+1) over sorted S (set_encoder.hpp:40-46). */
uint64_t gtdo_encode(const int* sorted_set, int k);
/* Inverse of gtdo_encode (set_encoder.hpp:61-73). */
void gtdo_decode(int nverts, int k, uint64_t code, int* out_sorted);

/* EdgeLowerBound::Get (edge_lower_bound.hpp:13-20) in exact integer form:
 * smallest d in [1, n] with (d - 1) * (2n - d) >= 2e. */
int gtdo_edge_lower_bound(int nverts, int nedges);

/* All-subsets DP table, T indexed by the subset bit mask (2^n bytes),
 * restating DynamicGPU's recurrence (dynamic_gpu.cu:68-112): a connected S
 * gets 1 + min_v T[S \ v], a disconnected S the max over its components.
 * nthreads > 1 splits each popcount level over pthreads. Returns 0, or -1 if
 * n is outside [1, 34]. */
int gtdo_dp_table(int n, const uint64_t* adj, uint8_t* table, int nthreads);

/* Canonical tree from a bit-mask-indexed table: the root of every connected
 * component is its first (smallest) vertex v with T[C \ v] = T[C] - 1, the
 * root DynamicCPU/DynamicCPUImprov/DynamicGPU store (dynamic_cpu.cpp:96-99,
 * dynamic_gpu.cu:84-87) and replay (dynamic_cpu.hpp:59-81). Writes td and
 * parent[]; returns 0. */
int gtdo_tree_from_table(int n, const uint64_t* adj, const uint8_t* table,
                         int* td, int* parent);

/* DynamicGPU::GetElimination (dynamic_gpu.hpp:48-64) on a bit-mask-indexed
 * table: repeatedly remove the stored root of the remaining set, which for a
 * disconnected set is the root of its first deepest component
 * (dynamic_gpu.cu:92-103). Writes popcount(subset) vertices; returns 0. */
int gtdo_get_elimination(int n, const uint64_t* adj, const uint8_t* table,
                         uint64_t subset, int* order);

/* gtdo_dp_table + gtdo_tree_from_table with an internally allocated table.
 * Returns 0, -1 bad n, -2 out of memory. */
int gtdo_dp_solve(int n, const uint64_t* adj, int nthreads, int* td,
                  int* parent);

/* DynamicCPUImprov (dynamic_cpu_improv.cpp:21-65): memoised recursion over
 * connected components keyed by bit mask, root = first argmin. n <= 64.
 * Returns 0, -1 bad n, -2 out of memory. *memo_entries (if non-null) gets the
 * number of memoised components. */
int gtdo_dp_improv(int n, const uint64_t* adj, int* td, int* parent,
                   int64_t* memo_entries);

/* EliminationTree replay (elimination_tree.cpp:24-70 + Decompose,
 * elimination_tree.hpp:193-215): eliminate order[0..n-1] in turn; each vertex
 * becomes a child of the vertex whose elimination created its component.
 * Returns 0, or -1 if order is not a permutation. */
/* BottomUpHeuristicGPU's DP (bottom_up_heuristic_gpu_algorithm.cu:57-258)
 * and its GetElimination order (n <= 30): order_out[n]. The heuristic's
 * tree is the EliminationTree replay of that order (gtdo_elimination_tree),
 * as BottomUpHeuristicGPU::Get does (bottom_up_heuristic.hpp:18-33). */
int gtdo_bottom_up(int n, const uint64_t* adj, int* order_out);

int gtdo_elimination_tree(int n, const uint64_t* adj, const int* order,
                          int* td, int* parent);

/* CheckIfTdDecompIsValid (common/utils/utils.hpp:50-86): parent[] is a tree
 * (forest allowed only if allow_forest), every edge joins an ancestor and a
 * descendant, and the height (in vertices) equals td. 1 valid, 0 not. */
int gtdo_check_valid(int n, const uint64_t* adj, int td, const int* parent,
                     int allow_forest);

/* Heuristics (incumbent seeds), 128-bit adjacency as adj2[2v], adj2[2v+1]:
 *   kind 0: HighestDegree(Variance(nullptr, 1.0, 0.2, 0.8)) (benchmark.cpp:50-55)
 *   kind 2: HighestDegreeHeuristic alone (highest_degree_heuristic.hpp:18-44)
 *   kind 3: VarianceHeuristic alone (variance_heuristic.hpp:24-78)
 * Returns 0 or -1 for an unknown kind / disconnected graph. */
int gtdo_heuristic(int n, const uint64_t* adj2, int kind, int* td,
                   int* parent);

/* BranchAndBound::Algorithm (branch_and_bound.cpp:51-114) with
 * EdgeLowerBound (lb_kind 0) or BasicLowerBound (lb_kind 1), incumbent from
 * gtdo_heuristic(heur_kind). 128-bit adjacency as above. node_limit <= 0
 * means unlimited. Returns 0 solved, 1 node limit hit (td/parent hold the best
 * found), -1 invalid input (disconnected, self loop, n out of range). */
int gtdo_bnb(int n, const uint64_t* adj2, int lb_kind, int heur_kind,
             int64_t node_limit, int* td, int* parent, int64_t* nodes);

#ifdef __cplusplus
}
#endif
#endif /* GTD_ORACLE_H_ */
