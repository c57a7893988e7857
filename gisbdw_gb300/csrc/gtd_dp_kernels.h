// Kernel parameters and launchers of the subset DP (K1). Host and device.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "gtd_dp_layout.h"

namespace gtd {

// One graph of a DP launch (40 bytes). A graph with n < lb is padded with
// isolated vertices up to lb (one tile); padding changes no treedepth of a
// real subset and the reconstruction never touches padded vertices.
struct DpGraph {
  uint64_t table_off = 0;  // byte offset of the graph's table in the table pool
  uint32_t tile_base = 0;  // first flag of the graph (graph-major tile count)
  uint32_t ntiles = 0;     // 2^nh
  uint32_t adj_off = 0;    // first adjacency mask; also the first output slot
  int32_t n = 0;           // real vertices
  int32_t nh = 0;          // high vertices (max(n - lb, 0))
  int32_t out_idx = 0;     // position of the graph in the caller's arrays (td_out)
  int32_t lb = 0;          // tile bits of this graph's table
};

// Passed by value as a __grid_constant__ kernel parameter: the binomial
// table is read through the constant cache.
struct DpBatchParams {
  uint32_t binom[kDpMaxHigh + 1][kDpMaxHigh + 1] = {};  // C(a, b)
  const DpGraph* graphs = nullptr;  // device descriptors; nullptr: only `single`
  DpGraph single;
  uint2* tile_map = nullptr;        // ticket -> (graph, local tile) (batches)
  const uint32_t* level_base = nullptr;  // [graph][level] first ticket (batches)
  int num_graphs = 1;
  int lb = 0;                       // tile bits of this launch (mixed batches: the largest)
  int mixed = 0;                    // 1: graphs carry their own tile bits (DpGraph::lb)
  uint32_t total_tiles = 0;
  uint8_t* table = nullptr;         // table pool
  uint32_t* flags = nullptr;        // one ready stamp per global tile
  uint32_t* ticket = nullptr;       // work counter, zeroed before each launch
  int32_t* error = nullptr;         // [0] code, [1] info
  const uint64_t* adj = nullptr;    // adjacency pool (device)
  uint32_t epoch = 0;               // flags equal to epoch are ready
  uint64_t timeout_ns = 0;          // bound of every dependency wait
  // reconstruction outputs (device): td_out[g], parent_out[adj_off + v],
  // order_out[adj_off + step]; query != 0 restricts a single graph to a subset
  uint64_t query = 0;
  int32_t* td_out = nullptr;
  int32_t* parent_out = nullptr;
  int32_t* order_out = nullptr;
};

void dp_fill_binom(DpBatchParams& p);
int dp_tile_occupancy(int lb);
// CTAs per SM of the mixed-tile-size kernel with tiles of up to lb bits.
int dp_mixed_occupancy(int lb);
cudaError_t dp_launch_validate(const DpBatchParams& p, cudaStream_t s);
cudaError_t dp_launch_fill_tile_map(const DpBatchParams& p, cudaStream_t s);
cudaError_t dp_launch_tiles(const DpBatchParams& p, int ctas, cudaStream_t s);
cudaError_t dp_launch_tree(const DpBatchParams& p, cudaStream_t s);
cudaError_t dp_launch_labels(const DpBatchParams& p, const uint64_t* subsets, int count, int32_t* td_out,
                             uint64_t* roots_out, cudaStream_t s);

}  // namespace gtd
