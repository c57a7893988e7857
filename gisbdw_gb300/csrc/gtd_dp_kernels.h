// Kernel parameters and launchers of the subset DP (K1). Host and device.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "gtd_dp_layout.h"

namespace gtd {

// Passed by value (it lives in the kernel parameter bank, so the binomial
// table and level offsets are read through the constant cache).
struct DpKernelParams {
  DpLayout lay;
  uint8_t* table = nullptr;        // 2^n bytes
  uint32_t* flags = nullptr;       // one ready stamp per tile
  uint32_t* ticket = nullptr;      // work counter, zeroed before each launch
  int32_t* error = nullptr;        // [0] code, [1] info
  const uint64_t* adj = nullptr;   // n masks, device memory
  uint32_t epoch = 0;              // flags equal to epoch are ready
  uint64_t timeout_ns = 0;         // bound of every dependency wait
};

int dp_tile_threads(int lb);
int dp_tile_occupancy(int lb);
cudaError_t dp_launch_tiles(const DpKernelParams& p, int ctas, cudaStream_t s);
cudaError_t dp_launch_tree(const DpKernelParams& p, uint64_t query, int32_t* td,
                           int32_t* parent, int32_t* order, cudaStream_t s);

}  // namespace gtd
