// gtd_dp_solve_noalloc: the subset DP for callers that cannot allocate
// device memory.
//
// Who needs it: code that runs where cudaMalloc is off limits — for example
// inside a host callback or a custom allocator's own hooks, under a memory
// pool that must not grow, or in a process that has handed all device memory
// to another framework up front. Such a caller owns its input and output
// buffers but cannot give this library room for the DP's scratch (the table,
// the per-tile ready flags and the work counter).
//
// So the scratch lives in one file-scope __device__ array of fixed size,
// loaded with the library: every GPU that loads libgtd.so holds these
// kNoallocScratchBytes (about 16.1 MiB) until the process exits. That bounds
// the graph size to n <= GTD_DP_NOALLOC_MAX_N (table 2^n bytes); larger n is
// rejected with GTD_INVALID_ARG.
//
// The array's name is only a host-side stand-in for the device symbol, so
// host code never passes it to a kernel: every call, with the caller's device
// current, looks the address up with cudaGetSymbolAddress (cheap once the
// module is loaded) and checks the result, so a context that was reset and
// made again (which reloads the module at a new address) is never written
// through a stale pointer. The first call on a device loads the module, so
// it should happen before any stream capture begins on that device.
//
// Every call shares the one array, which keeps what the previous call left:
// the work counter and error word are cleared on each call, and tile flags
// carry a per-device epoch that increases with every call (the flags are
// cleared when it wraps, gtd_noalloc_epoch.h). Calls whose GPU work
// overlaps — on two streams, or from two host threads — race on the array
// and give undefined results.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>

#include "../../include/gtd.h"
#include "gtd_device.cuh"
#include "gtd_dp_kernels.h"
#include "gtd_noalloc_epoch.h"

namespace gtd {
namespace {

constexpr int kNoallocTileBits = 10;
constexpr size_t kNoallocTableBytes = size_t(1) << GTD_DP_NOALLOC_MAX_N;
// Tiles of the largest accepted graph: make_dp_layout(n, 10) keeps 10 tile
// bits for 10 <= n <= 24 (2^(n - 10) tiles) and one tile below that.
constexpr size_t kNoallocMaxTiles = size_t(1) << (GTD_DP_NOALLOC_MAX_N - kNoallocTileBits);
static_assert(kNoallocTileBits >= kDpMinTileBits && kNoallocTileBits <= kDpMaxTileBits,
              "make_dp_layout must keep the fixed tile size");
constexpr size_t kNoallocFlagsOffset = kNoallocTableBytes;
constexpr size_t kNoallocCtrlOffset = kNoallocFlagsOffset + kNoallocMaxTiles * sizeof(uint32_t);
constexpr size_t kNoallocScratchBytes = kNoallocCtrlOffset + 256;

// The scratch: [table 2^24 B][flags][control: ticket, error code, error info].
__device__ __align__(256) uint8_t g_noalloc_scratch[kNoallocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_epoch_mutex;
uint32_t g_epoch[kMaxDevices] = {};

gtd_status map_error(int32_t code) {
  switch (code) {
    case kDevOk: return GTD_OK;
    case kDevInvalidInput: return GTD_INVALID_ARG;
    case kDevWaitTimeout: return GTD_TIMEOUT;
    default: return GTD_ABORTED;
  }
}

}  // namespace
}  // namespace gtd

extern "C" gtd_status gtd_dp_solve_noalloc(const uint64_t* d_adj, int n, int32_t* d_td,
                                           int32_t* d_parent, int32_t* d_order, void* stream) {
  using namespace gtd;
  if (!d_adj || !d_td || !d_parent)
    return GTD_INVALID_ARG;
  if (n < 2 || n > GTD_DP_NOALLOC_MAX_N)
    return GTD_INVALID_ARG;  // beyond the fixed scratch (2^n-byte table)
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return GTD_CUDA_ERROR;
  // The scratch's address in the current context (see the top of the file).
  void* sym = nullptr;
  if (cudaGetSymbolAddress(&sym, g_noalloc_scratch) != cudaSuccess || !sym)
    return GTD_CUDA_ERROR;
  uint8_t* const base = static_cast<uint8_t*>(sym);
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1)
    return GTD_CUDA_ERROR;
  cudaStream_t s = static_cast<cudaStream_t>(stream);

  const DpLayout L = make_dp_layout(n, kNoallocTileBits);
  if (L.ntiles > kNoallocMaxTiles)
    return GTD_INVALID_ARG;
  DpBatchParams p;
  dp_fill_binom(p);
  p.single.ntiles = L.ntiles;
  p.single.n = n;
  p.single.nh = L.nh;
  p.single.lb = L.lb;
  p.num_graphs = 1;
  p.lb = L.lb;
  p.total_tiles = L.ntiles;
  p.table = base;
  p.flags = reinterpret_cast<uint32_t*>(base + kNoallocFlagsOffset);
  int32_t* ctrl = reinterpret_cast<int32_t*>(base + kNoallocCtrlOffset);
  p.ticket = reinterpret_cast<uint32_t*>(ctrl);
  p.error = ctrl + 1;
  p.adj = d_adj;
  p.timeout_ns = 10ull * 1000 * 1000 * 1000;
  p.td_out = d_td;
  p.parent_out = d_parent;
  p.order_out = d_order;
  bool clear_flags = false;
  {
    std::lock_guard<std::mutex> lock(g_epoch_mutex);
    g_epoch[dev] = noalloc_next_epoch(g_epoch[dev], &clear_flags);
    p.epoch = g_epoch[dev];
  }
  if (clear_flags && cudaMemsetAsync(p.flags, 0, kNoallocMaxTiles * sizeof(uint32_t), s) != cudaSuccess)
    return GTD_CUDA_ERROR;  // wrapped: no stale stamp may match the new epoch

  int occ = dp_tile_occupancy(p.lb);
  if (occ < 1)
    occ = 1;
  long long ctas = static_cast<long long>(sms) * occ;
  if (ctas > p.total_tiles)
    ctas = p.total_tiles;
  if (cudaMemsetAsync(ctrl, 0, 4 * sizeof(int32_t), s) != cudaSuccess)
    return GTD_CUDA_ERROR;
  if (dp_launch_validate(p, s) != cudaSuccess)
    return GTD_CUDA_ERROR;
  if (dp_launch_tiles(p, static_cast<int>(ctas), s) != cudaSuccess)
    return GTD_CUDA_ERROR;
  if (dp_launch_tree(p, s) != cudaSuccess)
    return GTD_CUDA_ERROR;
  int32_t code = 0;
  if (cudaMemcpyAsync(&code, p.error, sizeof(int32_t), cudaMemcpyDeviceToHost, s) != cudaSuccess)
    return GTD_CUDA_ERROR;
  if (cudaStreamSynchronize(s) != cudaSuccess)
    return GTD_CUDA_ERROR;
  return map_error(code);
}
