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
// kNoallocScratchBytes (about 16.3 MiB) until the process exits. That bounds
// the graph size to n <= GTD_DP_NOALLOC_MAX_N (table 2^n bytes); larger n is
// rejected with GTD_INVALID_ARG.
//
// The array's name is only a host-side stand-in for the device symbol, so
// host code never passes it to a kernel: on the first call on each device,
// with that device current, the address is looked up once with
// cudaGetSymbolAddress and cached. That first call should therefore happen
// before any stream capture begins on the device.
//
// Every call shares the one array, which keeps what the previous call left:
// the work counter and error word are cleared on each call, and tile flags
// carry a per-device epoch that increases with every call (the flags are
// cleared when it wraps). Calls whose GPU work overlaps — on two streams, or
// from two host threads — race on the array and give undefined results.
#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>
#include <mutex>

#include "../../include/gtd.h"
#include "gtd_device.cuh"
#include "gtd_dp_kernels.h"

namespace gtd {
namespace {

constexpr int kNoallocTileBits = 10;
constexpr size_t kNoallocTableBytes = size_t(1) << GTD_DP_NOALLOC_MAX_N;
// Tiles of the largest accepted graph at the smallest tile size the layout
// can choose (n = 24 keeps lb = 10 unless n < 10; 2^14 tiles).
constexpr size_t kNoallocMaxTiles = size_t(1) << (GTD_DP_NOALLOC_MAX_N - 8);
constexpr size_t kNoallocFlagsOffset = kNoallocTableBytes;
constexpr size_t kNoallocCtrlOffset = kNoallocFlagsOffset + kNoallocMaxTiles * sizeof(uint32_t);
constexpr size_t kNoallocScratchBytes = kNoallocCtrlOffset + 256;

// The scratch: [table 2^24 B][flags][control: ticket, error code, error info].
__device__ __align__(256) uint8_t g_noalloc_scratch[kNoallocScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mutex;
uint8_t* g_scratch_ptr[kMaxDevices] = {};
int g_num_sms[kMaxDevices] = {};
std::atomic<uint32_t> g_epoch[kMaxDevices];

// Once per device, with that device current: resolve the array's device
// address. Returns nullptr (and the CUDA error in *err) on failure.
uint8_t* scratch_for_device(int dev, cudaError_t* err) {
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (g_scratch_ptr[dev])
    return g_scratch_ptr[dev];
  void* ptr = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
  if (e != cudaSuccess) {
    *err = e;
    return nullptr;
  }
  int sms = 0;
  e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) {
    *err = e;
    return nullptr;
  }
  g_num_sms[dev] = sms;
  g_scratch_ptr[dev] = static_cast<uint8_t*>(ptr);
  return g_scratch_ptr[dev];
}

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
  cudaError_t err = cudaSuccess;
  uint8_t* base = scratch_for_device(dev, &err);
  if (!base)
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
  uint32_t epoch = g_epoch[dev].fetch_add(1) + 1;
  if (epoch == 0 || epoch == 0xffffffffu) {
    // wrapped: clear every flag so that no stale stamp matches
    if (cudaMemsetAsync(p.flags, 0, kNoallocMaxTiles * sizeof(uint32_t), s) != cudaSuccess)
      return GTD_CUDA_ERROR;
    g_epoch[dev].store(1);
    epoch = 1;
  }
  p.epoch = epoch;

  int occ = dp_tile_occupancy(p.lb);
  if (occ < 1)
    occ = 1;
  long long ctas = static_cast<long long>(g_num_sms[dev]) * occ;
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
