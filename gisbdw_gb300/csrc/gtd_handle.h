// Handle state and helpers shared by the C-ABI translation units (host only).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/gtd.h"
#include "gtd_device.cuh"
#include "gtd_dp_kernels.h"

namespace gtd {

// Device control/IO block of a handle (int32 words):
//   [0] ticket  [1] error code  [2] error info  [3] reserved
//   [4] td      [8 .. 8+64) parent   [72 .. 72+64) order
constexpr int kIoTicket = 0;
constexpr int kIoError = 1;
constexpr int kIoTd = 4;
constexpr int kIoParent = 8;
constexpr int kIoOrder = 72;
constexpr int kIoWords = 256;
// Byte offsets inside the handle's 4096-byte pinned staging block.
constexpr size_t kPinnedIo = 1024;     // IO block copies (kIoOrder + 64 words)
constexpr size_t kPinnedAbort = 4092;  // gtd_abort's source word

// Flag stamp reserved for CUDA-graph replays (the graph zeroes the flags
// first); direct launches cycle their epochs through [1, kGraphEpoch).
constexpr uint32_t kGraphEpoch = 0xFFFFFFFEu;
constexpr int kTuneLbMin = 8;
constexpr int kTuneLbMax = 12;

}  // namespace gtd

struct gtd_bnb_state;  // branch-and-bound buffers (gtd_bnb.cu)
void gtd_bnb_release(struct gtd_handle_s* h);

struct gtd_handle_s {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::string last_error;

  // Subset DP buffers (shared by single and batched solves).
  uint8_t* d_table = nullptr;
  size_t table_cap = 0;
  uint32_t* d_flags = nullptr;
  size_t flags_cap = 0;  // number of tiles
  uint32_t epoch = 0;
  int32_t* d_io = nullptr;   // control/IO block
  uint64_t* d_adj = nullptr; // kDpMaxN masks
  void* h_pinned = nullptr;  // staging for adj (in) and the IO block (out); word kPinnedAbort: abort code
  cudaStream_t abort_stream = nullptr;  // gtd_abort's copy of the abort code (non-blocking)
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};

  // Batched DP buffers.
  gtd::DpGraph* d_bgraphs = nullptr;
  size_t bgraphs_cap = 0;
  uint2* d_tile_map = nullptr;
  size_t tile_map_cap = 0;
  uint32_t* d_level_base = nullptr;
  size_t level_base_cap = 0;
  uint64_t* d_badj = nullptr;
  size_t badj_cap = 0;
  int32_t* d_btd = nullptr;
  size_t btd_cap = 0;
  int32_t* d_bparent = nullptr;
  size_t bparent_cap = 0;
  void* h_bstage = nullptr;  // pinned: adjacency pool in, td + parent out
  size_t bstage_cap = 0;
  cudaGraphExec_t bgraph = nullptr;
  uint64_t bgraph_key = 0;
  bool bgraph_valid = false;
  gtd::DpBatchParams bparams;
  gtd_dp_batch_stats bstats = {};
  // Autotuner: subsets per millisecond by n and tile bits (0 = unmeasured).
  float tune[GTD_DP_MAX_N + 1][gtd::kTuneLbMax + 1] = {};
  // Mixed-size kernel throughput over the one-size kernel's, per largest tile
  // size (0 = unmeasured), from the autotuner.
  float tune_mixed_eff[gtd::kTuneLbMax + 1] = {};
  // CTAs per SM of the one-size DP kernel per tile size (0 = not asked yet):
  // a property of the kernel and the device, looked up once per handle.
  int dp_occ[gtd::kDpMaxTileBits + 1] = {};

  gtd_bnb_state* bnb = nullptr;
  void* d_scratch = nullptr;  // general device scratch (labels, GNN batches)
  size_t scratch_cap = 0;
  uint8_t* d_bu = nullptr;    // bottom-up heuristic: forests, heights, history
  size_t bu_cap = 0;

  // Last DP solve (for gtd_dp_query / gtd_sync).
  bool have_table = false;
  bool pending_stats = false;
  gtd::DpBatchParams last_params;
  gtd_dp_stats last_stats = {};
};

namespace gtd {

gtd_status fail(gtd_handle h, gtd_status s, const std::string& msg);
gtd_status cuda_fail(gtd_handle h, cudaError_t e, const char* what);
gtd_status check_adjacency(gtd_handle h, const uint64_t* adj, int n);
gtd_status map_device_error(gtd_handle h, int32_t code, int32_t info);
// Grows a device buffer to at least `bytes` (contents not kept). On failure
// *ptr is null and *cap 0 (the old buffer is already freed).
cudaError_t ensure_device(void** ptr, size_t* cap, size_t bytes);

// ensure_device on a typed field of the handle, capacity in elements: the
// field is updated whether or not the allocation succeeds, so it never keeps
// a freed pointer.
template <typename T>
cudaError_t ensure_field(T** field, size_t* cap_elems, size_t count) {
  void* q = *field;
  size_t bytes = *cap_elems * sizeof(T);
  const cudaError_t e = ensure_device(&q, &bytes, count * sizeof(T));
  *field = static_cast<T*>(q);
  *cap_elems = bytes / sizeof(T);
  return e;
}

// Test fault injection (gtd_inject_fault), process-wide: consumes one
// pending device-allocation failure (true: fail this allocation), one
// pending DP stall (true: the launch skips its first tile) or one pending
// table poisoning (true: fill the DP table with 0xFF before the launch).
bool take_alloc_fault();
bool take_stall_fault();
bool take_poison_fault();
// Grows the flag array; fresh flags are zeroed and the epoch restarts.
gtd_status ensure_flags(gtd_handle h, size_t tiles);
// Next epoch for a direct (non-graph) launch.
gtd_status next_epoch(gtd_handle h, uint32_t* epoch);

// Makes the handle's device current for the duration of a call and restores
// the caller's device afterwards.
struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev) {
    if (cudaGetDevice(&prev) != cudaSuccess)
      prev = -1;
    if (prev != dev)
      cudaSetDevice(dev);
  }
  ~DeviceGuard() {
    int cur = -1;
    if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev)
      cudaSetDevice(prev);
  }
};

}  // namespace gtd

#define GTD_CUDA(h, call)                      \
  do {                                         \
    cudaError_t e_ = (call);                   \
    if (e_ != cudaSuccess)                     \
      return ::gtd::cuda_fail((h), e_, #call); \
  } while (0)
