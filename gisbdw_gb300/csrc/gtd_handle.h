// Handle state shared by the C-ABI translation units (host only).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "../../include/gtd.h"
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

}  // namespace gtd

struct gtd_handle_s {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::string last_error;

  // Subset DP buffers.
  uint8_t* d_table = nullptr;
  size_t table_cap = 0;
  uint32_t* d_flags = nullptr;
  size_t flags_cap = 0;  // number of tiles
  uint32_t epoch = 0;
  int32_t* d_io = nullptr;   // control/IO block
  uint64_t* d_adj = nullptr; // kDpMaxN masks
  void* h_pinned = nullptr;  // staging for adj (in) and the IO block (out)
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};

  // Last DP solve (for gtd_dp_query / gtd_sync).
  bool have_table = false;
  bool pending_stats = false;
  gtd::DpKernelParams last_params;
  gtd_dp_stats last_stats = {};
};

namespace gtd {
gtd_status fail(gtd_handle h, gtd_status s, const std::string& msg);
gtd_status cuda_fail(gtd_handle h, cudaError_t e, const char* what);
}  // namespace gtd
