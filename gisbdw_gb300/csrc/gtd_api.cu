// C ABI of the gtd library: handles and the single-graph subset-DP entry
// points. Errors never cross the ABI as exceptions; every call returns a
// gtd_status and keeps a message for gtd_last_error.
#include <cuda_runtime.h>

#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>

#include "gtd_handle.h"

namespace gtd {

gtd_status fail(gtd_handle h, gtd_status s, const std::string& msg) {
  if (h)
    h->last_error = msg;
  return s;
}

gtd_status cuda_fail(gtd_handle h, cudaError_t e, const char* what) {
  std::string m = std::string(what) + ": " + cudaGetErrorString(e);
  return fail(h, e == cudaErrorMemoryAllocation ? GTD_OOM : GTD_CUDA_ERROR, m);
}

gtd_status check_adjacency(gtd_handle h, const uint64_t* adj, int n) {
  const uint64_t allowed = n >= 64 ? ~0ull : ((1ull << n) - 1);
  for (int v = 0; v < n; ++v) {
    if ((adj[v] >> v) & 1ull)
      return fail(h, GTD_INVALID_ARG, "Self loops are not allowed (vertex " + std::to_string(v) + ")");
    if (adj[v] & ~allowed)
      return fail(h, GTD_INVALID_ARG, "adjacency of vertex " + std::to_string(v) + " has a bit >= n");
    for (uint64_t s = adj[v]; s; s &= s - 1) {
      int u = __builtin_ctzll(s);
      if (!((adj[u] >> v) & 1ull))
        return fail(h, GTD_INVALID_ARG, "adjacency is not symmetric at (" + std::to_string(v) + ", " +
                                            std::to_string(u) + ")");
    }
  }
  return GTD_OK;
}

gtd_status map_device_error(gtd_handle h, int32_t code, int32_t info) {
  switch (code) {
    case kDevOk:
      return GTD_OK;
    case kDevInvalidInput:
      return fail(h, GTD_INVALID_ARG,
                  "adjacency rejected on the device (self loop, bit >= n or asymmetric; graph " +
                      std::to_string(info) + ")");
    case kDevWaitTimeout:
      return fail(h, GTD_TIMEOUT, "a tile dependency wait exceeded its deadline");
    case kDevNoRoot:
      return fail(h, GTD_ABORTED, "tree reconstruction found no optimal root (graph " + std::to_string(info) + ")");
    case kDevDeadline:
      return fail(h, GTD_TIMEOUT, "search deadline reached");
    case kDevOverflow:
      return fail(h, GTD_ABORTED, "a bounded device buffer overflowed (info " + std::to_string(info) + ")");
    default:
      return fail(h, GTD_ABORTED, "device error " + std::to_string(code));
  }
}

namespace {
std::atomic<int> g_alloc_faults{0};  // pending: the n-th allocation from now fails (0 = none)
std::atomic<int> g_stall_faults{0};  // pending: DP launches that skip their first tile
std::atomic<int> g_poison_faults{0};  // pending: DP solves whose table is filled with 0xFF first

bool take_counted(std::atomic<int>& pending) {
  int n = pending.load();
  while (n > 0) {
    if (pending.compare_exchange_weak(n, n - 1))
      return true;
  }
  return false;
}
}  // namespace

bool take_alloc_fault() {
  int n = g_alloc_faults.load();
  while (n > 0) {
    if (g_alloc_faults.compare_exchange_weak(n, n - 1))
      return n == 1;
  }
  return false;
}

bool take_stall_fault() { return take_counted(g_stall_faults); }

bool take_poison_fault() { return take_counted(g_poison_faults); }

cudaError_t ensure_device(void** ptr, size_t* cap, size_t bytes) {
  if (*cap >= bytes && *ptr)
    return cudaSuccess;
  if (*ptr)
    cudaFree(*ptr);
  *ptr = nullptr;
  *cap = 0;
  const size_t want = bytes < 256 ? 256 : bytes;
  if (take_alloc_fault())
    return cudaErrorMemoryAllocation;
  cudaError_t e = cudaMalloc(ptr, want);
  if (e == cudaSuccess)
    *cap = want;
  return e;
}

gtd_status ensure_flags(gtd_handle h, size_t tiles) {
  if (h->flags_cap >= tiles && h->d_flags)
    return GTD_OK;
  GTD_CUDA(h, ensure_field(&h->d_flags, &h->flags_cap, tiles));
  GTD_CUDA(h, cudaMemsetAsync(h->d_flags, 0, h->flags_cap * sizeof(uint32_t), h->stream));
  h->epoch = 0;
  return GTD_OK;
}

gtd_status next_epoch(gtd_handle h, uint32_t* epoch) {
  if (++h->epoch >= kGraphEpoch) {
    GTD_CUDA(h, cudaMemsetAsync(h->d_flags, 0, h->flags_cap * sizeof(uint32_t), h->stream));
    h->epoch = 1;
  }
  *epoch = h->epoch;
  return GTD_OK;
}

namespace {

// Tile bits measured best on GB300 (1 KB tiles up to n = 25, 2 KB above:
// n = 30 3.51 ms with 11 bits vs 3.76 ms with 10 and 4.72 ms with 12).
int default_tile_bits(int n) { return n >= 26 ? 11 : 10; }

// Allocates (or grows) the table and flag buffers and enqueues the
// validation, DP and tree kernels for one graph. Outputs go to
// td/parent/order (device pointers, possibly the handle's IO block).
gtd_status dp_enqueue(gtd_handle h, const uint64_t* d_adj, int n, const gtd_dp_opts* opts,
                      int32_t* d_td, int32_t* d_parent, int32_t* d_order) {
  const int tile_bits = (opts && opts->tile_bits > 0) ? opts->tile_bits : default_tile_bits(n);
  const DpLayout L = make_dp_layout(n, tile_bits);
  const size_t table_bytes = size_t(1) << n;
  if (h->table_cap < table_bytes)
    h->have_table = false;
  GTD_CUDA(h, ensure_field(&h->d_table, &h->table_cap, table_bytes));
  gtd_status s = ensure_flags(h, L.ntiles);
  if (s != GTD_OK)
    return s;

  DpBatchParams p;
  dp_fill_binom(p);
  p.single.table_off = 0;
  p.single.tile_base = 0;
  p.single.ntiles = L.ntiles;
  p.single.adj_off = 0;
  p.single.n = n;
  p.single.nh = L.nh;
  p.single.lb = L.lb;
  p.single.out_idx = 0;
  p.num_graphs = 1;
  p.lb = L.lb;
  p.total_tiles = L.ntiles;
  p.table = h->d_table;
  p.flags = h->d_flags;
  p.ticket = reinterpret_cast<uint32_t*>(h->d_io + kIoTicket);
  p.error = h->d_io + kIoError;
  p.adj = d_adj;
  s = next_epoch(h, &p.epoch);
  if (s != GTD_OK)
    return s;
  p.timeout_ns = (opts && opts->timeout_ns) ? opts->timeout_ns : 10ull * 1000 * 1000 * 1000;
  p.td_out = d_td;
  p.parent_out = d_parent;
  p.order_out = d_order;

  if (h->dp_occ[p.lb] <= 0)
    h->dp_occ[p.lb] = dp_tile_occupancy(p.lb);
  int occ = h->dp_occ[p.lb];
  if (opts && opts->ctas_per_sm > 0 && opts->ctas_per_sm < occ)
    occ = opts->ctas_per_sm;
  if (occ < 1)
    occ = 1;
  long long ctas = static_cast<long long>(h->num_sms) * occ;
  if (ctas > p.total_tiles)
    ctas = p.total_tiles;

  GTD_CUDA(h, cudaMemsetAsync(h->d_io, 0, 4 * sizeof(int32_t), h->stream));
  if (take_poison_fault())  // test injection: every byte must be written before it is read
    GTD_CUDA(h, cudaMemsetAsync(h->d_table, 0xFF, h->table_cap, h->stream));
  if (take_stall_fault())  // test injection: ticket 0 (the level-0 tile) is never taken
    GTD_CUDA(h, cudaMemsetAsync(h->d_io + kIoTicket, 1, 1, h->stream));
  GTD_CUDA(h, dp_launch_validate(p, h->stream));
  GTD_CUDA(h, cudaEventRecord(h->ev[0], h->stream));
  GTD_CUDA(h, dp_launch_tiles(p, static_cast<int>(ctas), h->stream));
  GTD_CUDA(h, cudaEventRecord(h->ev[1], h->stream));
  GTD_CUDA(h, dp_launch_tree(p, h->stream));
  GTD_CUDA(h, cudaEventRecord(h->ev[2], h->stream));

  h->last_params = p;
  h->have_table = true;
  h->pending_stats = true;
  gtd_dp_stats& st = h->last_stats;
  st = gtd_dp_stats{};
  st.table_bytes = table_bytes;
  st.alg_bytes = table_bytes + static_cast<uint64_t>(n) * (table_bytes / 2);
  st.tile_bits = p.lb;
  st.tiles = static_cast<int>(p.total_tiles);
  st.ctas = static_cast<int>(ctas);
  return GTD_OK;
}

void collect_stats(gtd_handle h) {
  if (!h->pending_stats)
    return;
  float a = 0, b = 0;
  if (cudaEventElapsedTime(&a, h->ev[0], h->ev[1]) == cudaSuccess)
    h->last_stats.dp_ms = a;
  if (cudaEventElapsedTime(&b, h->ev[1], h->ev[2]) == cudaSuccess)
    h->last_stats.tree_ms = b;
  h->pending_stats = false;
}

}  // namespace
}  // namespace gtd

using namespace gtd;

extern "C" {

const char* gtd_status_string(gtd_status s) {
  switch (s) {
    case GTD_OK: return "GTD_OK";
    case GTD_INVALID_ARG: return "GTD_INVALID_ARG";
    case GTD_NOT_CONNECTED: return "GTD_NOT_CONNECTED";
    case GTD_OOM: return "GTD_OOM";
    case GTD_TIMEOUT: return "GTD_TIMEOUT";
    case GTD_ABORTED: return "GTD_ABORTED";
    case GTD_CUDA_ERROR: return "GTD_CUDA_ERROR";
    case GTD_NO_RESULT: return "GTD_NO_RESULT";
  }
  return "GTD_UNKNOWN";
}

const char* gtd_last_error(gtd_handle h) { return h ? h->last_error.c_str() : "null handle"; }

gtd_status gtd_create(gtd_handle* out, int device, void* stream) {
  if (!out)
    return GTD_INVALID_ARG;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0)
    return GTD_CUDA_ERROR;
  if (device < 0 || device >= count)
    return GTD_INVALID_ARG;
  gtd_handle h = new (std::nothrow) gtd_handle_s();
  if (!h)
    return GTD_OOM;
  DeviceGuard g(device);
  h->device = device;
  cudaError_t e = cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess) {
    if (stream) {
      h->stream = static_cast<cudaStream_t>(stream);
    } else {
      e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
      h->own_stream = true;
    }
  }
  if (e == cudaSuccess)
    e = cudaStreamCreateWithFlags(&h->abort_stream, cudaStreamNonBlocking);
  for (int i = 0; i < 4 && e == cudaSuccess; ++i)
    e = cudaEventCreate(&h->ev[i]);
  if (e == cudaSuccess)
    e = cudaMalloc(&h->d_io, kIoWords * sizeof(int32_t));
  if (e == cudaSuccess)
    e = cudaMalloc(&h->d_adj, kDpMaxN * sizeof(uint64_t));
  if (e == cudaSuccess)
    e = cudaMallocHost(&h->h_pinned, 4096);
  if (e == cudaSuccess)
    e = cudaMemsetAsync(h->d_io, 0, kIoWords * sizeof(int32_t), h->stream);
  if (e == cudaSuccess)
    e = cudaStreamSynchronize(h->stream);
  if (e != cudaSuccess) {
    gtd_destroy(h);
    return e == cudaErrorMemoryAllocation ? GTD_OOM : GTD_CUDA_ERROR;
  }
  *out = h;
  return GTD_OK;
}

gtd_status gtd_destroy(gtd_handle h) {
  if (!h)
    return GTD_INVALID_ARG;
  {
    DeviceGuard g(h->device);
    if (h->stream)
      cudaStreamSynchronize(h->stream);
    if (h->bgraph)
      cudaGraphExecDestroy(h->bgraph);
    gtd_bnb_release(h);
    cudaFree(h->d_table);
    cudaFree(h->d_flags);
    cudaFree(h->d_io);
    cudaFree(h->d_adj);
    cudaFree(h->d_bgraphs);
    cudaFree(h->d_tile_map);
    cudaFree(h->d_level_base);
    cudaFree(h->d_badj);
    cudaFree(h->d_btd);
    cudaFree(h->d_bparent);
    cudaFree(h->d_scratch);
    cudaFree(h->d_bu);
    if (h->h_pinned)
      cudaFreeHost(h->h_pinned);
    if (h->h_bstage)
      cudaFreeHost(h->h_bstage);
    for (auto& e : h->ev)
      if (e)
        cudaEventDestroy(e);
    if (h->own_stream && h->stream)
      cudaStreamDestroy(h->stream);
    if (h->abort_stream)
      cudaStreamDestroy(h->abort_stream);
  }
  delete h;
  return GTD_OK;
}

gtd_status gtd_dp_solve(gtd_handle h, const uint64_t* adj, int n, int32_t* td_out, int32_t* parent_out,
                        int32_t* order_out, const gtd_dp_opts* opts, gtd_dp_stats* stats) {
  if (!h)
    return GTD_INVALID_ARG;
  if (!adj || !td_out || !parent_out)
    return fail(h, GTD_INVALID_ARG, "null pointer argument");
  if (n < 1 || n > GTD_DP_MAX_N)
    return fail(h, GTD_INVALID_ARG, "n must be in [1, " + std::to_string(GTD_DP_MAX_N) + "]");
  gtd_status s = check_adjacency(h, adj, n);
  if (s != GTD_OK)
    return s;
  const auto t0 = std::chrono::steady_clock::now();
  DeviceGuard g(h->device);
  if (n == 1) {
    *td_out = 1;
    parent_out[0] = -1;
    if (order_out)
      order_out[0] = 0;
    h->have_table = false;
    if (stats)
      *stats = gtd_dp_stats{};
    return GTD_OK;
  }
  uint64_t* h_adj = static_cast<uint64_t*>(h->h_pinned);
  std::memcpy(h_adj, adj, sizeof(uint64_t) * n);
  GTD_CUDA(h, cudaMemcpyAsync(h->d_adj, h_adj, sizeof(uint64_t) * n, cudaMemcpyHostToDevice, h->stream));
  s = dp_enqueue(h, h->d_adj, n, opts, h->d_io + kIoTd, h->d_io + kIoParent, h->d_io + kIoOrder);
  if (s != GTD_OK)
    return s;
  int32_t* h_io = reinterpret_cast<int32_t*>(static_cast<char*>(h->h_pinned) + kPinnedIo);
  GTD_CUDA(h, cudaMemcpyAsync(h_io, h->d_io, (kIoOrder + 64) * sizeof(int32_t), cudaMemcpyDeviceToHost,
                              h->stream));
  GTD_CUDA(h, cudaStreamSynchronize(h->stream));
  collect_stats(h);
  s = map_device_error(h, h_io[kIoError], h_io[kIoError + 1]);
  if (s != GTD_OK) {
    h->have_table = false;
    return s;
  }
  *td_out = h_io[kIoTd];
  std::memcpy(parent_out, h_io + kIoParent, sizeof(int32_t) * n);
  if (order_out)
    std::memcpy(order_out, h_io + kIoOrder, sizeof(int32_t) * n);
  h->last_stats.total_ms =
      std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (stats)
    *stats = h->last_stats;
  return GTD_OK;
}

gtd_status gtd_dp_solve_device(gtd_handle h, const uint64_t* d_adj, int n, int32_t* d_td, int32_t* d_parent,
                               int32_t* d_order, const gtd_dp_opts* opts) {
  if (!h)
    return GTD_INVALID_ARG;
  if (!d_adj || !d_td || !d_parent)
    return fail(h, GTD_INVALID_ARG, "null pointer argument");
  if (n < 2 || n > GTD_DP_MAX_N)
    return fail(h, GTD_INVALID_ARG, "device solve needs n in [2, " + std::to_string(GTD_DP_MAX_N) + "]");
  DeviceGuard g(h->device);
  return dp_enqueue(h, d_adj, n, opts, d_td, d_parent, d_order);
}

gtd_status gtd_sync(gtd_handle h, gtd_dp_stats* stats) {
  if (!h)
    return GTD_INVALID_ARG;
  DeviceGuard g(h->device);
  int32_t* h_io = reinterpret_cast<int32_t*>(static_cast<char*>(h->h_pinned) + kPinnedIo);
  GTD_CUDA(h, cudaMemcpyAsync(h_io, h->d_io, 4 * sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
  GTD_CUDA(h, cudaStreamSynchronize(h->stream));
  collect_stats(h);
  if (stats)
    *stats = h->last_stats;
  gtd_status s = map_device_error(h, h_io[kIoError], h_io[kIoError + 1]);
  if (s != GTD_OK)
    h->have_table = false;
  return s;
}

gtd_status gtd_dp_query(gtd_handle h, uint64_t subset_mask, int32_t* td_out, int32_t* order_out) {
  if (!h)
    return GTD_INVALID_ARG;
  if (!h->have_table)
    return fail(h, GTD_NO_RESULT, "no DP table: solve a graph first");
  const int n = h->last_params.single.n;
  if (n < 64 && (subset_mask >> n))
    return fail(h, GTD_INVALID_ARG, "subset has a vertex >= n");
  if (!td_out)
    return fail(h, GTD_INVALID_ARG, "null td_out");
  if (subset_mask == 0) {
    *td_out = 0;
    return GTD_OK;
  }
  DeviceGuard g(h->device);
  DpBatchParams p = h->last_params;
  p.query = subset_mask;
  p.td_out = h->d_io + kIoTd;
  p.parent_out = nullptr;
  p.order_out = order_out ? h->d_io + kIoOrder : nullptr;
  GTD_CUDA(h, cudaMemsetAsync(h->d_io + kIoError, 0, 2 * sizeof(int32_t), h->stream));
  GTD_CUDA(h, dp_launch_tree(p, h->stream));
  int32_t* h_io = reinterpret_cast<int32_t*>(static_cast<char*>(h->h_pinned) + kPinnedIo);
  GTD_CUDA(h, cudaMemcpyAsync(h_io, h->d_io, (kIoOrder + 64) * sizeof(int32_t), cudaMemcpyDeviceToHost,
                              h->stream));
  GTD_CUDA(h, cudaStreamSynchronize(h->stream));
  gtd_status s = map_device_error(h, h_io[kIoError], h_io[kIoError + 1]);
  if (s != GTD_OK)
    return s;
  *td_out = h_io[kIoTd];
  if (order_out)
    std::memcpy(order_out, h_io + kIoOrder, sizeof(int32_t) * __builtin_popcountll(subset_mask));
  return GTD_OK;
}

gtd_status gtd_dp_table(gtd_handle h, const uint8_t** d_table, uint64_t* bytes, int* n, int* tile_bits) {
  if (!h)
    return GTD_INVALID_ARG;
  if (!h->have_table)
    return fail(h, GTD_NO_RESULT, "no DP table: solve a graph first");
  if (d_table)
    *d_table = h->d_table;
  if (bytes)
    *bytes = uint64_t(1) << h->last_params.single.n;
  if (n)
    *n = h->last_params.single.n;
  if (tile_bits)
    *tile_bits = h->last_params.lb;
  return GTD_OK;
}

gtd_status gtd_dp_read_table(gtd_handle h, uint8_t* out, uint64_t bytes) {
  if (!h)
    return GTD_INVALID_ARG;
  if (!h->have_table)
    return fail(h, GTD_NO_RESULT, "no DP table: solve a graph first");
  const uint64_t need = uint64_t(1) << h->last_params.single.n;
  if (!out || bytes < need)
    return fail(h, GTD_INVALID_ARG, "output buffer smaller than the table");
  DeviceGuard g(h->device);
  GTD_CUDA(h, cudaMemcpyAsync(out, h->d_table, need, cudaMemcpyDeviceToHost, h->stream));
  GTD_CUDA(h, cudaStreamSynchronize(h->stream));
  return GTD_OK;
}

gtd_status gtd_dp_labels(gtd_handle h, const uint64_t* subsets, int count, int32_t* td_out,
                         uint64_t* roots_out) {
  if (!h)
    return GTD_INVALID_ARG;
  if (!h->have_table)
    return fail(h, GTD_NO_RESULT, "no DP table: solve a graph first");
  if (!subsets || !td_out || !roots_out || count < 0)
    return fail(h, GTD_INVALID_ARG, "null pointer argument");
  if (count == 0)
    return GTD_OK;
  const int n = h->last_params.single.n;
  for (int i = 0; i < count; ++i)
    if (n < 64 && (subsets[i] >> n))
      return fail(h, GTD_INVALID_ARG, "subset has a vertex >= n");
  DeviceGuard g(h->device);
  const size_t bytes = size_t(count) * (2 * sizeof(uint64_t) + sizeof(int32_t));
  GTD_CUDA(h, ensure_device(&h->d_scratch, &h->scratch_cap, bytes));
  uint64_t* d_sub = static_cast<uint64_t*>(h->d_scratch);
  uint64_t* d_roots = d_sub + count;
  int32_t* d_td = reinterpret_cast<int32_t*>(d_roots + count);
  GTD_CUDA(h, cudaMemcpyAsync(d_sub, subsets, count * sizeof(uint64_t), cudaMemcpyHostToDevice, h->stream));
  GTD_CUDA(h, dp_launch_labels(h->last_params, d_sub, count, d_td, d_roots, h->stream));
  GTD_CUDA(h, cudaMemcpyAsync(td_out, d_td, count * sizeof(int32_t), cudaMemcpyDeviceToHost, h->stream));
  GTD_CUDA(h, cudaMemcpyAsync(roots_out, d_roots, count * sizeof(uint64_t), cudaMemcpyDeviceToHost, h->stream));
  GTD_CUDA(h, cudaStreamSynchronize(h->stream));
  return GTD_OK;
}

gtd_status gtd_abort(gtd_handle h) {
  if (!h)
    return GTD_INVALID_ARG;
  // Only the abort stream and the pinned abort word are touched, so this may
  // run while another host thread is inside a call on the same handle. The
  // persistent kernels poll the error word and stop; the host loops see it.
  DeviceGuard g(h->device);
  int32_t* word = reinterpret_cast<int32_t*>(static_cast<char*>(h->h_pinned) + kPinnedAbort);
  *word = kDevAborted;
  cudaError_t e = cudaMemcpyAsync(h->d_io + kIoError, word, sizeof(int32_t), cudaMemcpyHostToDevice,
                                  h->abort_stream);
  if (e == cudaSuccess)
    e = cudaStreamSynchronize(h->abort_stream);
  return e == cudaSuccess ? GTD_OK : GTD_CUDA_ERROR;
}

gtd_status gtd_inject_fault(int kind, int count) {
  if (count < 0)
    return GTD_INVALID_ARG;
  switch (kind) {
    case GTD_FAULT_NONE:
      g_alloc_faults.store(0);
      g_stall_faults.store(0);
      g_poison_faults.store(0);
      return GTD_OK;
    case GTD_FAULT_ALLOC:
      g_alloc_faults.store(count);
      return GTD_OK;
    case GTD_FAULT_STALL:
      g_stall_faults.store(count);
      return GTD_OK;
    case GTD_FAULT_POISON:
      g_poison_faults.store(count);
      return GTD_OK;
    default:
      return GTD_INVALID_ARG;
  }
}

uint64_t gtd_dp_table_index(int n, int tile_bits, uint64_t subset_mask) {
  if (n < 2 || n > GTD_DP_MAX_N)
    return ~0ull;
  DpLayout L = make_dp_layout(n, tile_bits);
  if (L.lb != tile_bits)
    return ~0ull;
  return L.index(subset_mask);
}

}  // extern "C"
