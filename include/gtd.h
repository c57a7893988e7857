/* gtd — GB300-native exact treedepth solvers, C ABI.
 *
 * Drop-in boundary for the exact solvers of Zackere/GiSBDW (Treedepth/src):
 * a graph goes in, its exact treedepth and an elimination tree come out.
 * Every entry point takes plain pointers and sizes, never throws, and returns
 * a gtd_status. The C++ layer in include/gtd/treedepth.hpp maps these codes
 * to the exception types the reference throws.
 *
 * Graphs: n vertices 0..n-1, adjacency as bit masks. adj[v] has bit u set iff
 * the undirected edge uv exists; masks must be symmetric with no self loops.
 * Trees: parent[v] is v's parent in the elimination tree, -1 for the root
 * (roots, for a disconnected graph's elimination forest). The tree height
 * (counted in vertices) equals the treedepth.
 *
 * Threading: a handle owns its device buffers and one CUDA stream; it is not
 * thread-safe. Use one handle per host thread.
 */
#ifndef GTD_H_
#define GTD_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  GTD_OK = 0,
  GTD_INVALID_ARG = 1, /* n out of range, self loop, asymmetric masks, bad pointer */
  GTD_NOT_CONNECTED = 2, /* input must be connected (branch and bound) */
  GTD_OOM = 3,           /* device allocation failed */
  GTD_TIMEOUT = 4,       /* a bounded wait or a deadline ran out */
  GTD_ABORTED = 5,       /* stopped by gtd_abort or another error */
  GTD_CUDA_ERROR = 6,    /* a CUDA runtime call failed */
  GTD_NO_RESULT = 7      /* query before a solve, or subset not available */
} gtd_status;

typedef struct gtd_handle_s* gtd_handle;

/* Largest n the subset DP accepts (table of 2^n bytes: 64 GiB at n = 36). */
#define GTD_DP_MAX_N 36

/* Creates a handle on CUDA device `device`. `stream` is a cudaStream_t to
 * run on, or NULL for a handle-owned stream. */
gtd_status gtd_create(gtd_handle* out, int device, void* stream);
gtd_status gtd_destroy(gtd_handle h);
const char* gtd_status_string(gtd_status s);
/* Human-readable detail of the last failure on this handle. */
const char* gtd_last_error(gtd_handle h);

/* Stops the call in flight on handle h: the persistent kernels see the
 * request at their next poll (every DP tile ticket and dependency wait,
 * every 64 branch-and-bound search nodes) and that call returns GTD_ABORTED
 * with its outputs undefined; the handle stays usable. This is the one call
 * that may be made from another host thread while a call on the same handle
 * runs. A request made while no call runs is dropped when the next call
 * starts (every call clears the handle's error word first). No counterpart
 * in the reference, whose solvers run to completion. */
gtd_status gtd_abort(gtd_handle h);

/* Fault injection for tests of the error paths (no counterpart in the
 * reference), process-wide:
 *   GTD_FAULT_ALLOC, c: the c-th device buffer allocation made by this
 *     library from now on fails as if the GPU were out of memory; the call
 *     returns GTD_OOM and the handle stays usable;
 *   GTD_FAULT_STALL, c: the next c single-graph DP solves (gtd_dp_solve,
 *     gtd_dp_solve_device) never take their first tile, so every tile that
 *     depends on it waits until its bound (gtd_dp_opts.timeout_ns) runs out:
 *     GTD_TIMEOUT, and the handle stays usable;
 *   GTD_FAULT_POISON, c: the next c subset-DP solves (single graphs and
 *     batches) first fill their table with 0xFF bytes (treedepth 127, a
 *     value no solve writes). Every table byte is written before any tile
 *     reads it, so results are unchanged; a tile read before its
 *     producer's stores were visible would see the poison and corrupt the
 *     result (the stress test of the tiles' release/acquire publication);
 *   GTD_FAULT_NONE: clears all. */
enum { GTD_FAULT_NONE = 0, GTD_FAULT_ALLOC = 1, GTD_FAULT_STALL = 2, GTD_FAULT_POISON = 3 };
gtd_status gtd_inject_fault(int kind, int count);

/* Options and statistics of one subset-DP solve. */
typedef struct {
  int tile_bits;        /* low vertices per tile (0 = autotuned default) */
  int ctas_per_sm;      /* persistent CTAs per SM (0 = default) */
  uint64_t timeout_ns;  /* bound on every in-kernel wait (0 = 10 s) */
} gtd_dp_opts;

typedef struct {
  float dp_ms;          /* DP kernel time, CUDA events on the handle's stream */
  float tree_ms;        /* tree reconstruction kernel */
  float total_ms;       /* whole call including copies */
  uint64_t table_bytes; /* 2^n */
  uint64_t alg_bytes;   /* 2^n + n 2^(n-1): one write + |S| one-byte gathers per subset */
  int tile_bits;
  int tiles;
  int ctas;
} gtd_dp_stats;

/* DynamicGPU (Treedepth/src/dynamic_gpu/dynamic_gpu.cu:171-201 Run, with
 * the reconstruction of dynamic_gpu.hpp:48-64 GetElimination and
 * main.cpp:187-195): exact treedepth of the graph and the elimination tree
 * whose every connected component is rooted at its first vertex v with
 * td(C - v) = td(C) - 1 (the reference's first-argmin root,
 * dynamic_gpu.cu:84-87). Host pointers: adj[n] in, td_out, parent_out[n]
 * and, if non-null, order_out[n] (the reference's GetElimination order) out.
 * The DP table stays on the device for gtd_dp_query until the next solve.
 * 1 <= n <= GTD_DP_MAX_N; disconnected graphs give an elimination forest. */
gtd_status gtd_dp_solve(gtd_handle h, const uint64_t* adj, int n,
                        int32_t* td_out, int32_t* parent_out,
                        int32_t* order_out, const gtd_dp_opts* opts,
                        gtd_dp_stats* stats);

/* Same computation with adjacency, td, parent and order in DEVICE memory;
 * enqueued on the handle's stream without a host synchronisation (stats and
 * errors are collected by gtd_sync). order_out may be NULL. */
gtd_status gtd_dp_solve_device(gtd_handle h, const uint64_t* d_adj, int n,
                               int32_t* d_td, int32_t* d_parent,
                               int32_t* d_order, const gtd_dp_opts* opts);

/* Waits for the handle's stream; reports in-kernel errors (timeouts) of
 * device-side solves and fills stats of the last DP solve if non-null. */
gtd_status gtd_sync(gtd_handle h, gtd_dp_stats* stats);

/* DynamicGPU::GetElimination (dynamic_gpu.hpp:48-64) on the table of the
 * last solve: treedepth of the subset `subset_mask` and its elimination
 * order (order_out[popcount(subset_mask)]; NULL to skip). */
gtd_status gtd_dp_query(gtd_handle h, uint64_t subset_mask, int32_t* td_out,
                        int32_t* order_out);

/* Device pointer and size of the last solve's table (for inspection in
 * tests): entry of subset S lives at gtd_dp_table_index(n, tile_bits, S).
 * Each byte holds td << 1 | connected (td in bits 1-6, bit 0 set iff the
 * induced subgraph is connected). */
gtd_status gtd_dp_table(gtd_handle h, const uint8_t** d_table, uint64_t* bytes,
                        int* n, int* tile_bits);
uint64_t gtd_dp_table_index(int n, int tile_bits, uint64_t subset_mask);

/* Copies the last solve's table (2^n bytes, tiled layout as above) to host
 * memory `out` of `bytes` bytes. */
gtd_status gtd_dp_read_table(gtd_handle h, uint8_t* out, uint64_t bytes);

/* ---- Batched subset DP ------------------------------------------------ */

/* One graph of a batch: n vertices; its adjacency masks are
 * adj_pool[offset .. offset + n) and its parent array is written to
 * parent_out[offset .. offset + n). */
typedef struct {
  int32_t n;
  int32_t offset;
} gtd_graph_desc;

typedef struct {
  int tile_bits;        /* 8..12 for every graph; 0 = planned per vertex
                           count from gtd_dp_autotune's results (else 10) */
  int ctas_per_sm;      /* 0 = occupancy limit */
  uint64_t timeout_ns;  /* bound on every in-kernel wait (0 = 10 s) */
  int use_cuda_graph;   /* capture the launch once, replay while the batch
                           (sizes, offsets, buffers) stays the same */
} gtd_dp_batch_opts;

typedef struct {
  float dp_ms;          /* device time of validate + DP + tree, CUDA events */
  float total_ms;       /* whole call including copies */
  uint64_t subsets;     /* sum of 2^n over the batch */
  uint64_t alg_bytes;   /* sum of 2^n + n 2^(n-1) */
  uint64_t table_bytes; /* table pool (graphs with n < tile bits padded) */
  int tile_bits;        /* the launch's largest tile size */
  int tiles;
  int ctas;
  int graph_replayed;   /* 1 if an existing CUDA graph was replayed */
  int tile_bits_by_n[GTD_DP_MAX_N + 1]; /* tile size of the graphs with n
                                           vertices (0: none in the batch) */
} gtd_dp_batch_stats;

/* DynamicGPU over many graphs of uneven size in ONE persistent launch
 * (every graph's tiles in one ticket order, largest graphs first), the
 * launch sequence optionally captured in a CUDA graph. Results are those of
 * gtd_dp_solve for every graph: td_out[i], and the tree of graph i in
 * parent_out[descs[i].offset ...]. Host pointers; adj_pool and parent_out
 * hold pool_len entries. 1 <= n <= GTD_DP_MAX_N per graph. */
gtd_status gtd_dp_solve_batch(gtd_handle h, const gtd_graph_desc* descs,
                              int count, const uint64_t* adj_pool,
                              int64_t pool_len, int32_t* td_out,
                              int32_t* parent_out,
                              const gtd_dp_batch_opts* opts,
                              gtd_dp_batch_stats* stats);

/* The same with adjacency pool and outputs in DEVICE memory (descs stay on
 * the host); enqueued on the handle's stream; gtd_dp_batch_sync waits,
 * reports in-kernel errors and fills the stats. */
gtd_status gtd_dp_solve_batch_device(gtd_handle h, const gtd_graph_desc* descs,
                                     int count, const uint64_t* d_adj_pool,
                                     int64_t pool_len, int32_t* d_td,
                                     int32_t* d_parent,
                                     const gtd_dp_batch_opts* opts);
gtd_status gtd_dp_batch_sync(gtd_handle h, gtd_dp_batch_stats* stats);

/* The autotuner: times the batched DP kernel for every n in [n_min, n_max]
 * and tile bits 8..12 on seeded random graphs (at least 2^26 subsets per
 * measurement) and keeps the rates in the handle; rates_out (may be NULL)
 * receives (n_max - n_min + 1) x 5 rates in subsets per microsecond, row n,
 * column tile bits - 8. At n_max it also times the mixed-size kernel (the
 * one that runs graphs of different tile sizes in one launch; it holds fewer
 * CTAs per SM) at each largest tile size 8..12: mixed_eff_out (may be NULL)
 * receives its 5 throughputs relative to the one-size kernel. Batches solved
 * with tile_bits = 0 then give each vertex count its own tile size when the
 * predicted time, mixed-kernel efficiency included, beats one size for all. */
gtd_status gtd_dp_autotune(gtd_handle h, int n_min, int n_max,
                           float* rates_out, float* mixed_eff_out);

/* Loads autotuner results (the layouts gtd_dp_autotune writes; 0 =
 * unknown; mixed_eff may be NULL: never mix sizes), e.g. saved from an
 * earlier process, so that a handle plans batches without measuring again.
 * 2 <= n_min <= n_max <= GTD_DP_MAX_N. */
gtd_status gtd_dp_set_rates(gtd_handle h, int n_min, int n_max,
                            const float* rates, const float* mixed_eff);

/* ---- Branch and bound -------------------------------------------------- */

/* Largest n of the branch and bound (memo keys hold 104 vertex bits). */
#define GTD_BNB_MAX_N 104

typedef struct {
  int memo_log2;        /* memo slots per graph = 2^memo_log2 (0 = sized from free HBM: a quarter,
                           at most 32 GiB, 2^16..2^24 slots of 16 bytes) */
  uint64_t deadline_ns; /* per-graph cap on time-to-proof (0 = 120 s) */
  int ctas_per_sm;      /* 0 = occupancy limit */
  const int32_t* level_hint; /* per graph, NULL or 0 = none: the decision level
                                k to try first (e.g. a learned td estimate);
                                it orders the search and never prunes */
  uint32_t first_budget; /* search nodes of an item's first run per pass (0 = 1024) */
  int window;            /* decision levels per graph run at a time (0 = 3) */
} gtd_bnb_opts;

typedef struct {
  float ms;             /* device time of search + reconstruction (events) */
  float total_ms;       /* whole call */
  uint64_t nodes;       /* search nodes over the batch */
  int32_t passes;       /* budgeted passes the one persistent launch ran */
} gtd_bnb_stats;

/* BranchAndBound (Treedepth/src/branch_and_bound/branch_and_bound.cpp:51-114)
 * and BnBGPU (bnb_gpu.cu:264-380) over a batch of connected graphs in ONE
 * persistent (cooperative) launch that runs passes of node-budgeted items
 * until every graph is proven or past its deadline (a batch too small to
 * fill the GPU is split into first-root x second-root items, so a single
 * graph uses n^2 warps): exact treedepth AND an elimination tree per graph (the
 * reference's GPU B&B returns the treedepth only). Graph i has n = descs[i].n
 * <= GTD_BNB_MAX_N vertices with 128-bit adjacency masks
 * adj2_pool[2 (offset + v)] (bits 0-63) and [2 (offset + v) + 1] (bits
 * 64-127). order_pool[offset + r] is the vertex tried r-th as a root (NULL:
 * ascending ids, the reference's DefaultAttemptOrder). seed_td[i] and the
 * tree seed_parent[offset ..] are the incumbent (a heuristic's result, e.g.
 * gtd_heuristic). Outputs: td_out[i], parent_out[offset ..], status_out[i]
 * (GTD_OK proven, GTD_TIMEOUT deadline hit: td/tree = best found),
 * proof_ms_out[i] (time from the launch's first item to the graph's proof)
 * and nodes_out[i] (search nodes), both optional. Disconnected graphs give
 * GTD_NOT_CONNECTED and self loops GTD_INVALID_ARG, as the reference's
 * std::invalid_argument (branch_and_bound.hpp:67-75). */
gtd_status gtd_bnb_solve_batch(gtd_handle h, const gtd_graph_desc* descs,
                               int count, const uint64_t* adj2_pool,
                               int64_t pool_len, const uint8_t* order_pool,
                               const int32_t* seed_td,
                               const int32_t* seed_parent, int32_t* td_out,
                               int32_t* parent_out, int32_t* status_out,
                               float* proof_ms_out, uint64_t* nodes_out,
                               const gtd_bnb_opts* opts, gtd_bnb_stats* stats);

/* The proven lower bound on the treedepth of every graph of the last
 * gtd_bnb_solve_batch call on h (count = that call's batch size): equal to
 * td_out for proven graphs, below it for graphs whose deadline ran out. */
gtd_status gtd_bnb_lower_bounds(gtd_handle h, int32_t* lb_out, int count);

/* Greedy elimination heuristics (host only), the reference's incumbent
 * seeds (src/branch_and_bound/heuristics/): kind 0 HighestDegree(Variance)
 * (benchmark.cpp:50-55), 1 HighestDegree, 2 Variance, 3 highest score first
 * (scores[n] required). adj2 as in gtd_bnb_solve_batch; the graph must be
 * connected. Writes the tree height and parent array. */
gtd_status gtd_heuristic(const uint64_t* adj2, int n, int kind,
                         const float* scores, int32_t* td_out,
                         int32_t* parent_out);

/* Largest n of gtd_bottom_up (one 32-byte forest row per subset). */
#define GTD_BOTTOM_UP_MAX_N 32

/* BottomUpHeuristicGPU (src/branch_and_bound/heuristics/bottom_up_heuristic.hpp:
 * 18-33 with its DP, bottom_up_heuristic_gpu_algorithm.cu:57-258), the
 * innermost incumbent heuristic of the reference's bnbGPU / bnbCPU chains
 * (main.cpp:170-186): level by level over all 2^n subsets, each subset keeps
 * one elimination forest, that of a child S - v with v added as the root of
 * its neighbours' trees, for the first v with the least height; the order of
 * last-added vertices from V down (GetElimination) is replayed into an
 * elimination tree. Host pointers: adj[n] in, td_out (the tree's height),
 * parent_out[n] and, if non-null, order_out[n] out. Needs 2^n + 66 C(n, n/2)
 * bytes of device memory (about 44 GB at n = 32). n > GTD_BOTTOM_UP_MAX_N
 * gives GTD_NO_RESULT, as the reference's Get returns its no-result sentinel
 * when the DP cannot run to the end (bottom_up_heuristic.hpp:24-32). */
gtd_status gtd_bottom_up(gtd_handle h, const uint64_t* adj, int n,
                         int32_t* td_out, int32_t* parent_out,
                         int32_t* order_out);

/* The same heuristics for many graphs in one GPU launch (one warp per
 * graph, n <= 128), trees identical to gtd_heuristic's: descs and the
 * (lo, hi) adjacency pool as for gtd_bnb_solve_batch; kind 0..3 as above
 * (kind 3 reads scores_pool[descs[i].offset + v]); td_out[count] and
 * parent_out[pool_len] (graph i's tree at descs[i].offset). Disconnected
 * graphs give an elimination forest. Host pointers. */
gtd_status gtd_heuristic_batch(gtd_handle h, const gtd_graph_desc* descs,
                               int count, const uint64_t* adj2_pool,
                               int64_t pool_len, int kind,
                               const float* scores_pool, int32_t* td_out,
                               int32_t* parent_out);

/* Training labels from the last single-graph DP solve: for subsets[i], its
 * treedepth td_out[i] and, when the subset is connected, the mask of its
 * optimal roots roots_out[i] (v with td(S - v) = td(S) - 1, the root set every
 * reference DP chooses from, dynamic_cpu.cpp:96-99). */
gtd_status gtd_dp_labels(gtd_handle h, const uint64_t* subsets, int count,
                         int32_t* td_out, uint64_t* roots_out);

/* ---- Learned branching order (no counterpart in the reference) --------- */

/* A message-passing GNN (input projection, `layers` mean-aggregation layers
 * of width `hidden` <= 64, ReLU) with a per-vertex root logit and a
 * per-graph treedepth estimate; BF16 weights, FP32 accumulation, own
 * forward / backward / Adam kernels. It orders the branch and bound's
 * candidates and seeds its incumbent; it never prunes. */
typedef struct gtd_gnn_s* gtd_gnn;

/* One batch of graphs: nodes of graph g are [graph_start[g],
 * graph_start[g + 1]); node v's neighbours (batch indices) are
 * nbr[nbr_start[v] .. nbr_start[v + 1]); x holds num_nodes x in_features
 * features. Labels (training only): root_label / node_mask per node (loss
 * over nodes with mask 1), td_label per graph. */
typedef struct {
  int num_nodes;
  int num_graphs;
  const float* x;
  const int32_t* graph_start;
  const int32_t* nbr_start;
  const int32_t* nbr;
  const float* root_label;
  const float* node_mask;
  const float* td_label;
} gtd_gnn_batch;

gtd_status gtd_gnn_create(gtd_handle h, int in_features, int hidden,
                          int layers, uint64_t seed, gtd_gnn* out);
gtd_status gtd_gnn_destroy(gtd_gnn g);
int64_t gtd_gnn_num_params(gtd_gnn g);
/* FP32 master parameters (the BF16 weights are their rounding). */
gtd_status gtd_gnn_get_params(gtd_gnn g, float* out);
gtd_status gtd_gnn_set_params(gtd_gnn g, const float* in);
gtd_status gtd_gnn_forward(gtd_gnn g, const gtd_gnn_batch* b,
                           float* logits_out, float* td_out);
/* Loss and its gradient w.r.t. every parameter (for checks). */
gtd_status gtd_gnn_gradients(gtd_gnn g, const gtd_gnn_batch* b,
                             float td_weight, float* grad_out,
                             float* loss_out);
/* One Adam step (lr, betas 0.9 / 0.999) on the batch's loss. */
gtd_status gtd_gnn_train_step(gtd_gnn g, const gtd_gnn_batch* b, float lr,
                              float td_weight, float* loss_out);

/* Host data pipeline of the GNN (n <= 128 per graph, adjacency as (lo, hi)
 * pairs per vertex like gtd_bnb_solve_batch). Features per vertex (8):
 * degree / 4, core number / 4, eccentricity / 8, mean neighbour degree / 4,
 * pendant flag, 1 / (1 + degree), n / 64, 1. */
gtd_status gtd_gnn_features(const uint64_t* adj2, int n, float* x_out);
/* Sizes of a packed batch: total vertices and total neighbour entries. */
gtd_status gtd_gnn_pack_sizes(const uint64_t* adj2_pool,
                              const gtd_graph_desc* descs, int count,
                              int64_t* nodes_out, int64_t* nbrs_out);
/* Features and CSR neighbour lists of graphs (the x / graph_start /
 * nbr_start / nbr arrays of a gtd_gnn_batch). */
gtd_status gtd_gnn_pack(const uint64_t* adj2_pool, const gtd_graph_desc* descs,
                        int count, float* x_out, int32_t* graph_start_out,
                        int32_t* nbr_start_out, int32_t* nbr_out);
/* Training labels from the exact DP: every base graph (2 <= n <= 24) is
 * solved on the GPU, then it and per_graph random connected induced
 * subgraphs (sizes uniform in [min_size, n], grown from a random vertex) are
 * labelled with td and the optimal-root mask (gtd_dp_labels). Up to
 * `capacity` samples are written relabelled 0..k-1 in vertex order:
 * sub_adj2_out (capacity * 48 words), sub_desc_out, root_out, td_out;
 * *num_out = samples written. Uses (and overwrites) the handle's DP table. */
gtd_status gtd_gnn_make_labels(gtd_handle h, const uint64_t* adj2_pool,
                               const gtd_graph_desc* descs, int count,
                               int per_graph, int min_size, uint64_t seed,
                               int capacity, uint64_t* sub_adj2_out,
                               gtd_graph_desc* sub_desc_out, uint64_t* root_out,
                               int32_t* td_out, int* num_out);

/* Largest n gtd_dp_solve_noalloc accepts (its fixed scratch holds a 2^n-byte
 * table: 16 MiB at n = 24). */
#define GTD_DP_NOALLOC_MAX_N 24

/* The subset DP for callers that cannot allocate device memory (code running
 * where cudaMalloc is not allowed, under a pool that must not grow, or next to
 * a framework that owns all device memory). This entry point has no
 * counterpart in the reference. It allocates nothing: no handle, no
 * cudaMalloc/cudaFree. Its scratch is one fixed __device__ array of about
 * 16.1 MiB that every GPU loading this library holds until process exit, so
 * it accepts 2 <= n <= GTD_DP_NOALLOC_MAX_N and rejects larger n with
 * GTD_INVALID_ARG. Inputs and outputs are DEVICE pointers owned by the
 * caller: adjacency d_adj[n]; outputs d_td (1 int), d_parent[n] and, if
 * non-null, d_order[n], with the same values as gtd_dp_solve. Runs on
 * `stream` (a cudaStream_t, NULL for the legacy default stream) on the
 * current device and returns after synchronising that stream. The first
 * call on each device looks up the scratch array's device address
 * (cudaGetSymbolAddress) with that device current; make that first call
 * before any stream capture. All calls share the one array and it keeps the
 * previous call's contents (the call clears what must start at zero): calls
 * whose GPU work overlaps, from two streams or two host threads, race. */
gtd_status gtd_dp_solve_noalloc(const uint64_t* d_adj, int n, int32_t* d_td,
                                int32_t* d_parent, int32_t* d_order,
                                void* stream);

#ifdef __cplusplus
}
#endif
#endif /* GTD_H_ */
