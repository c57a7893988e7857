// A small message-passing GNN that scores vertices as roots of an optimal
// elimination tree, with hand-written forward, backward and Adam kernels.
// It is used only to ORDER the branch and bound's candidates and to seed its
// incumbent (greedy elimination by score); it never prunes, so every
// treedepth stays proven by the exact search. No counterpart exists in the
// reference.
//
// Network (hidden H = 64 by default, L = 3 layers):
//   h0      = relu(x W_in + b_in)                       x: per-vertex features
//   a_l(v)  = mean_{u in N(v)} h_l(u)                   (0 for isolated v)
//   h_{l+1} = relu(h_l Ws_l + a_l Wn_l + b_l)
//   logit_v = h_L(v) . w_out + b_out                    root score
//   td_g    = mean_{v in g} h_L(v) . w_g + b_g          treedepth estimate
// Weights are stored in BF16 (a BF16 copy of an FP32 master kept by Adam);
// every product accumulates in FP32. Loss: masked mean binary cross entropy
// of the root logits + td_weight * mean squared td error.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "gtd_handle.h"

namespace gtd {
namespace {

constexpr int kNodesPerBlock = 16;
constexpr int kMaxK = 64;

__device__ __forceinline__ float bf(const __nv_bfloat16 x) { return __bfloat162float(x); }

// Z = X1 W1 (+ X2 W2) + bias; Hout = relu(Z). X rows of K floats, W K x H
// (row major, BF16), one thread per output channel, kNodesPerBlock nodes per
// block, weights staged in shared memory.
__global__ void node_linear(int N, int K, int H, const float* __restrict__ X1, const __nv_bfloat16* __restrict__ W1,
                            const float* __restrict__ X2, const __nv_bfloat16* __restrict__ W2,
                            const __nv_bfloat16* __restrict__ bias, float* __restrict__ Z, float* __restrict__ Hout) {
  __shared__ float w1[kMaxK * kMaxK], w2[kMaxK * kMaxK];
  __shared__ float x1[kNodesPerBlock][kMaxK], x2[kNodesPerBlock][kMaxK];
  const int j = threadIdx.x;
  for (int t = threadIdx.x; t < K * H; t += blockDim.x) {
    w1[t] = bf(W1[t]);
    if (X2)
      w2[t] = bf(W2[t]);
  }
  const int v0 = blockIdx.x * kNodesPerBlock;
  for (int t = threadIdx.x; t < kNodesPerBlock * K; t += blockDim.x) {
    const int r = t / K, i = t % K;
    const int v = v0 + r;
    x1[r][i] = v < N ? X1[size_t(v) * K + i] : 0.f;
    if (X2)
      x2[r][i] = v < N ? X2[size_t(v) * K + i] : 0.f;
  }
  __syncthreads();
  if (j >= H)
    return;
  float acc[kNodesPerBlock];
  const float b = bf(bias[j]);
#pragma unroll
  for (int r = 0; r < kNodesPerBlock; ++r)
    acc[r] = b;
  for (int i = 0; i < K; ++i) {
    const float wa = w1[i * H + j];
#pragma unroll
    for (int r = 0; r < kNodesPerBlock; ++r)
      acc[r] = fmaf(x1[r][i], wa, acc[r]);
  }
  if (X2)
    for (int i = 0; i < K; ++i) {
      const float wb = w2[i * H + j];
#pragma unroll
      for (int r = 0; r < kNodesPerBlock; ++r)
        acc[r] = fmaf(x2[r][i], wb, acc[r]);
    }
#pragma unroll
  for (int r = 0; r < kNodesPerBlock; ++r) {
    const int v = v0 + r;
    if (v < N) {
      Z[size_t(v) * H + j] = acc[r];
      Hout[size_t(v) * H + j] = fmaxf(acc[r], 0.f);
    }
  }
}

// dX = dZ W^T (W K x H): one thread per input channel i.
__global__ void node_linear_t(int N, int K, int H, const float* __restrict__ dZ, const __nv_bfloat16* __restrict__ W,
                              float* __restrict__ dX) {
  __shared__ float w[kMaxK * kMaxK];
  __shared__ float dz[kNodesPerBlock][kMaxK];
  for (int t = threadIdx.x; t < K * H; t += blockDim.x)
    w[t] = bf(W[t]);
  const int v0 = blockIdx.x * kNodesPerBlock;
  for (int t = threadIdx.x; t < kNodesPerBlock * H; t += blockDim.x) {
    const int r = t / H, j = t % H;
    const int v = v0 + r;
    dz[r][j] = v < N ? dZ[size_t(v) * H + j] : 0.f;
  }
  __syncthreads();
  const int i = threadIdx.x;
  if (i >= K)
    return;
  float acc[kNodesPerBlock] = {};
  for (int j = 0; j < H; ++j) {
    const float wij = w[i * H + j];
#pragma unroll
    for (int r = 0; r < kNodesPerBlock; ++r)
      acc[r] = fmaf(dz[r][j], wij, acc[r]);
  }
#pragma unroll
  for (int r = 0; r < kNodesPerBlock; ++r) {
    const int v = v0 + r;
    if (v < N)
      dX[size_t(v) * K + i] = acc[r];
  }
}

// Partial X^T dZ (and column sums of dZ) of a chunk of 64 nodes per block,
// written to part[block][K * H + H]; reduce_partials adds the chunks in a
// fixed order, so the gradient (and training) is deterministic.
__global__ void weight_grad(int N, int K, int H, const float* __restrict__ X, const float* __restrict__ dZ,
                            float* __restrict__ part) {
  constexpr int kChunk = 64;
  __shared__ float xs[kChunk][kMaxK], ds[kChunk][kMaxK];
  const int v0 = blockIdx.x * kChunk;
  const int nv = min(kChunk, N - v0);
  for (int t = threadIdx.x; t < kChunk * kMaxK; t += blockDim.x) {
    const int r = t / kMaxK, c = t % kMaxK;
    xs[r][c] = (r < nv && c < K) ? X[size_t(v0 + r) * K + c] : 0.f;
    ds[r][c] = (r < nv && c < H) ? dZ[size_t(v0 + r) * H + c] : 0.f;
  }
  __syncthreads();
  float* out = part + size_t(blockIdx.x) * (K * H + H);
  for (int t = threadIdx.x; t < K * H; t += blockDim.x) {
    const int i = t / H, j = t % H;
    float acc = 0.f;
    for (int r = 0; r < nv; ++r)
      acc = fmaf(xs[r][i], ds[r][j], acc);
    out[t] = acc;
  }
  for (int j = threadIdx.x; j < H; j += blockDim.x) {
    float acc = 0.f;
    for (int r = 0; r < nv; ++r)
      acc += ds[r][j];
    out[K * H + j] = acc;
  }
}

// dW += sum over chunks of the partials, db likewise (when non-null).
__global__ void reduce_partials(int chunks, int KH, int H, const float* __restrict__ part, float* __restrict__ dW,
                                float* __restrict__ db) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= KH + H || (t >= KH && !db))
    return;
  float acc = 0.f;
  for (int c = 0; c < chunks; ++c)
    acc += part[size_t(c) * (KH + H) + t];
  if (t < KH)
    dW[t] += acc;
  else
    db[t - KH] += acc;
}

// a(v) = mean over neighbours of h(u); one thread per (v, channel).
__global__ void aggregate(int N, int H, const int32_t* __restrict__ nbr_start, const int32_t* __restrict__ nbr,
                          const float* __restrict__ h, float* __restrict__ a) {
  const size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= size_t(N) * H)
    return;
  const int v = static_cast<int>(t / H), j = static_cast<int>(t % H);
  const int s = nbr_start[v], e = nbr_start[v + 1];
  float acc = 0.f;
  for (int k = s; k < e; ++k)
    acc += h[size_t(nbr[k]) * H + j];
  a[t] = e > s ? acc / float(e - s) : 0.f;
}

// Backward of the mean: dh(u) += sum over neighbours v of da(v) / deg(v)
// (adjacency is symmetric, so this is a gather, no atomics).
__global__ void aggregate_t(int N, int H, const int32_t* __restrict__ nbr_start, const int32_t* __restrict__ nbr,
                            const float* __restrict__ da, float* __restrict__ dh) {
  const size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= size_t(N) * H)
    return;
  const int u = static_cast<int>(t / H), j = static_cast<int>(t % H);
  float acc = 0.f;
  for (int k = nbr_start[u]; k < nbr_start[u + 1]; ++k) {
    const int v = nbr[k];
    const int dv = nbr_start[v + 1] - nbr_start[v];
    acc += da[size_t(v) * H + j] / float(dv);
  }
  dh[t] += acc;
}

__global__ void relu_mask(size_t count, const float* __restrict__ z, const float* __restrict__ dh,
                          float* __restrict__ dz) {
  const size_t t = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t < count)
    dz[t] = z[t] > 0.f ? dh[t] : 0.f;
}

// Heads: logits per node; pooled mean per graph; td estimate per graph.
__global__ void heads_forward(int N, int G, int H, const float* __restrict__ h, const int32_t* __restrict__ gstart,
                              const __nv_bfloat16* __restrict__ w_out, const __nv_bfloat16* __restrict__ b_out,
                              const __nv_bfloat16* __restrict__ w_g, const __nv_bfloat16* __restrict__ b_g,
                              float* __restrict__ logits, float* __restrict__ pooled, float* __restrict__ td_est) {
  // blocks [0, ceil(N/128)) do logits; the next G blocks do the graphs
  const int nb = (N + 127) / 128;
  if (static_cast<int>(blockIdx.x) < nb) {
    const int v = blockIdx.x * 128 + threadIdx.x;
    if (v < N) {
      float acc = bf(b_out[0]);
      for (int j = 0; j < H; ++j)
        acc = fmaf(h[size_t(v) * H + j], bf(w_out[j]), acc);
      logits[v] = acc;
    }
    return;
  }
  const int g = blockIdx.x - nb;
  if (g >= G)
    return;
  __shared__ float part[128];
  const int s = gstart[g], e = gstart[g + 1];
  const int j = threadIdx.x;
  float m = 0.f;
  if (j < H) {
    for (int v = s; v < e; ++v)
      m += h[size_t(v) * H + j];
    m = e > s ? m / float(e - s) : 0.f;
    pooled[size_t(g) * H + j] = m;
  }
  part[threadIdx.x] = j < H ? m * bf(w_g[j]) : 0.f;
  __syncthreads();
  for (int off = 64; off > 0; off >>= 1) {
    if (threadIdx.x < off)
      part[threadIdx.x] += part[threadIdx.x + off];
    __syncthreads();
  }
  if (threadIdx.x == 0)
    td_est[g] = part[0] + bf(b_g[0]);
}

// Loss and the head gradients w.r.t. the logits and td estimates: writes
// dlogit (per node), dtd (per graph) and dh_L = dlogit w_out + dtd w_g / |g|.
__global__ void heads_backward(int N, int G, int H, const int32_t* __restrict__ gstart,
                               const int32_t* __restrict__ graph_of, const float* __restrict__ logits,
                               const float* __restrict__ td_est, const float* __restrict__ y,
                               const float* __restrict__ mask, const float* __restrict__ td_label, float inv_mask_sum,
                               float td_weight, const __nv_bfloat16* __restrict__ w_out,
                               const __nv_bfloat16* __restrict__ w_g, float* __restrict__ dlogit,
                               float* __restrict__ dtd, float* __restrict__ dh, float* __restrict__ loss) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= N)
    return;
  const float z = logits[v];
  const float m = mask[v];
  const float sig = 1.f / (1.f + expf(-z));
  const float dl = m * (sig - y[v]) * inv_mask_sum;
  atomicAdd(loss, m * (fmaxf(z, 0.f) - z * y[v] + log1pf(expf(-fabsf(z)))) * inv_mask_sum);
  dlogit[v] = dl;
  const int g = graph_of[v];
  const float diff = td_est[g] - td_label[g];
  const float dt = 2.f * td_weight * diff / float(G);
  if (v == gstart[g]) {
    dtd[g] = dt;
    atomicAdd(loss, td_weight * diff * diff / float(G));
  }
  const float ng = float(gstart[g + 1] - gstart[g]);
  for (int j = 0; j < H; ++j)
    dh[size_t(v) * H + j] = dl * bf(w_out[j]) + dt * bf(w_g[j]) / ng;
}

__global__ void adam_step(int64_t n, float* __restrict__ master, float* __restrict__ m, float* __restrict__ v,
                          const float* __restrict__ g, __nv_bfloat16* __restrict__ w, float lr, float b1, float b2,
                          float eps, float c1, float c2) {
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= n)
    return;
  const float gt = g[t];
  const float mt = b1 * m[t] + (1.f - b1) * gt;
  const float vt = b2 * v[t] + (1.f - b2) * gt * gt;
  m[t] = mt;
  v[t] = vt;
  const float upd = lr * (mt / c1) / (sqrtf(vt / c2) + eps);
  const float nm = master[t] - upd;
  master[t] = nm;
  w[t] = __float2bfloat16_rn(nm);
}

__global__ void to_bf16(int64_t n, const float* __restrict__ src, __nv_bfloat16* __restrict__ dst) {
  const int64_t t = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t < n)
    dst[t] = __float2bfloat16_rn(src[t]);
}

unsigned blocks_for(size_t n, unsigned t) { return static_cast<unsigned>((n + t - 1) / t); }

}  // namespace
}  // namespace gtd

struct gtd_gnn_s {
  gtd_handle h = nullptr;
  int fin = 0, hid = 0, layers = 0;
  int64_t nparams = 0;
  float* master = nullptr;
  float* m = nullptr;
  float* v = nullptr;
  float* grad = nullptr;
  __nv_bfloat16* w = nullptr;
  int64_t step = 0;
  // batch and activation buffers (grown as needed)
  void* buf = nullptr;
  size_t buf_cap = 0;
};

namespace {

struct Layout {
  int64_t w_in, b_in, layer0, layer_stride, head;
  int64_t ws(int l, int H) const { return layer0 + l * layer_stride; }
  int64_t wn(int l, int H) const { return layer0 + l * layer_stride + int64_t(H) * H; }
  int64_t b(int l, int H) const { return layer0 + l * layer_stride + 2 * int64_t(H) * H; }
};

Layout layout_of(const gtd_gnn_s* g) {
  const int64_t H = g->hid;
  Layout L;
  L.w_in = 0;
  L.b_in = int64_t(g->fin) * H;
  L.layer0 = L.b_in + H;
  L.layer_stride = 2 * H * H + H;
  L.head = L.layer0 + g->layers * L.layer_stride;
  return L;
}

// Device views of one batch plus activations, carved from g->buf.
struct Views {
  float* x;
  int32_t *gstart, *nbr_start, *nbr, *graph_of;
  float *y, *mask, *td_label;
  float *Z, *Hs, *A;  // (L + 1) x N x H, (L + 1) x N x H, L x N x H
  float *logits, *pooled, *td_est, *loss;
  float *dh, *dz, *da, *tmp, *dlogit, *dtd;
  float* part;  // weight-gradient partials, one row per 64-node chunk
};

gtd_status prepare(gtd_gnn g, const gtd_gnn_batch* b, bool train, Views& V) {
  gtd_handle h = g->h;
  const size_t N = size_t(b->num_nodes), G = size_t(b->num_graphs), H = size_t(g->hid), L = size_t(g->layers);
  const size_t E = size_t(b->nbr_start[b->num_nodes]);
  auto al = [](size_t bytes) { return (bytes + 255) & ~size_t(255); };
  size_t off = 0;
  auto take = [&](size_t bytes) {
    const size_t o = off;
    off += al(bytes);
    return o;
  };
  const size_t ox = take(N * g->fin * 4), ogs = take((G + 1) * 4), ons = take((N + 1) * 4), onb = take(E * 4 + 4),
               ogo = take(N * 4), oy = take(N * 4), om = take(N * 4), otd = take(G * 4),
               oZ = take((L + 1) * N * H * 4), oH = take((L + 1) * N * H * 4), oA = take(L * N * H * 4),
               olog = take(N * 4), opool = take(G * H * 4), otde = take(G * 4), oloss = take(4), odh = take(N * H * 4),
               odz = take(N * H * 4), oda = take(N * H * 4), otmp = take(N * H * 4), odl = take(N * 4),
               odt = take(G * 4),
               opart = take(((std::max(N, G) + 63) / 64) * (size_t(std::max(g->fin, g->hid)) * H + H) * 4);
  GTD_CUDA(h, gtd::ensure_device(&g->buf, &g->buf_cap, off));
  char* base = static_cast<char*>(g->buf);
  V.x = reinterpret_cast<float*>(base + ox);
  V.gstart = reinterpret_cast<int32_t*>(base + ogs);
  V.nbr_start = reinterpret_cast<int32_t*>(base + ons);
  V.nbr = reinterpret_cast<int32_t*>(base + onb);
  V.graph_of = reinterpret_cast<int32_t*>(base + ogo);
  V.y = reinterpret_cast<float*>(base + oy);
  V.mask = reinterpret_cast<float*>(base + om);
  V.td_label = reinterpret_cast<float*>(base + otd);
  V.Z = reinterpret_cast<float*>(base + oZ);
  V.Hs = reinterpret_cast<float*>(base + oH);
  V.A = reinterpret_cast<float*>(base + oA);
  V.logits = reinterpret_cast<float*>(base + olog);
  V.pooled = reinterpret_cast<float*>(base + opool);
  V.td_est = reinterpret_cast<float*>(base + otde);
  V.loss = reinterpret_cast<float*>(base + oloss);
  V.dh = reinterpret_cast<float*>(base + odh);
  V.dz = reinterpret_cast<float*>(base + odz);
  V.da = reinterpret_cast<float*>(base + oda);
  V.tmp = reinterpret_cast<float*>(base + otmp);
  V.dlogit = reinterpret_cast<float*>(base + odl);
  V.dtd = reinterpret_cast<float*>(base + odt);
  V.part = reinterpret_cast<float*>(base + opart);
  cudaStream_t s = h->stream;
  GTD_CUDA(h, cudaMemcpyAsync(V.x, b->x, N * g->fin * 4, cudaMemcpyHostToDevice, s));
  GTD_CUDA(h, cudaMemcpyAsync(V.gstart, b->graph_start, (G + 1) * 4, cudaMemcpyHostToDevice, s));
  GTD_CUDA(h, cudaMemcpyAsync(V.nbr_start, b->nbr_start, (N + 1) * 4, cudaMemcpyHostToDevice, s));
  if (E)
    GTD_CUDA(h, cudaMemcpyAsync(V.nbr, b->nbr, E * 4, cudaMemcpyHostToDevice, s));
  // graph of every node, from the ranges
  std::vector<int32_t> go(N);
  for (size_t gi = 0; gi < G; ++gi)
    for (int32_t v = b->graph_start[gi]; v < b->graph_start[gi + 1]; ++v)
      go[v] = static_cast<int32_t>(gi);
  GTD_CUDA(h, cudaMemcpyAsync(V.graph_of, go.data(), N * 4, cudaMemcpyHostToDevice, s));
  if (train) {
    GTD_CUDA(h, cudaMemcpyAsync(V.y, b->root_label, N * 4, cudaMemcpyHostToDevice, s));
    GTD_CUDA(h, cudaMemcpyAsync(V.mask, b->node_mask, N * 4, cudaMemcpyHostToDevice, s));
    GTD_CUDA(h, cudaMemcpyAsync(V.td_label, b->td_label, G * 4, cudaMemcpyHostToDevice, s));
  }
  // the copies above read host arrays that the caller may reuse right after
  GTD_CUDA(h, cudaStreamSynchronize(s));
  return GTD_OK;
}

gtd_status forward(gtd_gnn g, const gtd_gnn_batch* b, const Views& V) {
  gtd_handle h = g->h;
  const int N = b->num_nodes, G = b->num_graphs, H = g->hid, L = g->layers;
  const Layout P = layout_of(g);
  cudaStream_t s = h->stream;
  const unsigned nb = gtd::blocks_for(size_t(N), gtd::kNodesPerBlock);
  const size_t NH = size_t(N) * H;
  gtd::node_linear<<<nb, 64, 0, s>>>(N, g->fin, H, V.x, g->w + P.w_in, nullptr, nullptr, g->w + P.b_in, V.Z, V.Hs);
  GTD_CUDA(h, cudaGetLastError());
  for (int l = 0; l < L; ++l) {
    gtd::aggregate<<<gtd::blocks_for(NH, 256), 256, 0, s>>>(N, H, V.nbr_start, V.nbr, V.Hs + l * NH, V.A + l * NH);
    gtd::node_linear<<<nb, 64, 0, s>>>(N, H, H, V.Hs + l * NH, g->w + P.ws(l, H), V.A + l * NH, g->w + P.wn(l, H),
                                       g->w + P.b(l, H), V.Z + (l + 1) * NH, V.Hs + (l + 1) * NH);
    GTD_CUDA(h, cudaGetLastError());
  }
  const unsigned hb = gtd::blocks_for(size_t(N), 128) + static_cast<unsigned>(G);
  gtd::heads_forward<<<hb, 128, 0, s>>>(N, G, H, V.Hs + L * NH, V.gstart, g->w + P.head, g->w + P.head + H,
                                        g->w + P.head + H + 1, g->w + P.head + 2 * H + 1, V.logits, V.pooled,
                                        V.td_est);
  GTD_CUDA(h, cudaGetLastError());
  return GTD_OK;
}

// Weight gradient of one linear map over N rows: per-chunk partials, then
// their ordered sum into dW (and db).
void wgrad(cudaStream_t s, int N, int K, int H, const float* X, const float* dZ, float* dW, float* db, float* part) {
  const unsigned chunks = gtd::blocks_for(size_t(N), 64);
  gtd::weight_grad<<<chunks, 256, 0, s>>>(N, K, H, X, dZ, part);
  gtd::reduce_partials<<<gtd::blocks_for(size_t(K) * H + H, 256), 256, 0, s>>>(static_cast<int>(chunks), K * H, H,
                                                                              part, dW, db);
}

gtd_status backward(gtd_gnn g, const gtd_gnn_batch* b, const Views& V, float td_weight) {
  gtd_handle h = g->h;
  const int N = b->num_nodes, G = b->num_graphs, H = g->hid, L = g->layers;
  const Layout P = layout_of(g);
  cudaStream_t s = h->stream;
  const size_t NH = size_t(N) * H;
  double msum = 0;
  for (int v = 0; v < N; ++v)
    msum += b->node_mask[v];
  const float inv = msum > 0 ? float(1.0 / msum) : 0.f;
  GTD_CUDA(h, cudaMemsetAsync(g->grad, 0, g->nparams * 4, s));
  GTD_CUDA(h, cudaMemsetAsync(V.loss, 0, 4, s));
  float* gr = g->grad;
  gtd::heads_backward<<<gtd::blocks_for(size_t(N), 128), 128, 0, s>>>(
      N, G, H, V.gstart, V.graph_of, V.logits, V.td_est, V.y, V.mask, V.td_label, inv, td_weight, g->w + P.head,
      g->w + P.head + H + 1, V.dlogit, V.dtd, V.dh, V.loss);
  // w_out, b_out from h_L and dlogit; w_g, b_g from the pooled means and dtd
  wgrad(s, N, H, 1, V.Hs + L * NH, V.dlogit, gr + P.head, gr + P.head + H, V.part);
  wgrad(s, G, H, 1, V.pooled, V.dtd, gr + P.head + H + 1, gr + P.head + 2 * H + 1, V.part);
  GTD_CUDA(h, cudaGetLastError());
  const unsigned nb = gtd::blocks_for(size_t(N), gtd::kNodesPerBlock);
  const unsigned eb = gtd::blocks_for(NH, 256);
  for (int l = L - 1; l >= 0; --l) {
    // dz = dh * relu'(z_{l+1})
    gtd::relu_mask<<<eb, 256, 0, s>>>(NH, V.Z + (l + 1) * NH, V.dh, V.dz);
    wgrad(s, N, H, H, V.Hs + l * NH, V.dz, gr + P.ws(l, H), gr + P.b(l, H), V.part);
    wgrad(s, N, H, H, V.A + l * NH, V.dz, gr + P.wn(l, H), nullptr, V.part);
    // dh_l = dz Ws^T + aggregate^T(dz Wn^T)
    gtd::node_linear_t<<<nb, 64, 0, s>>>(N, H, H, V.dz, g->w + P.wn(l, H), V.da);
    gtd::node_linear_t<<<nb, 64, 0, s>>>(N, H, H, V.dz, g->w + P.ws(l, H), V.tmp);
    gtd::aggregate_t<<<eb, 256, 0, s>>>(N, H, V.nbr_start, V.nbr, V.da, V.tmp);
    GTD_CUDA(h, cudaMemcpyAsync(V.dh, V.tmp, NH * 4, cudaMemcpyDeviceToDevice, s));
    GTD_CUDA(h, cudaGetLastError());
  }
  gtd::relu_mask<<<eb, 256, 0, s>>>(NH, V.Z, V.dh, V.dz);
  wgrad(s, N, g->fin, H, V.x, V.dz, gr + P.w_in, gr + P.b_in, V.part);
  GTD_CUDA(h, cudaGetLastError());
  return GTD_OK;
}

uint64_t splitmix(uint64_t& s) {
  s += 0x9E3779B97F4A7C15ull;
  uint64_t z = s;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

}  // namespace

using namespace gtd;

extern "C" {

gtd_status gtd_gnn_create(gtd_handle h, int in_features, int hidden, int layers, uint64_t seed, gtd_gnn* out) {
  if (!h || !out)
    return GTD_INVALID_ARG;
  if (in_features < 1 || in_features > kMaxK || hidden < 1 || hidden > kMaxK || layers < 1 || layers > 8)
    return fail(h, GTD_INVALID_ARG, "GNN shape out of range (features, hidden <= 64, layers <= 8)");
  DeviceGuard dg(h->device);
  gtd_gnn g = new (std::nothrow) gtd_gnn_s();
  if (!g)
    return GTD_OOM;
  g->h = h;
  g->fin = in_features;
  g->hid = hidden;
  g->layers = layers;
  const Layout P = layout_of(g);
  g->nparams = P.head + 2 * hidden + 2;
  const size_t bytes = size_t(g->nparams) * 4;
  cudaError_t e = cudaMalloc(&g->master, bytes);
  if (e == cudaSuccess)
    e = cudaMalloc(&g->m, bytes);
  if (e == cudaSuccess)
    e = cudaMalloc(&g->v, bytes);
  if (e == cudaSuccess)
    e = cudaMalloc(&g->grad, bytes);
  if (e == cudaSuccess)
    e = cudaMalloc(&g->w, size_t(g->nparams) * 2);
  if (e != cudaSuccess) {
    gtd_gnn_destroy(g);
    return cuda_fail(h, e, "gtd_gnn_create");
  }
  // Glorot-uniform weights, zero biases, from a seeded splitmix64 stream.
  std::vector<float> p(g->nparams, 0.f);
  uint64_t st = seed;
  auto fill = [&](int64_t off, int fan_in, int fan_out) {
    const double lim = std::sqrt(6.0 / (fan_in + fan_out));
    for (int64_t i = 0; i < int64_t(fan_in) * fan_out; ++i)
      p[off + i] = float((double(splitmix(st) >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0) * lim);
  };
  fill(P.w_in, in_features, hidden);
  for (int l = 0; l < layers; ++l) {
    fill(P.ws(l, hidden), hidden, hidden);
    fill(P.wn(l, hidden), hidden, hidden);
  }
  fill(P.head, hidden, 1);
  fill(P.head + hidden + 1, hidden, 1);
  gtd_status s = gtd_gnn_set_params(g, p.data());
  if (s != GTD_OK) {
    gtd_gnn_destroy(g);
    return s;
  }
  *out = g;
  return GTD_OK;
}

gtd_status gtd_gnn_destroy(gtd_gnn g) {
  if (!g)
    return GTD_INVALID_ARG;
  DeviceGuard dg(g->h->device);
  cudaFree(g->master);
  cudaFree(g->m);
  cudaFree(g->v);
  cudaFree(g->grad);
  cudaFree(g->w);
  cudaFree(g->buf);
  delete g;
  return GTD_OK;
}

int64_t gtd_gnn_num_params(gtd_gnn g) { return g ? g->nparams : -1; }

gtd_status gtd_gnn_get_params(gtd_gnn g, float* out) {
  if (!g || !out)
    return GTD_INVALID_ARG;
  DeviceGuard dg(g->h->device);
  GTD_CUDA(g->h, cudaMemcpyAsync(out, g->master, g->nparams * 4, cudaMemcpyDeviceToHost, g->h->stream));
  GTD_CUDA(g->h, cudaStreamSynchronize(g->h->stream));
  return GTD_OK;
}

gtd_status gtd_gnn_set_params(gtd_gnn g, const float* in) {
  if (!g || !in)
    return GTD_INVALID_ARG;
  DeviceGuard dg(g->h->device);
  cudaStream_t s = g->h->stream;
  GTD_CUDA(g->h, cudaMemcpyAsync(g->master, in, g->nparams * 4, cudaMemcpyHostToDevice, s));
  GTD_CUDA(g->h, cudaMemsetAsync(g->m, 0, g->nparams * 4, s));
  GTD_CUDA(g->h, cudaMemsetAsync(g->v, 0, g->nparams * 4, s));
  to_bf16<<<blocks_for(size_t(g->nparams), 256), 256, 0, s>>>(g->nparams, g->master, g->w);
  GTD_CUDA(g->h, cudaGetLastError());
  GTD_CUDA(g->h, cudaStreamSynchronize(s));
  g->step = 0;
  return GTD_OK;
}

static gtd_status check_batch(gtd_gnn g, const gtd_gnn_batch* b, bool train) {
  if (!g || !b || b->num_nodes < 1 || b->num_graphs < 1 || !b->x || !b->graph_start || !b->nbr_start ||
      (b->nbr_start[b->num_nodes] > 0 && !b->nbr))
    return fail(g ? g->h : nullptr, GTD_INVALID_ARG, "malformed GNN batch");
  if (train && (!b->root_label || !b->node_mask || !b->td_label))
    return fail(g->h, GTD_INVALID_ARG, "training batch without labels");
  if (b->graph_start[0] != 0 || b->graph_start[b->num_graphs] != b->num_nodes)
    return fail(g->h, GTD_INVALID_ARG, "graph ranges do not cover the nodes");
  return GTD_OK;
}

gtd_status gtd_gnn_forward(gtd_gnn g, const gtd_gnn_batch* b, float* logits_out, float* td_out) {
  gtd_status s = check_batch(g, b, false);
  if (s != GTD_OK)
    return s;
  DeviceGuard dg(g->h->device);
  Views V;
  if ((s = prepare(g, b, false, V)) != GTD_OK)
    return s;
  if ((s = forward(g, b, V)) != GTD_OK)
    return s;
  cudaStream_t st = g->h->stream;
  if (logits_out)
    GTD_CUDA(g->h, cudaMemcpyAsync(logits_out, V.logits, size_t(b->num_nodes) * 4, cudaMemcpyDeviceToHost, st));
  if (td_out)
    GTD_CUDA(g->h, cudaMemcpyAsync(td_out, V.td_est, size_t(b->num_graphs) * 4, cudaMemcpyDeviceToHost, st));
  GTD_CUDA(g->h, cudaStreamSynchronize(st));
  return GTD_OK;
}

gtd_status gtd_gnn_gradients(gtd_gnn g, const gtd_gnn_batch* b, float td_weight, float* grad_out, float* loss_out) {
  gtd_status s = check_batch(g, b, true);
  if (s != GTD_OK)
    return s;
  DeviceGuard dg(g->h->device);
  Views V;
  if ((s = prepare(g, b, true, V)) != GTD_OK)
    return s;
  if ((s = forward(g, b, V)) != GTD_OK)
    return s;
  if ((s = backward(g, b, V, td_weight)) != GTD_OK)
    return s;
  cudaStream_t st = g->h->stream;
  if (grad_out)
    GTD_CUDA(g->h, cudaMemcpyAsync(grad_out, g->grad, g->nparams * 4, cudaMemcpyDeviceToHost, st));
  if (loss_out)
    GTD_CUDA(g->h, cudaMemcpyAsync(loss_out, V.loss, 4, cudaMemcpyDeviceToHost, st));
  GTD_CUDA(g->h, cudaStreamSynchronize(st));
  return GTD_OK;
}

gtd_status gtd_gnn_train_step(gtd_gnn g, const gtd_gnn_batch* b, float lr, float td_weight, float* loss_out) {
  gtd_status s = check_batch(g, b, true);
  if (s != GTD_OK)
    return s;
  DeviceGuard dg(g->h->device);
  Views V;
  if ((s = prepare(g, b, true, V)) != GTD_OK)
    return s;
  if ((s = forward(g, b, V)) != GTD_OK)
    return s;
  if ((s = backward(g, b, V, td_weight)) != GTD_OK)
    return s;
  ++g->step;
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - std::pow(b1, float(g->step)), c2 = 1.f - std::pow(b2, float(g->step));
  cudaStream_t st = g->h->stream;
  adam_step<<<blocks_for(size_t(g->nparams), 256), 256, 0, st>>>(g->nparams, g->master, g->m, g->v, g->grad, g->w,
                                                                  lr, b1, b2, 1e-8f, c1, c2);
  GTD_CUDA(g->h, cudaGetLastError());
  if (loss_out)
    GTD_CUDA(g->h, cudaMemcpyAsync(loss_out, V.loss, 4, cudaMemcpyDeviceToHost, st));
  GTD_CUDA(g->h, cudaStreamSynchronize(st));
  return GTD_OK;
}

}  // extern "C"
