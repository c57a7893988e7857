/* ORACLE — TEST INFRASTRUCTURE ONLY (see gtd_oracle.h).
 *
 * CPU restatement of the reference's exact treedepth algorithms. Each
 * function names the reference file:line it follows. Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU legs load this library.
 */
#define _GNU_SOURCE
#include "gtd_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

typedef unsigned __int128 m128;

static inline int pop64(uint64_t x) { return __builtin_popcountll(x); }
static inline int ctz64(uint64_t x) { return __builtin_ctzll(x); }
static inline int pop128(m128 x) {
  return pop64((uint64_t)x) + pop64((uint64_t)(x >> 64));
}
static inline int ctz128(m128 x) {
  uint64_t lo = (uint64_t)x;
  return lo ? ctz64(lo) : 64 + ctz64((uint64_t)(x >> 64));
}
static inline m128 bit128(int v) { return (m128)1 << v; }

/* ---- set encoder: set_encoder.cu:6-17, set_encoder.hpp:40-73 ---------- */

uint64_t gtdo_nchoosek(uint64_t n, uint64_t k) {
  if (k > n)
    return 0;
  if (k > n / 2)
    k = n - k;
  uint64_t r = 1;
  for (uint64_t i = 1; i <= k; ++i, --n)
    r = r * n / i;
  return r;
}

uint64_t gtdo_encode(const int* s, int k) {
  uint64_t r = 0;
  for (int i = 0; i < k; ++i)
    r += gtdo_nchoosek((uint64_t)s[i], (uint64_t)(i + 1));
  return r;
}

void gtdo_decode(int nverts, int k, uint64_t code, int* out) {
  while (k > 0) {
    uint64_t c = gtdo_nchoosek((uint64_t)(--nverts), (uint64_t)k);
    if (code >= c) {
      out[--k] = nverts;
      code -= c;
    }
  }
}

/* ---- lower bound: edge_lower_bound.hpp:13-20 -------------------------- */
/* ceil(0.5 + n - sqrt(0.25 + n^2 - n - 2e)) equals the smallest integer d
 * with d >= that value; for 1 <= d <= n that is (d-1)(2n-d) >= 2e (square
 * both sides of sqrt((n-1/2)^2 - 2e) >= n + 1/2 - d). */
int gtdo_edge_lower_bound(int n, int e) {
  if (n <= 0)
    return 0;
  for (int d = 1; d <= n; ++d)
    if ((int64_t)(d - 1) * (2 * n - d) >= 2 * (int64_t)e)
      return d;
  return n;
}

/* ---- subset DP: dynamic_gpu.cu:68-112 ------------------------------- */

static inline uint64_t component64(uint64_t S, int v, const uint64_t* adj) {
  uint64_t reach = 1ull << v, frontier = reach;
  while (frontier) {
    uint64_t nb = 0;
    while (frontier) {
      nb |= adj[ctz64(frontier)];
      frontier &= frontier - 1;
    }
    nb &= S & ~reach;
    reach |= nb;
    frontier = nb;
  }
  return reach;
}

/* Value of one subset given all its proper subsets: connected -> 1 + min over
 * S \ v (dynamic_gpu.cu:68-89), disconnected -> max over components
 * (dynamic_gpu.cu:90-111). */
static inline uint8_t dp_value(uint64_t S, const uint64_t* adj,
                               const uint8_t* T) {
  if (pop64(S) == 1)
    return 1;
  uint64_t c0 = component64(S, ctz64(S), adj);
  if (c0 == S) {
    uint8_t best = 255;
    for (uint64_t r = S; r; r &= r - 1) {
      uint8_t t = T[S & ~(1ull << ctz64(r))];
      if (t < best)
        best = t;
    }
    return (uint8_t)(best + 1);
  }
  uint8_t mx = T[c0];
  for (uint64_t rest = S & ~c0; rest;) {
    uint64_t c = component64(rest, ctz64(rest), adj);
    rest &= ~c;
    if (T[c] > mx)
      mx = T[c];
  }
  return mx;
}

static inline uint64_t gosper_next(uint64_t x) {
  uint64_t c = x & (~x + 1), r = x + c;
  return (((r ^ x) >> 2) / c) | r;
}

typedef struct {
  int n, k;
  const uint64_t* adj;
  uint8_t* T;
  uint64_t first_rank, count;
} level_job;

static void* level_worker(void* p) {
  level_job* j = (level_job*)p;
  if (!j->count)
    return NULL;
  int elems[64];
  gtdo_decode(j->n, j->k, j->first_rank, elems);
  uint64_t S = 0;
  for (int i = 0; i < j->k; ++i)
    S |= 1ull << elems[i];
  for (uint64_t i = 0; i < j->count; ++i) {
    j->T[S] = dp_value(S, j->adj, j->T);
    if (i + 1 < j->count)
      S = gosper_next(S);
  }
  return NULL;
}

int gtdo_dp_table(int n, const uint64_t* adj, uint8_t* T, int nthreads) {
  if (n < 1 || n > 34)
    return -1;
  if (nthreads < 1)
    nthreads = 1;
  if (nthreads > 256)
    nthreads = 256;
  T[0] = 0;
  for (int k = 1; k <= n; ++k) {
    uint64_t total = gtdo_nchoosek((uint64_t)n, (uint64_t)k);
    int nt = (total < 4096 || nthreads == 1) ? 1 : nthreads;
    level_job jobs[256];
    pthread_t th[256];
    for (int t = 0; t < nt; ++t) {
      uint64_t a = total * (uint64_t)t / (uint64_t)nt;
      uint64_t b = total * (uint64_t)(t + 1) / (uint64_t)nt;
      jobs[t] = (level_job){n, k, adj, T, a, b - a};
    }
    if (nt == 1) {
      level_worker(&jobs[0]);
    } else {
      for (int t = 0; t < nt; ++t)
        pthread_create(&th[t], NULL, level_worker, &jobs[t]);
      for (int t = 0; t < nt; ++t)
        pthread_join(th[t], NULL);
    }
  }
  return 0;
}

/* Canonical tree: dynamic_cpu.hpp:59-81 replays, for the first remaining
 * component, its stored root (first argmin, dynamic_cpu.cpp:96-99). The tree
 * only depends on the root chosen per component, so a work list of
 * (component, owner) pairs gives the same parent array. */
int gtdo_tree_from_table(int n, const uint64_t* adj, const uint8_t* T, int* td,
                         int* parent) {
  uint64_t full = n == 64 ? ~0ull : ((1ull << n) - 1);
  uint64_t cm[64];
  int co[64], cd[64], top = 0, height = 0;
  for (uint64_t rest = full; rest;) {
    uint64_t c = component64(rest, ctz64(rest), adj);
    rest &= ~c;
    cm[top] = c;
    co[top] = -1;
    cd[top++] = 1;
  }
  while (top > 0) {
    --top;
    uint64_t C = cm[top];
    int owner = co[top], depth = cd[top], r = -1;
    if (pop64(C) == 1) {
      r = ctz64(C);
    } else {
      uint8_t want = (uint8_t)(T[C] - 1);
      for (uint64_t s = C; s; s &= s - 1) {
        int v = ctz64(s);
        if (T[C & ~(1ull << v)] == want) {
          r = v;
          break;
        }
      }
      if (r < 0)
        return -1;
    }
    parent[r] = owner;
    if (depth > height)
      height = depth;
    for (uint64_t rest = C & ~(1ull << r); rest;) {
      uint64_t c = component64(rest, ctz64(rest), adj);
      rest &= ~c;
      cm[top] = c;
      co[top] = r;
      cd[top++] = depth + 1;
    }
  }
  *td = height;
  return 0;
}

/* Root of a connected set: first v with T[C \ v] = T[C] - 1. */
static int first_root(uint64_t C, const uint8_t* T) {
  if (pop64(C) == 1)
    return ctz64(C);
  uint8_t want = (uint8_t)(T[C] - 1);
  for (uint64_t s = C; s; s &= s - 1)
    if (T[C & ~(1ull << ctz64(s))] == want)
      return ctz64(s);
  return -1;
}

int gtdo_get_elimination(int n, const uint64_t* adj, const uint8_t* T,
                         uint64_t subset, int* order) {
  (void)n;
  int step = 0;
  while (subset) {
    uint64_t best = 0;
    uint8_t best_td = 0;
    for (uint64_t rest = subset; rest;) {
      uint64_t c = component64(rest, ctz64(rest), adj);
      rest &= ~c;
      if (!best || T[c] > best_td) {
        best = c;
        best_td = T[c];
      }
    }
    int r = first_root(best, T);
    if (r < 0)
      return -1;
    order[step++] = r;
    subset &= ~(1ull << r);
  }
  return 0;
}

int gtdo_dp_solve(int n, const uint64_t* adj, int nthreads, int* td,
                  int* parent) {
  if (n < 1 || n > 34)
    return -1;
  uint8_t* T = (uint8_t*)malloc((size_t)1 << n);
  if (!T)
    return -2;
  int rc = gtdo_dp_table(n, adj, T, nthreads);
  if (rc == 0)
    rc = gtdo_tree_from_table(n, adj, T, td, parent);
  free(T);
  return rc;
}

/* ---- DynamicCPUImprov: dynamic_cpu_improv.cpp:21-65 ------------------ */

typedef struct {
  uint64_t* keys;
  uint8_t* td;
  int8_t* root;
  uint64_t cap, used;
} memo_t;

static inline uint64_t mix64(uint64_t x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdull;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ull;
  x ^= x >> 33;
  return x;
}

static int memo_init(memo_t* m, uint64_t cap) {
  m->cap = cap;
  m->used = 0;
  m->keys = (uint64_t*)calloc(cap, sizeof(uint64_t));
  m->td = (uint8_t*)malloc(cap);
  m->root = (int8_t*)malloc(cap);
  return (m->keys && m->td && m->root) ? 0 : -2;
}

static void memo_free(memo_t* m) {
  free(m->keys);
  free(m->td);
  free(m->root);
}

static int64_t memo_find(const memo_t* m, uint64_t key) {
  uint64_t i = mix64(key) & (m->cap - 1);
  while (m->keys[i]) {
    if (m->keys[i] == key)
      return (int64_t)i;
    i = (i + 1) & (m->cap - 1);
  }
  return -1;
}

static int memo_put(memo_t* m, uint64_t key, uint8_t td, int8_t root) {
  if ((m->used + 1) * 2 > m->cap) {
    memo_t g;
    if (memo_init(&g, m->cap * 2))
      return -2;
    for (uint64_t i = 0; i < m->cap; ++i)
      if (m->keys[i]) {
        uint64_t j = mix64(m->keys[i]) & (g.cap - 1);
        while (g.keys[j])
          j = (j + 1) & (g.cap - 1);
        g.keys[j] = m->keys[i];
        g.td[j] = m->td[i];
        g.root[j] = m->root[i];
      }
    g.used = m->used;
    memo_free(m);
    *m = g;
  }
  uint64_t i = mix64(key) & (m->cap - 1);
  while (m->keys[i] && m->keys[i] != key)
    i = (i + 1) & (m->cap - 1);
  if (!m->keys[i])
    m->used++;
  m->keys[i] = key;
  m->td[i] = td;
  m->root[i] = root;
  return 0;
}

typedef struct {
  const uint64_t* adj;
  memo_t memo;
  int oom;
} improv_ctx;

/* Run(component) of dynamic_cpu_improv.cpp:21-46: try every vertex of the
 * component in ascending order, recurse into the components left behind,
 * keep the first strict minimum. Singletons are pre-seeded there
 * (dynamic_cpu_improv.hpp:61-62); here they are answered directly. */
static int improv_run(improv_ctx* c, uint64_t C) {
  if (pop64(C) == 1)
    return 1;
  int64_t h = memo_find(&c->memo, C);
  if (h >= 0)
    return c->memo.td[h];
  int best = 1 << 30, broot = -1;
  for (uint64_t s = C; s; s &= s - 1) {
    int v = ctz64(s);
    int tdcomp = 0;
    for (uint64_t rest = C & ~(1ull << v); rest;) {
      uint64_t comp = component64(rest, ctz64(rest), c->adj);
      rest &= ~comp;
      int t = improv_run(c, comp);
      if (t > tdcomp)
        tdcomp = t;
    }
    ++tdcomp;
    if (best > tdcomp) {
      best = tdcomp;
      broot = v;
    }
  }
  if (memo_put(&c->memo, C, (uint8_t)best, (int8_t)broot))
    c->oom = 1;
  return best;
}

int gtdo_dp_improv(int n, const uint64_t* adj, int* td, int* parent,
                   int64_t* memo_entries) {
  if (n < 1 || n > 64)
    return -1;
  improv_ctx c = {adj, {0}, 0};
  if (memo_init(&c.memo, 1u << 16))
    return -2;
  uint64_t full = n == 64 ? ~0ull : ((1ull << n) - 1);
  /* GetTDDecompImpl (dynamic_cpu_improv.cpp:48-65): replay stored roots. */
  uint64_t cm[64];
  int co[64], cd[64], top = 0, height = 0;
  for (uint64_t rest = full; rest;) {
    uint64_t comp = component64(rest, ctz64(rest), adj);
    rest &= ~comp;
    improv_run(&c, comp);
    cm[top] = comp;
    co[top] = -1;
    cd[top++] = 1;
  }
  int rc = c.oom ? -2 : 0;
  while (rc == 0 && top > 0) {
    --top;
    uint64_t C = cm[top];
    int owner = co[top], depth = cd[top], r;
    if (pop64(C) == 1) {
      r = ctz64(C);
    } else {
      int64_t h = memo_find(&c.memo, C);
      if (h < 0) {
        rc = -2;
        break;
      }
      r = c.memo.root[h];
    }
    parent[r] = owner;
    if (depth > height)
      height = depth;
    for (uint64_t rest = C & ~(1ull << r); rest;) {
      uint64_t comp = component64(rest, ctz64(rest), adj);
      rest &= ~comp;
      cm[top] = comp;
      co[top] = r;
      cd[top++] = depth + 1;
    }
  }
  *td = height;
  if (memo_entries)
    *memo_entries = (int64_t)c.memo.used;
  memo_free(&c.memo);
  return rc;
}

/* ---- EliminationTree replay: elimination_tree.cpp:24-70 -------------- */

int gtdo_elimination_tree(int n, const uint64_t* adj, const int* order,
                          int* td, int* parent) {
  if (n < 1 || n > 64)
    return -1;
  uint64_t remaining = n == 64 ? ~0ull : ((1ull << n) - 1);
  int owner[64], cdepth[64], height = 0;
  for (int v = 0; v < n; ++v) {
    owner[v] = -1;
    cdepth[v] = 0;
  }
  for (int i = 0; i < n; ++i) {
    int v = order[i];
    if (v < 0 || v >= n || !(remaining >> v & 1))
      return -1;
    parent[v] = owner[v];
    if (cdepth[v] + 1 > height)
      height = cdepth[v] + 1;
    uint64_t C = component64(remaining, v, adj);
    remaining &= ~(1ull << v);
    for (uint64_t s = C & ~(1ull << v); s; s &= s - 1) {
      int u = ctz64(s);
      owner[u] = v;
      cdepth[u] = cdepth[v] + 1;
    }
  }
  *td = height;
  return 0;
}

/* ---- BottomUpHeuristicGPU: bottom_up_heuristic_gpu_algorithm.cu ------ */

/* ext_array_union_find::Find (ext_array_union_find.hpp:10-22): root of
 * elem with path compression. Entries >= 0 are parents, a negative entry
 * -v marks a root whose tree has value (height) v. */
static int8_t uf_find(int8_t* uf, int8_t elem) {
  int8_t root = elem;
  while (uf[root] >= 0)
    root = uf[root];
  while (elem != root) {
    int8_t prev = uf[elem];
    uf[elem] = root;
    elem = prev;
  }
  return root;
}

/* ext_array_union_find::Union (ext_array_union_find.hpp:24-33): s2's tree
 * goes under s1, s1's value becomes max(own, value(s2) + 1), and the running
 * maximum at val_ix follows it. */
static void uf_union(int8_t* uf, int8_t s1, int8_t s2, int val_ix) {
  if (s1 == s2)
    return;
  int8_t new_val = (int8_t)-uf[s1];
  if (new_val <= -uf[s2])
    new_val = (int8_t)(-uf[s2] + 1);
  if (uf[val_ix] < new_val)
    uf[val_ix] = new_val;
  uf[s1] = (int8_t)-new_val;
  uf[s2] = s1;
}

/* The bottom-up heuristic DP (Run :211-258, DynamicStepKernel :57-94): level
 * i keeps one union-find forest per i-subset S (n + 2 entries: the forest,
 * the last vertex added, the forest's height). S's forest is its child
 * S \ s_j's forest with s_j added as the root over the trees of its
 * neighbours in S, for the first j (ascending vertex) with the least height.
 * GetElimination (bottom_up_heuristic_gpu_algorithm.hpp:104-120) then reads
 * the last vertex of V, of V minus it, and so on: that order is order_out.
 * Level 0: every entry -1, height 1 (:222-223). */
int gtdo_bottom_up(int n, const uint64_t* adj, int* order_out) {
  if (n < 1 || n > 30)
    return -1;
  const int W = n + 2;
  uint64_t maxc = 0;
  for (int k = 0; k <= n; ++k)
    if (gtdo_nchoosek((uint64_t)n, (uint64_t)k) > maxc)
      maxc = gtdo_nchoosek((uint64_t)n, (uint64_t)k);
  int8_t* prev = (int8_t*)malloc((size_t)maxc * W);
  int8_t* next = (int8_t*)malloc((size_t)maxc * W);
  int8_t* last = (int8_t*)malloc(((size_t)1 << n) + 1); /* history: last vertex per (level, rank) */
  uint64_t lvl_off[65];
  if (!prev || !next || !last) {
    free(prev);
    free(next);
    free(last);
    return -2;
  }
  lvl_off[0] = 0;
  for (int k = 0; k < n; ++k)
    lvl_off[k + 1] = lvl_off[k] + gtdo_nchoosek((uint64_t)n, (uint64_t)k);
  for (int j = 0; j < W; ++j)
    prev[j] = -1;
  prev[n + 1] = 1;
  last[0] = -1;
  int8_t uf[66];
  int set[64];
  for (int i = 1; i <= n; ++i) {
    const uint64_t count = gtdo_nchoosek((uint64_t)n, (uint64_t)i);
    for (uint64_t r = 0; r < count; ++r) {
      gtdo_decode(n, i, r, set);
      int8_t best = (int8_t)(i + 1);
      int8_t* out = next + (size_t)r * W;
      for (int j = 0; j < i; ++j) {
        /* the child S \ s_j: its colex rank skips position j */
        uint64_t code = 0;
        for (int q = 0, pos = 0; q < i; ++q)
          if (q != j)
            code += gtdo_nchoosek((uint64_t)set[q], (uint64_t)(++pos));
        memcpy(uf, prev + (size_t)code * W, (size_t)W);
        const int v = set[j];
        uf[n] = (int8_t)v;
        for (uint64_t nb = adj[v]; nb; nb &= nb - 1) {
          const int u = ctz64(nb);
          int in = 0;
          for (int q = 0; q < i; ++q)
            in |= set[q] == u;
          if (in)
            uf_union(uf, (int8_t)v, uf_find(uf, (int8_t)u), n + 1);
        }
        if (uf[n + 1] < best) {
          best = uf[n + 1];
          memcpy(out, uf, (size_t)W);
        }
      }
      last[lvl_off[i] + r] = out[n];
    }
    int8_t* t = prev;
    prev = next;
    next = t;
  }
  /* GetElimination(n, n, 0) */
  int rem[64], k = n;
  for (int v = 0; v < n; ++v)
    rem[v] = v;
  for (int step = 0; step < n; ++step) {
    const uint64_t code = gtdo_encode(rem, k);
    const int v = last[lvl_off[k] + code];
    order_out[step] = v;
    int w = 0;
    for (int q = 0; q < k; ++q)
      if (rem[q] != v)
        rem[w++] = rem[q];
    --k;
  }
  free(prev);
  free(next);
  free(last);
  return 0;
}

/* ---- validity: common/utils/utils.hpp:50-86 ------------------------- */

int gtdo_check_valid(int n, const uint64_t* adj, int td, const int* parent,
                     int allow_forest) {
  if (n < 1 || n > 64)
    return 0;
  int depth[64], roots = 0, height = 0;
  for (int v = 0; v < n; ++v) {
    if (parent[v] < -1 || parent[v] >= n || parent[v] == v)
      return 0;
    depth[v] = 0;
  }
  for (int v = 0; v < n; ++v) {
    int d = 0, u = v;
    while (u >= 0 && d <= n) {
      ++d;
      u = parent[u];
    }
    if (d > n)
      return 0; /* cycle */
    depth[v] = d;
    if (parent[v] == -1)
      ++roots;
    if (d > height)
      height = d;
  }
  if (roots < 1 || (!allow_forest && roots != 1))
    return 0;
  for (int v = 0; v < n; ++v)
    for (uint64_t s = adj[v]; s; s &= s - 1) {
      int u = ctz64(s);
      int a = v, b = u;
      if (depth[a] < depth[b]) {
        int t = a;
        a = b;
        b = t;
      }
      while (depth[a] > depth[b])
        a = parent[a];
      if (a != b)
        return 0;
    }
  return height == td;
}

/* ---- 128-bit helpers for heuristics and branch and bound ------------- */

static inline m128 load_adj(const uint64_t* adj2, int v) {
  return (m128)adj2[2 * v] | ((m128)adj2[2 * v + 1] << 64);
}

static inline m128 component128(m128 S, int v, const m128* adj) {
  m128 reach = bit128(v), frontier = reach;
  while (frontier) {
    m128 nb = 0;
    while (frontier) {
      nb |= adj[ctz128(frontier)];
      frontier &= frontier - 1;
    }
    nb &= S & ~reach;
    reach |= nb;
    frontier = nb;
  }
  return reach;
}

static int edges_in(m128 C, const m128* adj) {
  int e = 0;
  for (m128 s = C; s; s &= s - 1)
    e += pop128(adj[ctz128(s)] & C);
  return e / 2;
}

static int load_graph128(int n, const uint64_t* adj2, m128* adj) {
  if (n < 1 || n > 128)
    return -1;
  m128 full = n == 128 ? ~(m128)0 : (bit128(n) - 1);
  for (int v = 0; v < n; ++v) {
    adj[v] = load_adj(adj2, v);
    if ((adj[v] >> v) & 1)
      return -1; /* self loop: elimination_tree.hpp:175-177 */
    if (adj[v] & ~full)
      return -1;
  }
  if (component128(full, 0, adj) != full)
    return -1; /* disconnected: elimination_tree.hpp:171-173 */
  return 0;
}

/* Greedy elimination shared by the heuristics: repeatedly pick a vertex of
 * the first component (the one holding the smallest remaining vertex,
 * ComponentCmp elimination_tree.hpp:67-72) and eliminate it. */
typedef int (*pick_fn)(m128 C, m128 remaining, const m128* adj);

/* highest_degree_heuristic.hpp:21-34: first vertex of maximum degree. */
static int pick_highest_degree(m128 C, m128 remaining, const m128* adj) {
  (void)remaining;
  int best = -1, bestdeg = -1;
  for (m128 s = C; s; s &= s - 1) {
    int v = ctz128(s);
    int d = pop128(adj[v] & C);
    if (d > bestdeg) {
      bestdeg = d;
      best = v;
    }
  }
  return best;
}

/* variance_heuristic.hpp:77-118 with A, D, E = 1.0, 0.2, 0.8 (float), the
 * arithmetic kept in the reference's float/double mix. */
static int pick_variance(m128 C, m128 remaining, const m128* adj) {
  (void)remaining;
  const float A = 1.0f, D = 0.2f, E = 0.8f;
  double best_coef = -1;
  int best_deg = -1, best = 0;
  for (m128 s = C; s; s &= s - 1) {
    int v = ctz128(s);
    int deg = pop128(adj[v] & C);
    int sizes[128], nc = 0;
    for (m128 rest = C & ~bit128(v); rest;) {
      m128 comp = component128(rest, ctz128(rest), adj);
      rest &= ~comp;
      sizes[nc++] = pop128(comp);
    }
    double acc = 0.0;
    for (int i = 0; i < nc; ++i)
      acc = acc + sizes[i];
    double avg = acc / nc;
    double gamma = 0.0;
    for (int i = 0; i < nc; ++i)
      gamma = gamma + (sizes[i] - avg) * (sizes[i] - avg);
    double coef = D / (sqrt(gamma + A)) + E * (float)nc;
    if (coef > best_coef || (coef == best_coef && deg > best_deg)) {
      best_coef = coef;
      best_deg = deg;
      best = v;
    }
  }
  return best;
}

static int greedy(int n, const m128* adj, pick_fn pick, int* parent) {
  m128 remaining = n == 128 ? ~(m128)0 : (bit128(n) - 1);
  int owner[128], cdepth[128], height = 0;
  for (int v = 0; v < n; ++v) {
    owner[v] = -1;
    cdepth[v] = 0;
  }
  while (remaining) {
    m128 C = component128(remaining, ctz128(remaining), adj);
    int v = pick(C, remaining, adj);
    parent[v] = owner[v];
    if (cdepth[v] + 1 > height)
      height = cdepth[v] + 1;
    remaining &= ~bit128(v);
    for (m128 s = C & ~bit128(v); s; s &= s - 1) {
      int u = ctz128(s);
      owner[u] = v;
      cdepth[u] = cdepth[v] + 1;
    }
  }
  return height;
}

static int heuristic128(int n, const m128* adj, int kind, int* td,
                        int* parent) {
  int tmp[128];
  switch (kind) {
    case 0: { /* HighestDegree(Variance): keep the inner result if better */
      int hd = greedy(n, adj, pick_highest_degree, parent);
      int va = greedy(n, adj, pick_variance, tmp);
      if (va < hd) {
        memcpy(parent, tmp, sizeof(int) * (size_t)n);
        hd = va;
      }
      *td = hd;
      return 0;
    }
    case 2:
      *td = greedy(n, adj, pick_highest_degree, parent);
      return 0;
    case 3:
      *td = greedy(n, adj, pick_variance, parent);
      return 0;
    default:
      return -1;
  }
}

int gtdo_heuristic(int n, const uint64_t* adj2, int kind, int* td,
                   int* parent) {
  m128 adj[128];
  if (load_graph128(n, adj2, adj))
    return -1;
  return heuristic128(n, adj, kind, td, parent);
}

/* ---- BranchAndBound::Algorithm: branch_and_bound.cpp:51-114 ---------- */

typedef struct {
  m128 mask;
  int depth, owner;
} comp_t;

typedef struct {
  int n, lb_kind;
  const m128* adj;
  int best_td;
  int best_parent[128];
  int cur_parent[128], vdepth[128];
  int64_t nodes, limit;
  int limited;
  comp_t* arena; /* (n + 1) levels x n components */
} bnb_ctx;

static int lower_bound(const bnb_ctx* c, m128 C) {
  int nv = pop128(C);
  if (c->lb_kind == 1)
    return nv > 1 ? 2 : 1; /* basic_lower_bound.hpp:11-17 */
  return gtdo_edge_lower_bound(nv, edges_in(C, c->adj));
}

static void bnb_rec(bnb_ctx* c, comp_t* comps, int nc, int level) {
  if (c->limited)
    return;
  if (c->limit > 0 && c->nodes >= c->limit) {
    c->limited = 1;
    return;
  }
  c->nodes++;
  if (nc == 0) { /* complete elimination: Decompose + keep if better */
    int h = 0;
    for (int v = 0; v < c->n; ++v)
      if (c->vdepth[v] > h)
        h = c->vdepth[v];
    if (h < c->best_td) {
      c->best_td = h;
      memcpy(c->best_parent, c->cur_parent, sizeof(int) * (size_t)c->n);
    }
    return;
  }
  for (int i = 1; i < nc; ++i)
    if (comps[i].depth + lower_bound(c, comps[i].mask) >= c->best_td)
      return;
  if (comps[0].depth + lower_bound(c, comps[0].mask) >= c->best_td)
    return;
  comp_t* next = c->arena + (size_t)(level + 1) * (size_t)c->n;
  m128 first = comps[0].mask;
  /* DefaultAttemptOrder (branch_and_bound.cpp:9-16): ascending ids. */
  for (m128 s = first; s; s &= s - 1) {
    int v = ctz128(s);
    c->cur_parent[v] = comps[0].owner;
    c->vdepth[v] = comps[0].depth + 1;
    /* children of v, then merge with comps[1..] by smallest vertex */
    comp_t kids[128];
    int nk = 0;
    for (m128 rest = first & ~bit128(v); rest;) {
      m128 comp = component128(rest, ctz128(rest), c->adj);
      rest &= ~comp;
      kids[nk++] = (comp_t){comp, comps[0].depth + 1, v};
    }
    int a = 1, b = 0, m = 0;
    while (a < nc || b < nk) {
      if (b >= nk || (a < nc && ctz128(comps[a].mask) < ctz128(kids[b].mask)))
        next[m++] = comps[a++];
      else
        next[m++] = kids[b++];
    }
    bnb_rec(c, next, m, level + 1);
    c->vdepth[v] = 0;
    if (c->limited)
      return;
  }
}

int gtdo_bnb(int n, const uint64_t* adj2, int lb_kind, int heur_kind,
             int64_t node_limit, int* td, int* parent, int64_t* nodes) {
  m128 adj[128];
  if (load_graph128(n, adj2, adj))
    return -1;
  bnb_ctx* c = (bnb_ctx*)calloc(1, sizeof(bnb_ctx));
  if (!c)
    return -2;
  c->n = n;
  c->lb_kind = lb_kind;
  c->adj = adj;
  c->limit = node_limit;
  c->arena = (comp_t*)malloc(sizeof(comp_t) * (size_t)(n + 2) * (size_t)n);
  if (!c->arena) {
    free(c);
    return -2;
  }
  if (heuristic128(n, adj, heur_kind, &c->best_td, c->best_parent)) {
    free(c->arena);
    free(c);
    return -1;
  }
  m128 full = n == 128 ? ~(m128)0 : (bit128(n) - 1);
  c->arena[0] = (comp_t){full, 0, -1};
  bnb_rec(c, c->arena, 1, 0);
  *td = c->best_td;
  memcpy(parent, c->best_parent, sizeof(int) * (size_t)n);
  if (nodes)
    *nodes = c->nodes;
  int rc = c->limited ? 1 : 0;
  free(c->arena);
  free(c);
  return rc;
}
