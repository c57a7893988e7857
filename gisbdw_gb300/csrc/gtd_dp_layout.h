// Layout of the subset-DP table in device memory (host and device code).
//
// Every subset S of the n vertices owns one byte, td(G[S]) << 1 | c, where
// c = 1 iff G[S] is connected. Vertices 0..lb-1 are the tile's "low"
// vertices and vertices lb..n-1 its "high" ones (nh = n - lb of them). The
// 2^lb subsets that share the same high part H form one tile of 2^lb
// contiguous bytes, indexed inside the tile by the low part's bit mask.
// Tiles are stored level by level in |H| order and, inside a level, in the
// combinatorial-number-system rank of H (colex order, the ranking of
// set_encoder.hpp:40-46 in the reference), so
//   index(S) = (level_off[|H|] + rank(H)) * 2^lb + (S & (2^lb - 1)).
// A tile's |H| children H \ h are whole tiles one level down: every
// cross-tile gather of the DP reads 2^lb contiguous bytes.
#pragma once

#include <cstdint>

#if defined(__CUDACC__)
#define GTD_HD __host__ __device__ __forceinline__
#else
#define GTD_HD inline
#endif

namespace gtd {

constexpr int kDpMaxN = 36;          // 2^36 B = 64 GiB table
constexpr int kDpMaxHigh = 26;       // nh <= 26: C(26, 13) < 2^32, 2^26 tiles
constexpr int kDpMinTileBits = 8;
constexpr int kDpMaxTileBits = 12;

struct DpLayout {
  int n = 0;
  int lb = 0;   // tile bits (low vertices per tile)
  int nh = 0;   // high vertices
  uint32_t ntiles = 0;
  uint32_t level_off[kDpMaxHigh + 2] = {};
  uint32_t binom[kDpMaxHigh + 1][kDpMaxHigh + 1] = {};  // C(a, b)

  GTD_HD uint32_t C(int a, int b) const { return (b < 0 || b > a) ? 0u : binom[a][b]; }

  // Colex rank of a subset of the high positions among sets of its size.
  GTD_HD uint32_t rank_high(uint32_t H) const {
    uint32_t r = 0;
    int q = 0;
    while (H) {
      int b = ctz_portable(H);
      r += binom[b][++q];
      H &= H - 1;
    }
    return r;
  }

  GTD_HD uint64_t index(uint64_t S) const {
    uint32_t H = static_cast<uint32_t>(S >> lb);
    int j = popcount_portable(H);
    uint64_t tile = static_cast<uint64_t>(level_off[j]) + rank_high(H);
    return (tile << lb) | (S & ((1ull << lb) - 1));
  }

  GTD_HD static int popcount_portable(uint32_t x) {
#if defined(__CUDA_ARCH__)
    return __popc(x);
#else
    return __builtin_popcount(x);
#endif
  }
  GTD_HD static int ctz_portable(uint32_t x) {
#if defined(__CUDA_ARCH__)
    return __ffs(x) - 1;
#else
    return __builtin_ctz(x);
#endif
  }
};

// Fills a layout for n vertices and the requested tile bits (clamped so
// that lb <= n and nh <= kDpMaxHigh). Host only.
inline DpLayout make_dp_layout(int n, int tile_bits) {
  DpLayout L;
  int lb = tile_bits;
  if (lb < kDpMinTileBits)
    lb = kDpMinTileBits;
  if (lb > kDpMaxTileBits)
    lb = kDpMaxTileBits;
  if (n - lb > kDpMaxHigh)
    lb = n - kDpMaxHigh;
  if (lb > n)
    lb = n;
  L.n = n;
  L.lb = lb;
  L.nh = n - lb;
  for (int a = 0; a <= kDpMaxHigh; ++a) {
    L.binom[a][0] = 1;
    for (int b = 1; b <= a; ++b)
      L.binom[a][b] = L.binom[a - 1][b - 1] + (b <= a - 1 ? L.binom[a - 1][b] : 0u);
  }
  L.level_off[0] = 0;
  for (int j = 0; j <= L.nh; ++j)
    L.level_off[j + 1] = L.level_off[j] + L.binom[L.nh][j];
  L.ntiles = L.level_off[L.nh + 1];
  return L;
}

}  // namespace gtd
