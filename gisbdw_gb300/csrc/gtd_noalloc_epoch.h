// Epoch of the no-allocation DP entry point's shared tile flags (host only).
//
// Every call stamps the tiles it finishes with a new epoch, so flags left by
// earlier calls never read as ready. Epochs run through 1 .. 0xFFFFFFFE; after
// the last one the next call starts again at 1 and must clear every flag
// first (a flag of an earlier call could hold 1).
#pragma once

#include <cstdint>

namespace gtd {

constexpr uint32_t kNoallocLastEpoch = 0xFFFFFFFEu;

// The epoch after `prev` (0 = no call yet); *clear is set when the flags must
// be cleared before the call that uses the returned epoch.
inline uint32_t noalloc_next_epoch(uint32_t prev, bool* clear) {
  if (prev >= kNoallocLastEpoch) {
    *clear = true;
    return 1u;
  }
  *clear = prev == 0;  // the process's first call clears them too (no reliance on load-time contents)
  return prev + 1;
}

}  // namespace gtd
