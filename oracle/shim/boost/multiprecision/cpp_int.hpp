// Boost-API shim (test infrastructure for oracle/_ref): uint128_t maps to the
// compiler's unsigned __int128 (std::hash for it exists under -std=gnu++17).
#pragma once
#include <functional>

namespace boost {
namespace multiprecision {
using uint128_t = unsigned __int128;
}  // namespace multiprecision
}  // namespace boost
