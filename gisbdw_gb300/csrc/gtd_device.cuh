// Device-side primitives shared by the gtd kernels (sm_103a): GPU-scope
// acquire/release flag accesses, the global timer, and the bounded wait that
// every cross-CTA dependency in this library goes through.
#pragma once

#include <cstdint>

namespace gtd {

// Error codes written by kernels into the handle's control block.
enum DeviceError : int32_t {
  kDevOk = 0,
  kDevInvalidInput = 1,  // adjacency not symmetric / self loop / bit >= n
  kDevWaitTimeout = 2,   // a dependency wait ran past its deadline
  kDevNoRoot = 3,        // tree reconstruction found no optimal root
  kDevAborted = 4,
  kDevDeadline = 5,      // per-graph search deadline reached
  kDevOverflow = 6,      // a bounded device buffer ran out
};

__device__ __forceinline__ uint32_t ld_acquire_u32(const uint32_t* p) {
  uint32_t v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ int32_t ld_relaxed_s32(const int32_t* p) {
  int32_t v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void st_release_u32(uint32_t* p, uint32_t v) {
  asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Records the first error (later ones are dropped).
__device__ __forceinline__ void raise_error(int32_t* err, int32_t code, int32_t info) {
  if (atomicCAS(err, 0, code) == 0)
    atomicExch(err + 1, info);
}

// Waits until *flag == want. Gives up (returns false) when the deadline
// passes or another thread has raised an error; never spins unbounded.
__device__ __forceinline__ bool wait_flag(const uint32_t* flag, uint32_t want,
                                          uint64_t timeout_ns, int32_t* err) {
  if (ld_acquire_u32(flag) == want)
    return true;
  const uint64_t deadline = global_ns() + timeout_ns;
  unsigned sleep_ns = 32;
  for (;;) {
    if (ld_acquire_u32(flag) == want)
      return true;
    if (ld_relaxed_s32(err) != 0)
      return false;
    if (global_ns() > deadline) {
      raise_error(err, kDevWaitTimeout, 0);
      return false;
    }
    __nanosleep(sleep_ns);
    if (sleep_ns < 2048)
      sleep_ns *= 2;
  }
}

}  // namespace gtd
