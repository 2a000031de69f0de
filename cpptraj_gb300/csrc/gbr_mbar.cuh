// gbr_mbar.cuh -- shared-memory mbarrier helpers with bounded waits.
//
// The tensor-core pair kernels (gbr_pair_tc.cu) wait on mbarriers for TMA
// copies and MMA commits.  Every such wait is bounded: after `limit` clock64
// cycles it records an error code in a global word and returns false, so a
// kernel never spins forever and the host reads the code after the launch.
// The same helper is run by the self-test kernel in gbr_selftest.cu.
#pragma once
#include <cstdint>

namespace gbr {

// About 2 s at 2 GHz.
constexpr long long kWaitCycles = 4000000000LL;

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint32_t bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint32_t bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(bar), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: false (and *err set to `code` unless already set) when the
// phase does not complete within `limit` cycles, or false at once when
// another thread already reported an error.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int* err, int code,
                                          long long limit = kWaitCycles) {
  if (mbar_try(bar, parity)) return true;
  const long long t0 = clock64();
  for (uint32_t it = 1;; ++it) {
    if (mbar_try(bar, parity)) return true;
    if ((it & 255u) == 0) {
      if (*(volatile int*)err != 0) return false;
      if (clock64() - t0 > limit) {
        atomicCAS(err, 0, code);
        return false;
      }
    }
  }
}

// Bounded wait that ignores the error flag (used to drain a kernel's own TMA
// copies before it exits).
__device__ __forceinline__ void mbar_wait_quiet(uint32_t bar, uint32_t parity, long long limit = kWaitCycles) {
  const long long t0 = clock64();
  while (!mbar_try(bar, parity)) {
    if (clock64() - t0 > limit) return;
  }
}

}  // namespace gbr
