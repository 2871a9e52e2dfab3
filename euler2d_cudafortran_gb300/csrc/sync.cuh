// sync.cuh -- bounded waits on shared-memory mbarriers.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace e2d {

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Waits for phase `parity` of the mbarrier at shared address `bar`, giving up
// after `limit_cycles` SM cycles; returns whether the phase completed.  Every
// wait in the library goes through here, so that a lost transfer or a missing
// arrival ends in a status the host can read instead of a hung GPU.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, long long limit_cycles) {
  const long long t0 = clock64();
  while (true) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    if (ok) return true;
    if (clock64() - t0 > limit_cycles) return false;
  }
}

// The limit of the step kernels' TMA wait: 2^31 cycles, about a second.
constexpr long long kTmaWaitCycles = 1ll << 31;

}  // namespace e2d
