// mbarrier helpers (inline PTX, sm_90+ forms used on sm_103a).
//
// Every wait is bounded: mbar_wait gives up after ~2^32 cycles (about 2 s at
// 2 GHz; a launch may pass a shorter limit) or when the error word is already set, records `code` in the error
// word and returns false, so that a kernel can stop, let its own copies land
// (mbar_drain) and return instead of spinning forever.
#pragma once
#include <cstdint>

namespace scess {

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Arrive once and add `bytes` to the transaction count of the current phase.
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait: false (and the error word set) after `limit` cycles (~2^32 by
// default) or when another role of the CTA (or another CTA) already gave up.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, unsigned *err,
                                          unsigned code, long long limit = 1ll << 32) {
  if (mbar_try_wait(bar, parity)) return true;
  const long long t0 = clock64();
  for (unsigned spin = 1;; spin++) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((spin & 1023u) == 0) {
      if (*(volatile unsigned *)err) return false;
      if (clock64() - t0 > limit) {
        atomicCAS(err, 0u, code);
        return false;
      }
    }
  }
}

// Bounded wait that ignores the error word: used to let issued copies land
// before the CTA exits (returns after ~2^32 cycles at the latest).
__device__ __forceinline__ void mbar_drain(uint64_t *bar, uint32_t parity) {
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity))
    if (clock64() - t0 > (1ll << 32)) return;
}

}  // namespace scess
