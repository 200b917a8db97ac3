// tma.cuh -- bulk asynchronous copies (TMA, cp.async.bulk) into shared
// memory with mbarrier completion, and bounded waits.
//
// Every wait here gives up after kTmaWaitCycles SM clocks (about a second):
// the caller then records a fault instead of spinning forever.  The fault is
// a word of mapped host memory (device_fault_word), so the host reads it
// after a call without another CUDA call (take_device_fault).
#pragma once

#include <cstdint>

namespace idrs {

constexpr long long kTmaWaitCycles = 1LL << 31;

// device address of the mapped fault word (allocated on first use)
int* device_fault_word();
// the fault word's value, cleared; 0 when no staged copy was lost
int take_device_fault();

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* b, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
// makes mbarrier initialisations visible to the async proxy (before any copy)
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// orders this thread's earlier generic-proxy shared accesses (and those the
// preceding barrier made visible to it) before later async-proxy writes
__device__ __forceinline__ void proxy_async_fence() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
// one arrival that also announces `bytes` of copies completing on b
__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* b, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
// wait for the phase of parity `parity` to complete; false after kTmaWaitCycles
__device__ __forceinline__ bool mbar_wait(uint64_t* b, unsigned parity) {
  if (mbar_try_wait(b, parity)) return true;
  const long long t0 = clock64();
  while (!mbar_try_wait(b, parity))
    if (clock64() - t0 > kTmaWaitCycles) return false;
  return true;
}
// the same for many waiting threads: between polls a thread sleeps, so
// waiting warps leave the issue slots to the warps that compute
__device__ __forceinline__ bool mbar_wait_sleep(uint64_t* b, unsigned parity) {
  if (mbar_try_wait(b, parity)) return true;
  const long long t0 = clock64();
  while (!mbar_try_wait(b, parity)) {
    __nanosleep(32);
    if (clock64() - t0 > kTmaWaitCycles) return false;
  }
  return true;
}
// bulk copy global -> shared: both addresses 16-byte aligned, bytes a
// multiple of 16; completes `bytes` of transactions on b
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, uint64_t* b) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(b))
               : "memory");
}

}  // namespace idrs
