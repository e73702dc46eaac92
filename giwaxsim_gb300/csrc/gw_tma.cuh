// Tensor-memory-accelerator (TMA) tile loads completed through an mbarrier,
// in inline PTX (sm_90 and later, sm_103a here).
//
// A tiled load cp.async.bulk.tensor.2d copies a box of a 2-D tensor map
// (made on the host with cuTensorMapEncodeTiled) into shared memory and
// reports its bytes to an mbarrier; the threads wait on the barrier's phase.
// Rules kept by the callers: the box's inner extent and the inner
// coordinate times the element size are multiples of 16 bytes, the shared
// destination is 128-byte aligned, and every wait is bounded.
#pragma once

#include <cuda.h>
#include <stdint.h>

__device__ __forceinline__ unsigned smem_u32(const void *p) {
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(count)
               : "memory");
  // make the initialised barrier visible to the asynchronous proxy
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// One arrival that also announces `bytes` of transactions to come.
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(
                   smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned phase) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(phase)
      : "memory");
  return ok != 0;
}

// Bounded wait for the barrier's phase: false after `limit` polls.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, unsigned phase,
                                                  unsigned limit) {
  for (unsigned it = 0; it < limit; ++it)
    if (mbar_try_wait(bar, phase)) return true;
  return false;
}

// Box at element coordinates (x inner, y outer) of the 2-D map into dst.
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map,
                                            int x, int y, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
      : "memory");
}
