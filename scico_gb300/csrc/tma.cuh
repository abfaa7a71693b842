// Tensor-map global->shared copies (cp.async.bulk.tensor, the TMA engine)
// completing on an mbarrier, with a bounded wait.  Inline PTX for sm_90+
// (sm_103a here).
#pragma once

#include <stdint.h>

namespace ct {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Make the initialised barrier visible to the async (TMA) proxy.
__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

// Tiled tensor-map load of one box at element coordinates (x, y, z) into
// shared memory, completing the box's bytes on `bar` (elements outside the
// tensor are filled with zeros and counted).  x * element size must be a
// multiple of 16 bytes; `tmap` is the address of a __grid_constant__
// CUtensorMap kernel parameter.
__device__ __forceinline__ void tensor_g2s_3d(void* dst_smem, const void* tmap, int x, int y, int z,
                                              uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, "
      "%4}], [%5];" ::"r"(smem_u32(dst_smem)),
      "l"(tmap), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.b32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

// Wait for phase `parity` of `bar`, at most `max_polls` polls (each poll may
// suspend the thread for a hardware-defined interval).  Returns false if the
// limit was reached.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t max_polls) {
  for (uint32_t k = 0; k < max_polls; ++k)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

}  // namespace ct
