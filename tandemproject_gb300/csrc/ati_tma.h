// ati_tma.h — tensor-memory-accelerator (TMA) staging helpers of the segmented line sweeps.
//
// A line tile of the eta or zeta sweeps is 32 consecutive lines of one block (32 neighbouring points of a grid
// row) over the whole line length: with the field plane of a block described as a 3-D (zeta lines) or 4-D
// (eta lines) tensor, one cp.async.bulk.tensor copy moves the tile into shared memory as [point][line] rows of
// 32 floats, completion counted on an mbarrier.  Waits on the mbarrier are bounded: a copy that has not landed
// after TMA_WAIT_TRIES polls makes the kernel record the failure instead of spinning on.
#pragma once
#include <cstdint>

namespace ati {

constexpr uint32_t TMA_WAIT_TRIES = 1u << 22;

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
// make the initialised barrier visible to the asynchronous (TMA) proxy
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
// true once phase `parity` of the barrier has completed
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n"
      ".reg .pred p;\n"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      "selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}
// bounded wait: false if the phase did not complete within TMA_WAIT_TRIES polls
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity) {
  for (uint32_t k = 0; k < TMA_WAIT_TRIES; k++)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

// the tensor maps live in global memory, written by a host copy before the launch: acquire them for the tensor-map
// proxy before their first use
__device__ __forceinline__ void tmap_acquire(const void *tmap) {
  asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;\n" ::"l"(tmap) : "memory");
}

// tile copies global -> shared (no multicast), completion on the mbarrier; x is the innermost coordinate
__device__ __forceinline__ void tma_load_3d(void *dst, const void *tmap, int x, int y, int z, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];\n" ::"r"(smem_u32(dst)),
      "l"(tmap), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tma_load_4d(void *dst, const void *tmap, int x, int y, int z, int w, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, "
      "%5}], [%6];\n" ::"r"(smem_u32(dst)),
      "l"(tmap), "r"(x), "r"(y), "r"(z), "r"(w), "r"(smem_u32(bar))
      : "memory");
}

// one tensor map (CUtensorMap, 128 bytes, 64-byte aligned) per block, array and direction
struct alignas(64) TmaMap {
  unsigned char bytes[128];
};

}  // namespace ati
