// e2d_tma.cuh -- inline-PTX helpers of the TMA-staged kernels: mbarriers
// with bounded waits and 3-D tiled bulk copies (cp.async.bulk.tensor) from a
// tensor map of this GPU's own memory into shared memory.
#pragma once

#include <cuda.h>

namespace e2d {

constexpr unsigned long long kWaitNs = 1000000000ull;  // bounded waits give up after 1 s

__device__ __forceinline__ unsigned int smem_u32(const void *p) { return (unsigned int)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned int count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory"); }
__device__ __forceinline__ void mbar_arrive_expect(unsigned long long *bar, unsigned int bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long *bar, unsigned int parity) {
  unsigned int ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0u;
}
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int x, int y, int z,
                                            unsigned long long *bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
      "[%5];\n" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

// Waits (every lane) for the completion of phase `parity` of *bar; false,
// for the whole warp, once kWaitNs have passed without it.
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned int parity) {
  bool ok = mbar_try_wait(bar, parity);
  if (!__all_sync(0xffffffffu, ok)) {
    const unsigned long long t0 = global_ns();
    while (!ok && global_ns() - t0 < kWaitNs) ok = mbar_try_wait(bar, parity);
    ok = __all_sync(0xffffffffu, ok);
  }
  return ok;
}

}  // namespace e2d
