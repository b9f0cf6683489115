// hyc_tma.cuh -- mbarrier and TMA (cp.async.bulk.tensor) helpers in inline
// PTX for the streaming kernels.  Every wait is bounded: after 2 s of wall
// time (globaltimer) it records the failure in an error flag and returns
// false, so a lost transaction ends the kernel with an error the host reads
// instead of a hang.
#pragma once
#include <cuda.h>
#include <cuda_runtime.h>

#include <cstdint>

namespace hyc {
namespace tma {

__device__ __forceinline__ uint32_t sa(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void bar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(sa(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_bar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
// orders this thread's earlier generic-proxy accesses of shared memory (and,
// after a CTA barrier, the CTA's) before its later TMA writes
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(sa(bar)), "r"(bytes) : "memory");
}
// one arrival (release) on an mbarrier
__device__ __forceinline__ void arrive(uint64_t *bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(sa(bar)) : "memory");
}
__device__ __forceinline__ bool try_wait(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(sa(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ uint64_t now_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Wait for the phase with the given parity to complete; false (and *err set)
// after 2 s.
__device__ __forceinline__ bool wait(uint64_t *bar, uint32_t parity, int *err) {
  if (try_wait(bar, parity)) return true;
  const uint64_t t0 = now_ns();
  for (;;) {
    if (try_wait(bar, parity)) return true;
    if (now_ns() - t0 > 2000000000ull) break;
  }
  if (err) atomicExch(err, 1);
  return false;
}
__device__ __forceinline__ void load3(void *dst, const CUtensorMap *map, uint64_t *bar, int x, int y, int z) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];" ::
          "r"(sa(dst)),
      "l"(map), "r"(x), "r"(y), "r"(z), "r"(sa(bar))
      : "memory");
}
}  // namespace tma
}  // namespace hyc
