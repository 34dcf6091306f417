// kb_tma.cuh -- bulk async copies and TMA tensor loads into shared memory,
// completed on mbarriers, with bounded waits (shared by the update, moment
// and batched kernels).
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

namespace kb {

// ---- bulk async copies (TMA engine) into shared memory, completed on an mbarrier.
// Every wait is bounded by the global timer: after KB_WAIT_NS the waiter
// gives up, and the caller records KB status bit 2 (timeout).
constexpr unsigned long long KB_WAIT_NS = 1000000000ull;  // 1 s

__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
// One bounded probe of an mbarrier phase.  The suspend-time hint lets the
// hardware park the waiting thread until the phase completes (or the hint
// runs out) instead of having it spin and take issue slots from other warps.
constexpr unsigned KB_SUSPEND_NS = 200000;  // 0.2 ms per probe
__device__ __forceinline__ bool mbar_try(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
      " selp.u32 %0, 1, 0, p;\n}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity), "r"(KB_SUSPEND_NS)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ void mbar_arrive(unsigned long long* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// true once the phase with this parity completed; false after limit_ns.
__device__ __forceinline__ bool mbar_wait_ns(unsigned long long* bar, unsigned parity,
                                             unsigned long long limit_ns) {
  if (mbar_try(bar, parity)) return true;
  const unsigned long long t0 = gtimer();
  while (!mbar_try(bar, parity))
    if (gtimer() - t0 > limit_ns) return false;
  return true;
}
// the wait every staging kernel uses: gives up after KB_WAIT_NS
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity) {
  return mbar_wait_ns(bar, parity, KB_WAIT_NS);
}
// global -> shared bulk copy; dst, src 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes,
                                         unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// A tensor map in global memory that was written before the launch (the
// table of a grouped launch): acquire it for the tensor-map proxy before the
// first copy that uses it.
__device__ __forceinline__ void tmap_acquire(const CUtensorMap* m) {
  asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(
                   reinterpret_cast<unsigned long long>(m))
               : "memory");
}

// 3D tiled tensor load (TMA) of one box into shared memory, completed on an
// mbarrier.  Coordinates outside the tensor read as zero.
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int c0, int c1,
                                            int c2, unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(c0), "r"(c1), "r"(c2),
      "r"(smem_u32(bar))
      : "memory");
}

}  // namespace kb
