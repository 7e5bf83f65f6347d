// lbm_pipeline.cuh - the pieces of the bulk-copy pipelines of the staged
// stream + collide kernels: mbarrier init / arrive / bounded wait and the
// cp.async.bulk global -> shared copy (inline PTX, sm_90 and later).
#pragma once
#include <cstdint>

namespace lbm {
namespace {

constexpr long long kWaitNs = 2000000000LL;   // 2 s bound on one wait

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ long long global_ns() {
  long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}
// try_wait with a suspend-time hint: the waiting thread sleeps until the
// phase completes or about `hint_ns` pass, instead of spinning
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity, unsigned hint_ns) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity), "r"(hint_ns)
      : "memory");
  return ok != 0;
}
// wait for the phase of parity `parity` of the barrier to complete, at most
// `limit_ns` nanoseconds
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity,
                                                  long long limit_ns) {
  if (mbar_try_wait(bar, parity, 20000u)) return true;
  const long long t0 = global_ns();
  for (int it = 0; it < (1 << 26); ++it) {
    if (mbar_try_wait(bar, parity, 20000u)) return true;
    if (global_ns() - t0 > limit_ns) return false;
  }
  return false;
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

}  // namespace
}  // namespace lbm
