// Shared-memory mbarrier and bulk-copy helpers (inline PTX, sm_90+ forms
// that sm_103a keeps), shared by the tensor-core Legendre kernels and the
// FFT (internal header).  Every wait is bounded by WAIT_LIMIT_NS of
// %globaltimer; the caller records an error code and stops on expiry.
#pragma once
#include <stdint.h>

namespace dccm {

constexpr unsigned long long WAIT_LIMIT_NS = 1000000000ull;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t *b, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *b) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(b)) : "memory");
}
__device__ __forceinline__ void mbar_arrive_tx(uint64_t *b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try(uint64_t *b, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(b)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ unsigned long long gtimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}
// Bounded wait for the phase of the given parity; false (and err set to
// code, first writer wins) if it did not complete within the limit.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *b, uint32_t parity, int *err, int code) {
  if (mbar_try(b, parity)) return true;
  const unsigned long long t0 = gtimer();
  for (uint32_t it = 1;; ++it) {
    if (mbar_try(b, parity)) return true;
    if ((it & 255) == 0 && gtimer() - t0 > WAIT_LIMIT_NS) {
      if (err) atomicCAS(err, 0, code);
      return false;
    }
  }
}
// Contiguous global -> shared copy by the bulk-copy engine (TMA, no tensor
// map): dst and src 16-byte aligned, bytes a multiple of 16; completes as
// transaction bytes on bar.
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(src)), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

}  // namespace dccm
