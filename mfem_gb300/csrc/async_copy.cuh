// Bulk asynchronous copies global -> shared memory (the TMA engine's
// one-dimensional form, cp.async.bulk) completed through mbarriers, with
// bounded waits.
//
// Every wait gives up after kMbarMaxPolls polls or kMbarTimeoutNs of the
// GPU's global timer, whichever comes first, and returns false; the caller
// raises an error flag the host reads, then drains its own copies in flight
// (again with a bounded wait) before the block exits.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace mfem_gpu {

constexpr unsigned int kMbarMaxPolls = 1u << 22;
constexpr unsigned long long kMbarTimeoutNs = 1000000000ull;  // 1 s

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ unsigned long long mbar_global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// One arrival completes a phase (with the transaction bytes expected by it).
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

// Makes barrier initialisation visible to the async proxy (the copy engine).
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Orders this thread's earlier generic-proxy accesses of shared memory
// before async-proxy writes it issues afterwards (refilling a stage the
// warp has just read).
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

// bytes from global src to shared dst, completing on bar.  dst, src 16-byte
// aligned, bytes a multiple of 16.  policy: an L2 cache policy
// (createpolicy) for the source lines.
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t bar,
                                         unsigned long long policy) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint"
      " [%0], [%1], %2, [%3], %4;" ::"r"(dst),
      "l"(src), "r"(bytes), "r"(bar), "l"(policy)
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(bar), "r"(parity)
      : "memory");
  return done != 0;
}

// Waits for the phase of the given parity to complete; false if the wait
// ran out (poll count or time).
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = mbar_global_ns();
  for (unsigned int polls = 1; polls < kMbarMaxPolls; ++polls) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((polls & 1023u) == 0 && mbar_global_ns() - t0 > kMbarTimeoutNs) return false;
  }
  return false;
}

// Loads of one ELL pair from shared memory by its 32-bit shared address.
__device__ __forceinline__ float2 lds_pair(uint32_t addr, float) {
  float2 v;
  asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(v.x), "=f"(v.y) : "r"(addr) : "memory");
  return v;
}
__device__ __forceinline__ double2 lds_pair(uint32_t addr, double) {
  double2 v;
  asm volatile("ld.shared.v2.f64 {%0, %1}, [%2];" : "=d"(v.x), "=d"(v.y) : "r"(addr) : "memory");
  return v;
}

}  // namespace mfem_gpu
