// afg_tma.cuh -- bulk asynchronous copies (TMA, cp.async.bulk) into shared
// memory with mbarrier completion, for sm_90 and later (here sm_103a).
//
// Waits are bounded by the global nanosecond timer: a wait that has not
// completed after kWaitLimitNs returns false, and the caller raises its
// error flag and drains its copies instead of spinning forever.
#pragma once
#include <cstdint>

namespace afg {

constexpr unsigned long long kWaitLimitNs = 1000000000ull;  // 1 s

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// one-time setup of an mbarrier expecting `count` arrivals per phase
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
// makes the initialised barriers visible to the asynchronous proxy
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
// orders earlier generic-proxy accesses of shared memory before later
// asynchronous-proxy writes (a stage is refilled after it was read)
__device__ __forceinline__ void fence_proxy_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// the calling thread's arrival, announcing `bytes` of copies on the phase
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// global -> shared bulk copy; dst, src 16-byte aligned, bytes a multiple of
// 16; completes `bytes` of the barrier's current phase
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// wait for the phase with the given parity; false after kWaitLimitNs
__device__ __forceinline__ bool mbar_wait(unsigned long long* bar, unsigned parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = global_ns();
  while (!mbar_try_wait(bar, parity))
    if (global_ns() - t0 > kWaitLimitNs) return false;
  return true;
}

}  // namespace afg

namespace afg {

// Check of the bounded-wait path used by the staged kernels: one thread
// announces `bytes` of copies on a fresh mbarrier and issues none, so the
// phase cannot complete; the wait gives up after kWaitLimitNs and raises
// *err exactly as a staged kernel does.  No copy is in flight when the CTA
// returns.
static __global__ void k_wait_check(unsigned bytes, unsigned* err) {
  __shared__ __align__(8) unsigned long long bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) mbar_arrive_expect_tx(&bar, bytes);
  __syncthreads();
  const bool ok = mbar_wait(&bar, 0);
  if (__syncthreads_or(!ok) && threadIdx.x == 0) atomicExch(err, 1u);
}

}  // namespace afg
