// eg_tma.cuh -- bulk asynchronous copies (TMA, cp.async.bulk) from global to
// shared memory completed on an mbarrier, and the barrier primitives around
// them (inline PTX for sm_103a).
//
// Rules the callers keep: source address, destination address and size are
// multiples of 16 bytes; one thread arms a barrier with the byte count of all
// the copies it then issues on it (mbarrier.arrive.expect_tx, barrier count
// 1); waits are bounded (mbar_wait gives up after kMbarWaitNs and the caller
// reports an error instead of spinning forever).
#pragma once
#include <stdint.h>

// time limit of one bounded mbarrier wait (nanoseconds of %globaltimer); a
// copy of a few hundred KB completes in microseconds
constexpr unsigned long long kMbarWaitNs = 200000000ull;  // 0.2 s

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// makes barrier initialisation visible to the async proxy (the copy engine)
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// orders this thread's earlier shared-memory accesses (generic proxy) before
// the async-proxy writes of copies it issues next
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

// bytes (multiple of 16) from global src (16-byte aligned) to shared dst
// (16-byte aligned); completion is counted on bar
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}

// one arrival (release semantics at CTA scope: this thread's and, after a
// barrier, its group's earlier shared-memory accesses happen before)
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// wait for the completion of phase `parity` of bar; false once kMbarWaitNs
// have passed (the caller raises its error flag)
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  if (mbar_try_wait(bar, parity)) return true;
  const unsigned long long t0 = global_ns();
  for (;;) {
    if (mbar_try_wait(bar, parity)) return true;
    if (global_ns() - t0 > kMbarWaitNs) return false;
  }
}

// barrier over `nthreads` threads (a multiple of 32) of the CTA, id 1..15
// (id 0 is __syncthreads)
__device__ __forceinline__ void named_sync(int id, int nthreads) {
  asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}
