// Bulk asynchronous copies (TMA, cp.async.bulk) into shared memory with
// mbarrier completion, and the bounded waits on them.
//
// A copy moves `bytes` (a multiple of 16) from 16-byte aligned global memory
// to 16-byte aligned shared memory and counts them against an mbarrier's
// transaction count.  The issuing thread first arms the barrier with the
// expected byte count (arrive.expect_tx); the barrier's phase completes when
// all bytes have landed.  Waiters poll the phase parity with try_wait, at most
// kTmaMaxPolls times: a wait that runs out increments a timeout counter in
// global memory (read back by vp_wait_timeouts()) and returns false instead
// of spinning on, so a fault in the memory system cannot hang the GPU.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <stdint.h>

namespace vp {
namespace tma {

constexpr unsigned kTmaMaxPolls = 1u << 22;  // try_wait returns after a bounded time each

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}

// Makes barrier initialisation visible to the async proxy (the copy engine).
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Orders this thread's earlier generic-proxy shared-memory accesses before
// later async-proxy ones (a stage read by the warp, then refilled by a copy).
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  uint32_t done;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(done)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

// Waits until the barrier's phase of the given parity has completed; false
// (and one count in *timeouts, from lane 0) if the bound ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity,
                                          unsigned long long* timeouts) {
  for (unsigned i = 0; i < kTmaMaxPolls; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  if ((threadIdx.x & 31) == 0) atomicAdd(timeouts, 1ull);
  return false;
}

// Tensor copy of one box of a 3-D tensor map (coordinates innermost first,
// elements) to shared dst, completing on bar.  Box elements outside the
// tensor read as zero; the barrier counts the whole box.
__device__ __forceinline__ void tensor3d_g2s(void* dst, const CUtensorMap* map, int c0, int c1,
                                             int c2, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];"
      ::"r"(smem_addr(dst)), "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2),
        "r"(smem_addr(bar))
      : "memory");
}

}  // namespace tma
}  // namespace vp
