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
#include <cudaTypedefs.h>
#include <stdint.h>

namespace vp {
namespace tma {

// cuTensorMapEncodeTiled, looked up once per process through the runtime (a
// thread-safe static initialiser; no link against the driver library), or
// nullptr where the driver does not offer it.
inline PFN_cuTensorMapEncodeTiled_v12000 encode_tiled_fn() {
  static const PFN_cuTensorMapEncodeTiled_v12000 fn = []() {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    const cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000,
                                                           cudaEnableDefault, &q);
    return (e == cudaSuccess && q == cudaDriverEntryPointSuccess)
               ? reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f)
               : nullptr;
  }();
  return fn;
}

// A float32 3-D tensor map (dims and box innermost first; strides in bytes of
// dims 1 and 2), zero fill outside the tensor.  The caller keeps the rules of
// tiled copies: base 16-byte aligned, strides multiples of 16 bytes, box
// inner extent a multiple of 16 bytes.
inline cudaError_t encode_3d_f32(CUtensorMap* map, const float* base, const uint64_t dims[3],
                                 const uint64_t strides[2], const uint32_t box[3]) {
  const PFN_cuTensorMapEncodeTiled_v12000 encode = encode_tiled_fn();
  if (encode == nullptr) return cudaErrorNotSupported;
  const cuuint64_t d[3] = {dims[0], dims[1], dims[2]};
  const cuuint64_t st[2] = {strides[0], strides[1]};
  const cuuint32_t bx[3] = {box[0], box[1], box[2]};
  const cuuint32_t estride[3] = {1, 1, 1};
  const CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<float*>(base),
                            d, st, bx, estride, CU_TENSOR_MAP_INTERLEAVE_NONE,
                            CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

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

// Waits until the barrier's phase of the given parity has completed, polling
// at most `polls` times; false (and one count in *timeouts, from lane 0) if
// the bound ran out.  With `abort`, the wait also gives up, uncounted, once
// *abort is nonzero (another warp of the block gave up first).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity,
                                          unsigned long long* timeouts,
                                          unsigned polls = kTmaMaxPolls,
                                          const volatile int* abort = nullptr) {
  for (unsigned i = 0; i < polls; ++i) {
    if (mbar_try_wait(bar, parity)) return true;
    if (abort && (i & 63u) == 63u && *abort) return false;
  }
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
