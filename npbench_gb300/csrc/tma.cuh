// TMA (cp.async.bulk.tensor) and mbarrier helpers for sm_103a, plus host-side
// tensor-map encoding.
//
// Every wait is bounded: mbar_wait() gives up after kWaitLimitNs of the
// global timer and returns false; kernels then record an error word and
// leave, so a lost copy never hangs the GPU.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <cstdint>

namespace npbgb {
namespace tma {

constexpr uint64_t kWaitLimitNs = 1000000000ull;  // one second

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ uint64_t globaltimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Makes a tensor map that the host copied into global memory visible to the
// tensormap proxy before the first copy that uses it.
__device__ __forceinline__ void fence_tensormap_acquire(const void* map) {
  asm volatile("fence.proxy.tensormap::generic.acquire.sys [%0], 128;" ::"l"(map) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n"
      ".reg .pred p;\n"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      "selp.u32 %0, 1, 0, p;\n"
      "}\n"
      : "=r"(done)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return done != 0;
}

// Waits for the phase with the given parity to complete; false once
// `limit_ns` of the global timer has passed.
__device__ __forceinline__ bool mbar_wait_for(uint64_t* bar, uint32_t parity, uint64_t limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = globaltimer();
  for (uint32_t n = 1;; ++n) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((n & 63u) == 0 && globaltimer() - t0 > limit_ns) return false;
  }
}

__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  return mbar_wait_for(bar, parity, kWaitLimitNs);
}

// 3D tiled bulk copy global -> shared, completing on `bar`.  x (the innermost
// coordinate) times the element size must be a multiple of 16 bytes.
__device__ __forceinline__ void load_3d(void* dst, const CUtensorMap* map, int x, int y, int z,
                                        uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
      : "memory");
}

// Host: encodes a 3D tiled tensor map over a C-ordered array with extents
// dims = {fastest, middle, slowest} and element size `esize` (4 or 8).
// Returns cudaSuccess or cudaErrorInvalidValue when a TMA rule is not met
// (16-byte aligned base and row strides, box inner extent a multiple of 16
// bytes, box extents <= 256).
cudaError_t encode_3d(CUtensorMap* map, int esize, const void* base, const uint64_t dims[3],
                      const uint32_t box[3]);

}  // namespace tma
}  // namespace npbgb
