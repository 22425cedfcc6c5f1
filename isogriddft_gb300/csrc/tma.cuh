// TMA (cp.async.bulk.tensor) and mbarrier helpers, plus host-side tensor-map
// encoding through the driver entry point (no link against libcuda).
#pragma once

#include <cuda.h>
#include <cudaTypedefs.h>

#include "common.cuh"

namespace igd {

// Device-side error word (bit 0: an mbarrier wait gave up).  Kernels get its
// address as a parameter; the host reads it with igd_error_flags().
enum : unsigned int { IGD_FLAG_WAIT_TIMEOUT = 1u };
unsigned int* device_error_word();  // host: address on the current device

__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Bounded wait: after ~2^24 polls (seconds) record a timeout flag and go on
// (the caller's results are then invalid and the host reports an error);
// never spins forever.
__device__ __forceinline__ void mbar_wait(uint64_t* bar, unsigned parity, unsigned* err) {
  for (int i = 0; i < (1 << 24); ++i)
    if (mbar_try_wait(bar, parity)) return;
  atomicOr(err, IGD_FLAG_WAIT_TIMEOUT);
}

__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, int c0, int c1, int c2, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];\n" ::
          "r"(smem_u32(dst)),
      "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void tma_load_4d(void* dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];\n" ::"r"(smem_u32(dst)),
      "l"(map), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
      : "memory");
}

// Host: tensor map of a dense row-major array with dims[0] fastest.
// Returns false when the TMA alignment rules are not met (caller falls back).
bool encode_tensor_map(CUtensorMap* map, bool f64, int rank, const void* base, const unsigned long long* dims,
                       const unsigned long long* stride_bytes, const unsigned* box);
// Same, optionally with the 128-byte swizzle (box rows of exactly 128 bytes).
bool encode_tensor_map_ex(CUtensorMap* map, bool f64, int rank, const void* base, const unsigned long long* dims,
                          const unsigned long long* stride_bytes, const unsigned* box, bool swizzle128);

}  // namespace igd
