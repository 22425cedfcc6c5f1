// Shared helpers for the IsoGridDFT GB300 kernels (sm_103a).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "isogrid_gb300.h"

#define IGD_HD __host__ __device__ __forceinline__

namespace igd {

// Status words returned by every C entry point (mirrored in include/isogrid_gb300.h).
static inline int launch_status() {
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? IGD_OK : IGD_ERR_CUDA;
}

static inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// ---------------------------------------------------------------- cp.async
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// 4- or 8-byte asynchronous global->shared copy; src_bytes = 0 zero-fills.
template <int BYTES>
__device__ __forceinline__ void cp_async_zfill(void* dst, const void* src, bool valid) {
  static_assert(BYTES == 4 || BYTES == 8, "element copies only");
  const int n = valid ? BYTES : 0;
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;\n" ::"r"(smem_u32(dst)), "l"(src), "n"(BYTES),
               "r"(n)
               : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

// ---------------------------------------------------------------- reductions
template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Block-wide FP64 sum of NV values per thread; result valid in thread 0.
template <int NV, int NTHREADS>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* scratch /* NV * NTHREADS/32 */) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int i = 0; i < NV; ++i) v[i] = warp_sum(v[i]);
  if (lane == 0) {
#pragma unroll
    for (int i = 0; i < NV; ++i) scratch[i * (NTHREADS / 32) + warp] = v[i];
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      double x = lane < NTHREADS / 32 ? scratch[i * (NTHREADS / 32) + lane] : 0.0;
      v[i] = warp_sum(x);
    }
  }
  __syncthreads();
}

// Block-wide FP64 sums of NV values followed by one atomicAdd per block and
// value (every thread of the block must call it).
template <int NV, int NTHREADS>
__device__ __forceinline__ void block_atomic_add(double* dst, double (&v)[NV]) {
  __shared__ double scratch[NV * (NTHREADS / 32)];
  block_sum<NV, NTHREADS>(v, scratch);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int i = 0; i < NV; ++i) atomicAdd(dst + i, v[i]);
  }
}

// Launch set-up shared by host threads (tma.cu).  The dynamic shared-memory
// limit of a kernel is process-wide, so it is raised under a lock and never
// lowered (a thread that lowered it could fail another thread's launch that
// needs more); returns IGD_OK or IGD_ERR_CUDA.
int ensure_dynamic_smem(const void* kernel, size_t bytes);
// Resident blocks per SM of a kernel at (threads, dynamic shared memory),
// computed once per (device, kernel, threads, bytes) under a lock; >= 1.
int blocks_per_sm(const void* kernel, int threads, size_t bytes);
// SM count of the current device (cached per device; 152 if the query fails).
int device_sm_count();

// TMA fast path of igd_hpsi_agrid (hpsi_agrid_tma.cu); -1 = not applicable.
int hpsi_agrid_tma_launch(int dtype, int closure, int nx, int ny, int nz, const void* coeffs, const void* veff,
                          const void* psi, void* out, int nb, long long ostride, double kscale, double vscale,
                          cudaStream_t st);

// The whole-row kernel as the Poisson operator of a Krylov solve (hpsi_agrid_zvec.cu):
// one FP32 orbital, production closure, out = kscale L psi with the six faces
// written as zero, and acc[0] += out . y (y = dot_y, or psi when dot_y is null),
// acc[1] += out . out (FP64 across blocks, accumulated); nothing runs while
// *skip != 0.  -1 when the row length or alignment is outside the kernel.
bool hpsi_agrid_krylov_applies(int nz, const void* coeffs);
int hpsi_agrid_krylov(int nx, int ny, int nz, const float* coeffs, const float* psi, float* out, double kscale,
                      const float* dot_y, double* dot_acc, const int* skip, cudaStream_t st);

// Whole-row z-vectorised fast path of igd_hpsi_agrid (hpsi_agrid_zvec.cu); -1 = not applicable.
int hpsi_agrid_zvec_launch(int dtype, int closure, int nx, int ny, int nz, const void* coeffs, const void* veff,
                           const void* psi, void* out, int nb, long long ostride, double kscale, double vscale,
                           cudaStream_t st);

}  // namespace igd
