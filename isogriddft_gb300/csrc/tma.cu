// Tensor-map encoding (driver API via the runtime entry-point query) and the
// device error word shared by kernels with bounded waits.
#include <mutex>

#include "tma.cuh"

namespace igd {

__device__ unsigned int g_error_flags = 0;

unsigned int* device_error_word() {
  static unsigned int* cached[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  if (!cached[dev]) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_error_flags) != cudaSuccess) return nullptr;
    cached[dev] = static_cast<unsigned int*>(p);
  }
  return cached[dev];
}

namespace {
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::once_flag g_once;

void resolve() {
  void* fn = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
      q == cudaDriverEntryPointSuccess)
    g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
}
}  // namespace

bool encode_tensor_map(CUtensorMap* map, bool f64, int rank, const void* base, const unsigned long long* dims,
                       const unsigned long long* stride_bytes, const unsigned* box) {
  std::call_once(g_once, resolve);
  if (!g_encode) return false;
  const unsigned es = f64 ? 8u : 4u;
  if ((reinterpret_cast<uintptr_t>(base) & 15u) != 0) return false;
  if ((box[0] * es) % 16u != 0) return false;
  for (int i = 0; i < rank - 1; ++i)
    if (stride_bytes[i] % 16u != 0) return false;
  for (int i = 0; i < rank; ++i)
    if (box[i] == 0 || box[i] > 256) return false;
  cuuint64_t gd[5], gs[4];
  cuuint32_t bx[5], es1[5];
  for (int i = 0; i < rank; ++i) {
    gd[i] = dims[i];
    bx[i] = box[i];
    es1[i] = 1;
  }
  for (int i = 0; i < rank - 1; ++i) gs[i] = stride_bytes[i];
  CUresult r = g_encode(map, f64 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, rank,
                        const_cast<void*>(base), gd, gs, bx, es1, CU_TENSOR_MAP_INTERLEAVE_NONE,
                        CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

}  // namespace igd

// Read (and optionally clear) the device error word; synchronises the stream.
extern "C" int igd_error_flags(unsigned int* flags_out, int clear, void* stream) {
  if (!flags_out) return IGD_ERR_ARG;
  cudaStream_t st = igd::as_stream(stream);
  if (cudaMemcpyFromSymbolAsync(flags_out, igd::g_error_flags, sizeof(unsigned), 0, cudaMemcpyDeviceToHost, st) !=
      cudaSuccess)
    return IGD_ERR_CUDA;
  if (clear) {
    const unsigned zero = 0;
    if (cudaMemcpyToSymbolAsync(igd::g_error_flags, &zero, sizeof(unsigned), 0, cudaMemcpyHostToDevice, st) !=
        cudaSuccess)
      return IGD_ERR_CUDA;
  }
  return cudaStreamSynchronize(st) == cudaSuccess ? IGD_OK : IGD_ERR_CUDA;
}
