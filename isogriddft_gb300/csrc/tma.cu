// Tensor-map encoding (driver API via the runtime entry-point query) and the
// device error word shared by kernels with bounded waits.
#include <atomic>
#include <map>
#include <mutex>
#include <tuple>
#include <utility>

#include "tma.cuh"

namespace igd {

// One error word per host thread (slot = the thread's number modulo the slot
// count), so that a thread that reads and clears its word neither sees nor
// wipes a timeout raised by another thread's kernels.
constexpr int kErrorSlots = 64;
__device__ unsigned int g_error_flags[kErrorSlots];

namespace {
std::atomic<int> g_next_error_slot{0};
int error_slot() {
  thread_local const int slot = g_next_error_slot.fetch_add(1, std::memory_order_relaxed) % kErrorSlots;
  return slot;
}
}  // namespace

unsigned int* device_error_word() {
  static std::atomic<unsigned int*> cached[64] = {};  // first calls on several threads store the same address
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  unsigned int* w = cached[dev].load(std::memory_order_acquire);
  if (!w) {
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_error_flags) != cudaSuccess) return nullptr;
    w = static_cast<unsigned int*>(p);
    cached[dev].store(w, std::memory_order_release);
  }
  return w + error_slot();
}

namespace {
std::mutex g_launch_mu;
std::map<std::pair<int, const void*>, size_t> g_smem_limit;                // (device, kernel) -> bytes
std::map<std::tuple<int, const void*, int, size_t>, int> g_blocks_per_sm;  // occupancy cache
}  // namespace

int ensure_dynamic_smem(const void* kernel, size_t bytes) {
  if (bytes <= 48 * 1024) return IGD_OK;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return IGD_ERR_CUDA;
  std::lock_guard<std::mutex> lk(g_launch_mu);
  size_t& have = g_smem_limit[{dev, kernel}];
  if (have >= bytes) return IGD_OK;
  if (cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes) != cudaSuccess)
    return IGD_ERR_CUDA;
  have = bytes;
  return IGD_OK;
}

int blocks_per_sm(const void* kernel, int threads, size_t bytes) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  std::lock_guard<std::mutex> lk(g_launch_mu);
  auto key = std::make_tuple(dev, kernel, threads, bytes);
  auto it = g_blocks_per_sm.find(key);
  if (it != g_blocks_per_sm.end()) return it->second;
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kernel, threads, bytes) != cudaSuccess || n < 1) {
    cudaGetLastError();  // leave no error behind for the caller's launch check
    n = 1;
  }
  g_blocks_per_sm[key] = n;
  return n;
}

int device_sm_count() {
  static std::atomic<int> cached[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
  int n = cached[dev].load(std::memory_order_relaxed);
  if (n > 0) return n;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 152;
  cached[dev].store(n, std::memory_order_relaxed);
  return n;
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
  return encode_tensor_map_ex(map, f64, rank, base, dims, stride_bytes, box, false);
}

bool encode_tensor_map_ex(CUtensorMap* map, bool f64, int rank, const void* base, const unsigned long long* dims,
                          const unsigned long long* stride_bytes, const unsigned* box, bool swizzle128) {
  std::call_once(g_once, resolve);
  if (!g_encode) return false;
  const unsigned es = f64 ? 8u : 4u;
  if ((reinterpret_cast<uintptr_t>(base) & 15u) != 0) return false;
  if ((box[0] * es) % 16u != 0) return false;
  if (swizzle128 && box[0] * es != 128u) return false;  // one 128-byte swizzle span per row
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
                        swizzle128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS;
}

}  // namespace igd

// Read (and optionally clear) the calling thread's device error word; synchronises the stream.
extern "C" int igd_error_flags(unsigned int* flags_out, int clear, void* stream) {
  if (!flags_out) return IGD_ERR_ARG;
  cudaStream_t st = igd::as_stream(stream);
  const size_t off = (size_t)igd::error_slot() * sizeof(unsigned);
  if (cudaMemcpyFromSymbolAsync(flags_out, igd::g_error_flags, sizeof(unsigned), off, cudaMemcpyDeviceToHost, st) !=
      cudaSuccess)
    return IGD_ERR_CUDA;
  if (clear) {
    const unsigned zero = 0;
    if (cudaMemcpyToSymbolAsync(igd::g_error_flags, &zero, sizeof(unsigned), off, cudaMemcpyHostToDevice, st) !=
        cudaSuccess)
      return IGD_ERR_CUDA;
  }
  return cudaStreamSynchronize(st) == cudaSuccess ? IGD_OK : IGD_ERR_CUDA;
}

namespace igd {
namespace {
// One thread waits on a fresh mbarrier that nothing arrives at: every poll fails,
// so after `polls` polls the wait gives up and records the timeout bit.
__global__ void selftest_wait_kernel(int polls, unsigned* err) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    mbar_fence_init();
  }
  __syncthreads();
  if (threadIdx.x != 0) return;
  for (int i = 0; i < polls; ++i)
    if (mbar_try_wait(&bar, 0)) return;
  atomicOr(err, IGD_FLAG_WAIT_TIMEOUT);
}
}  // namespace
}  // namespace igd

// Failure-path self-test of the bounded in-kernel waits (no fault, no hang).
extern "C" int igd_selftest_wait_timeout(int polls, void* stream) {
  if (polls < 1 || polls > (1 << 16)) return IGD_ERR_ARG;
  unsigned* err = igd::device_error_word();
  if (!err) return IGD_ERR_CUDA;
  igd::selftest_wait_kernel<<<1, 32, 0, igd::as_stream(stream)>>>(polls, err);
  return igd::launch_status();
}
