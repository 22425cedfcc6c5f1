// Tall-skinny block linear algebra of the eigensolver (K6 Gram, K7 rotation).
//
// Orbital blocks are row-major (k, n): each orbital is one contiguous field.
// Gram: G[i][j] = sum_p A_i[p] W[p] B_j[p]  (weighted_overlap_matrix,
// ks/eigensolver.py:246-272; _weighted_overlap_columns, ks/eigensolver_jax.py:105)
// Rotation: out_j = sum_i A_i C1[i][j] + sum_i B_i C2[i][j]  (basis @ coeffs and
// the two-part compressions of ks/eigensolver_jax.py:178-251).
// FP32 data: products and per-thread sums (at most 64 points) in FP32, block
// and cross-block accumulation in FP64; FP64 data: FP64 throughout.  Cross-block
// sums are deterministic (per-block partials reduced in a second kernel).
#include "common.cuh"
#include "gram_tc.cuh"
#include "tma.cuh"

namespace igd {
namespace {

constexpr int GTH = 256;   // threads per Gram block
constexpr long long kGramTcMinPoints = 1LL << 18;  // below this the CUDA-core kernels have less set-up
thread_local int g_gram_path = 0;                   // igd_gram_select
thread_local int g_gram_last = 0;                   // kernel of this thread's last Gram (1 tensor, 2 pipe, 3 tiled)
constexpr int GPT = 64;    // points per thread and block column (FP32 partial sums stay short)

// Register-tiled tall-skinny Gram.  Block (x, y): tile y of TR x TR outputs
// (rows i0.., columns j0..) over the points of column slice x; each thread
// streams its points straight from global memory (TR + TR + 1 coalesced loads,
// TR^2 FMAs per point) into TR^2 register accumulators of T, then the block
// reduces them in FP64 into part[x][a][b].
template <typename T, int TR>
__global__ void __launch_bounds__(GTH) gram_tile_kernel(long long n, int a, int b, const T* __restrict__ A,
                                                        long long sa, const T* __restrict__ B, long long sb,
                                                        const double* __restrict__ w, double* __restrict__ part) {
  const int tb = (b + TR - 1) / TR;
  const int i0 = (blockIdx.y / tb) * TR, j0 = (blockIdx.y % tb) * TR;
  T acc[TR][TR];
#pragma unroll
  for (int r = 0; r < TR; ++r)
#pragma unroll
    for (int c = 0; c < TR; ++c) acc[r][c] = T(0);
  const T* Ar[TR];
  const T* Br[TR];
#pragma unroll
  for (int r = 0; r < TR; ++r) {
    Ar[r] = i0 + r < a ? A + (long long)(i0 + r) * sa : nullptr;
    Br[r] = j0 + r < b ? B + (long long)(j0 + r) * sb : nullptr;
  }
#pragma unroll 2
  for (long long p = blockIdx.x * (long long)GTH + threadIdx.x; p < n; p += (long long)gridDim.x * GTH) {
    T av[TR], bv[TR];
    const T wp = w ? T(w[p]) : T(1);
#pragma unroll
    for (int r = 0; r < TR; ++r) {
      av[r] = Ar[r] ? Ar[r][p] : T(0);
      bv[r] = Br[r] ? Br[r][p] * wp : T(0);
    }
#pragma unroll
    for (int r = 0; r < TR; ++r)
#pragma unroll
      for (int c = 0; c < TR; ++c) acc[r][c] += av[r] * bv[c];
  }
  // one output row at a time keeps the reduction's registers small
  __shared__ double scratch[TR * (GTH / 32)];
  double* pb = part + (long long)blockIdx.x * a * b;
#pragma unroll
  for (int r = 0; r < TR; ++r) {
    double v[TR];
#pragma unroll
    for (int c = 0; c < TR; ++c) v[c] = (double)acc[r][c];
    block_sum<TR, GTH>(v, scratch);
    if (threadIdx.x == 0 && i0 + r < a) {
#pragma unroll
      for (int c = 0; c < TR; ++c)
        if (j0 + c < b) pb[(long long)(i0 + r) * b + j0 + c] = v[c];
    }
  }
}

// 16-byte asynchronous global->shared copy; the bytes beyond src_bytes are zero-filled.
__device__ __forceinline__ void cp16_zfill(void* dst, const void* src, int src_bytes) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(smem_u32(dst)), "l"(src), "r"(src_bytes)
               : "memory");
}

template <typename T>
struct GVec;
template <>
struct GVec<float> {
  using V = float4;
  static constexpr int W = 4;
  __device__ static float dot(const float4& x, const float4& y) { return x.x * y.x + x.y * y.y + x.z * y.z + x.w * y.w; }
};
template <>
struct GVec<double> {
  using V = double2;
  static constexpr int W = 2;
  __device__ static double dot(const double2& x, const double2& y) { return x.x * y.x + x.y * y.y; }
};

// Pipelined tall-skinny Gram: every value of A, B and w comes from global
// memory once, by 16-byte cp.async copies into a double-buffered shared chunk
// of P points (all rows; rows padded to a multiple of 4 and their stride by
// one vector against bank conflicts) while the previous chunk is summed.  Each
// group of TPT threads owns a 4 x 4 output tile and sums its share of a chunk
// with 16-byte shared loads (8 loads, 64 FMAs per 4 FP32 points); B is scaled
// by w in shared memory once per chunk.  FP32: per-thread sums of at most 32
// points, compensated (Neumaier) FP32 accumulation across chunks, FP64 tile
// reduction over the group's lanes and across blocks (per-block partials).
template <typename T>
__global__ void __launch_bounds__(GTH) gram_pipe_kernel(long long n, int a, int b, const T* __restrict__ A,
                                                        long long sa, const T* __restrict__ B, long long sb,
                                                        const double* __restrict__ w, double* __restrict__ part, int P,
                                                        int TPT) {
  using G = GVec<T>;
  using V = typename G::V;
  constexpr int VW = G::W;
  extern __shared__ __align__(16) unsigned char gsm[];
  const int ap = (a + 3) & ~3, bp = (b + 3) & ~3, PP = P + VW;
  const size_t rows = (size_t)(ap + bp) * PP;
  T* const buf0 = reinterpret_cast<T*>(gsm);
  double* const wb0 = reinterpret_cast<double*>(buf0 + 2 * rows);
  const int tb = bp / 4, ntiles = (ap / 4) * tb;
  const int tid = threadIdx.x, tile = tid / TPT, lt = tid % TPT;
  const bool act = tile < ntiles;
  const int i0 = act ? (tile / tb) * 4 : 0, j0 = act ? (tile % tb) * 4 : 0;
  const int vpr = P / VW;  // vectors per row of a chunk
  // padding rows stay zero (never copied into)
  for (int q = 0; q < 2; ++q) {
    T* As = buf0 + q * rows;
    for (int e = tid; e < (ap - a) * PP; e += GTH) As[(size_t)a * PP + e] = T(0);
    for (int e = tid; e < (bp - b) * PP; e += GTH) As[(size_t)(ap + b) * PP + e] = T(0);
  }
  const long long nchunks = (n + P - 1) / P;
  auto issue = [&](long long c, int q) {
    const long long p0 = c * P;
    T* As = buf0 + q * rows;
    T* Bs = As + (size_t)ap * PP;
    for (int e = tid; e < (a + b) * vpr; e += GTH) {
      const int row = e / vpr, v = e - row * vpr;
      const long long p = p0 + (long long)v * VW, left = n - p;
      const int bytes = left >= VW ? 16 : (left > 0 ? (int)left * (int)sizeof(T) : 0);
      if (row < a)
        cp16_zfill(As + (size_t)row * PP + v * VW, A + (long long)row * sa + (bytes ? p : 0), bytes);
      else
        cp16_zfill(Bs + (size_t)(row - a) * PP + v * VW, B + (long long)(row - a) * sb + (bytes ? p : 0), bytes);
    }
    if (w) {
      double* wq = wb0 + q * P;
      for (int e = tid; e < P / 2; e += GTH) {
        const long long p = p0 + 2 * e, left = n - p;
        const int bytes = left >= 2 ? 16 : (left > 0 ? 8 : 0);
        cp16_zfill(wq + 2 * e, w + (bytes ? p : 0), bytes);
      }
    }
  };
  T hi[4][4], lo[4][4];
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) hi[r][c] = lo[r][c] = T(0);
  long long c = blockIdx.x;
  if (c < nchunks) issue(c, 0);
  cp_async_commit();
  for (int q = 0; c < nchunks; c += gridDim.x, q ^= 1) {
    if (c + gridDim.x < nchunks) issue(c + gridDim.x, q ^ 1);
    cp_async_commit();
    cp_async_wait<1>();  // chunk c has landed (the next may still be in flight)
    __syncthreads();
    T* As = buf0 + q * rows;
    T* Bs = As + (size_t)ap * PP;
    if (w) {
      const double* wq = wb0 + q * P;
      for (int e = tid; e < b * P; e += GTH) {
        const int j = e / P, x = e - j * P;
        Bs[(size_t)j * PP + x] *= T(wq[x]);
      }
      __syncthreads();
    }
    if (act) {
      const V* Av = reinterpret_cast<const V*>(As + (size_t)i0 * PP);
      const V* Bv = reinterpret_cast<const V*>(Bs + (size_t)j0 * PP);
      const int rowv = PP / VW;
      for (int g0 = lt; g0 < vpr; g0 += 8 * TPT) {
        T sacc[4][4];
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
          for (int cc = 0; cc < 4; ++cc) sacc[r][cc] = T(0);
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int g = g0 + u * TPT;
          if (g < vpr) {
            V av[4], bv[4];
#pragma unroll
            for (int r = 0; r < 4; ++r) av[r] = Av[r * rowv + g];
#pragma unroll
            for (int cc = 0; cc < 4; ++cc) bv[cc] = Bv[cc * rowv + g];
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
              for (int cc = 0; cc < 4; ++cc) sacc[r][cc] += G::dot(av[r], bv[cc]);
          }
        }
#pragma unroll
        for (int r = 0; r < 4; ++r)
#pragma unroll
          for (int cc = 0; cc < 4; ++cc) {
            if constexpr (sizeof(T) == 8) {
              hi[r][cc] += sacc[r][cc];
            } else {  // Neumaier: the rounding error of each addition goes to lo
              const T t = hi[r][cc] + sacc[r][cc];
              lo[r][cc] += fabsf(hi[r][cc]) >= fabsf(sacc[r][cc]) ? (hi[r][cc] - t) + sacc[r][cc]
                                                                  : (sacc[r][cc] - t) + hi[r][cc];
              hi[r][cc] = t;
            }
          }
      }
    }
    __syncthreads();  // buffer q is refilled by the next iteration's copies
  }
  cp_async_wait<0>();
  // FP64 sum over the TPT contiguous lanes of each tile group
  double v[4][4];
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int cc = 0; cc < 4; ++cc) v[r][cc] = (double)hi[r][cc] + (double)lo[r][cc];
  for (int off = TPT / 2; off > 0; off >>= 1)
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int cc = 0; cc < 4; ++cc) v[r][cc] += __shfl_down_sync(0xffffffffu, v[r][cc], off);
  if (act && lt == 0) {
    double* pb = part + (long long)blockIdx.x * a * b;
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
      for (int cc = 0; cc < 4; ++cc)
        if (i0 + r < a && j0 + cc < b) pb[(long long)(i0 + r) * b + j0 + cc] = v[r][cc];
  }
}

// out[e] (+)= sum over blocks of part[k][e]: one warp per output (lanes stride
// over the blocks, then a fixed-order shuffle tree: deterministic).
__global__ void gram_reduce_kernel(int nblocks, int ab, const double* __restrict__ part, double* __restrict__ out,
                                   int accumulate) {
  const int lane = threadIdx.x & 31;
  for (int e = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; e < ab; e += (gridDim.x * blockDim.x) >> 5) {
    double s = 0.0;
    for (int k = lane; k < nblocks; k += 32) s += part[(long long)k * ab + e];
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    if (lane == 0) out[e] = accumulate ? out[e] + s : s;
  }
}

constexpr int RTH = 256;

// out[j][p] (+)= sum_i A[i][p] C1[i][j] + sum_i B[i][p] C2[i][j] for j in
// [j0, j0 + RC); RC in {4, 8, 16, 32} is the smallest that covers c (or 32).
template <typename T, int RC>
__global__ void __launch_bounds__(RTH) rotate_kernel(long long n, int a, const T* __restrict__ A, long long sa,
                                                     const double* __restrict__ C1, int b, const T* __restrict__ B,
                                                     long long sb, const double* __restrict__ C2, int c,
                                                     T* __restrict__ out, long long so, int accumulate) {
  extern __shared__ __align__(16) unsigned char rsm[];
  T* cs = reinterpret_cast<T*>(rsm);  // (a + b) x RC
  const int j0 = blockIdx.y * RC;
  const int nj = min(RC, c - j0);
  for (int e = threadIdx.x; e < (a + b) * RC; e += RTH) {
    const int i = e / RC, jj = e - i * RC;
    double v = 0.0;
    if (jj < nj) v = i < a ? C1[(long long)i * c + j0 + jj] : C2[(long long)(i - a) * c + j0 + jj];
    cs[e] = T(v);
  }
  __syncthreads();
  for (long long p = blockIdx.x * (long long)RTH + threadIdx.x; p < n; p += (long long)gridDim.x * RTH) {
    T acc[RC];
#pragma unroll
    for (int jj = 0; jj < RC; ++jj) acc[jj] = T(0);
    // rows in batches of 8: the batch's loads are all in flight before its FMAs
    auto rows = [&](const T* __restrict__ M, long long sm, int m, const T* coef) {
      int i = 0;
      for (; i + 8 <= m; i += 8) {
        T x[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) x[u] = M[(long long)(i + u) * sm + p];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const T* row = coef + (i + u) * RC;
#pragma unroll
          for (int jj = 0; jj < RC; ++jj) acc[jj] += x[u] * row[jj];
        }
      }
      for (; i < m; ++i) {
        const T x = M[(long long)i * sm + p];
        const T* row = coef + i * RC;
#pragma unroll
        for (int jj = 0; jj < RC; ++jj) acc[jj] += x * row[jj];
      }
    };
    rows(A, sa, a, cs);
    if (b) rows(B, sb, b, cs + a * RC);
#pragma unroll
    for (int jj = 0; jj < RC; ++jj)
      if (jj < nj) {
        T* o = out + (long long)(j0 + jj) * so + p;
        *o = accumulate ? *o + acc[jj] : acc[jj];
      }
  }
}

template <typename T, int RC>
int rotate_launch(long long n, int a, const T* A, long long sa, const double* C1, int b, const T* B, long long sb,
                  const double* C2, int c, T* out, long long so, int accumulate, cudaStream_t st) {
  const size_t smem = (size_t)(a + b) * RC * sizeof(T);
  if (smem > 200 * 1024) return IGD_ERR_TOO_LARGE;
  if (ensure_dynamic_smem(reinterpret_cast<const void*>(rotate_kernel<T, RC>), smem) != IGD_OK) return IGD_ERR_CUDA;
  const long long blocks = std::min<long long>((n + RTH - 1) / RTH, 152LL * 8);
  dim3 grid((unsigned)blocks, (c + RC - 1) / RC);
  rotate_kernel<T, RC><<<grid, RTH, smem, st>>>(n, a, A, sa, C1, b, B, sb, C2, c, out, so, accumulate);
  return IGD_OK;
}

template <typename T>
int rotate_dispatch(long long n, int a, const T* A, long long sa, const double* C1, int b, const T* B, long long sb,
                    const double* C2, int c, T* out, long long so, int accumulate, cudaStream_t st) {
  if (c <= 4) return rotate_launch<T, 4>(n, a, A, sa, C1, b, B, sb, C2, c, out, so, accumulate, st);
  if (c <= 8) return rotate_launch<T, 8>(n, a, A, sa, C1, b, B, sb, C2, c, out, so, accumulate, st);
  if (c <= 16) return rotate_launch<T, 16>(n, a, A, sa, C1, b, B, sb, C2, c, out, so, accumulate, st);
  return rotate_launch<T, 32>(n, a, A, sa, C1, b, B, sb, C2, c, out, so, accumulate, st);
}

// Blocks (and per-block partials) of a Gram: one column slice of GTH x GPT
// points per block for the register-tiled kernel, a persistent grid of up to
// 608 blocks (4 per SM) for the pipelined one.
inline int gram_tiled_blocks(long long n) {
  const long long per = (long long)GTH * GPT;
  return (int)std::max<long long>(1, std::min<long long>((n + per - 1) / per, 4096));
}
inline int gram_pipe_blocks(long long n) { return (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 608)); }
inline int gram_blocks(long long n) { return std::max(gram_tiled_blocks(n), gram_pipe_blocks(n)); }

// Chunk length P (points, a power of two) and threads per output tile TPT of
// gram_pipe_kernel, with its shared-memory bytes; false when it does not apply
// (more than 64 x 64 outputs, unaligned rows, or no chunk fits 96 KB).
template <typename T>
bool gram_pipe_plan(int a, int b, const void* A, long long sa, const void* B, long long sb, const double* w, int* P,
                    int* TPT, size_t* smem) {
  constexpr int VW = 16 / (int)sizeof(T);
  auto al = [](const void* q) { return (reinterpret_cast<uintptr_t>(q) & 15u) == 0; };
  if (!al(A) || !al(B) || (w && !al(w)) || sa % VW != 0 || sb % VW != 0) return false;
  const int ap = (a + 3) & ~3, bp = (b + 3) & ~3, ntiles = (ap / 4) * (bp / 4);
  if (ntiles > GTH) return false;
  auto bytes = [&](int p) { return 2 * ((size_t)(ap + bp) * (p + VW) * sizeof(T) + (size_t)p * sizeof(double)); };
  int p = 256;
  while (p > 32 && bytes(p) > 96 * 1024) p >>= 1;
  if (bytes(p) > 96 * 1024) return false;
  int tpt = 32;
  while (tpt > 1 && (tpt * ntiles > GTH || p / VW < tpt)) tpt >>= 1;
  *P = p;
  *TPT = tpt;
  *smem = bytes(p);
  return true;
}

template <typename T>
int gram_pipe_launch(long long n, int a, int b, const T* A, long long sa, const T* B, long long sb, const double* w,
                     double* part, int nb, cudaStream_t st) {
  int P = 0, TPT = 0;
  size_t smem = 0;
  if (!gram_pipe_plan<T>(a, b, A, sa, B, sb, w, &P, &TPT, &smem)) return -1;
  if (ensure_dynamic_smem(reinterpret_cast<const void*>(gram_pipe_kernel<T>), smem) != IGD_OK) return IGD_ERR_CUDA;
  gram_pipe_kernel<T><<<nb, GTH, smem, st>>>(n, a, b, A, sa, B, sb, w, part, P, TPT);
  return IGD_OK;
}

// Damped Jacobi sweep for (T + sigma) t = r on k columns:
// first: t = dinv r; else t += omega dinv (r - tt - sigma t), tt = T t.
template <typename T>
__global__ void jacobi_kernel(long long n, int k, const T* __restrict__ r, long long sr, T* __restrict__ t,
                              long long st, const T* __restrict__ tt, long long stt, const T* __restrict__ dinv,
                              T sigma, T omega, int first) {
  const int c = blockIdx.y;  // one column per grid row: no division per element
  const T* rc = r + c * sr;
  T* tc = t + c * st;
  const T* ttc = first ? nullptr : tt + c * stt;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += (long long)gridDim.x * blockDim.x) {
    const T rv = rc[p], di = dinv[p];
    if (first)
      tc[p] = di * rv;
    else
      tc[p] += omega * di * (rv - ttc[p] - sigma * tc[p]);
  }
}

}  // namespace
}  // namespace igd

using namespace igd;

// Residual preconditioner step (see jacobi_kernel); dinv = 1 / (diag(T) + sigma).
extern "C" int igd_precond_jacobi(int dtype, long long n, int k, const void* r, long long sr, void* t, long long st,
                                  const void* tt, long long stt, const void* dinv, double sigma, double omega,
                                  int first, void* stream) {
  if (n <= 0 || k <= 0 || k > 65535 || !r || !t || !dinv || (!first && !tt)) return IGD_ERR_ARG;
  cudaStream_t s = as_stream(stream);
  const dim3 blocks((unsigned)std::max<long long>(1, std::min<long long>((n + 255) / 256, 152LL * 16 / k + 1)),
                    (unsigned)k);
  if (dtype == IGD_F32)
    jacobi_kernel<float><<<blocks, 256, 0, s>>>(n, k, static_cast<const float*>(r), sr, static_cast<float*>(t), st,
                                                static_cast<const float*>(tt), stt, static_cast<const float*>(dinv),
                                                (float)sigma, (float)omega, first);
  else if (dtype == IGD_F64)
    jacobi_kernel<double><<<blocks, 256, 0, s>>>(n, k, static_cast<const double*>(r), sr, static_cast<double*>(t), st,
                                                 static_cast<const double*>(tt), stt,
                                                 static_cast<const double*>(dinv), sigma, omega, first);
  else
    return IGD_ERR_DTYPE;
  return launch_status();
}

// Gram kernel choice for the calling host thread (tests): 0 automatic, 1 the
// tcgen05 kernel where it applies, 2 the pipelined CUDA-core kernel, 3 the
// register-tiled kernel.
extern "C" int igd_gram_select(int path) {
  if (path < 0 || path > 3) return IGD_ERR_ARG;
  g_gram_path = path;
  return IGD_OK;
}

// Kernel used by the calling thread's last igd_block_gram (0 before any call).
extern "C" int igd_gram_last_path(void) { return g_gram_last; }

extern "C" long long igd_block_gram_workspace_bytes(long long n, int a, int b) {
  if (n <= 0 || a <= 0 || b <= 0) return -1;
  return (long long)gram_blocks(n) * a * b * (long long)sizeof(double);
}

// out (a x b, FP64, row-major) [+]= A W B^T for row-major blocks A (a x n, row
// stride sa) and B (b x n, stride sb); w (n doubles) may be NULL.
extern "C" int igd_block_gram(int dtype, long long n, int a, const void* A, long long sa, int b, const void* B,
                              long long sb, const double* w, double* out, int accumulate, void* workspace,
                              long long workspace_bytes, void* stream) {
  if (n <= 0 || a <= 0 || b <= 0 || !A || !B || !out || !workspace) return IGD_ERR_ARG;
  if (workspace_bytes < igd_block_gram_workspace_bytes(n, a, b)) return IGD_ERR_ARG;
  if (dtype != IGD_F32 && dtype != IGD_F64) return IGD_ERR_DTYPE;
  cudaStream_t st = as_stream(stream);
  int nb = gram_pipe_blocks(n);
  double* part = static_cast<double*>(workspace);
  const int path = g_gram_path;
  // FP32: the tcgen05 3xTF32 kernel (outputs up to 64 x 64, 16-byte rows) on large grids
  if (dtype == IGD_F32 && (path == 1 || (path == 0 && n >= kGramTcMinPoints))) {
    const int r = gram_tc_launch(n, a, b, static_cast<const float*>(A), sa, static_cast<const float*>(B), sb, w, part,
                                 gram_blocks(n), device_error_word(), st);
    if (r > 0) {
      g_gram_last = 1;
      const int ab = a * b;
      gram_reduce_kernel<<<std::min((ab * 32 + 255) / 256, 1024), 256, 0, st>>>(r, ab, part, out, accumulate);
      return launch_status();
    }
    if (r != -1) return r;
  }
  // the pipelined kernel when rows are 16-byte aligned and outputs <= 64 x 64, else the register-tiled one
  const int e = path == 3 ? -1
                : dtype == IGD_F32 ? gram_pipe_launch<float>(n, a, b, static_cast<const float*>(A), sa,
                                                             static_cast<const float*>(B), sb, w, part, nb, st)
                                   : gram_pipe_launch<double>(n, a, b, static_cast<const double*>(A), sa,
                                                              static_cast<const double*>(B), sb, w, part, nb, st);
  if (e > 0) return e;
  if (e < 0) nb = gram_tiled_blocks(n);
  g_gram_last = e == 0 ? 2 : 3;
  if (e == 0) {
    // launched
  } else if (dtype == IGD_F32) {
    constexpr int TR = 4;
    dim3 grid(nb, ((a + TR - 1) / TR) * ((b + TR - 1) / TR));
    gram_tile_kernel<float, TR><<<grid, GTH, 0, st>>>(n, a, b, static_cast<const float*>(A), sa,
                                                      static_cast<const float*>(B), sb, w, part);
  } else {
    constexpr int TR = 4;
    dim3 grid(nb, ((a + TR - 1) / TR) * ((b + TR - 1) / TR));
    gram_tile_kernel<double, TR><<<grid, GTH, 0, st>>>(n, a, b, static_cast<const double*>(A), sa,
                                                       static_cast<const double*>(B), sb, w, part);
  }
  const int ab = a * b;
  gram_reduce_kernel<<<std::min((ab * 32 + 255) / 256, 1024), 256, 0, st>>>(nb, ab, part, out, accumulate);
  return launch_status();
}

// out (c x n, row stride so) [+]= A^T C1 + B^T C2 with FP64 coefficient matrices
// C1 (a x c) and C2 (b x c) on the device (B / C2 may be absent with b = 0).
// out must not alias A or B.
extern "C" int igd_block_rotate(int dtype, long long n, int a, const void* A, long long sa, const double* C1, int b,
                                const void* B, long long sb, const double* C2, int c, void* out, long long so,
                                int accumulate, void* stream) {
  if (n <= 0 || a < 0 || b < 0 || a + b == 0 || c <= 0 || !out || (a && (!A || !C1)) || (b && (!B || !C2)))
    return IGD_ERR_ARG;
  cudaStream_t st = as_stream(stream);
  int e;
  if (dtype == IGD_F32)
    e = rotate_dispatch<float>(n, a, static_cast<const float*>(A), sa, C1, b, static_cast<const float*>(B), sb, C2, c,
                               static_cast<float*>(out), so, accumulate, st);
  else if (dtype == IGD_F64)
    e = rotate_dispatch<double>(n, a, static_cast<const double*>(A), sa, C1, b, static_cast<const double*>(B), sb, C2,
                                c, static_cast<double*>(out), so, accumulate, st);
  else
    return IGD_ERR_DTYPE;
  if (e != IGD_OK) return e;
  return launch_status();
}

// Stream-ordered host-to-device copy of small coefficient matrices from pinned
// staging memory (one runtime call, none of a framework's dispatch).
extern "C" int igd_copy_h2d(void* dst, const void* src, long long bytes, void* stream) {
  if (!dst || !src || bytes < 0) return IGD_ERR_ARG;
  if (bytes == 0) return IGD_OK;
  return cudaMemcpyAsync(dst, src, (size_t)bytes, cudaMemcpyHostToDevice, as_stream(stream)) == cudaSuccess
             ? IGD_OK
             : IGD_ERR_CUDA;
}
