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

namespace igd {
namespace {

constexpr int GTH = 256;   // threads per Gram block
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

__global__ void gram_reduce_kernel(int nblocks, int ab, const double* __restrict__ part, double* __restrict__ out,
                                   int accumulate) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ab; e += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int k = 0; k < nblocks; ++k) s += part[(long long)k * ab + e];
    out[e] = accumulate ? out[e] + s : s;
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
    for (int i = 0; i < a; ++i) {
      const T x = A[(long long)i * sa + p];
      const T* row = cs + i * RC;
#pragma unroll
      for (int jj = 0; jj < RC; ++jj) acc[jj] += x * row[jj];
    }
    for (int i = 0; i < b; ++i) {
      const T x = B[(long long)i * sb + p];
      const T* row = cs + (a + i) * RC;
#pragma unroll
      for (int jj = 0; jj < RC; ++jj) acc[jj] += x * row[jj];
    }
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
  if (smem > 48 * 1024) {
    static bool raised = false;  // one attribute call per instantiation
    if (!raised) {
      if (cudaFuncSetAttribute(rotate_kernel<T, RC>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024) !=
          cudaSuccess)
        return IGD_ERR_CUDA;
      raised = true;
    }
  }
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

inline int gram_blocks(long long n) {
  const long long per = (long long)GTH * GPT;
  return (int)std::max<long long>(1, std::min<long long>((n + per - 1) / per, 4096));
}

// Damped Jacobi sweep for (T + sigma) t = r on k columns:
// first: t = dinv r; else t += omega dinv (r - tt - sigma t), tt = T t.
template <typename T>
__global__ void jacobi_kernel(long long n, int k, const T* __restrict__ r, long long sr, T* __restrict__ t,
                              long long st, const T* __restrict__ tt, long long stt, const T* __restrict__ dinv,
                              T sigma, T omega, int first) {
  const long long total = n * k;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(e / n);
    const long long p = e - (long long)c * n;
    const T rv = r[c * sr + p], di = dinv[p];
    T* tp = t + c * st + p;
    if (first)
      *tp = di * rv;
    else
      *tp += omega * di * (rv - tt[c * stt + p] - sigma * *tp);
  }
}

}  // namespace
}  // namespace igd

using namespace igd;

// Residual preconditioner step (see jacobi_kernel); dinv = 1 / (diag(T) + sigma).
extern "C" int igd_precond_jacobi(int dtype, long long n, int k, const void* r, long long sr, void* t, long long st,
                                  const void* tt, long long stt, const void* dinv, double sigma, double omega,
                                  int first, void* stream) {
  if (n <= 0 || k <= 0 || !r || !t || !dinv || (!first && !tt)) return IGD_ERR_ARG;
  cudaStream_t s = as_stream(stream);
  const int blocks = (int)std::min<long long>((n * k + 255) / 256, 152LL * 16);
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
  const int nb = gram_blocks(n);
  double* part = static_cast<double*>(workspace);
  if (dtype == IGD_F32) {
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
  gram_reduce_kernel<<<(ab + 255) / 256, 256, 0, st>>>(nb, ab, part, out, accumulate);
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
