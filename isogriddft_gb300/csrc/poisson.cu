// Open-boundary Poisson interior solve (K4): BiCGSTAB with device-resident
// scalars, FP64 or FP32-inner + FP64 iterative refinement.
//
// Solves -L u = f on the interior with u = 0 on the six faces, where L is the
// monitor-grid Laplacian with the np.gradient closure (the operator of
// poisson/open_boundary.py:1017-1064, applied through igd_hpsi_agrid with
// kscale = -1) or the legacy 7-point Laplacian (open_boundary.py:1216-1226,
// through igd_hpsi_legacy).  Convergence is the SciPy rule the reference uses:
// ||r||_2 <= rtol ||f||_2 with x0 = 0.  Every vector is a full (nx, ny, nz)
// field whose face entries are kept at zero.
#include <cmath>
#include <cstring>
#include <vector>

#include "common.cuh"

namespace igd {

// hpsi entry points used as the operator (declared in isogrid_gb300.h).

namespace {

constexpr int PB = 256;

struct KState {
  double rho, rho_prev, alpha, omega;
  double acc_rv, acc_ss, acc_ts, acc_tt, acc_rr, acc_rhr;
  double bnorm2, rnorm2;
  int iters, done, status, pad;
};

// Grids of this solver have fewer than 2^31 points (checked at entry), so
// the face test uses 32-bit unsigned division.
__device__ __forceinline__ bool on_face(long long i, int nx, int ny, int nz) {
  const unsigned pl = (unsigned)ny * (unsigned)nz, ii = (unsigned)i;
  const unsigned x = ii / pl, r = ii - x * pl;
  const unsigned y = r / (unsigned)nz, z = r - y * (unsigned)nz;
  return x == 0 || x == (unsigned)nx - 1 || y == 0 || y == (unsigned)ny - 1 || z == 0 || z == (unsigned)nz - 1;
}

// Block-level FP64 sums, one atomic per block and accumulator (a per-warp
// atomic on one address serialises thousands of updates per reduction).
__device__ __forceinline__ void acc_add(double* dst, double v) {
  __shared__ double scratch[PB / 32];
  double a[1] = {v};
  block_sum<1, PB>(a, scratch);
  if (threadIdx.x == 0) atomicAdd(dst, a[0]);
}

__device__ __forceinline__ void acc_add2(double* d0, double v0, double* d1, double v1) {
  __shared__ double scratch[2 * (PB / 32)];
  double a[2] = {v0, v1};
  block_sum<2, PB>(a, scratch);
  if (threadIdx.x == 0) {
    atomicAdd(d0, a[0]);
    atomicAdd(d1, a[1]);
  }
}

inline int pblocks(long long n) { return (int)std::min<long long>((n + PB - 1) / PB, 152LL * 4); }

// r = f (masked), rhat = r, p = v = 0, x = 0; bnorm2 = ||f||^2.
template <typename T>
__global__ void k_init(long long n, int nx, int ny, int nz, const T* __restrict__ f, T* x, T* r, T* rh, T* p, T* v,
                       KState* s) {
  double a = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const T fi = on_face(i, nx, ny, nz) ? T(0) : f[i];
    r[i] = fi;
    rh[i] = fi;
    p[i] = T(0);
    v[i] = T(0);
    x[i] = T(0);
    a += (double)fi * (double)fi;
  }
  acc_add(&s->bnorm2, a);
}

__global__ void k_state_init(KState* s) {
  memset(s, 0, sizeof(KState));
  s->rho = s->rho_prev = s->alpha = s->omega = 1.0;
}

// After init: rho = rhat.r = bnorm2; done if ||f|| == 0.
__global__ void k_after_init(KState* s, double rtol) {
  s->rho = s->bnorm2;
  s->rnorm2 = s->bnorm2;
  s->acc_rhr = s->bnorm2;
  if (s->bnorm2 == 0.0) s->done = 1;
}

// p = r + beta (p - omega v), beta = (rho / rho_prev) (alpha / omega); zero acc_rv.
// (faces stay zero: v = A p carries stencil values on the faces)
template <typename T>
__global__ void k_update_p(long long n, int nx, int ny, int nz, const T* __restrict__ r, T* __restrict__ p,
                           const T* __restrict__ v, const KState* s) {
  if (s->done) return;
  const double beta = (s->rho / s->rho_prev) * (s->alpha / s->omega);
  const T b = T(beta), om = T(s->omega);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    p[i] = on_face(i, nx, ny, nz) ? T(0) : r[i] + b * (p[i] - om * v[i]);
}

// acc_rv = rhat . v over the interior (rhat is zero on faces).
template <typename T>
__global__ void k_dot_rv(long long n, const T* __restrict__ rh, const T* __restrict__ v, KState* s) {
  if (s->done) return;
  double a = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    a += (double)rh[i] * (double)v[i];
  acc_add(&s->acc_rv, a);
}

__global__ void k_alpha(KState* s) {
  if (s->done) return;
  if (!(fabs(s->acc_rv) > 1e-300) || !isfinite(s->acc_rv)) {
    s->status = IGD_ERR_BREAKDOWN;
    s->done = 1;
    return;
  }
  s->alpha = s->rho / s->acc_rv;
  s->acc_ss = s->acc_ts = s->acc_tt = 0.0;
}

// s_vec = r - alpha v (faces zero); acc_ss.
template <typename T>
__global__ void k_update_s(long long n, int nx, int ny, int nz, const T* __restrict__ r, const T* __restrict__ v,
                           T* __restrict__ sv, KState* s) {
  if (s->done) return;
  const T al = T(s->alpha);
  double a = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const T val = on_face(i, nx, ny, nz) ? T(0) : r[i] - al * v[i];
    sv[i] = val;
    a += (double)val * (double)val;
  }
  acc_add(&s->acc_ss, a);
}

// acc_ts = t.s, acc_tt = t.t over the interior.
template <typename T>
__global__ void k_dot_ts(long long n, int nx, int ny, int nz, const T* __restrict__ t, const T* __restrict__ sv,
                         KState* s) {
  if (s->done) return;
  double a = 0.0, b = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    if (on_face(i, nx, ny, nz)) continue;
    const double ti = (double)t[i];
    a += ti * (double)sv[i];
    b += ti * ti;
  }
  acc_add2(&s->acc_ts, a, &s->acc_tt, b);
}

__global__ void k_omega(KState* s) {
  if (s->done) return;
  if (!(s->acc_tt > 0.0) || !isfinite(s->acc_tt)) {
    s->status = IGD_ERR_BREAKDOWN;
    s->done = 1;
    return;
  }
  s->omega = s->acc_ts / s->acc_tt;
  s->acc_rr = s->acc_rhr = 0.0;
}

// x += alpha p + omega s; r = s - omega t (faces zero); acc_rr, acc_rhr.
template <typename T>
__global__ void k_update_xr(long long n, int nx, int ny, int nz, T* __restrict__ x, T* __restrict__ r,
                            const T* __restrict__ p, const T* __restrict__ sv, const T* __restrict__ t,
                            const T* __restrict__ rh, KState* s) {
  if (s->done) return;
  const T al = T(s->alpha), om = T(s->omega);
  double a = 0.0, b = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const bool f = on_face(i, nx, ny, nz);
    x[i] = f ? T(0) : x[i] + al * p[i] + om * sv[i];
    const T ri = f ? T(0) : sv[i] - om * t[i];
    r[i] = ri;
    a += (double)ri * (double)ri;
    b += (double)rh[i] * (double)ri;
  }
  acc_add2(&s->acc_rr, a, &s->acc_rhr, b);
}

__global__ void k_next(KState* s, double rtol2, int maxit) {
  if (s->done) return;
  s->iters += 1;
  s->rnorm2 = s->acc_rr;
  s->rho_prev = s->rho;
  s->rho = s->acc_rhr;
  s->acc_rv = 0.0;
  if (!isfinite(s->acc_rr)) {
    s->status = IGD_ERR_NONFINITE;
    s->done = 1;
  } else if (s->acc_rr <= rtol2 * s->bnorm2) {
    s->done = 1;
  } else if (!(fabs(s->rho) > 1e-300) || s->omega == 0.0) {
    s->status = IGD_ERR_BREAKDOWN;
    s->done = 1;
  } else if (s->iters >= maxit) {
    s->status = IGD_ERR_NOT_CONVERGED;
    s->done = 1;
  }
}


// ---- 16-byte vector forms of the per-iteration kernels (nz a multiple of the
// vector width, so one vector never crosses a grid row; 16-byte aligned data).
// Each thread sums its few vectors in the data type (FP32 inside the mixed
// solve: GB300's FP64 pipe would otherwise bound these kernels) and hands one
// FP64 value to the block reduction.
template <typename T>
struct VecT;
template <>
struct VecT<float> {
  using V = float4;
  static constexpr int E = 4;
};
template <>
struct VecT<double> {
  using V = double2;
  static constexpr int E = 2;
};

template <typename T>
__device__ __forceinline__ void ldv(const T* __restrict__ p, long long v, T (&o)[VecT<T>::E]) {
  const typename VecT<T>::V q = reinterpret_cast<const typename VecT<T>::V*>(p)[v];
  memcpy(o, &q, sizeof(q));
}
template <typename T>
__device__ __forceinline__ void stv(T* __restrict__ p, long long v, const T (&o)[VecT<T>::E]) {
  typename VecT<T>::V q;
  memcpy(&q, o, sizeof(q));
  reinterpret_cast<typename VecT<T>::V*>(p)[v] = q;
}
// Face flags of the E elements of vector v (bit e set: element e on a face).
template <int E>
__device__ __forceinline__ unsigned face_bits(long long v, int nx, int ny, int nz) {
  const unsigned i = (unsigned)(v * E), pl = (unsigned)ny * (unsigned)nz;
  const unsigned x = i / pl, r = i - x * pl, y = r / (unsigned)nz, z0 = r - y * (unsigned)nz;
  if (x == 0 || x == (unsigned)nx - 1 || y == 0 || y == (unsigned)ny - 1) return (1u << E) - 1u;
  unsigned b = 0;
  if (z0 == 0) b |= 1u;
  if (z0 + E == (unsigned)nz) b |= 1u << (E - 1);
  return b;
}

template <typename T>
__global__ void kv_update_p(long long nv, int nx, int ny, int nz, const T* __restrict__ r, T* __restrict__ p,
                            const T* __restrict__ v, const KState* s) {
  constexpr int E = VecT<T>::E;
  if (s->done) return;
  const double beta = (s->rho / s->rho_prev) * (s->alpha / s->omega);
  const T b = T(beta), om = T(s->omega);
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < nv; q += (long long)gridDim.x * blockDim.x) {
    T rr[E], pp[E], vv[E];
    ldv(r, q, rr);
    ldv(p, q, pp);
    ldv(v, q, vv);
    const unsigned f = face_bits<E>(q, nx, ny, nz);
#pragma unroll
    for (int e = 0; e < E; ++e) pp[e] = (f >> e) & 1u ? T(0) : rr[e] + b * (pp[e] - om * vv[e]);
    stv(p, q, pp);
  }
}

template <typename T>
__global__ void kv_dot_rv(long long nv, const T* __restrict__ rh, const T* __restrict__ v, KState* s) {
  constexpr int E = VecT<T>::E;
  if (s->done) return;
  T a = T(0);  // per-thread sum of a few vectors in the data type; FP64 across threads
#pragma unroll 4
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < nv; q += (long long)gridDim.x * blockDim.x) {
    T x[E], y[E];
    ldv(rh, q, x);
    ldv(v, q, y);
#pragma unroll
    for (int e = 0; e < E; ++e) a += x[e] * y[e];
  }
  acc_add(&s->acc_rv, (double)a);
}

template <typename T>
__global__ void kv_update_s(long long nv, int nx, int ny, int nz, const T* __restrict__ r, const T* __restrict__ v,
                            T* __restrict__ sv, KState* s) {
  constexpr int E = VecT<T>::E;
  if (s->done) return;
  const T al = T(s->alpha);
  T a = T(0);
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < nv; q += (long long)gridDim.x * blockDim.x) {
    T rr[E], vv[E], o[E];
    ldv(r, q, rr);
    ldv(v, q, vv);
    const unsigned f = face_bits<E>(q, nx, ny, nz);
#pragma unroll
    for (int e = 0; e < E; ++e) {
      o[e] = (f >> e) & 1u ? T(0) : rr[e] - al * vv[e];
      a += o[e] * o[e];
    }
    stv(sv, q, o);
  }
  acc_add(&s->acc_ss, (double)a);
}

template <typename T>
__global__ void kv_dot_ts(long long nv, int nx, int ny, int nz, const T* __restrict__ t, const T* __restrict__ sv,
                          KState* s) {
  constexpr int E = VecT<T>::E;
  if (s->done) return;
  T a = T(0), b = T(0);
#pragma unroll 2
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < nv; q += (long long)gridDim.x * blockDim.x) {
    T tt[E], ss[E];
    ldv(t, q, tt);
    ldv(sv, q, ss);
    const unsigned f = face_bits<E>(q, nx, ny, nz);
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const T ti = (f >> e) & 1u ? T(0) : tt[e];
      a += ti * ss[e];
      b += ti * ti;
    }
  }
  acc_add2(&s->acc_ts, (double)a, &s->acc_tt, (double)b);
}

template <typename T>
__global__ void kv_update_xr(long long nv, int nx, int ny, int nz, T* __restrict__ x, T* __restrict__ r,
                             const T* __restrict__ p, const T* __restrict__ sv, const T* __restrict__ t,
                             const T* __restrict__ rh, KState* s) {
  constexpr int E = VecT<T>::E;
  if (s->done) return;
  const T al = T(s->alpha), om = T(s->omega);
  T a = T(0), b = T(0);
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < nv; q += (long long)gridDim.x * blockDim.x) {
    T xx[E], pp[E], ss[E], tt[E], hh[E], rr[E];
    ldv(x, q, xx);
    ldv(p, q, pp);
    ldv(sv, q, ss);
    ldv(t, q, tt);
    ldv(rh, q, hh);
    const unsigned f = face_bits<E>(q, nx, ny, nz);
#pragma unroll
    for (int e = 0; e < E; ++e) {
      const bool fc = (f >> e) & 1u;
      xx[e] = fc ? T(0) : xx[e] + al * pp[e] + om * ss[e];
      rr[e] = fc ? T(0) : ss[e] - om * tt[e];
      a += rr[e] * rr[e];
      b += hh[e] * rr[e];
    }
    stv(x, q, xx);
    stv(r, q, rr);
  }
  acc_add2(&s->acc_rr, (double)a, &s->acc_rhr, (double)b);
}

// residual res = f - A u (faces zero); accumulates ||res||^2 and max |res|.
__global__ void k_residual(long long n, int nx, int ny, int nz, const double* __restrict__ f,
                           const double* __restrict__ Au, double* __restrict__ res, double* norm2,
                           unsigned long long* maxabs) {
  double a = 0.0, m = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double ri = on_face(i, nx, ny, nz) ? 0.0 : f[i] - Au[i];
    res[i] = ri;
    a += ri * ri;
    m = fmax(m, fabs(ri));
  }
  m = warp_max(m);
  if ((threadIdx.x & 31) == 0) atomicMax(maxabs, (unsigned long long)__double_as_longlong(m));  // m >= 0
  acc_add(norm2, a);
}

__global__ void k_cast_scaled(long long n, const double* __restrict__ a, float* __restrict__ b, double scale) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    b[i] = (float)(a[i] * scale);
}

__global__ void k_axpy_masked(long long n, int nx, int ny, int nz, double* __restrict__ x, const float* __restrict__ d,
                              double scale) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    x[i] = on_face(i, nx, ny, nz) ? 0.0 : x[i] + scale * (double)d[i];
}

struct Problem {
  int kind, nx, ny, nz;
  long long n;
  const void* c64;
  const void* c32;
  cudaStream_t st;
};

template <typename T>
int apply_op(const Problem& P, const T* x, T* y) {
  const int dt = sizeof(T) == 8 ? IGD_F64 : IGD_F32;
  if (P.kind == IGD_GRID_MONITOR)
    return igd_hpsi_agrid(dt, IGD_CLOSURE_PRODUCTION, P.nx, P.ny, P.nz, sizeof(T) == 8 ? P.c64 : P.c32, nullptr, x, y,
                          1, P.n, -1.0, 0.0, P.st);
  return igd_hpsi_legacy(dt, P.nx, P.ny, P.nz, static_cast<const double*>(P.c64), nullptr, x, y, 1, P.n, -1.0, 0.0,
                         P.st);
}

template <typename T>
size_t krylov_bytes(long long n) {
  return 6 * (size_t)n * sizeof(T) + 256;
}

// A private non-blocking stream per host thread and device for graph capture
// (the caller's stream may be the legacy default stream, which cannot be
// captured; solves on several threads capture concurrently).
cudaStream_t capture_stream() {
  static thread_local cudaStream_t streams[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  if (!streams[dev] && cudaStreamCreateWithFlags(&streams[dev], cudaStreamNonBlocking) != cudaSuccess)
    streams[dev] = nullptr;
  return streams[dev];
}

// BiCGSTAB on T vectors: solves A x = f (x0 = 0).  Returns a status; iters / rel set.
template <typename T>
int bicgstab(const Problem& P, const T* f, T* x, double rtol, int maxit, unsigned char* ws, int* iters, double* rel,
             double* bnorm = nullptr) {
  const long long n = P.n;
  T* r = reinterpret_cast<T*>(ws);
  T *rh = r + n, *p = rh + n, *v = p + n, *sv = v + n, *t = sv + n;
  KState* S = reinterpret_cast<KState*>(ws + 6 * (size_t)n * sizeof(T));
  const int nb = pblocks(n);
  cudaStream_t st = P.st;
  k_state_init<<<1, 1, 0, st>>>(S);
  k_init<T><<<nb, PB, 0, st>>>(n, P.nx, P.ny, P.nz, f, x, r, rh, p, v, S);
  k_after_init<<<1, 1, 0, st>>>(S, rtol);
  const double rtol2 = rtol * rtol;
  KState h;
  const int chunk = 8;
  constexpr int E = VecT<T>::E;
  const auto al16 = [](const void* q) { return (reinterpret_cast<uintptr_t>(q) & 15u) == 0; };
  const bool vec = P.nz % E == 0 && al16(x) && al16(r) && al16(rh) && al16(p) && al16(v) && al16(sv) && al16(t);
  const long long nv = n / E;
  const int nbv = pblocks(nv);
  // One chunk of `chunk` iterations on stream q (direct launches or graph capture).
  auto issue_chunk = [&](cudaStream_t q) -> int {
    Problem Q = P;
    Q.st = q;
    for (int c = 0; c < chunk; ++c) {
      if (vec)
        kv_update_p<T><<<nbv, PB, 0, q>>>(nv, P.nx, P.ny, P.nz, r, p, v, S);
      else
        k_update_p<T><<<nb, PB, 0, q>>>(n, P.nx, P.ny, P.nz, r, p, v, S);
      int e = apply_op<T>(Q, p, v);
      if (e) return e;
      if (vec)
        kv_dot_rv<T><<<nbv, PB, 0, q>>>(nv, rh, v, S);
      else
        k_dot_rv<T><<<nb, PB, 0, q>>>(n, rh, v, S);
      k_alpha<<<1, 1, 0, q>>>(S);
      if (vec)
        kv_update_s<T><<<nbv, PB, 0, q>>>(nv, P.nx, P.ny, P.nz, r, v, sv, S);
      else
        k_update_s<T><<<nb, PB, 0, q>>>(n, P.nx, P.ny, P.nz, r, v, sv, S);
      e = apply_op<T>(Q, sv, t);
      if (e) return e;
      if (vec)
        kv_dot_ts<T><<<nbv, PB, 0, q>>>(nv, P.nx, P.ny, P.nz, t, sv, S);
      else
        k_dot_ts<T><<<nb, PB, 0, q>>>(n, P.nx, P.ny, P.nz, t, sv, S);
      k_omega<<<1, 1, 0, q>>>(S);
      if (vec)
        kv_update_xr<T><<<nbv, PB, 0, q>>>(nv, P.nx, P.ny, P.nz, x, r, p, sv, t, rh, S);
      else
        k_update_xr<T><<<nb, PB, 0, q>>>(n, P.nx, P.ny, P.nz, x, r, p, sv, t, rh, S);
      k_next<<<1, 1, 0, q>>>(S, rtol2, maxit);
    }
    return 0;
  };
  // After a first direct chunk (first-call set-up of every kernel happens outside
  // a capture), later chunks replay a CUDA graph of one chunk captured on a
  // private stream: one launch instead of ~10 per iteration.  Falls back to
  // direct launches if capture is unavailable.
  cudaGraphExec_t gexec = nullptr;
  struct GraphGuard {
    cudaGraphExec_t* e;
    ~GraphGuard() {
      if (*e) cudaGraphExecDestroy(*e);
    }
  } guard{&gexec};
  for (int done_iters = 0;;) {
    if (done_iters == chunk && !gexec) {
      cudaStream_t cs = capture_stream();
      cudaGraph_t graph = nullptr;
      if (cs && cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
        const int e = issue_chunk(cs);
        const cudaError_t ce = cudaStreamEndCapture(cs, &graph);
        if (e == 0 && ce == cudaSuccess && graph) {
          if (cudaGraphInstantiate(&gexec, graph, 0) != cudaSuccess) gexec = nullptr;
        }
        if (graph) cudaGraphDestroy(graph);
      }
      cudaGetLastError();  // a failed capture leaves no sticky error; clear the last one
    }
    if (gexec) {
      if (cudaGraphLaunch(gexec, st) != cudaSuccess) return IGD_ERR_CUDA;
    } else {
      const int e = issue_chunk(st);
      if (e) return e;
    }

    if (cudaMemcpyAsync(&h, S, sizeof(KState), cudaMemcpyDeviceToHost, st) != cudaSuccess) return IGD_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return IGD_ERR_CUDA;
    done_iters += chunk;
    if (h.done || done_iters > maxit + chunk) break;
  }
  *iters = h.iters;
  *rel = h.bnorm2 > 0 ? std::sqrt(h.rnorm2 / h.bnorm2) : 0.0;
  if (bnorm) *bnorm = std::sqrt(h.bnorm2);
  return h.status == IGD_ERR_NOT_CONVERGED ? IGD_OK : h.status;  // non-convergence is reported via rel
}

// ---- Fused FP32 BiCGSTAB for the monitor-grid operator of the whole-row
// kernel (hpsi_agrid_krylov): the operator writes zero faces and returns the
// dot products r^.v, t.s and t.t from its epilogue, so every vector keeps zero
// faces without masks, and the scalars alpha, beta, omega and the stopping
// test are recomputed by the vector kernels from rotating banks of sums:
// iteration j of a chunk accumulates into bank j % 4, reads banks j-1 and j-2,
// and its first kernel clears bank j+1 (chunks are a multiple of 4 long).
// Per iteration: p update, v = A p (+ r^.v), s update, t = A s (+ t.s, t.t),
// x / r update (+ r.r, r^.r): five launches, no single-thread kernels.
// The arithmetic is the same BiCGSTAB as bicgstab<T> above.
enum { B_RV = 0, B_VV = 1, B_TS = 2, B_TT = 3, B_RR = 4, B_RHR = 5, B_N = 6 };
struct FState {
  double bnorm2;
  double bank[4][B_N];
  int done, stop, status, chunk, base, pad[3];
};
static_assert(sizeof(FState) <= 256, "FState must fit the 256-byte state slot of the Krylov workspace");

__global__ void kf_state_init(FState* s) { memset(s, 0, sizeof(FState)); }

// r = rhat = f (faces zero), x = p = v = 0; bnorm2 = ||f||^2
__global__ void kf_init(long long nv, int nx, int ny, int nz, const float* __restrict__ f, float* x, float* r,
                        float* rh, float* p, float* v, FState* s) {
  float a = 0.f;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < nv; q += (long long)gridDim.x * blockDim.x) {
    float ff[4];
    ldv<float>(f, q, ff);
    const unsigned fb = face_bits<4>(q, nx, ny, nz);
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      ff[e] = (fb >> e) & 1u ? 0.f : ff[e];
      a += ff[e] * ff[e];
    }
    const float z[4] = {0.f, 0.f, 0.f, 0.f};
    stv<float>(r, q, ff);
    stv<float>(rh, q, ff);
    stv<float>(x, q, z);
    stv<float>(p, q, z);
    stv<float>(v, q, z);
  }
  acc_add(&s->bnorm2, (double)a);
}

// bank 3 stands for iteration -1: rho_0 = r^.r_0 = ||f||^2 = ||r_0||^2
__global__ void kf_after_init(FState* s) {
  s->bank[3][B_RR] = s->bnorm2;
  s->bank[3][B_RHR] = s->bnorm2;
  if (s->bnorm2 == 0.0) s->done = 1;
}

__global__ void kf_chunk_begin(FState* s, int chunk_len) {
  if (s->done) return;
  s->base = s->chunk * chunk_len;
  s->chunk += 1;
}

// every block reaches the same decision; one thread records it
__device__ __forceinline__ void f_stop(FState* s, int j, int status) {
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    s->status = status;
    s->stop = j;
    s->done = 1;
  }
}

// Iteration j, part 1: the stopping test on the previous iteration (k_next of
// bicgstab<T>), then p = r + beta (p - omega v), beta = (rho_k / rho_{k-1})
// (alpha_{k-1} / omega_{k-1}) (p = r on the first iteration); clears bank j+1.
__global__ void kf_p(long long nv, const float* __restrict__ r, float* __restrict__ p, const float* __restrict__ v,
                     FState* s, int j, double rtol2, int maxit) {
  // the scalar work (FP64 divisions, slow on GB300's FP64 pipe) once per block;
  // stop: -1 go on, -2 stopped before, else the status this iteration stops with
  __shared__ float sc[2];
  __shared__ int stop;
  if (threadIdx.x == 0) {
    int st = -1;
    float bt = 0.f, om = 0.f;
    if (s->done) {
      st = -2;
    } else {
      const double* b1 = s->bank[(j + 3) & 3];  // iteration j - 1
      const double* b2 = s->bank[(j + 2) & 3];  // iteration j - 2
      const int k = s->base + j;                // iterations completed
      const double rr = b1[B_RR];
      if (!isfinite(rr)) {
        st = IGD_ERR_NONFINITE;
      } else if (k > 0 && rr <= rtol2 * s->bnorm2) {
        st = IGD_OK;
      } else {
        if (k > 0) {
          const double rho = b1[B_RHR], rho_prev = b2[B_RHR];
          const double alpha = rho_prev / b1[B_RV], omega = b1[B_TS] / b1[B_TT];
          if (!(fabs(rho) > 1e-300) || omega == 0.0) st = IGD_ERR_BREAKDOWN;
          bt = (float)((rho / rho_prev) * (alpha / omega));
          om = (float)omega;
        }
        if (st < 0 && k >= maxit) st = IGD_ERR_NOT_CONVERGED;
      }
      if (st >= 0) f_stop(s, j, st);  // every block decides alike; block 0 records it
    }
    stop = st;
    sc[0] = bt;
    sc[1] = om;
  }
  __syncthreads();
  if (stop != -1) return;
  const float bt = sc[0], om = sc[1];
  if (blockIdx.x == 0 && threadIdx.x < B_N) s->bank[(j + 1) & 3][threadIdx.x] = 0.0;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < nv; q += (long long)gridDim.x * blockDim.x) {
    float rr4[4], pp[4], vv[4];
    ldv<float>(r, q, rr4);
    ldv<float>(p, q, pp);
    ldv<float>(v, q, vv);
#pragma unroll
    for (int e = 0; e < 4; ++e) pp[e] = rr4[e] + bt * (pp[e] - om * vv[e]);
    stv<float>(p, q, pp);
  }
}

// Part 2 (after v = A p and r^.v): alpha = rho_k / r^.v; s = r - alpha v.
__global__ void kf_s(long long nv, const float* __restrict__ r, const float* __restrict__ v, float* __restrict__ sv,
                     FState* s, int j) {
  __shared__ float sal;
  __shared__ int go;
  if (threadIdx.x == 0) {
    go = 0;
    if (!s->done) {
      const double rv = s->bank[j & 3][B_RV];
      if (!(fabs(rv) > 1e-300) || !isfinite(rv)) {
        f_stop(s, j, IGD_ERR_BREAKDOWN);
      } else {
        sal = (float)(s->bank[(j + 3) & 3][B_RHR] / rv);
        go = 1;
      }
    }
  }
  __syncthreads();
  if (!go) return;
  const float al = sal;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < nv; q += (long long)gridDim.x * blockDim.x) {
    float rr4[4], vv[4], o[4];
    ldv<float>(r, q, rr4);
    ldv<float>(v, q, vv);
#pragma unroll
    for (int e = 0; e < 4; ++e) o[e] = rr4[e] - al * vv[e];
    stv<float>(sv, q, o);
  }
}

// Part 3 (after t = A s, t.s, t.t): omega = t.s / t.t; x += alpha p + omega s;
// r = s - omega t; r.r and r^.r into bank j.
__global__ void kf_xr(long long nv, float* __restrict__ x, float* __restrict__ r, const float* __restrict__ p,
                      const float* __restrict__ sv, const float* __restrict__ t, const float* __restrict__ rh,
                      FState* s, int j) {
  double* b0 = s->bank[j & 3];
  __shared__ float sc[2];
  __shared__ int go;
  if (threadIdx.x == 0) {
    go = 0;
    if (!s->done) {
      const double tt = b0[B_TT];
      if (!(tt > 0.0) || !isfinite(tt)) {
        f_stop(s, j, IGD_ERR_BREAKDOWN);
      } else {
        sc[0] = (float)(s->bank[(j + 3) & 3][B_RHR] / b0[B_RV]);
        sc[1] = (float)(b0[B_TS] / tt);
        go = 1;
      }
    }
  }
  __syncthreads();
  if (!go) return;
  const float al = sc[0], om = sc[1];
  float a = 0.f, b = 0.f;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < nv; q += (long long)gridDim.x * blockDim.x) {
    float xx[4], pp[4], ss[4], tv[4], hh[4], ro[4];
    ldv<float>(x, q, xx);
    ldv<float>(p, q, pp);
    ldv<float>(sv, q, ss);
    ldv<float>(t, q, tv);
    ldv<float>(rh, q, hh);
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      xx[e] = xx[e] + al * pp[e] + om * ss[e];
      ro[e] = ss[e] - om * tv[e];
      a += ro[e] * ro[e];
      b += hh[e] * ro[e];
    }
    stv<float>(x, q, xx);
    stv<float>(r, q, ro);
  }
  acc_add2(&b0[B_RR], (double)a, &b0[B_RHR], (double)b);
}

// igd_poisson_select: 0 = the fused FP32 path wherever it applies, 1 = never (per host thread).
thread_local int g_poisson_path = 0;
bool fused_poisson_enabled() { return g_poisson_path == 0; }

// The fused path applies: monitor grid, FP32 whole-row operator, 16-byte vectors.
bool fused_applies(const Problem& P, const void* a, const void* b, const void* ws) {
  const auto al16 = [](const void* q) { return (reinterpret_cast<uintptr_t>(q) & 15u) == 0; };
  return P.kind == IGD_GRID_MONITOR && P.c32 && hpsi_agrid_krylov_applies(P.nz, P.c32) && P.n % 4 == 0 && al16(a) &&
         al16(b) && al16(ws);
}

int bicgstab_fused(const Problem& P, const float* f, float* x, double rtol, int maxit, unsigned char* ws, int* iters,
                   double* rel) {
  const long long n = P.n, nv = n / 4;
  float* r = reinterpret_cast<float*>(ws);
  float *rh = r + n, *p = rh + n, *v = p + n, *sv = v + n, *t = sv + n;
  FState* S = reinterpret_cast<FState*>(ws + 6 * (size_t)n * sizeof(float));
  const float* c32 = static_cast<const float*>(P.c32);
  const int nbv = pblocks(nv);
  cudaStream_t st = P.st;
  kf_state_init<<<1, 1, 0, st>>>(S);
  kf_init<<<nbv, PB, 0, st>>>(nv, P.nx, P.ny, P.nz, f, x, r, rh, p, v, S);
  kf_after_init<<<1, 1, 0, st>>>(S);
  const double rtol2 = rtol * rtol;
  constexpr int chunk = 8;  // a multiple of the 4 banks
  auto issue_chunk = [&](cudaStream_t q) -> int {
    kf_chunk_begin<<<1, 1, 0, q>>>(S, chunk);
    for (int j = 0; j < chunk; ++j) {
      double* bank = S->bank[j & 3];
      kf_p<<<nbv, PB, 0, q>>>(nv, r, p, v, S, j, rtol2, maxit);
      int e = hpsi_agrid_krylov(P.nx, P.ny, P.nz, c32, p, v, -1.0, rh, bank + B_RV, &S->done, q);
      if (e) return e < 0 ? IGD_ERR_ARG : e;
      kf_s<<<nbv, PB, 0, q>>>(nv, r, v, sv, S, j);
      e = hpsi_agrid_krylov(P.nx, P.ny, P.nz, c32, sv, t, -1.0, nullptr, bank + B_TS, &S->done, q);
      if (e) return e < 0 ? IGD_ERR_ARG : e;
      kf_xr<<<nbv, PB, 0, q>>>(nv, x, r, p, sv, t, rh, S, j);
    }
    return launch_status();
  };
  // the first chunk runs directly (first-call set-up outside any capture), later
  // ones replay one captured chunk (one launch instead of 41)
  cudaGraphExec_t gexec = nullptr;
  struct GraphGuard {
    cudaGraphExec_t* e;
    ~GraphGuard() {
      if (*e) cudaGraphExecDestroy(*e);
    }
  } guard{&gexec};
  FState h;
  int launched = 0;
  for (;;) {
    if (launched == chunk && !gexec) {
      cudaStream_t cs = capture_stream();
      cudaGraph_t graph = nullptr;
      if (cs && cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
        const int e = issue_chunk(cs);
        const cudaError_t ce = cudaStreamEndCapture(cs, &graph);
        if (e == 0 && ce == cudaSuccess && graph) {
          if (cudaGraphInstantiate(&gexec, graph, 0) != cudaSuccess) gexec = nullptr;
        }
        if (graph) cudaGraphDestroy(graph);
      }
      cudaGetLastError();  // a failed capture leaves no sticky error; clear the last one
    }
    if (gexec) {
      if (cudaGraphLaunch(gexec, st) != cudaSuccess) return IGD_ERR_CUDA;
    } else {
      const int e = issue_chunk(st);
      if (e) return e;
    }
    if (cudaMemcpyAsync(&h, S, sizeof(FState), cudaMemcpyDeviceToHost, st) != cudaSuccess) return IGD_ERR_CUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return IGD_ERR_CUDA;
    launched += chunk;
    if (h.done || launched > maxit + chunk) break;
  }
  // iterations completed, and the residual of the last one (bank of iteration stop - 1)
  *iters = h.done ? h.base + h.stop : std::min(launched, maxit);
  const double rr = h.done ? h.bank[(h.stop + 3) & 3][B_RR] : h.bank[(chunk - 1) & 3][B_RR];
  *rel = h.bnorm2 > 0 ? std::sqrt(rr / h.bnorm2) : 0.0;
  return h.status == IGD_ERR_NOT_CONVERGED ? IGD_OK : h.status;  // non-convergence is reported via rel
}

__global__ void k_zero_u64(unsigned long long* a, double* b) {
  *a = 0ull;
  *b = 0.0;
}

// u += d on the interior (faces stay zero).
__global__ void k_add_masked(long long n, int nx, int ny, int nz, double* __restrict__ u, const double* __restrict__ d) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    u[i] = on_face(i, nx, ny, nz) ? 0.0 : u[i] + d[i];
}

// ||f||_2 over the interior (res = f masked; zero_buf is set to zero here).
int rhs_norm(const Problem& P, const double* f, double* zero_buf, double* res, double* scal, double* norm) {
  if (cudaMemsetAsync(zero_buf, 0, P.n * sizeof(double), P.st) != cudaSuccess) return IGD_ERR_CUDA;
  unsigned long long* mx = reinterpret_cast<unsigned long long*>(scal + 1);
  k_zero_u64<<<1, 1, 0, P.st>>>(mx, scal);
  k_residual<<<pblocks(P.n), PB, 0, P.st>>>(P.n, P.nx, P.ny, P.nz, f, zero_buf, res, scal, mx);
  double h[2];
  if (cudaMemcpyAsync(h, scal, 2 * sizeof(double), cudaMemcpyDeviceToHost, P.st) != cudaSuccess) return IGD_ERR_CUDA;
  if (cudaStreamSynchronize(P.st) != cudaSuccess) return IGD_ERR_CUDA;
  *norm = std::sqrt(h[0]);
  return IGD_OK;
}

// true FP64 residual of u: res = f - A u; returns ||res||_2 and max |res| on the host.
int true_residual(const Problem& P, const double* f, const double* u, double* Au, double* res, double* scal,
                  double* norm, double* maxabs) {
  int e = apply_op<double>(P, u, Au);
  if (e) return e;
  unsigned long long* mx = reinterpret_cast<unsigned long long*>(scal + 1);
  k_zero_u64<<<1, 1, 0, P.st>>>(mx, scal);
  k_residual<<<pblocks(P.n), PB, 0, P.st>>>(P.n, P.nx, P.ny, P.nz, f, Au, res, scal, mx);
  double h[2];
  if (cudaMemcpyAsync(h, scal, 2 * sizeof(double), cudaMemcpyDeviceToHost, P.st) != cudaSuccess) return IGD_ERR_CUDA;
  if (cudaStreamSynchronize(P.st) != cudaSuccess) return IGD_ERR_CUDA;
  unsigned long long bits;
  std::memcpy(&bits, &h[1], 8);
  *norm = std::sqrt(h[0]);
  *maxabs = __builtin_bit_cast(double, bits);
  return IGD_OK;
}

}  // namespace
}  // namespace igd

using namespace igd;

// Test hook: 0 = the fused FP32 BiCGSTAB (operator-epilogue dots, no scalar
// kernels) wherever it applies, 1 = the unfused iteration; per host thread.
extern "C" int igd_poisson_select(int path) {
  if (path < 0 || path > 1) return IGD_ERR_ARG;
  g_poisson_path = path;
  return IGD_OK;
}

extern "C" long long igd_poisson_workspace_bytes(int precision, long long n) {
  if (n <= 0) return -1;
  const size_t base = 2 * (size_t)n * sizeof(double) + 256;  // A u, residual, scalars
  if (precision == IGD_PREC_FP64) return (long long)(base + krylov_bytes<double>(n));
  if (precision == IGD_PREC_MIXED) return (long long)(base + 2 * (size_t)n * sizeof(float) + krylov_bytes<float>(n));
  return -1;
}

static int poisson_solve(int grid_kind, int precision, int nx, int ny, int nz, const void* op_coeffs64,
                         const void* op_coeffs32, const double* f, double* u, double rtol, int max_iterations,
                         void* workspace, long long workspace_bytes, double* info, void* stream, bool from_u) {
  if (nx < 3 || ny < 3 || nz < 3 || !f || !u || !workspace || !op_coeffs64 || rtol <= 0 || max_iterations < 1)
    return IGD_ERR_ARG;
  if ((long long)nx * ny * nz >= (1LL << 31)) return IGD_ERR_TOO_LARGE;
  if (grid_kind != IGD_GRID_MONITOR && grid_kind != IGD_GRID_LEGACY) return IGD_ERR_ARG;
  const long long n = (long long)nx * ny * nz;
  const long long need = igd_poisson_workspace_bytes(precision, n);
  if (need < 0 || workspace_bytes < need) return IGD_ERR_ARG;
  if (precision == IGD_PREC_MIXED && grid_kind == IGD_GRID_MONITOR && !op_coeffs32) return IGD_ERR_ARG;
  Problem P{grid_kind, nx, ny, nz, n, op_coeffs64, op_coeffs32, as_stream(stream)};
  unsigned char* w = static_cast<unsigned char*>(workspace);
  double* Au = reinterpret_cast<double*>(w);
  double* res = Au + n;
  double* scal = res + n;  // 2 doubles (+ padding)
  unsigned char* kry = w + 2 * (size_t)n * sizeof(double) + 256;
  int iters = 0, rounds = 0, status = IGD_OK;
  double rel = 0.0, rnorm = 0.0, rmax = 0.0, fnorm = 0.0;
  if (precision == IGD_PREC_FP64 && !from_u) {
    status = bicgstab<double>(P, f, u, rtol, max_iterations, kry, &iters, &rel, &fnorm);
    rounds = 1;
  } else if (precision == IGD_PREC_FP64) {
    // one correction solve A d = f - A u0 to rtol ||f|| / ||f - A u0||, then u = u0 + d
    int e = rhs_norm(P, f, Au, res, scal, &fnorm);
    if (e) return e;
    e = true_residual(P, f, u, Au, res, scal, &rnorm, &rmax);
    if (e) return e;
    if (rnorm > rtol * fnorm) {
      double inner_rel = 0.0;
      status = bicgstab<double>(P, res, Au, rtol * fnorm / rnorm, max_iterations, kry, &iters, &inner_rel);
      k_add_masked<<<pblocks(n), PB, 0, P.st>>>(n, nx, ny, nz, u, Au);
      rounds = 1;
    }
  } else if (precision == IGD_PREC_MIXED) {
    float* r32 = reinterpret_cast<float*>(kry);
    float* d32 = r32 + n;
    unsigned char* k32 = kry + 2 * (size_t)n * sizeof(float);
    const bool fused = fused_poisson_enabled() && fused_applies(P, r32, d32, k32);
    int e;
    if (from_u) {
      e = rhs_norm(P, f, Au, res, scal, &fnorm);
      if (e) return e;
      e = true_residual(P, f, u, Au, res, scal, &rnorm, &rmax);  // res = f - A u0
      if (e) return e;
    } else {
      cudaMemsetAsync(u, 0, n * sizeof(double), P.st);
      e = true_residual(P, f, u, Au, res, scal, &fnorm, &rmax);  // res = f (masked)
      if (e) return e;
      rnorm = fnorm;
    }
    while (rnorm > rtol * fnorm && iters < max_iterations && rounds < 16) {
      k_cast_scaled<<<pblocks(n), PB, 0, P.st>>>(n, res, r32, 1.0 / rnorm);
      int it = 0;
      double inner_rel = 0.0;
      const double inner_tol = std::max(1e-5, 0.5 * rtol * fnorm / rnorm);
      status = fused ? bicgstab_fused(P, r32, d32, inner_tol, max_iterations - iters, k32, &it, &inner_rel)
                     : bicgstab<float>(P, r32, d32, inner_tol, max_iterations - iters, k32, &it, &inner_rel);
      iters += it;
      ++rounds;
      if (status != IGD_OK) break;
      k_axpy_masked<<<pblocks(n), PB, 0, P.st>>>(n, nx, ny, nz, u, d32, rnorm);
      e = true_residual(P, f, u, Au, res, scal, &rnorm, &rmax);
      if (e) return e;
      if (it == 0) break;
    }
    rel = fnorm > 0 ? rnorm / fnorm : 0.0;
  } else {
    return IGD_ERR_ARG;
  }
  {
    const int e = true_residual(P, f, u, Au, res, scal, &rnorm, &rmax);
    if (e) return e;
    if (fnorm > 0.0) rel = rnorm / fnorm;
  }
  if (info) {
    info[0] = iters;
    info[1] = rel;
    info[2] = status;
    info[3] = rounds;
    info[4] = rnorm;
    info[5] = rmax;
  }
  return status == IGD_ERR_BREAKDOWN ? IGD_ERR_BREAKDOWN : launch_status();
}

extern "C" int igd_poisson_solve(int grid_kind, int precision, int nx, int ny, int nz, const void* op_coeffs64,
                                 const void* op_coeffs32, const double* f, double* u, double rtol, int max_iterations,
                                 void* workspace, long long workspace_bytes, double* info, void* stream) {
  return poisson_solve(grid_kind, precision, nx, ny, nz, op_coeffs64, op_coeffs32, f, u, rtol, max_iterations,
                       workspace, workspace_bytes, info, stream, false);
}

extern "C" int igd_poisson_solve_from(int grid_kind, int precision, int nx, int ny, int nz, const void* op_coeffs64,
                                      const void* op_coeffs32, const double* f, double* u, double rtol,
                                      int max_iterations, void* workspace, long long workspace_bytes, double* info,
                                      void* stream) {
  return poisson_solve(grid_kind, precision, nx, ny, nz, op_coeffs64, op_coeffs32, f, u, rtol, max_iterations,
                       workspace, workspace_bytes, info, stream, true);
}
