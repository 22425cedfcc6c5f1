// The JAX route of the monitor-grid Poisson solve (poisson/poisson_jax.py:675-750):
// preconditioned CG on the interior -L (production closure) from x = 0, stopping
// when max |r| < tolerance, with the route's three preconditioners:
//   diag      (:248-273)  z = dinv r, dinv = 1 / (2 sum_a g^aa / h_a^2) (floored),
//   separable (:312-383)  z = S D^-1 S r, S the orthonormal Dirichlet sine transform
//                         along each axis, D the separable constant-stiffness spectrum
//                         (applied in FP32: a preconditioner changes the path, not the
//                         fixed point),
//   line      (:411-579)  tridiagonal solves along the stiffest axis (the Thomas
//                         factorisation comes from the host; the apply is FMAs only).
// FP64 vectors and operator; every field is a full (nx, ny, nz) field with zero faces.
// Scalars stay on the device; the host reads them once per 8 iterations.
#include <cmath>
#include <cstring>

#include "common.cuh"

namespace igd {
namespace {

constexpr int CB = 256;
inline int cblocks(long long n) { return (int)std::min<long long>((n + CB - 1) / CB, 152LL * 8); }

struct PState {
  double rz, den, rznew, alpha, beta;
  unsigned long long rmax_bits;
  int it, done, converged, pad;
};

__device__ __forceinline__ bool face_pt(long long i, int nx, int ny, int nz) {
  const unsigned pl = (unsigned)ny * (unsigned)nz, ii = (unsigned)i;
  const unsigned x = ii / pl, r = ii - x * pl;
  const unsigned y = r / (unsigned)nz, z = r - y * (unsigned)nz;
  return x == 0 || x == (unsigned)nx - 1 || y == 0 || y == (unsigned)ny - 1 || z == 0 || z == (unsigned)nz - 1;
}

__device__ __forceinline__ void block_add(double* dst, double v) {
  __shared__ double scratch[CB / 32];
  double a[1] = {v};
  block_sum<1, CB>(a, scratch);
  if (threadIdx.x == 0) atomicAdd(dst, a[0]);
}

__global__ void pcg_state_init(PState* s) { memset(s, 0, sizeof(PState)); }

// r = f on the interior (faces zero), x = 0
__global__ void pcg_init(long long n, int nx, int ny, int nz, const double* __restrict__ f, double* __restrict__ x,
                         double* __restrict__ r) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    r[i] = face_pt(i, nx, ny, nz) ? 0.0 : f[i];
    x[i] = 0.0;
  }
}

__global__ void pcg_dot(long long n, const double* __restrict__ a, const double* __restrict__ b, double* acc,
                        const PState* s) {
  if (s->done) return;
  double t = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    t += a[i] * b[i];
  block_add(acc, t);
}

__global__ void pcg_copy(long long n, const double* __restrict__ a, double* __restrict__ b) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    b[i] = a[i];
}

// den = p.Ap: stop below 1e-20 in magnitude, else alpha = rz / den; clears the max |r| word
__global__ void pcg_alpha(PState* s) {
  if (s->done) return;
  if (!(fabs(s->den) > 1.0e-20)) {
    s->done = 1;
    return;
  }
  s->alpha = s->rz / s->den;
  s->rmax_bits = 0ull;
}

// x += alpha p; r -= alpha Ap (faces stay zero); max |r| over the interior
__global__ void pcg_xr(long long n, int nx, int ny, int nz, double* __restrict__ x, double* __restrict__ r,
                       const double* __restrict__ p, const double* __restrict__ ap, PState* s) {
  if (s->done) return;
  const double al = s->alpha;
  double m = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    if (face_pt(i, nx, ny, nz)) continue;
    x[i] += al * p[i];
    const double ri = r[i] - al * ap[i];
    r[i] = ri;
    m = fmax(m, fabs(ri));
  }
  m = warp_max(m);
  if ((threadIdx.x & 31) == 0) atomicMax(&s->rmax_bits, (unsigned long long)__double_as_longlong(m));  // m >= 0
}

// iteration count and the stopping test max |r| < tolerance; clears rznew
__global__ void pcg_check(PState* s, double tol, int maxit) {
  if (s->done) return;
  s->it += 1;
  const double rmax = __longlong_as_double((long long)s->rmax_bits);
  if (rmax < tol) {
    s->done = 1;
    s->converged = 1;
  } else if (s->it >= maxit) {
    s->done = 1;
  }
  s->rznew = 0.0;
}

// beta = rz_new / rz (stop when |rz| <= 1e-30); clears den
__global__ void pcg_beta(PState* s) {
  if (s->done) return;
  if (!(fabs(s->rz) > 1.0e-30)) {
    s->done = 1;
    return;
  }
  s->beta = s->rznew / s->rz;
  s->rz = s->rznew;
  s->den = 0.0;
}

__global__ void pcg_p(long long n, double* __restrict__ p, const double* __restrict__ z, const PState* s) {
  if (s->done) return;
  const double b = s->beta;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    p[i] = z[i] + b * p[i];
}

// ---- preconditioners (z = M r; every one leaves the faces of z zero)
__global__ void pc_none(long long n, const double* __restrict__ r, double* __restrict__ z, const PState* s) {
  if (s->done) return;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    z[i] = r[i];
}

__global__ void pc_diag(long long n, const double* __restrict__ r, const double* __restrict__ dinv,
                        double* __restrict__ z, const PState* s) {
  if (s->done) return;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    z[i] = dinv[i] * r[i];  // dinv is zero on the faces
}

// Tridiagonal solves along `axis` with the host factorisation: lower[i] (the
// sub-diagonal), cprime[i] and inv_den[i] at every interior point (full-field
// index): d_i = (r_i - lower_i d_{i-1}) inv_den_i, z_m = d_m, z_i = d_i - c'_i z_{i+1}.
// One thread per interior line.
__global__ void pc_line(int nx, int ny, int nz, int axis, const double* __restrict__ r,
                        const double* __restrict__ lower, const double* __restrict__ cprime,
                        const double* __restrict__ inv_den, double* __restrict__ z, const PState* s) {
  if (s->done) return;
  const long long sx = (long long)ny * nz, sy = nz;
  const int n0 = axis == 0 ? ny - 2 : nx - 2;  // the two other interior extents
  const int n1 = axis == 2 ? ny - 2 : nz - 2;
  const int m = (axis == 0 ? nx : axis == 1 ? ny : nz) - 2;
  const long long step = axis == 0 ? sx : axis == 1 ? sy : 1;
  const long long lines = (long long)n0 * n1;
  for (long long l = blockIdx.x * (long long)blockDim.x + threadIdx.x; l < lines;
       l += (long long)gridDim.x * blockDim.x) {
    const int a = (int)(l / n1) + 1, b = (int)(l % n1) + 1;
    long long base;
    if (axis == 0)
      base = a * sy + b;            // (x = 0, y = a, z = b)
    else if (axis == 1)
      base = a * sx + b;            // (x = a, y = 0, z = b)
    else
      base = a * sx + (long long)b * sy;  // (x = a, y = b, z = 0)
    double d = 0.0;
    for (int i = 1; i <= m; ++i) {
      const long long q = base + i * step;
      d = (r[q] - lower[q] * d) * inv_den[q];
      z[q] = d;
    }
    double zn = z[base + m * step];
    for (int i = m - 1; i >= 1; --i) {
      const long long q = base + i * step;
      zn = z[q] - cprime[q] * zn;
      z[q] = zn;
    }
  }
}

// separable: interior of r to a compact FP32 block (mx, my, mz)
__global__ void sep_gather(int nx, int ny, int nz, const double* __restrict__ r, float* __restrict__ t,
                           const PState* s) {
  if (s->done) return;
  const long long mx = nx - 2, my = ny - 2, mz = nz - 2, tot = mx * my * mz;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot; e += (long long)gridDim.x * blockDim.x) {
    const long long i = e / (my * mz), rem = e - i * my * mz, j = rem / mz, k = rem - j * mz;
    t[e] = (float)r[((i + 1) * ny + (j + 1)) * (long long)nz + (k + 1)];
  }
}

// u = S_a t along axis a (S symmetric orthonormal, m_a x m_a); optional pointwise scale after
__global__ void sep_mode(int mx, int my, int mz, int axis, const float* __restrict__ S, const float* __restrict__ t,
                         float* __restrict__ u, const float* __restrict__ scale, const PState* s) {
  if (s->done) return;
  const long long tot = (long long)mx * my * mz;
  const int m = axis == 0 ? mx : axis == 1 ? my : mz;
  const long long stride = axis == 0 ? (long long)my * mz : axis == 1 ? mz : 1;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < tot; e += (long long)gridDim.x * blockDim.x) {
    const long long i = e / ((long long)my * mz), rem = e - i * my * mz, j = rem / mz, k = rem - j * mz;
    const int idx = axis == 0 ? (int)i : axis == 1 ? (int)j : (int)k;
    const long long line0 = e - (long long)idx * stride;
    const float* Srow = S + (long long)idx * m;
    float acc = 0.f;
    for (int l = 0; l < m; ++l) acc = fmaf(Srow[l], t[line0 + l * stride], acc);
    u[e] = scale ? acc * scale[e] : acc;
  }
}

// compact FP32 block back into the interior of z (faces zero)
__global__ void sep_scatter(long long n, int nx, int ny, int nz, const float* __restrict__ t, double* __restrict__ z,
                            const PState* s) {
  if (s->done) return;
  const int my = ny - 2, mz = nz - 2;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n; q += (long long)gridDim.x * blockDim.x) {
    const long long x = q / ((long long)ny * nz), rem = q - x * ny * nz, y = rem / nz, zz = rem - y * nz;
    const bool face = x == 0 || x == nx - 1 || y == 0 || y == ny - 1 || zz == 0 || zz == nz - 1;
    z[q] = face ? 0.0 : (double)t[((x - 1) * my + (y - 1)) * (long long)mz + (zz - 1)];
  }
}

struct Pcg {
  int nx, ny, nz;
  long long n;
  int kind, axis;
  const double* c64;
  const double* pc;
  const float* pc32;
  double *r, *p, *z, *ap;
  float *t0, *t1;
  PState* S;
  cudaStream_t st;
};

int precondition(const Pcg& G) {
  const long long n = G.n;
  const int nb = cblocks(n);
  switch (G.kind) {
    case IGD_PCG_NONE:
      pc_none<<<nb, CB, 0, G.st>>>(n, G.r, G.z, G.S);
      break;
    case IGD_PCG_DIAG:
      pc_diag<<<nb, CB, 0, G.st>>>(n, G.r, G.pc, G.z, G.S);
      break;
    case IGD_PCG_LINE: {
      const long long lines = G.axis == 0 ? (long long)(G.ny - 2) * (G.nz - 2)
                              : G.axis == 1 ? (long long)(G.nx - 2) * (G.nz - 2)
                                            : (long long)(G.nx - 2) * (G.ny - 2);
      pc_line<<<cblocks(lines), CB, 0, G.st>>>(G.nx, G.ny, G.nz, G.axis, G.r, G.pc, G.pc + n, G.pc + 2 * n, G.z,
                                               G.S);
      break;
    }
    case IGD_PCG_SEPARABLE: {
      const int mx = G.nx - 2, my = G.ny - 2, mz = G.nz - 2;
      const long long mt = (long long)mx * my * mz;
      const float *Sx = G.pc32, *Sy = Sx + (long long)mx * mx, *Sz = Sy + (long long)my * my,
                  *inv = Sz + (long long)mz * mz;
      const int mb = cblocks(mt);
      sep_gather<<<mb, CB, 0, G.st>>>(G.nx, G.ny, G.nz, G.r, G.t0, G.S);
      sep_mode<<<mb, CB, 0, G.st>>>(mx, my, mz, 0, Sx, G.t0, G.t1, nullptr, G.S);
      sep_mode<<<mb, CB, 0, G.st>>>(mx, my, mz, 1, Sy, G.t1, G.t0, nullptr, G.S);
      sep_mode<<<mb, CB, 0, G.st>>>(mx, my, mz, 2, Sz, G.t0, G.t1, inv, G.S);  // spectral coefficients / D
      sep_mode<<<mb, CB, 0, G.st>>>(mx, my, mz, 0, Sx, G.t1, G.t0, nullptr, G.S);
      sep_mode<<<mb, CB, 0, G.st>>>(mx, my, mz, 1, Sy, G.t0, G.t1, nullptr, G.S);
      sep_mode<<<mb, CB, 0, G.st>>>(mx, my, mz, 2, Sz, G.t1, G.t0, nullptr, G.S);
      sep_scatter<<<nb, CB, 0, G.st>>>(n, G.nx, G.ny, G.nz, G.t0, G.z, G.S);
      break;
    }
    default:
      return IGD_ERR_ARG;
  }
  return IGD_OK;
}

int apply_A(const Pcg& G, const double* x, double* y) {
  return igd_hpsi_agrid(IGD_F64, IGD_CLOSURE_PRODUCTION, G.nx, G.ny, G.nz, G.c64, nullptr, x, y, 1, G.n, -1.0, 0.0,
                        G.st);
}

}  // namespace
}  // namespace igd

using namespace igd;

extern "C" long long igd_poisson_pcg_workspace_bytes(int precond, int nx, int ny, int nz) {
  if (nx < 3 || ny < 3 || nz < 3 || precond < IGD_PCG_NONE || precond > IGD_PCG_LINE) return -1;
  const long long n = (long long)nx * ny * nz, mt = (long long)(nx - 2) * (ny - 2) * (nz - 2);
  long long b = 4 * n * (long long)sizeof(double) + 256;
  if (precond == IGD_PCG_SEPARABLE) b += 2 * ((mt * (long long)sizeof(float) + 255) / 256 * 256);
  return b;
}

extern "C" int igd_poisson_pcg(int nx, int ny, int nz, const double* op_coeffs64, const double* f, double* x,
                               double tolerance, int max_iterations, int precond, const double* pc_data,
                               const float* pc_data32, int pc_axis, void* workspace, long long workspace_bytes,
                               double* info, void* stream) {
  if (nx < 3 || ny < 3 || nz < 3 || !op_coeffs64 || !f || !x || !workspace || !(tolerance > 0.0) ||
      max_iterations < 1)
    return IGD_ERR_ARG;
  if ((long long)nx * ny * nz >= (1LL << 31)) return IGD_ERR_TOO_LARGE;
  if ((precond == IGD_PCG_DIAG || precond == IGD_PCG_LINE) && !pc_data) return IGD_ERR_ARG;
  if (precond == IGD_PCG_SEPARABLE && !pc_data32) return IGD_ERR_ARG;
  if (precond == IGD_PCG_LINE && (pc_axis < 0 || pc_axis > 2)) return IGD_ERR_ARG;
  const long long need = igd_poisson_pcg_workspace_bytes(precond, nx, ny, nz);
  if (need < 0 || workspace_bytes < need) return IGD_ERR_ARG;
  const long long n = (long long)nx * ny * nz;
  unsigned char* w = static_cast<unsigned char*>(workspace);
  Pcg G;
  G.nx = nx;
  G.ny = ny;
  G.nz = nz;
  G.n = n;
  G.kind = precond;
  G.axis = pc_axis;
  G.c64 = op_coeffs64;
  G.pc = pc_data;
  G.pc32 = pc_data32;
  G.r = reinterpret_cast<double*>(w);
  G.p = G.r + n;
  G.z = G.p + n;
  G.ap = G.z + n;
  G.S = reinterpret_cast<PState*>(w + 4 * n * sizeof(double));
  const long long mt = (long long)(nx - 2) * (ny - 2) * (nz - 2);
  G.t0 = reinterpret_cast<float*>(w + 4 * n * sizeof(double) + 256);
  G.t1 = G.t0 + (mt + 63) / 64 * 64;
  G.st = as_stream(stream);
  const int nb = cblocks(n);
  pcg_state_init<<<1, 1, 0, G.st>>>(G.S);
  pcg_init<<<nb, CB, 0, G.st>>>(n, nx, ny, nz, f, x, G.r);
  // the line solves write interior points only: the faces of z start (and stay) zero
  if (precond == IGD_PCG_LINE && cudaMemsetAsync(G.z, 0, n * sizeof(double), G.st) != cudaSuccess)
    return IGD_ERR_CUDA;
  int e = precondition(G);
  if (e) return e;
  pcg_dot<<<nb, CB, 0, G.st>>>(n, G.r, G.z, &G.S->rz, G.S);
  pcg_copy<<<nb, CB, 0, G.st>>>(n, G.z, G.p);
  PState h;
  std::memset(&h, 0, sizeof(h));
  for (int launched = 0; launched < max_iterations + 8;) {
    for (int c = 0; c < 8; ++c) {
      e = apply_A(G, G.p, G.ap);
      if (e) return e;
      pcg_dot<<<nb, CB, 0, G.st>>>(n, G.p, G.ap, &G.S->den, G.S);
      pcg_alpha<<<1, 1, 0, G.st>>>(G.S);
      pcg_xr<<<nb, CB, 0, G.st>>>(n, nx, ny, nz, x, G.r, G.p, G.ap, G.S);
      pcg_check<<<1, 1, 0, G.st>>>(G.S, tolerance, max_iterations);
      e = precondition(G);
      if (e) return e;
      pcg_dot<<<nb, CB, 0, G.st>>>(n, G.r, G.z, &G.S->rznew, G.S);
      pcg_beta<<<1, 1, 0, G.st>>>(G.S);
      pcg_p<<<nb, CB, 0, G.st>>>(n, G.p, G.z, G.S);
    }
    launched += 8;
    if (cudaMemcpyAsync(&h, G.S, sizeof(PState), cudaMemcpyDeviceToHost, G.st) != cudaSuccess) return IGD_ERR_CUDA;
    if (cudaStreamSynchronize(G.st) != cudaSuccess) return IGD_ERR_CUDA;
    if (h.done) break;
  }
  if (info) {
    info[0] = h.it;
    info[1] = __builtin_bit_cast(double, h.rmax_bits);
    info[2] = h.converged;
  }
  return launch_status();
}
