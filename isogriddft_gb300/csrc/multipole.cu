// Multipole boundary of the open-boundary Poisson problem (K5), RHS assembly
// and FP64 weighted reductions.
//
// poisson/open_boundary.py: nodal moments through integrate_field :816-851,
// incident-node fractions :206-220 and nodal-region moments :267-296,
// corrected moments from a per-cell quadratic least-squares fit over the
// 4x4x4 node neighbourhood with 2x2x2 sub-cell trilinear quadrature :299-464,
// the legacy_split boundary correction :559-719, boundary potential from the
// moments :467-495, and the split RHS 4 pi rho + L(b) :1143-1146.
// Moments are 10 doubles: q, p_x, p_y, p_z, Q_xx, Q_xy, Q_xz, Q_yy, Q_yz, Q_zz.
#include "common.cuh"

namespace igd {
namespace {

constexpr int MB = 256;
inline int mblocks(long long n) { return (int)std::min<long long>((n + MB - 1) / MB, 152LL * 8); }

__device__ __forceinline__ void moment_terms(double w, double dx, double dy, double dz, double m[10]) {
  const double r2 = dx * dx + dy * dy + dz * dz;
  m[0] += w;
  m[1] += w * dx;
  m[2] += w * dy;
  m[3] += w * dz;
  m[4] += w * (3.0 * dx * dx - r2);
  m[5] += w * (3.0 * dx * dy);
  m[6] += w * (3.0 * dx * dz);
  m[7] += w * (3.0 * dy * dy - r2);
  m[8] += w * (3.0 * dy * dz);
  m[9] += w * (3.0 * dz * dz - r2);
}

template <int K>
__device__ __forceinline__ void flush(double (&v)[K], double* out) {
  block_atomic_add<K, MB>(out, v);
}

__global__ void zero_kernel(double* out, int k) {
  if (threadIdx.x < k) out[threadIdx.x] = 0.0;
}

// sum rho * W * frac * (1, d, 3 d d - r^2) about center.
__global__ void nodal_moments_kernel(long long n, const double* __restrict__ rho, const double* __restrict__ w,
                                     const double* __restrict__ x, const double* __restrict__ y,
                                     const double* __restrict__ z, const double* __restrict__ frac, double cx,
                                     double cy, double cz, double* out) {
  double m[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double wt = rho[i] * w[i];
    if (frac) wt *= frac[i];
    moment_terms(wt, x[i] - cx, y[i] - cy, z[i] - cz, m);
  }
  flush<10>(m, out);
}

__device__ __forceinline__ double tri(const double c[8], double u, double v, double t) {
  const double um = 1.0 - u, vm = 1.0 - v, tm = 1.0 - t;
  return um * vm * tm * c[0] + u * vm * tm * c[1] + um * v * tm * c[2] + u * v * tm * c[3] + um * vm * t * c[4] +
         u * vm * t * c[5] + um * v * t * c[6] + u * v * t * c[7];
}

// Least-squares quadratic through the 64 nodes around cell (i, j, k); returns
// coefficients in local coordinates xi = (r - c) / L.  Normal equations with
// Cholesky in FP64 (the local scaling keeps them well conditioned).
__device__ bool quad_fit(const double* __restrict__ X, const double* __restrict__ Y, const double* __restrict__ Z,
                         const double* __restrict__ R, int ny, int nz, int i, int j, int k, double c[3], double L,
                         double coef[10]) {
  double G[55];
  double b[10];
#pragma unroll
  for (int a = 0; a < 55; ++a) G[a] = 0.0;
#pragma unroll
  for (int a = 0; a < 10; ++a) b[a] = 0.0;
  const long long pl = (long long)ny * nz;
  for (int di = -1; di <= 2; ++di)
    for (int dj = -1; dj <= 2; ++dj)
      for (int dk = -1; dk <= 2; ++dk) {
        const long long g = (long long)(i + di) * pl + (long long)(j + dj) * nz + (k + dk);
        const double u = (X[g] - c[0]) / L, v = (Y[g] - c[1]) / L, t = (Z[g] - c[2]) / L;
        const double f[10] = {1.0, u, v, t, u * u, v * v, t * t, u * v, u * t, v * t};
        const double rv = R[g];
        int idx = 0;
#pragma unroll
        for (int a = 0; a < 10; ++a) {
          b[a] += f[a] * rv;
#pragma unroll
          for (int e = 0; e <= a; ++e) G[idx++] += f[a] * f[e];
        }
      }
  // Cholesky G = L L^T in place (packed lower), then solve.
  int ia = 0;
  for (int a = 0; a < 10; ++a) {
    const int rowa = a * (a + 1) / 2;
    for (int e = 0; e <= a; ++e) {
      const int rowe = e * (e + 1) / 2;
      double s = G[rowa + e];
      for (int q = 0; q < e; ++q) s -= G[rowa + q] * G[rowe + q];
      if (a == e) {
        if (!(s > 0.0)) return false;
        G[rowa + a] = sqrt(s);
      } else {
        G[rowa + e] = s / G[rowe + e];
      }
    }
    ia += a + 1;
  }
  double y[10];
  for (int a = 0; a < 10; ++a) {
    const int rowa = a * (a + 1) / 2;
    double s = b[a];
    for (int q = 0; q < a; ++q) s -= G[rowa + q] * y[q];
    y[a] = s / G[rowa + a];
  }
  for (int a = 9; a >= 0; --a) {
    double s = y[a];
    for (int q = a + 1; q < 10; ++q) s -= G[q * (q + 1) / 2 + a] * coef[q];
    coef[a] = s / G[a * (a + 1) / 2 + a];
  }
  return true;
}

// mode 0: corrected moments (weight rho_quad J dV about center);
// mode 1: legacy_split pass 1 (|delta| and |delta| r sums, delta = (rho_quad - rho_tri) J dV);
// mode 2: legacy_split pass 2 (moments of delta about center).
__global__ void cell_quadrature_kernel(int nx, int ny, int nz, const double* __restrict__ X,
                                       const double* __restrict__ Y, const double* __restrict__ Z,
                                       const double* __restrict__ J, const double* __restrict__ R,
                                       const int* __restrict__ cells, int ncells, double dvol, int mode, double cx,
                                       double cy, double cz, double* out, int* fail) {
  double m[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  const long long pl = (long long)ny * nz;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ncells; t += gridDim.x * blockDim.x) {
    const int i = cells[3 * t], j = cells[3 * t + 1], k = cells[3 * t + 2];
    double cx8[8], cy8[8], cz8[8], cj8[8], cr8[8];
    int q = 0;
    for (int dk = 0; dk < 2; ++dk)
      for (int dj = 0; dj < 2; ++dj)
        for (int di = 0; di < 2; ++di) {
          const long long g = (long long)(i + di) * pl + (long long)(j + dj) * nz + (k + dk);
          cx8[q] = X[g];
          cy8[q] = Y[g];
          cz8[q] = Z[g];
          cj8[q] = J[g];
          cr8[q] = R[g];
          ++q;
        }
    double c[3] = {0, 0, 0};
    for (int a = 0; a < 8; ++a) {
      c[0] += cx8[a];
      c[1] += cy8[a];
      c[2] += cz8[a];
    }
    c[0] *= 0.125;
    c[1] *= 0.125;
    c[2] *= 0.125;
    const double Ls = fmax(fmax(fabs(cx8[7] - cx8[0]), fabs(cy8[7] - cy8[0])), fabs(cz8[7] - cz8[0])) + 1e-300;
    double coef[10];
    if (!quad_fit(X, Y, Z, R, ny, nz, i, j, k, c, Ls, coef)) {
      atomicOr(fail, 1);
      continue;
    }
    for (int s = 0; s < 8; ++s) {
      const double u = ((s >> 2) & 1) ? 0.75 : 0.25;  // sample (ix, iy, iz) with z fastest
      const double v = ((s >> 1) & 1) ? 0.75 : 0.25;
      const double w = (s & 1) ? 0.75 : 0.25;
      const double xs = tri(cx8, u, v, w), ys = tri(cy8, u, v, w), zs = tri(cz8, u, v, w);
      const double js = tri(cj8, u, v, w), rt = tri(cr8, u, v, w);
      const double a = (xs - c[0]) / Ls, b = (ys - c[1]) / Ls, d = (zs - c[2]) / Ls;
      const double rq = coef[0] + coef[1] * a + coef[2] * b + coef[3] * d + coef[4] * a * a + coef[5] * b * b +
                        coef[6] * d * d + coef[7] * a * b + coef[8] * a * d + coef[9] * b * d;
      if (mode == 0) {
        moment_terms(rq * js * dvol, xs - cx, ys - cy, zs - cz, m);
      } else {
        const double delta = (rq - rt) * js * dvol;
        if (mode == 1) {
          const double ad = fabs(delta);
          m[0] += ad;
          m[1] += ad * xs;
          m[2] += ad * ys;
          m[3] += ad * zs;
        } else {
          moment_terms(delta, xs - cx, ys - cy, zs - cz, m);
        }
      }
    }
  }
  flush<10>(m, out);
}

// Boundary potential on the faces from moments about center (order 0..2):
// q/r + p.d/r^3 + 1/2 d.Q.d / r^5 with the reference's contraction.  add != 0
// accumulates into out; otherwise faces are set and the interior zeroed.
__global__ void boundary_kernel(int nx, int ny, int nz, const double* __restrict__ X, const double* __restrict__ Y,
                                const double* __restrict__ Z, const double* __restrict__ mom, int order, double cx,
                                double cy, double cz, double* __restrict__ out, int add) {
  const long long n = (long long)nx * ny * nz, pl = (long long)ny * nz;
  const double q = mom[0], px = mom[1], py = mom[2], pz = mom[3];
  const double Qxx = mom[4], Qxy = mom[5], Qxz = mom[6], Qyy = mom[7], Qyz = mom[8], Qzz = mom[9];
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i / pl), r = (int)(i - (long long)x * pl), y = r / nz, z = r - y * nz;
    const bool face = x == 0 || x == nx - 1 || y == 0 || y == ny - 1 || z == 0 || z == nz - 1;
    if (!face) {
      if (!add) out[i] = 0.0;
      continue;
    }
    const double dx = X[i] - cx, dy = Y[i] - cy, dz = Z[i] - cz;
    const double rr = sqrt(dx * dx + dy * dy + dz * dz);
    double v = q / rr;
    if (order >= 1) v += (px * dx + py * dy + pz * dz) / (rr * rr * rr);
    if (order >= 2) {
      const double c = Qxx * dx * dx + 2.0 * Qxy * dx * dy + 2.0 * Qxz * dx * dz + Qyy * dy * dy +
                       2.0 * Qyz * dy * dz + Qzz * dz * dz;
      v += 0.5 * c / (rr * rr * rr * rr * rr);
    }
    out[i] = add ? out[i] + v : v;
  }
}

// f = 4 pi rho + Lb on the interior, 0 on the faces.
__global__ void rhs_kernel(int nx, int ny, int nz, const double* __restrict__ rho, const double* __restrict__ Lb,
                           double* __restrict__ f) {
  const long long n = (long long)nx * ny * nz, pl = (long long)ny * nz;
  const double fp = 4.0 * 3.14159265358979323846;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i / pl), r = (int)(i - (long long)x * pl), y = r / nz, z = r - y * nz;
    const bool face = x == 0 || x == nx - 1 || y == 0 || y == ny - 1 || z == 0 || z == nz - 1;
    f[i] = face ? 0.0 : fp * rho[i] + Lb[i];
  }
}

// v = b on faces, u inside.
__global__ void compose_kernel(int nx, int ny, int nz, const double* __restrict__ b, const double* __restrict__ u,
                               double* __restrict__ v) {
  const long long n = (long long)nx * ny * nz, pl = (long long)ny * nz;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i / pl), r = (int)(i - (long long)x * pl), y = r / nz, z = r - y * nz;
    const bool face = x == 0 || x == nx - 1 || y == 0 || y == ny - 1 || z == 0 || z == nz - 1;
    v[i] = face ? b[i] : u[i];
  }
}

template <typename T>
__global__ void wsum_kernel(long long n, const T* __restrict__ a, const T* __restrict__ b, const double* __restrict__ w,
                            double* out) {
  double s[1] = {0.0};
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double t = (double)a[i];
    if (b) t *= (double)b[i];
    if (w) t *= w[i];
    s[0] += t;
  }
  flush<1>(s, out);
}

}  // namespace
}  // namespace igd

using namespace igd;

// out[10] (device) = sum over points of rho W frac (1, d, 3 d d - r^2) about (cx, cy, cz).
extern "C" int igd_multipole_nodal_moments(long long n, const double* rho, const double* cell_volumes,
                                           const double* x, const double* y, const double* z, const double* frac,
                                           double cx, double cy, double cz, double* out, void* stream) {
  if (n <= 0 || !rho || !cell_volumes || !x || !y || !z || !out) return IGD_ERR_ARG;
  cudaStream_t st = as_stream(stream);
  zero_kernel<<<1, 32, 0, st>>>(out, 10);
  nodal_moments_kernel<<<mblocks(n), MB, 0, st>>>(n, rho, cell_volumes, x, y, z, frac, cx, cy, cz, out);
  return launch_status();
}

// Quadratic-fit sub-cell quadrature over `ncells` selected cells (cells: 3 ints
// (i, j, k) per cell, each 1 <= i <= nx-3 etc.).  mode 0: corrected moments;
// 1: legacy_split |delta| sums (out[0] = sum |delta|, out[1..3] = sum |delta| r);
// 2: legacy_split moments of delta.  *fail (device int) is set if a fit is singular.
extern "C" int igd_multipole_cell_quadrature(int nx, int ny, int nz, const double* x, const double* y,
                                             const double* z, const double* jacobian, const double* rho,
                                             const int* cells, int ncells, double subcell_volume, int mode, double cx,
                                             double cy, double cz, double* out, int* fail, void* stream) {
  if (nx < 4 || ny < 4 || nz < 4 || !x || !y || !z || !jacobian || !rho || !out || !fail || mode < 0 || mode > 2 ||
      ncells < 0 || (ncells > 0 && !cells))
    return IGD_ERR_ARG;
  cudaStream_t st = as_stream(stream);
  zero_kernel<<<1, 32, 0, st>>>(out, 10);
  if (ncells > 0)
    cell_quadrature_kernel<<<(ncells + MB - 1) / MB, MB, 0, st>>>(nx, ny, nz, x, y, z, jacobian, rho, cells, ncells,
                                                                   subcell_volume, mode, cx, cy, cz, out, fail);
  return launch_status();
}

// Face values of the multipole potential (order <= 2) about (cx, cy, cz); add = 0 sets
// the faces and zeroes the interior, add = 1 accumulates on the faces.
extern "C" int igd_multipole_boundary(int nx, int ny, int nz, const double* x, const double* y, const double* z,
                                      const double* moments, int order, double cx, double cy, double cz, double* out,
                                      int add, void* stream) {
  if (nx < 2 || ny < 2 || nz < 2 || !x || !y || !z || !moments || !out || order < 0 || order > 2) return IGD_ERR_ARG;
  const long long n = (long long)nx * ny * nz;
  boundary_kernel<<<mblocks(n), MB, 0, as_stream(stream)>>>(nx, ny, nz, x, y, z, moments, order, cx, cy, cz, out, add);
  return launch_status();
}

// f = 4 pi rho + Lb inside, 0 on the faces (open_boundary.py:1143-1146).
extern "C" int igd_poisson_rhs(int nx, int ny, int nz, const double* rho, const double* Lb, double* f, void* stream) {
  if (nx < 3 || ny < 3 || nz < 3 || !rho || !Lb || !f) return IGD_ERR_ARG;
  rhs_kernel<<<mblocks((long long)nx * ny * nz), MB, 0, as_stream(stream)>>>(nx, ny, nz, rho, Lb, f);
  return launch_status();
}

// v = b on the faces, u inside (open_boundary.py:1173-1174).
extern "C" int igd_poisson_compose(int nx, int ny, int nz, const double* b, const double* u, double* v, void* stream) {
  if (nx < 3 || ny < 3 || nz < 3 || !b || !u || !v) return IGD_ERR_ARG;
  compose_kernel<<<mblocks((long long)nx * ny * nz), MB, 0, as_stream(stream)>>>(nx, ny, nz, b, u, v);
  return launch_status();
}

// *out (device) = sum a[i] * b[i] * w[i] in FP64 (b, w may be NULL): integrate_field
// (ops/kinetic.py:61-66) and evaluate_hartree_energy (poisson/hartree.py:117-129).
extern "C" int igd_weighted_sum(int dtype, long long n, const void* a, const void* b, const double* w, double* out,
                                void* stream) {
  if (n <= 0 || !a || !out) return IGD_ERR_ARG;
  cudaStream_t st = as_stream(stream);
  zero_kernel<<<1, 32, 0, st>>>(out, 1);
  if (dtype == IGD_F64)
    wsum_kernel<double><<<mblocks(n), MB, 0, st>>>(n, static_cast<const double*>(a), static_cast<const double*>(b), w,
                                                   out);
  else if (dtype == IGD_F32)
    wsum_kernel<float><<<mblocks(n), MB, 0, st>>>(n, static_cast<const float*>(a), static_cast<const float*>(b), w,
                                                  out);
  else
    return IGD_ERR_DTYPE;
  return launch_status();
}
