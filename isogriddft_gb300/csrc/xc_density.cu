// Pointwise LSDA exchange-correlation (K9) and spin-density build (K10).
//
// LSDA: the reference evaluates "lda,vwn" through PySCF/libxc
// (xc/lsda.py:70-121): Slater exchange plus the VWN5 correlation fit of
// Vosko, Wilk and Nusair (Can. J. Phys. 58, 1200 (1980)) with its spin
// interpolation; PW92 (Perdew and Wang, PRB 45, 13244 (1992)) is offered as
// an option.  Written from those published forms: per channel
//   G(x) = A [ln(x^2/X) + 2b/Q atan(Q/(2x+b))
//             - b x0/X(x0) (ln((x-x0)^2/X) + 2(b+2x0)/Q atan(Q/(2x+b)))],
// x = sqrt(rs), X = x^2 + b x + c, Q = sqrt(4c - b^2);
// eps_c = eps_P + alpha f(z)(1-z^4)/f''(0) + (eps_F - eps_P) f(z) z^4 and
// v_s = eps - rs/3 d eps/d rs +- (1 -+ z) d eps/dz.  Density validation and
// clipping follow xc/lsda.py:57-67; points below 1e-15 total density give 0.
//
// Density: rho_s = sum_i occ_i |psi_i|^2 (scf/driver.py:663-676), its integral
// and renormalisation (:679-690) and the weighted residual (:693-702).
#include "common.cuh"

namespace igd {
namespace {

constexpr int XB = 256;
inline int xblocks(long long n) { return (int)std::min<long long>((n + XB - 1) / XB, 152LL * 8); }

template <typename M>
struct VwnChan {
  M A, b, c, x0;
};

template <typename M>
__device__ __forceinline__ void vwn_channel(M x, const VwnChan<M>& p, M& g, M& dgdx) {
  const M X = x * x + p.b * x + p.c;
  const M X0 = p.x0 * p.x0 + p.b * p.x0 + p.c;
  const M Q = sqrt(M(4) * p.c - p.b * p.b);
  const M t = M(2) * x + p.b;
  const M at = atan(Q / t);
  const M k = p.b * p.x0 / X0;
  g = p.A * (log(x * x / X) + (M(2) * p.b / Q) * at -
             k * (log((x - p.x0) * (x - p.x0) / X) + (M(2) * (p.b + M(2) * p.x0) / Q) * at));
  const M den = t * t + Q * Q;
  dgdx = p.A * (M(2) / x - t / X - M(4) * p.b / den -
                k * (M(2) / (x - p.x0) - t / X - M(4) * (p.b + M(2) * p.x0) / den));
}

template <typename M>
struct PwChan {
  M A, a1, b1, b2, b3, b4;
};

template <typename M>
__device__ __forceinline__ void pw_channel(M rs, const PwChan<M>& p, M& g, M& dgdrs) {
  const M s = sqrt(rs);
  const M qd = M(2) * p.A * (p.b1 * s + p.b2 * rs + p.b3 * rs * s + p.b4 * rs * rs);
  const M dqd = M(2) * p.A * (M(0.5) * p.b1 / s + p.b2 + M(1.5) * p.b3 * s + M(2) * p.b4 * rs);
  const M lg = log1p(M(1) / qd);
  g = -M(2) * p.A * (M(1) + p.a1 * rs) * lg;
  dgdrs = -M(2) * p.A * p.a1 * lg + M(2) * p.A * (M(1) + p.a1 * rs) * dqd / (qd * qd + qd);
}

// Math in M (float or double); I/O in T; energy reduction in FP64.
template <typename T, typename M, int FUNC>
__global__ void lsda_kernel(long long n, const T* __restrict__ ru_in, const T* __restrict__ rd_in, T* __restrict__ eps,
                            T* __restrict__ vu, T* __restrict__ vd, T* __restrict__ edens,
                            const double* __restrict__ w, double* energy, int* flags) {
  const M pi = M(3.14159265358979323846);
  const M fpp = M(4) / (M(9) * (cbrt(M(2)) - M(1)));
  const M fden = M(2) * cbrt(M(2)) - M(2);
  const M cx = cbrt(M(6) / pi);
  double e_acc = 0.0;
  int fl = 0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double ru64 = (double)ru_in[i], rd64 = (double)rd_in[i];
    if (!isfinite(ru64) || !isfinite(rd64)) fl |= 1;
    if (ru64 < -1.0e-14 || rd64 < -1.0e-14) fl |= 2;
    ru64 = fmax(ru64, 0.0);
    rd64 = fmax(rd64, 0.0);
    const double rho64 = ru64 + rd64;
    M e_out = M(0), vu_out = M(0), vd_out = M(0);
    if (rho64 >= 1.0e-15) {
      const M u = M(ru64), d = M(rd64), r = M(rho64);
      const M cu = cbrt(u), cd = cbrt(d);
      const M ex = -M(0.75) * cx * (u * cu + d * cd);
      const M vxu = -cx * cu, vxd = -cx * cd;
      M z = (u - d) / r;
      z = z > M(1) ? M(1) : (z < M(-1) ? M(-1) : z);
      const M rs = cbrt(M(3) / (M(4) * pi * r));
      M gp, dgp, gf, dgf, ga, dga;
      if (FUNC == 0) {
        const M x = sqrt(rs);
        const VwnChan<M> P{M(0.0310907), M(3.72744), M(12.9352), M(-0.10498)};
        const VwnChan<M> F{M(0.01554535), M(7.06042), M(18.0578), M(-0.32500)};
        const VwnChan<M> Al{M(-1) / (M(6) * pi * pi), M(1.13107), M(13.0045), M(-0.0047584)};
        vwn_channel(x, P, gp, dgp);
        vwn_channel(x, F, gf, dgf);
        vwn_channel(x, Al, ga, dga);
        const M to_rs = M(1) / (M(2) * x);
        dgp *= to_rs;
        dgf *= to_rs;
        dga *= to_rs;
      } else {
        const PwChan<M> P{M(0.031091), M(0.21370), M(7.5957), M(3.5876), M(1.6382), M(0.49294)};
        const PwChan<M> F{M(0.015545), M(0.20548), M(14.1189), M(6.1977), M(3.3662), M(0.62517)};
        const PwChan<M> Al{M(0.016887), M(0.11125), M(10.357), M(3.6231), M(0.88026), M(0.49671)};
        pw_channel(rs, P, gp, dgp);
        pw_channel(rs, F, gf, dgf);
        pw_channel(rs, Al, ga, dga);
        ga = -ga;
        dga = -dga;
      }
      // 1 +- z from the spin densities directly (no cancellation when one spin is tiny)
      const M opz = M(2) * u / r, omz = M(2) * d / r;
      const M a = cbrt(opz), b = cbrt(omz);
      const M f = (opz * a + omz * b - M(2)) / fden;
      const M df = (M(4) / M(3)) * (a - b) / fden;
      const M z3 = z * z * z, z4 = z3 * z;
      const M ec = gp + ga * f * (M(1) - z4) / fpp + (gf - gp) * f * z4;
      const M decrs = dgp + dga * f * (M(1) - z4) / fpp + (dgf - dgp) * f * z4;
      const M decz = ga * (df * (M(1) - z4) - M(4) * z3 * f) / fpp + (gf - gp) * (df * z4 + M(4) * z3 * f);
      const M base = ec - rs / M(3) * decrs;
      e_out = ex / r + ec;
      vu_out = vxu + base + omz * decz;
      vd_out = vxd + base - opz * decz;
    }
    if (eps) eps[i] = T(e_out);
    if (vu) vu[i] = T(vu_out);
    if (vd) vd[i] = T(vd_out);
    const double ed = rho64 * (double)e_out;
    if (edens) edens[i] = T(ed);
    if (w) e_acc += ed * w[i];
  }
  if (energy) {
    double a[1] = {e_acc};
    block_atomic_add<1, XB>(energy, a);
  }
  if (fl) atomicOr(flags, fl);
}

// rho = sum_i occ_i psi_i^2 (FP64 out); *integral += sum rho W.
template <typename T>
__global__ void density_kernel(long long n, int nb, long long stride, const T* __restrict__ psi,
                               const double* __restrict__ occ, const double* __restrict__ w, double* __restrict__ rho,
                               double* integral, int accumulate) {
  double acc = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    // sum over orbitals in the orbital type (FP32 orbitals: FP32 squares and sum,
    // GB300's FP64 pipe would bound the kernel), stored and integrated in FP64
    T t = T(0);
    for (int o = 0; o < nb; ++o) {
      const T p = psi[(long long)o * stride + i];
      t += T(occ[o]) * p * p;
    }
    const double r = (accumulate ? rho[i] : 0.0) + (double)t;
    rho[i] = r;
    if (w) acc += r * w[i];
  }
  if (integral) {
    double a[1] = {acc};
    block_atomic_add<1, XB>(integral, a);
  }
}

// 16-byte form for FP32 orbitals (4 consecutive points per thread; n and the
// orbital stride multiples of 4, 16-byte aligned data): occupations converted
// to FP32 once per block into shared memory (a per-point FP64 conversion would
// bound the kernel on GB300's FP64 pipe), FP32 squares and sum over orbitals,
// FP64 density and integral.
constexpr int DENS_MAXNB = 64;
__global__ void density_v4_kernel(long long n4, int nb, long long stride, const float* __restrict__ psi,
                                  const double* __restrict__ occ, const double* __restrict__ w,
                                  double* __restrict__ rho, double* integral, int accumulate) {
  __shared__ float so[DENS_MAXNB];
  for (int o = threadIdx.x; o < nb; o += blockDim.x) so[o] = (float)occ[o];
  __syncthreads();
  double acc = 0.0;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n4; q += (long long)gridDim.x * blockDim.x) {
    float4 t = make_float4(0.f, 0.f, 0.f, 0.f);
    const float* pq = psi + 4 * q;
#pragma unroll 4
    for (int o = 0; o < nb; ++o) {
      const float4 p = __ldg(reinterpret_cast<const float4*>(pq + (long long)o * stride));
      const float c = so[o];
      t.x = fmaf(c * p.x, p.x, t.x);
      t.y = fmaf(c * p.y, p.y, t.y);
      t.z = fmaf(c * p.z, p.z, t.z);
      t.w = fmaf(c * p.w, p.w, t.w);
    }
    double2* r2 = reinterpret_cast<double2*>(rho + 4 * q);
    double2 a = make_double2((double)t.x, (double)t.y), b = make_double2((double)t.z, (double)t.w);
    if (accumulate) {
      const double2 ra = r2[0], rb = r2[1];
      a.x += ra.x;
      a.y += ra.y;
      b.x += rb.x;
      b.y += rb.y;
    }
    r2[0] = a;
    r2[1] = b;
    if (w) {
      const double2 wa = __ldg(reinterpret_cast<const double2*>(w + 4 * q)),
                    wb = __ldg(reinterpret_cast<const double2*>(w + 4 * q + 2));
      acc += a.x * wa.x + a.y * wa.y + b.x * wb.x + b.y * wb.y;
    }
  }
  if (integral) {
    double v[1] = {acc};
    block_atomic_add<1, XB>(integral, v);
  }
}

// rho *= target / integral (integral read on the device; no host sync).
__global__ void renorm_kernel(long long n, double* __restrict__ rho, const double* integral, double target,
                              int* flags) {
  const double s = *integral;
  if (!(s > 0.0)) {
    if (blockIdx.x == 0 && threadIdx.x == 0) atomicOr(flags, 4);
    return;
  }
  const double f = target / s;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    rho[i] *= f;
}

// sum ((up_o - up_i)^2 + (dn_o - dn_i)^2) W
__global__ void residual2_kernel(long long n, const double* __restrict__ ui, const double* __restrict__ di,
                                 const double* __restrict__ uo, const double* __restrict__ dout,
                                 const double* __restrict__ w, double* out) {
  double acc = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double a = uo[i] - ui[i], b = dout[i] - di[i];
    acc += (a * a + b * b) * w[i];
  }
  double a[1] = {acc};
  block_atomic_add<1, XB>(out, a);
}

__global__ void zero1(double* p) { *p = 0.0; }

}  // namespace
}  // namespace igd

using namespace igd;

// LSDA on n points.  dtype = I/O type, math = IGD_F64 or IGD_F32 arithmetic,
// functional 0 = Slater + VWN5 ("lda,vwn"), 1 = Slater + PW92.  Any output may be
// NULL.  energy (device double) = sum rho eps W when w and energy are given
// (zeroed first).  flags (device int) |= 1 non-finite input, 2 negative below
// -1e-14 (the caller raises).
extern "C" int igd_lsda(int dtype, int math, int functional, long long n, const void* rho_up, const void* rho_down,
                        void* eps, void* v_up, void* v_down, void* energy_density, const double* w, double* energy,
                        int* flags, void* stream) {
  if (n <= 0 || !rho_up || !rho_down || !flags || functional < 0 || functional > 1) return IGD_ERR_ARG;
  cudaStream_t st = as_stream(stream);
  if (energy) zero1<<<1, 1, 0, st>>>(energy);
  const int g = xblocks(n);
#define IGD_LSDA_LAUNCH(T, M, F)                                                                                   \
  lsda_kernel<T, M, F><<<g, XB, 0, st>>>(n, static_cast<const T*>(rho_up), static_cast<const T*>(rho_down),        \
                                         static_cast<T*>(eps), static_cast<T*>(v_up), static_cast<T*>(v_down),     \
                                         static_cast<T*>(energy_density), w, energy, flags)
  if (dtype == IGD_F64 && math == IGD_F64) {
    if (functional == 0) IGD_LSDA_LAUNCH(double, double, 0); else IGD_LSDA_LAUNCH(double, double, 1);
  } else if (dtype == IGD_F64 && math == IGD_F32) {
    if (functional == 0) IGD_LSDA_LAUNCH(double, float, 0); else IGD_LSDA_LAUNCH(double, float, 1);
  } else if (dtype == IGD_F32 && math == IGD_F32) {
    if (functional == 0) IGD_LSDA_LAUNCH(float, float, 0); else IGD_LSDA_LAUNCH(float, float, 1);
  } else if (dtype == IGD_F32 && math == IGD_F64) {
    if (functional == 0) IGD_LSDA_LAUNCH(float, double, 0); else IGD_LSDA_LAUNCH(float, double, 1);
  } else {
    return IGD_ERR_DTYPE;
  }
#undef IGD_LSDA_LAUNCH
  return launch_status();
}

// rho (FP64, n) = [rho +] sum_i occupations[i] psi_i^2 over nb orbitals of `dtype`
// separated by stride elements; occupations: nb device doubles.  integral (device,
// may be NULL) = sum rho W (zeroed first).
extern "C" int igd_density(int dtype, long long n, int nb, long long stride, const void* psi, const double* occupations,
                           const double* w, double* rho, double* integral, int accumulate, void* stream) {
  if (n <= 0 || nb < 0 || !rho || (nb > 0 && (!psi || !occupations))) return IGD_ERR_ARG;
  cudaStream_t st = as_stream(stream);
  if (integral) zero1<<<1, 1, 0, st>>>(integral);
  if (dtype == IGD_F64)
    density_kernel<double><<<xblocks(n), XB, 0, st>>>(n, nb, stride, static_cast<const double*>(psi), occupations, w,
                                                      rho, integral, accumulate);
  else if (dtype == IGD_F32 && n % 4 == 0 && stride % 4 == 0 && nb <= DENS_MAXNB &&
           ((reinterpret_cast<uintptr_t>(psi) | reinterpret_cast<uintptr_t>(rho) | reinterpret_cast<uintptr_t>(w)) &
            15u) == 0)
    density_v4_kernel<<<xblocks(n / 4), XB, 0, st>>>(n / 4, nb, stride, static_cast<const float*>(psi), occupations,
                                                     w, rho, integral, accumulate);
  else if (dtype == IGD_F32)
    density_kernel<float><<<xblocks(n), XB, 0, st>>>(n, nb, stride, static_cast<const float*>(psi), occupations, w,
                                                     rho, integral, accumulate);
  else
    return IGD_ERR_DTYPE;
  return launch_status();
}

// rho *= target / *integral on the device (flags |= 4 when the integral is not positive).
extern "C" int igd_density_renormalize(long long n, double* rho, const double* integral, double target, int* flags,
                                       void* stream) {
  if (n <= 0 || !rho || !integral || !flags) return IGD_ERR_ARG;
  renorm_kernel<<<xblocks(n), XB, 0, as_stream(stream)>>>(n, rho, integral, target, flags);
  return launch_status();
}

// *out = sum ((up_out - up_in)^2 + (dn_out - dn_in)^2) W (square of _density_residual).
extern "C" int igd_density_residual2(long long n, const double* up_in, const double* dn_in, const double* up_out,
                                     const double* dn_out, const double* w, double* out, void* stream) {
  if (n <= 0 || !up_in || !dn_in || !up_out || !dn_out || !w || !out) return IGD_ERR_ARG;
  cudaStream_t st = as_stream(stream);
  zero1<<<1, 1, 0, st>>>(out);
  residual2_kernel<<<xblocks(n), XB, 0, st>>>(n, up_in, dn_in, up_out, dn_out, w, out);
  return launch_status();
}
