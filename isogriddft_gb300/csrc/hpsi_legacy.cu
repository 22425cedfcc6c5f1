// Legacy separable sinh-grid H.Psi (K2): ops/kinetic.py:87-153.
//
// Per axis the reference forms face fluxes (psi[i+1]-psi[i])/(du h_face) with
// zero ghosts and divides their difference by du h[i]; the host folds that
// into two coefficient vectors per axis, cm and cp, so that
//   lap_axis(i) = cp[i] (psi[i+1] - psi[i]) - cm[i] (psi[i] - psi[i-1]),
// psi[-1] = psi[n] = 0.  Each thread marches along x over a chunk of
// planes, keeping psi[i-1], psi[i], psi[i+1] in registers.
#include "common.cuh"

namespace igd {
namespace {

// One thread per (column, x-chunk): the march covers xc consecutive planes,
// xc chosen on the host so that small grids still fill every SM.
template <typename T>
__global__ void __launch_bounds__(256) hpsi_legacy_kernel(const double* __restrict__ cf, const T* __restrict__ veff,
                                                          const T* __restrict__ psi, T* __restrict__ out, int nx,
                                                          int ny, int nz, int nb, long long ostride, T kscale,
                                                          T vscale, int xc) {
  const long long plane = (long long)ny * nz;
  const int nchunks = (nx + xc - 1) / xc;
  const long long cols = plane * nb;
  const long long work = cols * nchunks;
  const double *cxm = cf, *cxp = cf + nx, *cym = cf + 2 * nx, *cyp = cym + ny, *czm = cf + 2 * nx + 2 * ny,
               *czp = czm + nz;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < work; t += (long long)gridDim.x * blockDim.x) {
    const int chunk = (int)(t / cols);
    const long long oc = t - (long long)chunk * cols;
    const int o = (int)(oc / plane);
    const long long col = oc - (long long)o * plane;
    const int j = (int)(col / nz), k = (int)(col - (long long)j * nz);
    const T* p = psi + (long long)o * ostride;
    T* q = out + (long long)o * ostride;
    const T ymc = T(cym[j]), ypc = T(cyp[j]), zmc = T(czm[k]), zpc = T(czp[k]);
    const int i0 = chunk * xc, i1 = min(nx, i0 + xc);
    T prev = i0 > 0 ? __ldg(p + (long long)(i0 - 1) * plane + col) : T(0);
    T cur = __ldg(p + (long long)i0 * plane + col), next;
    for (int i = i0; i < i1; ++i) {
      const long long g = (long long)i * plane + col;
      next = (i + 1 < nx) ? __ldg(p + g + plane) : T(0);
      const T ym = j > 0 ? __ldg(p + g - nz) : T(0);
      const T yp = j + 1 < ny ? __ldg(p + g + nz) : T(0);
      const T zm = k > 0 ? __ldg(p + g - 1) : T(0);
      const T zp = k + 1 < nz ? __ldg(p + g + 1) : T(0);
      const T lap = (T(cxp[i]) * (next - cur) - T(cxm[i]) * (cur - prev)) + (ypc * (yp - cur) - ymc * (cur - ym)) +
                    (zpc * (zp - cur) - zmc * (cur - zm));
      const T v = veff ? __ldg(veff + g) : T(0);
      q[g] = kscale * lap + vscale * v * cur;
      prev = cur;
      cur = next;
    }
  }
}

}  // namespace
}  // namespace igd

using namespace igd;

extern "C" int igd_hpsi_legacy(int dtype, int nx, int ny, int nz, const double* axis_coeffs, const void* veff,
                               const void* psi, void* out, int nb, long long orbital_stride, double kscale,
                               double vscale, void* stream) {
  if (nx < 2 || ny < 2 || nz < 2 || nb < 1 || !axis_coeffs || !psi || !out) return IGD_ERR_ARG;
  if (nb > 1 && orbital_stride < (long long)nx * ny * nz) return IGD_ERR_ARG;
  const long long cols = (long long)ny * nz * nb;
  // enough threads for ~8 resident 256-thread blocks on each of 152 SMs
  const long long target = 152LL * 8 * 256;
  const int xc = (int)std::max<long long>(1, std::min<long long>(nx, (cols * nx + target - 1) / target));
  const long long work = cols * ((nx + xc - 1) / xc);
  const int blocks = (int)std::min<long long>((work + 255) / 256, 152LL * 64);
  cudaStream_t st = as_stream(stream);
  if (dtype == IGD_F32)
    hpsi_legacy_kernel<float><<<blocks, 256, 0, st>>>(axis_coeffs, static_cast<const float*>(veff),
                                                      static_cast<const float*>(psi), static_cast<float*>(out), nx, ny,
                                                      nz, nb, orbital_stride, (float)kscale, (float)vscale, xc);
  else if (dtype == IGD_F64)
    hpsi_legacy_kernel<double><<<blocks, 256, 0, st>>>(axis_coeffs, static_cast<const double*>(veff),
                                                       static_cast<const double*>(psi), static_cast<double*>(out), nx,
                                                       ny, nz, nb, orbital_stride, kscale, vscale, xc);
  else
    return IGD_ERR_DTYPE;
  return launch_status();
}
