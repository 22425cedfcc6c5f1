// GTH pseudopotential terms: local potential (setup, per geometry) and the
// separable nonlocal action over compact atom-centred spheres (K3).
//
// Local: V(r) = -Z erf(r / (sqrt2 rloc)) / r + exp(-r^2 / 2 rloc^2)
//               sum_i C_i (r / rloc)^(2i),  r = 0: -Z sqrt(2/pi) / rloc
// (pseudo/local.py:138-205), summed over atoms (:303-357).
// Nonlocal: V_nl psi = sum_{atom,l,m} sum_ij p_i h_ij <p_j | psi>_W
// (pseudo/nonlocal.py:209-283).  The reference evaluates the projectors on the
// whole grid; here they are tabulated once per geometry on the points where
// they exceed 1e-17 of their peak (a sphere around each atom), stored as
// (point index, value) lists, and applied as a gather-dot followed by a
// scatter-add into H psi.
#include "common.cuh"

namespace igd {
namespace {

constexpr int LB = 256;
inline int lblocks(long long n) { return (int)std::min<long long>((n + LB - 1) / LB, 152LL * 8); }

// atoms: 8 doubles each (x, y, z, Z_ion, rloc, C1, C2, C3)
__global__ void local_potential_kernel(long long n, const double* __restrict__ X, const double* __restrict__ Y,
                                       const double* __restrict__ Z, int natoms, const double* __restrict__ atoms,
                                       double* __restrict__ out) {
  const double s2 = sqrt(2.0), s2pi = sqrt(2.0 / 3.14159265358979323846);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double v = 0.0;
    for (int a = 0; a < natoms; ++a) {
      const double* p = atoms + 8 * a;
      const double dx = X[i] - p[0], dy = Y[i] - p[1], dz = Z[i] - p[2];
      const double r = sqrt(dx * dx + dy * dy + dz * dz);
      const double zion = p[3], rl = p[4];
      const double coul = r == 0.0 ? -zion * s2pi / rl : -zion * erf(r / (s2 * rl)) / r;
      const double sr = r / rl, s2r = sr * sr;
      const double poly = p[5] + p[6] * s2r + p[7] * s2r * s2r;
      v += coul + exp(-0.5 * s2r) * poly;
    }
    out[i] = v;
  }
}

// dV/dr of one atom's local GTH potential (the radial derivative of
// local_potential_kernel's expression).  Near r = 0 the Coulomb part uses the
// series of erf(x)/x, whose derivative vanishes at the origin.
__device__ __forceinline__ double local_dvdr(double r, const double* p) {
  const double zion = p[3], rl = p[4];
  const double a = 1.0 / (sqrt(2.0) * rl), x = a * r;
  const double c2pi = 2.0 / sqrt(3.14159265358979323846);
  double dcoul;
  if (x < 1.0e-2) {
    // d/dx [erf(x)/x] = (2/sqrt(pi)) (-2x/3 + 2x^3/5 - x^5/7)
    const double x2 = x * x;
    dcoul = -zion * a * a * c2pi * x * (-2.0 / 3.0 + x2 * (2.0 / 5.0 - x2 / 7.0));
  } else {
    dcoul = -zion * (c2pi * a * exp(-x * x) / r - erf(x) / (r * r));
  }
  const double s = r / rl, s2 = s * s;
  const double poly = p[5] + p[6] * s2 + p[7] * s2 * s2;
  const double dpoly = (2.0 * p[6] * s + 4.0 * p[7] * s2 * s) / rl;
  const double g = exp(-0.5 * s2);
  return dcoul + g * (dpoly - r / (rl * rl) * poly);
}

// Hellmann-Feynman local force on each atom: F_a = sum_i rho_i W_i V_a'(r) (r_i - R_a)/r.
// One block-level FP64 reduction per atom and component into out[3 * natoms].
constexpr int FB = 256;
__global__ void local_force_kernel(long long n, const double* __restrict__ X, const double* __restrict__ Y,
                                   const double* __restrict__ Z, const double* __restrict__ rho,
                                   const double* __restrict__ w, int a0, int na, const double* __restrict__ atoms,
                                   double* __restrict__ out) {
  double f[3 * 4] = {};
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double q = rho[i] * w[i];
    for (int a = 0; a < na; ++a) {
      const double* p = atoms + 8 * (a0 + a);
      const double dx = X[i] - p[0], dy = Y[i] - p[1], dz = Z[i] - p[2];
      const double r = sqrt(dx * dx + dy * dy + dz * dz);
      if (r == 0.0) continue;
      const double c = q * local_dvdr(r, p) / r;
      f[3 * a] += c * dx;
      f[3 * a + 1] += c * dy;
      f[3 * a + 2] += c * dz;
    }
  }
  __shared__ double scratch[12 * (FB / 32)];
  block_sum<12, FB>(f, scratch);
  if (threadIdx.x == 0)
    for (int k = 0; k < 3 * na; ++k) atomicAdd(out + 3 * a0 + k, f[k]);
}

// c[j * nb + o] = sum_p val[j][p] W[idx[p]] psi_o[idx[p]] over the projector's
// point list (offsets[j] .. offsets[j+1]).  One block per (projector, orbital).
template <typename T>
__global__ void nl_gather_kernel(int nproj, const long long* __restrict__ offsets, const int* __restrict__ idx,
                                 const double* __restrict__ val, const double* __restrict__ w,
                                 const T* __restrict__ psi, long long stride, int nb, double* __restrict__ c) {
  const int j = blockIdx.x, o = blockIdx.y;
  if (j >= nproj || o >= nb) return;
  double s = 0.0;
  for (long long q = offsets[j] + threadIdx.x; q < offsets[j + 1]; q += blockDim.x) {
    const int g = idx[q];
    s += val[q] * w[g] * (double)psi[(long long)o * stride + g];
  }
  __shared__ double red[32];
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    double t = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    t = warp_sum(t);
    if (threadIdx.x == 0) c[(long long)j * nb + o] = t;
  }
}

// d = H c within each (atom, l, m) group: groups[g] = (first projector, count);
// hmat: per group count x count doubles at hoff[g].
__global__ void nl_contract_kernel(int ngroups, const int* __restrict__ groups, const long long* __restrict__ hoff,
                                   const double* __restrict__ hmat, const double* __restrict__ c, int nb,
                                   double* __restrict__ d) {
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ngroups * nb; e += gridDim.x * blockDim.x) {
    const int g = e / nb, o = e - g * nb;
    const int first = groups[2 * g], cnt = groups[2 * g + 1];
    const double* H = hmat + hoff[g];
    for (int a = 0; a < cnt; ++a) {
      double s = 0.0;
      for (int b = 0; b < cnt; ++b) s += H[a * cnt + b] * c[(long long)(first + b) * nb + o];
      d[(long long)(first + a) * nb + o] = s;
    }
  }
}

// out_o[idx[p]] += scale * d[j][o] * val[j][p] (atomic: spheres overlap)
template <typename T>
__global__ void nl_scatter_kernel(int nproj, const long long* __restrict__ offsets, const int* __restrict__ idx,
                                  const double* __restrict__ val, const double* __restrict__ d, T* __restrict__ out,
                                  long long stride, int nb, double scale) {
  const int j = blockIdx.x, o = blockIdx.y;
  if (j >= nproj || o >= nb) return;
  const double coef = scale * d[(long long)j * nb + o];
  if (coef == 0.0) return;
  for (long long q = offsets[j] + threadIdx.x; q < offsets[j + 1]; q += blockDim.x)
    atomicAdd(out + (long long)o * stride + idx[q], T(coef * val[q]));
}

}  // namespace
}  // namespace igd

using namespace igd;

extern "C" int igd_gth_local_potential(long long n, const double* x, const double* y, const double* z, int natoms,
                                       const double* atoms, double* out, void* stream) {
  if (n <= 0 || !x || !y || !z || !out || natoms < 0 || (natoms && !atoms)) return IGD_ERR_ARG;
  local_potential_kernel<<<lblocks(n), LB, 0, as_stream(stream)>>>(n, x, y, z, natoms, atoms, out);
  return launch_status();
}

// Hellmann-Feynman force of the local GTH potential, F_a = -dE_loc/dR_a for
// E_loc = sum_i rho_i W_i V_loc(r_i); out: 3 * natoms doubles (overwritten).
extern "C" int igd_gth_local_force(long long n, const double* x, const double* y, const double* z,
                                   const double* rho, const double* w, int natoms, const double* atoms, double* out,
                                   void* stream) {
  if (n <= 0 || !x || !y || !z || !rho || !w || !out || natoms < 1 || !atoms) return IGD_ERR_ARG;
  cudaStream_t st = as_stream(stream);
  if (cudaMemsetAsync(out, 0, sizeof(double) * 3 * natoms, st) != cudaSuccess) return IGD_ERR_CUDA;
  // up to 4 atoms per pass (12 accumulators per thread)
  const int blocks = (int)std::min<long long>((n + FB - 1) / FB, 152LL * 4);
  for (int a0 = 0; a0 < natoms; a0 += 4) {
    const int na = std::min(4, natoms - a0);
    local_force_kernel<<<blocks, FB, 0, st>>>(n, x, y, z, rho, w, a0, na, atoms, out);
  }
  return launch_status();
}

// Apply scale * V_nl to nb orbitals psi (stride elements apart), adding into out.
// Projectors: nproj point lists (offsets[nproj+1] into idx / val); ngroups
// (atom, l, m) groups with their h matrices.  workspace: 2 * nproj * nb doubles.
extern "C" int igd_gth_nonlocal_apply(int dtype, int nproj, const long long* offsets, const int* idx,
                                      const double* val, int ngroups, const int* groups, const long long* hoff,
                                      const double* hmat, const double* w, const void* psi, void* out, int nb,
                                      long long stride, double scale, double* workspace, void* stream) {
  if (nproj < 0 || nb < 1 || !psi || !out || (nproj > 0 && (!offsets || !idx || !val || !groups || !hoff || !hmat ||
                                                            !w || !workspace)))
    return IGD_ERR_ARG;
  if (nproj == 0) return IGD_OK;
  cudaStream_t st = as_stream(stream);
  double* c = workspace;
  double* d = workspace + (long long)nproj * nb;
  dim3 grid(nproj, nb);
  if (dtype == IGD_F32) {
    nl_gather_kernel<float><<<grid, 256, 0, st>>>(nproj, offsets, idx, val, w, static_cast<const float*>(psi), stride,
                                                  nb, c);
    nl_contract_kernel<<<(ngroups * nb + 127) / 128, 128, 0, st>>>(ngroups, groups, hoff, hmat, c, nb, d);
    nl_scatter_kernel<float><<<grid, 256, 0, st>>>(nproj, offsets, idx, val, d, static_cast<float*>(out), stride, nb,
                                                   scale);
  } else if (dtype == IGD_F64) {
    nl_gather_kernel<double><<<grid, 256, 0, st>>>(nproj, offsets, idx, val, w, static_cast<const double*>(psi),
                                                   stride, nb, c);
    nl_contract_kernel<<<(ngroups * nb + 127) / 128, 128, 0, st>>>(ngroups, groups, hoff, hmat, c, nb, d);
    nl_scatter_kernel<double><<<grid, 256, 0, st>>>(nproj, offsets, idx, val, d, static_cast<double*>(out), stride,
                                                    nb, scale);
  } else {
    return IGD_ERR_DTYPE;
  }
  return launch_status();
}

// Projections out[j * nb + o] = <p_j | psi_o>_W (the gather stage of the
// nonlocal apply; with gradient tables in val, <d p_j / d x_k | psi_o>_W).
extern "C" int igd_gth_projections(int dtype, int nproj, const long long* offsets, const int* idx, const double* val,
                                   const double* w, const void* psi, int nb, long long stride, double* out,
                                   void* stream) {
  if (nproj < 0 || nb < 1 || !psi || !out || (nproj > 0 && (!offsets || !idx || !val || !w))) return IGD_ERR_ARG;
  if (nproj == 0) return IGD_OK;
  cudaStream_t st = as_stream(stream);
  dim3 grid(nproj, nb);
  if (dtype == IGD_F32)
    nl_gather_kernel<float><<<grid, 256, 0, st>>>(nproj, offsets, idx, val, w, static_cast<const float*>(psi), stride,
                                                  nb, out);
  else if (dtype == IGD_F64)
    nl_gather_kernel<double><<<grid, 256, 0, st>>>(nproj, offsets, idx, val, w, static_cast<const double*>(psi),
                                                   stride, nb, out);
  else
    return IGD_ERR_DTYPE;
  return launch_status();
}
