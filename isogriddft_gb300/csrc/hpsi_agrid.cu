// Fused monitor A-grid H.Psi stencil (K1) and its geometry pre-folding.
//
// Replaces ops/kinetic.py:212-358 (flux form T psi = -1/2 J^-1 d_a(J g^ab d_b psi)
// with centred differences applied twice) plus the v_eff * psi term of
// ks/eigensolver.py:753-756, for a block of orbitals in one pass.
//
// Both edge closures are centred differences with a ghost value beyond each
// face: zero for the trial fix (ops/kinetic.py:165-187) and the quadratic
// extrapolation 3 f0 - 3 f1 + f2 for np.gradient(edge_order=2)
// (ops/kinetic.py:202-209), which reproduces (-3 f0 + 4 f1 - f2)/(2h).
// The same rule applies to psi (gradient pass) and to the fluxes
// (divergence pass).
//
// Work decomposition: a CTA owns a 32 (z) x 8 (y) column tile and marches
// along x over a chunk of planes, for NB orbitals at once so every geometry
// value is read once per CTA.  psi planes (tile + 2-point halo) stream through
// a 4-slot shared-memory ring with cp.async zero-fill; fluxes F^y, F^z of the
// current plane live in shared memory (1-point halo), F^x in registers.
#include <algorithm>
#include <cstdlib>
#include <initializer_list>

#include "common.cuh"

namespace igd {
namespace {

// Block = WY warps x 32 lanes; lane C / warp R compute fluxes at global
// (j0-1+R, k0-1+C); lanes 1..30 of warps 1..WY-2 emit the output tile.
constexpr int WZ = 32, WY = 16, NT = WZ * WY;
constexpr int OZ = WZ - 2, OY = WY - 2;
constexpr int PZ = WZ + 2, PY = WY + 2;  // psi tile: 1-point halo around the flux points
constexpr int RING = 6;                  // planes s-1, s, s+1 resident; s+2..s+4 in flight
constexpr int AHEAD = RING - 2;
constexpr int LOADS = (PY * PZ + NT - 1) / NT;

template <typename T>
struct Coeffs {
  const T* axx;
  const T* ayy;
  const T* azz;
  const T* axy;
  const T* axz;
  const T* ayz;
  const T* ij;
};

template <typename T, int NB>
struct Smem {
  T ring[RING][NB][PY][PZ];
  T fy[2][NB][WY][WZ];
};

__device__ __forceinline__ int slot_of(int p) { return (p + RING) % RING; }

// Production closure: psi cells one step beyond the y / z faces get 3 f0 - 3 f1 + f2.
template <typename T, int NB>
__device__ __forceinline__ void ghost_fill_yz(Smem<T, NB>& sm, int p, int ny, int nz, int j0, int k0) {
  const int sl = slot_of(p);
  const int ylo = 1 - j0, yhi = ny - j0 + 2, zlo = 1 - k0, zhi = nz - k0 + 2;
  for (int idx = threadIdx.x; idx < NB * 2 * PZ; idx += NT) {
    const int o = idx / (2 * PZ), side = (idx / PZ) & 1, zz = idx % PZ;
    const int k = k0 - 2 + zz, yy = side ? yhi : ylo, d = side ? -1 : 1;
    if (k < 0 || k >= nz || yy < 0 || yy >= PY) continue;
    auto& a = sm.ring[sl][o];
    a[yy][zz] = T(3) * a[yy + d][zz] - T(3) * a[yy + 2 * d][zz] + a[yy + 3 * d][zz];
  }
  for (int idx = threadIdx.x; idx < NB * 2 * PY; idx += NT) {
    const int o = idx / (2 * PY), side = (idx / PY) & 1, yy = idx % PY;
    const int j = j0 - 2 + yy, zz = side ? zhi : zlo, d = side ? -1 : 1;
    if (j < 0 || j >= ny || zz < 0 || zz >= PZ) continue;
    auto& a = sm.ring[sl][o];
    a[yy][zz] = T(3) * a[yy][zz + d] - T(3) * a[yy][zz + 2 * d] + a[yy][zz + 3 * d];
  }
}

// Ghost plane p from planes p+d, p+2d, p+3d (zero for the trial fix).
template <typename T, int NB, bool PROD>
__device__ __forceinline__ void ghost_plane(Smem<T, NB>& sm, int p, int d) {
  const int s0 = slot_of(p), s1 = slot_of(p + d), s2 = slot_of(p + 2 * d), s3 = slot_of(p + 3 * d);
  T* a0 = &sm.ring[s0][0][0][0];
  const T* a1 = &sm.ring[s1][0][0][0];
  const T* a2 = &sm.ring[s2][0][0][0];
  const T* a3 = &sm.ring[s3][0][0][0];
  for (int idx = threadIdx.x; idx < NB * PY * PZ; idx += NT)
    a0[idx] = PROD ? T(3) * a1[idx] - T(3) * a2[idx] + a3[idx] : T(0);
}

template <typename T, int NB, bool PROD>
__global__ void __launch_bounds__(NT) hpsi_agrid_kernel(Coeffs<T> c, const T* __restrict__ veff,
                                                        const T* __restrict__ psi, T* __restrict__ out, int nx,
                                                        int ny, int nz, int nb, long long ostride, T kscale,
                                                        T vscale, int chunk, int tiles_z) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Smem<T, NB>& sm = *reinterpret_cast<Smem<T, NB>*>(smem_raw);

  const int tid = threadIdx.x, C = tid & (WZ - 1), R = tid / WZ;
  const int tzi = blockIdx.x % tiles_z, tyi = blockIdx.x / tiles_z;
  const int k0 = min(tzi * OZ, max(nz - OZ, 0));
  const int j0 = min(tyi * OY, max(ny - OY, 0));
  const int x0 = blockIdx.y * chunk, x1 = min(nx, x0 + chunk);
  const int o0 = blockIdx.z * NB;
  const long long plane = (long long)ny * nz;

  const int j = j0 - 1 + R, k = k0 - 1 + C;
  const bool real = j >= 0 && j < ny && k >= 0 && k < nz;
  const bool emit = real && R >= 1 && R <= OY && C >= 1 && C <= OZ;
  const long long col = real ? (long long)j * nz + k : 0;
  // block-uniform face flags
  const bool yface = (j0 == 0) || (ny - j0 <= OY);
  const bool zface = (k0 == 0) || (nz - k0 <= OZ);

  // per-thread psi-tile load slots (precomputed offsets)
  int ld_sm[LOADS];
  long long ld_off[LOADS];
  bool ld_ok[LOADS];
#pragma unroll
  for (int l = 0; l < LOADS; ++l) {
    const int e = tid + l * NT;
    const int yy = e / PZ, zz = e - yy * PZ;
    const int jj = j0 - 2 + yy, kk = k0 - 2 + zz;
    ld_ok[l] = e < PY * PZ && jj >= 0 && jj < ny && kk >= 0 && kk < nz;
    ld_sm[l] = e < PY * PZ ? e : 0;
    ld_off[l] = ld_ok[l] ? (long long)jj * nz + kk : 0;
  }
  int nvalid_o = nb - o0;
  if (nvalid_o > NB) nvalid_o = NB;
  auto load_plane = [&](int p) {
    const T* base = psi + (long long)p * plane;
    T* dst0 = &sm.ring[slot_of(p)][0][0][0];
#pragma unroll
    for (int o = 0; o < NB; ++o) {
      const T* b = base + (long long)(o0 + o) * ostride;
#pragma unroll
      for (int l = 0; l < LOADS; ++l) {
        if (tid + l * NT < PY * PZ) {
          const bool ok = ld_ok[l] && o < nvalid_o;
          cp_async_zfill<sizeof(T)>(dst0 + o * PY * PZ + ld_sm[l], ok ? b + ld_off[l] : psi, ok);
        }
      }
    }
  };

  const int sb = x0 == 0 ? 0 : min(x0 - 1, max(nx - 3, 0));  // F^x(nx-3) needed by the last-face ghost
  const int se = x1 == nx ? nx - 1 : x1;
  const int last = min(nx - 1, se + 1);
  const int pro_lo = max(sb - 1, 0), pro_hi = min(sb + AHEAD - 1, last);
  for (int p = pro_lo; p <= pro_hi; ++p) load_plane(p);
  cp_async_commit();

  // geometry of plane sb (flux coefficients) and sb-1 (output scaling) in registers
  auto ldg0 = [&](const T* a, long long g) { return real ? __ldg(a + g) : T(0); };
  T gxx, gyy, gzz, gxy, gxz, gyz, gij, gv;
  {
    const long long g = (long long)sb * plane + col;
    gxx = ldg0(c.axx, g); gyy = ldg0(c.ayy, g); gzz = ldg0(c.azz, g);
    gxy = ldg0(c.axy, g); gxz = ldg0(c.axz, g); gyz = ldg0(c.ayz, g);
    gij = ldg0(c.ij, g); gv = veff ? ldg0(veff, g) : T(0);
  }
  cp_async_wait<0>();
  __syncthreads();
  if (PROD && (yface || zface)) {
    for (int p = pro_lo; p <= pro_hi; ++p) ghost_fill_yz<T, NB>(sm, p, ny, nz, j0, k0);
    __syncthreads();
  }
  if (sb == 0) {
    ghost_plane<T, NB, PROD>(sm, -1, +1);
    __syncthreads();
  }

  const int yy0 = R + 1, zz0 = C + 1;  // own cell inside the psi tile
  T pm1[NB], p0[NB], pp1[NB], fxm2[NB], fxm1[NB], fx0[NB], fzp[NB], pend[NB];
#pragma unroll
  for (int o = 0; o < NB; ++o) {
    pm1[o] = sm.ring[slot_of(sb - 1)][o][yy0][zz0];
    p0[o] = sm.ring[slot_of(sb)][o][yy0][zz0];
    pp1[o] = T(0);
    fxm2[o] = fxm1[o] = fx0[o] = fzp[o] = pend[o] = T(0);
  }
  T ij_prev = T(0), v_prev = T(0), pend_ij = T(0);

  for (int s = sb; s <= se; ++s) {
    const int buf = s & 1;
    // ---- stream: issue plane s+AHEAD, wait for plane s+1
    const int pn = s + AHEAD;
    if (pn > pro_hi && pn <= last) load_plane(pn);
    cp_async_commit();
    cp_async_wait<AHEAD - 1>();
    __syncthreads();
    if (s + 1 == nx) {
      ghost_plane<T, NB, PROD>(sm, nx, -1);
      __syncthreads();
    } else if (PROD && (yface || zface) && s + 1 > pro_hi) {
      ghost_fill_yz<T, NB>(sm, s + 1, ny, nz, j0, k0);
      __syncthreads();
    }
    // geometry of plane s (registers) -> issue loads for plane s+1
    const T axx = gxx, ayy = gyy, azz = gzz, axy = gxy, axz = gxz, ayz = gyz;
    const T ij_s = gij, v_s = gv;
    if (s + 1 <= se) {
      const long long g = (long long)(s + 1) * plane + col;
      gxx = ldg0(c.axx, g); gyy = ldg0(c.ayy, g); gzz = ldg0(c.azz, g);
      gxy = ldg0(c.axy, g); gxz = ldg0(c.axz, g); gyz = ldg0(c.ayz, g);
      gij = ldg0(c.ij, g); gv = veff ? ldg0(veff, g) : T(0);
    }
    // ---- fluxes of plane s at every (R, C)
    T fzc[NB];
    const int sl0 = slot_of(s), slp = slot_of(s + 1);
#pragma unroll
    for (int o = 0; o < NB; ++o) {
      if (s > sb) {
        pm1[o] = p0[o];
        p0[o] = pp1[o];
      }
      pp1[o] = sm.ring[slp][o][yy0][zz0];
      const T gx = pp1[o] - pm1[o];
      const T gy = sm.ring[sl0][o][yy0 + 1][zz0] - sm.ring[sl0][o][yy0 - 1][zz0];
      const T gz = sm.ring[sl0][o][yy0][zz0 + 1] - sm.ring[sl0][o][yy0][zz0 - 1];
      fxm2[o] = fxm1[o];
      fxm1[o] = fx0[o];
      fx0[o] = axx * gx + axy * gy + axz * gz;
      sm.fy[buf][o][R][C] = axy * gx + ayy * gy + ayz * gz;
      fzc[o] = axz * gx + ayz * gy + azz * gz;
    }
    if (zface) {  // F^z ghosts at k = -1 / nz from the three inner lanes
      const bool lo = (k == -1), hi = (k == nz);
#pragma unroll
      for (int o = 0; o < NB; ++o) {
        const T d1 = __shfl_down_sync(0xffffffffu, fzc[o], 1), d2 = __shfl_down_sync(0xffffffffu, fzc[o], 2),
                d3 = __shfl_down_sync(0xffffffffu, fzc[o], 3);
        const T u1 = __shfl_up_sync(0xffffffffu, fzc[o], 1), u2 = __shfl_up_sync(0xffffffffu, fzc[o], 2),
                u3 = __shfl_up_sync(0xffffffffu, fzc[o], 3);
        if (lo) fzc[o] = PROD ? T(3) * d1 - T(3) * d2 + d3 : T(0);
        if (hi) fzc[o] = PROD ? T(3) * u1 - T(3) * u2 + u3 : T(0);
      }
    }
    __syncthreads();
    if (yface && (j == -1 || j == ny)) {  // F^y ghost rows from the three inner rows
      const int d = (j == -1) ? 1 : -1;
#pragma unroll
      for (int o = 0; o < NB; ++o)
        sm.fy[buf][o][R][C] = PROD ? T(3) * sm.fy[buf][o][R + d][C] - T(3) * sm.fy[buf][o][R + 2 * d][C] +
                                         sm.fy[buf][o][R + 3 * d][C]
                                   : T(0);
    }
    if (yface) __syncthreads();

    // ---- output plane s-1 (F^x from registers, F^y from smem of step s-1, F^z via shuffles)
    const int op = s - 1;
    const bool do_out = emit && op >= x0 && op < x1;
    const int pb = op & 1;
#pragma unroll
    for (int o = 0; o < NB; ++o) {
      const T zd = __shfl_down_sync(0xffffffffu, fzp[o], 1) - __shfl_up_sync(0xffffffffu, fzp[o], 1);
      if (do_out && o < nvalid_o) {
        const T div = (fx0[o] - fxm2[o]) + (sm.fy[pb][o][R + 1][C] - sm.fy[pb][o][R - 1][C]) + zd;
        const T val = kscale * ij_prev * div + vscale * v_prev * pm1[o];
        if (PROD && op == 0)
          pend[o] = val;  // finished at s = 2, once F^x(2) is known
        else
          out[(long long)(o0 + o) * ostride + (long long)op * plane + col] = val;
      }
      fzp[o] = fzc[o];
    }
    if (PROD && op == 0) pend_ij = ij_prev;
    if (PROD && s == 2 && x0 == 0 && emit) {
      // x = -1 flux ghost 3 F(0) - 3 F(1) + F(2); the plane-0 value above used 0.
#pragma unroll
      for (int o = 0; o < NB; ++o)
        if (o < nvalid_o)
          out[(long long)(o0 + o) * ostride + col] = pend[o] - kscale * pend_ij * (T(3) * fxm2[o] - T(3) * fxm1[o] + fx0[o]);
    }
    ij_prev = ij_s;
    v_prev = v_s;
  }

  // ---- epilogue: plane nx-1 (F^x ghost beyond the last face)
  if (x1 == nx) {
    const int op = nx - 1, pb = op & 1;
#pragma unroll
    for (int o = 0; o < NB; ++o) {
      const T zd = __shfl_down_sync(0xffffffffu, fzp[o], 1) - __shfl_up_sync(0xffffffffu, fzp[o], 1);
      if (emit && o < nvalid_o) {
        const T ghost = PROD ? T(3) * fx0[o] - T(3) * fxm1[o] + fxm2[o] : T(0);
        const T div = (ghost - fxm1[o]) + (sm.fy[pb][o][R + 1][C] - sm.fy[pb][o][R - 1][C]) + zd;
        out[(long long)(o0 + o) * ostride + (long long)op * plane + col] =
            kscale * ij_prev * div + vscale * v_prev * p0[o];
      }
    }
  }
}

template <typename T>
__global__ void prepare_geometry_kernel(long long n, double sxx, double syy, double szz, double sxy, double sxz,
                                        double syz, const double* __restrict__ jac, const double* __restrict__ gi,
                                        T* __restrict__ outc) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double J = jac[i];
    const double* G = gi + 9 * i;
    outc[0 * n + i] = T(J * G[0] * sxx);
    outc[1 * n + i] = T(J * G[4] * syy);
    outc[2 * n + i] = T(J * G[8] * szz);
    outc[3 * n + i] = T(J * 0.5 * (G[1] + G[3]) * sxy);
    outc[4 * n + i] = T(J * 0.5 * (G[2] + G[6]) * sxz);
    outc[5 * n + i] = T(J * 0.5 * (G[5] + G[7]) * syz);
    outc[6 * n + i] = T(1.0 / J);
  }
}

template <typename T, int NB, bool PROD>
int launch_hpsi(const void* coeffs, const void* veff, const void* psi, void* out, int nx, int ny, int nz, int nb,
                long long ostride, double kscale, double vscale, cudaStream_t st) {
  const long long n = (long long)nx * ny * nz;
  const T* cb = static_cast<const T*>(coeffs);
  Coeffs<T> c{cb, cb + n, cb + 2 * n, cb + 3 * n, cb + 4 * n, cb + 5 * n, cb + 6 * n};
  const int tiles_z = (nz + OZ - 1) / OZ, tiles_y = (ny + OY - 1) / OY;
  const int groups = (nb + NB - 1) / NB;
  // chunk the march so the grid fills the GPU (152 SMs x several CTAs)
  int chunks = 1;
  const long long base = (long long)tiles_z * tiles_y * groups;
  while (base * chunks < 2 * 152 && nx / (chunks * 2) >= 16) chunks *= 2;
  int chunk = (nx + chunks - 1) / chunks;
  if (chunk < 3) chunk = 3;
  chunks = (nx + chunk - 1) / chunk;
  const size_t smem = sizeof(Smem<T, NB>);
  auto kern = hpsi_agrid_kernel<T, NB, PROD>;
  if (ensure_dynamic_smem(reinterpret_cast<const void*>(kern), smem) != IGD_OK) return IGD_ERR_CUDA;
  dim3 grid(tiles_z * tiles_y, chunks, groups);
  kern<<<grid, NT, smem, st>>>(c, static_cast<const T*>(veff), static_cast<const T*>(psi), static_cast<T*>(out), nx,
                               ny, nz, nb, ostride, T(kscale), T(vscale), chunk, tiles_z);
  return launch_status();
}

template <typename T, bool PROD>
int dispatch_nb(const void* coeffs, const void* veff, const void* psi, void* out, int nx, int ny, int nz, int nb,
                long long ostride, double kscale, double vscale, cudaStream_t st) {
  constexpr int NBMAX = 4;
  if (nb >= NBMAX) return launch_hpsi<T, NBMAX, PROD>(coeffs, veff, psi, out, nx, ny, nz, nb, ostride, kscale, vscale, st);
  if (nb >= 4) return launch_hpsi<T, 4, PROD>(coeffs, veff, psi, out, nx, ny, nz, nb, ostride, kscale, vscale, st);
  if (nb >= 2) return launch_hpsi<T, 2, PROD>(coeffs, veff, psi, out, nx, ny, nz, nb, ostride, kscale, vscale, st);
  return launch_hpsi<T, 1, PROD>(coeffs, veff, psi, out, nx, ny, nz, nb, ostride, kscale, vscale, st);
}

}  // namespace
}  // namespace igd

using namespace igd;

// Kernel selection (a test hook) of the calling host thread: 0 = fastest
// applicable kernel, 1 = skip the whole-row kernel, 2 = the cp.async kernel
// only.  IGD_HPSI_FALLBACK=1 in the environment starts every thread at 2.
static thread_local int g_hpsi_path = -1;

static int hpsi_path() {
  if (g_hpsi_path < 0) {
    const char* e = getenv("IGD_HPSI_FALLBACK");
    g_hpsi_path = (e && e[0] == '1') ? 2 : 0;
  }
  return g_hpsi_path;
}

extern "C" int igd_hpsi_select(int path) {
  if (path < 0 || path > 2) return IGD_ERR_ARG;
  g_hpsi_path = path;
  return IGD_OK;
}

extern "C" int igd_agrid_prepare_geometry(int dtype, int nx, int ny, int nz, double hx, double hy, double hz,
                                          const double* jacobian, const double* inverse_metric, void* coeffs,
                                          void* stream) {
  if (nx < 3 || ny < 3 || nz < 3 || !jacobian || !inverse_metric || !coeffs || hx <= 0 || hy <= 0 || hz <= 0)
    return IGD_ERR_ARG;
  const long long n = (long long)nx * ny * nz;
  const double sxx = 1.0 / (4 * hx * hx), syy = 1.0 / (4 * hy * hy), szz = 1.0 / (4 * hz * hz);
  const double sxy = 1.0 / (4 * hx * hy), sxz = 1.0 / (4 * hx * hz), syz = 1.0 / (4 * hy * hz);
  const int blocks = (int)std::min<long long>((n + 255) / 256, 152 * 16);
  cudaStream_t st = as_stream(stream);
  if (dtype == IGD_F32)
    prepare_geometry_kernel<float><<<blocks, 256, 0, st>>>(n, sxx, syy, szz, sxy, sxz, syz, jacobian, inverse_metric,
                                                            static_cast<float*>(coeffs));
  else if (dtype == IGD_F64)
    prepare_geometry_kernel<double><<<blocks, 256, 0, st>>>(n, sxx, syy, szz, sxy, sxz, syz, jacobian,
                                                             inverse_metric, static_cast<double*>(coeffs));
  else
    return IGD_ERR_DTYPE;
  return launch_status();
}

extern "C" int igd_hpsi_agrid(int dtype, int closure, int nx, int ny, int nz, const void* coeffs, const void* veff,
                              const void* psi, void* out, int nb, long long orbital_stride, double kscale,
                              double vscale, void* stream) {
  if (nx < 3 || ny < 3 || nz < 3 || nb < 1 || !coeffs || !psi || !out) return IGD_ERR_ARG;
  if (nb > 1 && orbital_stride < (long long)nx * ny * nz) return IGD_ERR_ARG;
  if (closure != IGD_CLOSURE_TRIAL_FIX && closure != IGD_CLOSURE_PRODUCTION) return IGD_ERR_ARG;
  const bool prod = closure == IGD_CLOSURE_PRODUCTION;
  cudaStream_t st = as_stream(stream);
  const int path = hpsi_path();
  if (path == 0) {
    const int t = hpsi_agrid_zvec_launch(dtype, closure, nx, ny, nz, coeffs, veff, psi, out, nb, orbital_stride,
                                         kscale, vscale, st);
    if (t >= 0) return t;
  }
  if (path <= 1) {
    const int t = hpsi_agrid_tma_launch(dtype, closure, nx, ny, nz, coeffs, veff, psi, out, nb, orbital_stride, kscale,
                                        vscale, st);
    if (t >= 0) return t;
  }
  if (dtype == IGD_F32)
    return prod ? dispatch_nb<float, true>(coeffs, veff, psi, out, nx, ny, nz, nb, orbital_stride, kscale, vscale, st)
                : dispatch_nb<float, false>(coeffs, veff, psi, out, nx, ny, nz, nb, orbital_stride, kscale, vscale, st);
  if (dtype == IGD_F64)
    return prod ? dispatch_nb<double, true>(coeffs, veff, psi, out, nx, ny, nz, nb, orbital_stride, kscale, vscale, st)
                : dispatch_nb<double, false>(coeffs, veff, psi, out, nx, ny, nz, nb, orbital_stride, kscale, vscale, st);
  return IGD_ERR_DTYPE;
}

// Copy streams and events of the calling host thread for igd_hpsi_agrid_host
// (created on first use, per device; non-blocking, so they never serialise
// against the legacy default stream).
namespace {
struct HostPipe {
  int dev = -1;
  cudaStream_t in = nullptr, out = nullptr;
  cudaEvent_t start = nullptr, copied = nullptr, applied = nullptr, done = nullptr;
  bool ready() const { return in && out && start && copied && applied && done; }
};
thread_local HostPipe g_pipe;

HostPipe* host_pipe() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return nullptr;
  if (g_pipe.dev != dev) {
    g_pipe = HostPipe{};  // streams of another device stay with it
    g_pipe.dev = dev;
    bool ok = cudaStreamCreateWithFlags(&g_pipe.in, cudaStreamNonBlocking) == cudaSuccess &&
              cudaStreamCreateWithFlags(&g_pipe.out, cudaStreamNonBlocking) == cudaSuccess;
    for (cudaEvent_t* e : {&g_pipe.start, &g_pipe.copied, &g_pipe.applied, &g_pipe.done})
      ok = ok && cudaEventCreateWithFlags(e, cudaEventDisableTiming) == cudaSuccess;
    if (!ok) {
      g_pipe.dev = -1;
      return nullptr;
    }
  }
  return g_pipe.ready() ? &g_pipe : nullptr;
}
}  // namespace

extern "C" int igd_hpsi_agrid_host(int dtype, int closure, int nx, int ny, int nz, const void* coeffs,
                                   const void* veff, const void* host_psi, void* host_out, int nb, double kscale,
                                   double vscale, void* dev_in, void* dev_out, int chunk, void* stream) {
  if (nx < 3 || ny < 3 || nz < 3 || nb < 1 || chunk < 0 || !coeffs || !host_psi || !host_out || !dev_in || !dev_out)
    return IGD_ERR_ARG;
  if (dtype != IGD_F32 && dtype != IGD_F64) return IGD_ERR_DTYPE;
  if (closure != IGD_CLOSURE_TRIAL_FIX && closure != IGD_CLOSURE_PRODUCTION) return IGD_ERR_ARG;
  HostPipe* hp = host_pipe();
  if (!hp) return IGD_ERR_CUDA;
  cudaStream_t st = as_stream(stream);
  const long long n = (long long)nx * ny * nz;
  const size_t es = dtype == IGD_F32 ? 4 : 8;
  // default: eight chunks (at 128^3 and 16 FP32 orbitals, chunks of 1, 2, 4, 8 and 16
  // orbitals took 1.03, 1.01, 1.03, 1.16 and 1.47 ms: small chunks shorten the pipeline's
  // fill and drain, while each copy has a fixed cost)
  const int ch = chunk == 0 ? std::max(1, (nb + 7) / 8) : chunk;
  const char* hin = static_cast<const char*>(host_psi);
  char* hout = static_cast<char*>(host_out);
  char* din = static_cast<char*>(dev_in);
  char* dout = static_cast<char*>(dev_out);
  // the scratch buffers' earlier users on `stream` come first
  if (cudaEventRecord(hp->start, st) != cudaSuccess || cudaStreamWaitEvent(hp->in, hp->start, 0) != cudaSuccess ||
      cudaStreamWaitEvent(hp->out, hp->start, 0) != cudaSuccess)
    return IGD_ERR_CUDA;
  int rc = IGD_OK;
  for (int i0 = 0; i0 < nb && rc == IGD_OK; i0 += ch) {
    const int k = std::min(ch, nb - i0);
    const size_t off = (size_t)i0 * n * es, bytes = (size_t)k * n * es;
    // each wait below binds to the record just before it, so one event per edge suffices
    if (cudaMemcpyAsync(din + off, hin + off, bytes, cudaMemcpyHostToDevice, hp->in) != cudaSuccess ||
        cudaEventRecord(hp->copied, hp->in) != cudaSuccess || cudaStreamWaitEvent(st, hp->copied, 0) != cudaSuccess) {
      rc = IGD_ERR_CUDA;
      break;
    }
    rc = igd_hpsi_agrid(dtype, closure, nx, ny, nz, coeffs, veff, din + off, dout + off, k, n, kscale, vscale, st);
    if (rc != IGD_OK) break;
    if (cudaEventRecord(hp->applied, st) != cudaSuccess || cudaStreamWaitEvent(hp->out, hp->applied, 0) != cudaSuccess ||
        cudaMemcpyAsync(hout + off, dout + off, bytes, cudaMemcpyDeviceToHost, hp->out) != cudaSuccess)
      rc = IGD_ERR_CUDA;
  }
  // `stream` resumes after the last copy out (also on an error, so later work on
  // `stream` never overtakes a copy still in flight), and the call returns once
  // that copy has landed in host_out
  if (cudaEventRecord(hp->done, hp->out) != cudaSuccess || cudaStreamWaitEvent(st, hp->done, 0) != cudaSuccess ||
      cudaEventSynchronize(hp->done) != cudaSuccess)
    rc = rc == IGD_OK ? IGD_ERR_CUDA : rc;
  return rc;
}
