// Whole-row, z-vectorised TMA A-grid H.Psi stencil (K1, fastest path).
//
// Same arithmetic as hpsi_agrid.cu / hpsi_agrid_tma.cu (flux form of
// ops/kinetic.py:212-358 with ghost-value closures, plus v_eff psi of
// ks/eigensolver.py:753-756), for rows of at most 128 points (nz a multiple
// of 4), or of at most 256 points (nz a multiple of 8) for one orbital (the
// Poisson operator): one warp owns one whole grid row and every lane four
// (C = 1) or eight (C = 2, two 4-point chunks) consecutive z points, so
// * psi, F^y and the own-point geometry move as 16-byte vectors (one shared
//   or global instruction per four points instead of one per point);
// * the z neighbours of psi and F^z cross lanes by one shuffle each way, and
//   the z-face ghosts (psi and F^z) are formed in registers by the first and
//   last active lane, so a tile carries no z halo at all;
// * psi planes arrive through the same 4-slot cp.async.bulk.tensor ring with
//   bounded mbarrier waits, the own-point geometry is pulled into L2 two planes
//   ahead by bulk prefetches, F^y is exchanged through shared memory (double
//   buffered by step parity, one CTA barrier per plane), and the x march
//   assembles each divergence over two steps.
// Tile: WY warps compute fluxes on rows j0-1 .. j0+WY-2; warps 1..WY-2 emit.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <type_traits>

#include "tma.cuh"

namespace igd {
namespace {

constexpr int ZP = 4;               // z points per chunk; a lane holds C chunks
template <int C>
__host__ __device__ constexpr int zmax() { return 32 * ZP * C; }  // row length covered by one warp
#ifndef IGD_ZVEC_WY
#define IGD_ZVEC_WY 12
#endif
constexpr int WY = IGD_ZVEC_WY, NT = 32 * WY;  // warps (flux rows) per CTA
constexpr int OY = WY - 2;
constexpr int RING = 4;
constexpr int PYT = WY + 2;         // psi rows j0-2 .. j0+WY-1

// largest orbital count per CTA for the trial-fix and production closures
#ifndef IGD_ZVEC_NB_TRIAL
#define IGD_ZVEC_NB_TRIAL 4
#endif
#ifndef IGD_ZVEC_NB_PROD
#define IGD_ZVEC_NB_PROD 4
#endif
// orbital groups smaller than this prefetch the next plane's geometry into registers
#ifndef IGD_ZVEC_REGPF_BELOW
#define IGD_ZVEC_REGPF_BELOW 4
#endif
// planes ahead that the geometry rows are pulled into L2
#ifndef IGD_ZVEC_PF
#define IGD_ZVEC_PF 2
#endif

template <int NB, int C>
struct alignas(128) ZSlot {
  float v[NB][PYT][zmax<C>()];
};

template <int NB, int C>
struct alignas(128) ZSmem {
  ZSlot<NB, C> psi[RING];
  float fy[2][NB][WY][zmax<C>()];  // F^y of plane s, by parity of the step
  uint64_t bar[RING];
};

struct ZArgs {
  int nx, ny, nz, nb;
  long long ostride, n;
  int tiles, hasv, groups, lanes;
  // Krylov mode (one orbital, the Poisson operator): faces written as zero,
  // dot epilogue acc[0] += sum out*y (y = dot_y, or the input when dot_y is
  // null), acc[1] += sum out*out; the launch does nothing while *skip != 0
  const float* dot_y;
  double* dot_acc;
  const int* skip;
};

// Per-thread FP32 part of a Krylov dot product (a few dozen rows per thread;
// GB300's FP64 pipe is too slow to accumulate in FP64 per step): summed in
// FP64 across the block and the grid.
struct DotF {
  float s = 0.f;
  __device__ __forceinline__ void add4(float4 a, float4 b) {
    s = fmaf(a.x, b.x, s);
    s = fmaf(a.y, b.y, s);
    s = fmaf(a.z, b.z, s);
    s = fmaf(a.w, b.w, s);
  }
};

__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ void st4(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }
__device__ __forceinline__ float4 ldg4(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }

// Own four points of one plane: 6 folded metric components, 1/J, v_eff.
struct Geo4 {
  float4 axx, ayy, azz, axy, axz, ayz, ij, v;
};

__device__ __forceinline__ Geo4 load_geo4(const float* __restrict__ c, const float* __restrict__ veff, long long n,
                                          long long at, bool hasv) {
  Geo4 g;
  g.axx = ldg4(c + at);
  g.ayy = ldg4(c + n + at);
  g.azz = ldg4(c + 2 * n + at);
  g.axy = ldg4(c + 3 * n + at);
  g.axz = ldg4(c + 4 * n + at);
  g.ayz = ldg4(c + 5 * n + at);
  g.ij = ldg4(c + 6 * n + at);
  g.v = hasv ? ldg4(veff + at) : make_float4(0.f, 0.f, 0.f, 0.f);
  return g;
}

// Pull `bytes` at p (16-byte aligned) from DRAM into L2 without occupying registers.
__device__ __forceinline__ void l2_prefetch(const void* p, unsigned bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;\n" ::"l"(p), "r"(bytes) : "memory");
}

// Production closure ghosts of psi on the rows just beyond the y faces of slot q
// (the z-face ghosts are formed in registers).
template <int NB, int C>
__device__ __forceinline__ void ghost_rows(ZSmem<NB, C>& sm, int q, int ny, int nz, int j0) {
  const int ylo = 1 - j0, yhi = ny - j0 + 2;
  for (int idx = threadIdx.x; idx < NB * 2 * nz; idx += NT) {
    const int o = idx / (2 * nz), side = (idx / nz) & 1, zz = idx % nz;
    const int yy = side ? yhi : ylo, d = side ? -1 : 1;
    if (yy < 0 || yy >= PYT) continue;
    auto& a = sm.psi[q].v[o];
    a[yy][zz] = 3.f * a[yy + d][zz] - 3.f * a[yy + 2 * d][zz] + a[yy + 3 * d][zz];
  }
}

// psi ghost plane in slot q0 from slots q1, q2, q3 (3 f1 - 3 f2 + f3; zero for the trial fix).
template <int NB, int C, bool PROD>
__device__ __forceinline__ void ghost_plane(ZSmem<NB, C>& sm, int q0, int q1, int q2, int q3) {
  constexpr int N4 = NB * PYT * zmax<C>() / 4;
  float4* a0 = reinterpret_cast<float4*>(&sm.psi[q0].v[0][0][0]);
  const float4* a1 = reinterpret_cast<const float4*>(&sm.psi[q1].v[0][0][0]);
  const float4* a2 = reinterpret_cast<const float4*>(&sm.psi[q2].v[0][0][0]);
  const float4* a3 = reinterpret_cast<const float4*>(&sm.psi[q3].v[0][0][0]);
  for (int i = threadIdx.x; i < N4; i += NT) {
    float4 r = make_float4(0.f, 0.f, 0.f, 0.f);
    if (PROD) {
      const float4 x = a1[i], y = a2[i], z = a3[i];
      r = make_float4(3.f * x.x - 3.f * y.x + z.x, 3.f * x.y - 3.f * y.y + z.y, 3.f * x.z - 3.f * y.z + z.z,
                      3.f * x.w - 3.f * y.w + z.w);
    }
    a0[i] = r;
  }
}

// One thread: arm slot q's barrier and issue the psi tile load of plane p.
template <int NB, int C>
__device__ __forceinline__ void issue(ZSmem<NB, C>& sm, int q, int p, const CUtensorMap* m, int j0, int o0) {
  constexpr unsigned PB = NB * PYT * zmax<C>() * sizeof(float);
  fence_proxy_async();
  mbar_arrive_expect_tx(&sm.bar[q], PB);
  tma_load_4d(&sm.psi[q].v[0][0][0], m, 0, j0 - 2, p, o0, &sm.bar[q]);
}

__device__ __forceinline__ float4 f4(float a, float b, float c, float d) { return make_float4(a, b, c, d); }

// Pointwise float4 arithmetic on the packed FP32x2 pipe (two lanes' worth of
// FP32 work per instruction; per component the same rounding as scalar FP32).
__device__ __forceinline__ float2 lo2(float4 v) { return make_float2(v.x, v.y); }
__device__ __forceinline__ float2 hi2(float4 v) { return make_float2(v.z, v.w); }
__device__ __forceinline__ float4 cat2(float2 a, float2 b) { return make_float4(a.x, a.y, b.x, b.y); }
__device__ __forceinline__ float2 dup2(float s) { return make_float2(s, s); }
__device__ __forceinline__ float4 operator+(float4 a, float4 b) {
  return cat2(__fadd2_rn(lo2(a), lo2(b)), __fadd2_rn(hi2(a), hi2(b)));
}
// a - b as fma(b, -1, a): exact negation, one rounding
__device__ __forceinline__ float4 operator-(float4 a, float4 b) {
  return cat2(__ffma2_rn(lo2(b), dup2(-1.f), lo2(a)), __ffma2_rn(hi2(b), dup2(-1.f), hi2(a)));
}
__device__ __forceinline__ float4 operator*(float4 a, float4 b) {
  return cat2(__fmul2_rn(lo2(a), lo2(b)), __fmul2_rn(hi2(a), hi2(b)));
}
__device__ __forceinline__ float4 operator*(float s, float4 b) {
  return cat2(__fmul2_rn(dup2(s), lo2(b)), __fmul2_rn(dup2(s), hi2(b)));
}
// a * b + c
__device__ __forceinline__ float4 fma4(float4 a, float4 b, float4 c) {
  return cat2(__ffma2_rn(lo2(a), lo2(b), lo2(c)), __ffma2_rn(hi2(a), hi2(b), hi2(c)));
}
__device__ __forceinline__ float4 fma4(float s, float4 b, float4 c) {
  return cat2(__ffma2_rn(dup2(s), lo2(b), lo2(c)), __ffma2_rn(dup2(s), hi2(b), hi2(c)));
}
// ghost value 3 f1 - 3 f2 + f3 of the production closure
__device__ __forceinline__ float4 ext3(float4 a, float4 b, float4 c) { return fma4(3.f, a, fma4(-3.f, b, c)); }
// a1 g1 + a2 g2 + a3 g3, pointwise
__device__ __forceinline__ float4 flux(float4 a1, float4 g1, float4 a2, float4 g2, float4 a3, float4 g3) {
  return fma4(a3, g3, fma4(a2, g2, a1 * g1));
}

// The x march over planes [x0, x1) of one work unit (a row tile and an orbital
// group); ``ph`` carries the per-slot mbarrier parities from one segment to the
// next (every load a segment issues is also waited on inside it).  Each lane
// holds C chunks of four z points (k = 0..C-1 at z0 + 4k).
template <int NB, int C, bool PROD, bool FULL, bool KRY>
__device__ __forceinline__ void march(ZSmem<NB, C>& sm, const CUtensorMap* mpsi, const float* __restrict__ coeffs,
                                      const float* __restrict__ veff, float* __restrict__ out, const ZArgs& a,
                                      float kscale, float vscale, unsigned* err, int unit, int x0, int x1,
                                      unsigned& ph, DotF& d0, DotF& d1) {
  static_assert(!KRY || NB == 1, "the Krylov mode serves one orbital");
  constexpr unsigned FM = 0xffffffffu;
  constexpr int ZMAX = zmax<C>();
  const int nx = a.nx, ny = a.ny, nz = a.nz;
  const int tid = threadIdx.x, lane = tid & 31, R = tid >> 5;
  // unit = tile * groups + orbital group
  const int grp = unit % a.groups, tile = unit / a.groups;
  const int j0 = min(tile * OY, max(ny - OY, 0));
  const int o0 = grp * NB;
  const long long plane = (long long)ny * nz;
  const int nvalid_o = FULL ? NB : min(NB, a.nb - o0);
  const bool hasv = a.hasv != 0;

  const int j = j0 - 1 + R, z0 = ZP * C * lane;
  const bool real = lane < a.lanes && j >= 0 && j < ny;
  const bool emit = real && R >= 1 && R <= OY;
  const long long col = real ? (long long)j * nz + z0 : 0;
  // flux ghost rows j = -1 / ny inside the tile; psi ghost rows inside the psi box
  const bool yface = (j0 == 0) || (ny - j0 <= OY);
  const bool yghost = (j0 <= 1) || (ny - j0 <= OY + 1);
  const bool zlo = lane == 0, zhi = lane == a.lanes - 1;
  const int yy0 = R + 1;

  const int sb = x0 == 0 ? 0 : min(x0 - 1, max(nx - 3, 0));
  const int se = x1 == nx ? nx - 1 : x1;
  const int last = min(nx - 1, se + 1);
  auto slot = [&](int p) { return (p - sb + 1) & (RING - 1); };

  const int pro_lo = max(sb - 1, 0), pro_hi = min(sb + 2, last);
  if (tid == 0)
    for (int p = pro_lo; p <= pro_hi; ++p) issue<NB, C>(sm, slot(p), p, mpsi, j0, o0);
  // Geometry: with four orbitals per CTA (or two chunks per lane), eight lanes pull
  // this warp's geometry rows into L2 two planes ahead and each step reads its own
  // points from L2 (no registers held across steps); with fewer orbitals the step
  // is too short to cover the L2 latency and the next plane's points are loaded
  // into registers one step ahead instead.
  constexpr bool REGPF = NB < IGD_ZVEC_REGPF_BELOW && C == 1;
  constexpr int PF = IGD_ZVEC_PF;
  // lanes 0..6 prefetch the 7 geometry rows, lane 7 the v_eff row
  const bool pf_lane = j >= 0 && j < ny && (lane < 7 || (lane == 7 && hasv));
  const float* const pf_src = lane < 7 ? coeffs + (long long)lane * a.n : veff;
  auto prefetch_geo = [&](int p) {
    if (pf_lane) l2_prefetch(pf_src + (long long)p * plane + (long long)j * nz, nz * 4);
  };
  Geo4 gn;
  if constexpr (REGPF)
    gn = load_geo4(coeffs, veff, a.n, (long long)sb * plane + col, hasv);
  else
    for (int p = sb; p < min(sb + PF, nx); ++p) prefetch_geo(p);
  for (int p = pro_lo; p <= pro_hi; ++p) {
    const int q = slot(p);
    mbar_wait(&sm.bar[q], (ph >> q) & 1u, err);
    ph ^= 1u << q;
  }
  if (PROD && yghost) {
    for (int p = pro_lo; p <= pro_hi; ++p) ghost_rows<NB, C>(sm, slot(p), ny, nz, j0);
    __syncthreads();
  }
  if (sb == 0) {
    ghost_plane<NB, C, PROD>(sm, slot(-1), slot(0), slot(1), slot(2));
    __syncthreads();
  }
  const float4 zero = f4(0.f, 0.f, 0.f, 0.f);
  float4 part[NB][C], fxp[NB][C];
  // Production closure: the x-face values live in two shared slots per (orbital, chunk,
  // thread) rather than in registers (they are touched in a few face steps only).
  // Slot A: F^x(0) from step 0 to step 2, then F^x(nx-3) until step nx-1.  Slot B: the
  // output of plane 0 (it needs the F^x ghost below the lower face, so it waits for
  // F^x(0..2)) from step 1 to step 2, then the F^x ghost above the upper face.
  float4* const face = reinterpret_cast<float4*>(reinterpret_cast<unsigned char*>(&sm) + sizeof(ZSmem<NB, C>));
  auto slot_a = [&](int o, int k) -> float4& { return face[((0 * NB + o) * C + k) * NT + tid]; };
  auto slot_b = [&](int o, int k) -> float4& { return face[((1 * NB + o) * C + k) * NT + tid]; };
  float4 kij_prev[C], vv_prev[C], kij0[C];
#pragma unroll
  for (int k = 0; k < C; ++k) {
#pragma unroll
    for (int o = 0; o < NB; ++o) part[o][k] = fxp[o][k] = zero;
    kij_prev[k] = vv_prev[k] = kij0[k] = zero;
  }
  float* const outb = out + (long long)o0 * a.ostride + col;
  const long long ostr = a.ostride;

  // flux closure of F^y on the ghost rows j = -1 / ny of buffer fb, then a barrier
  auto fix_fy = [&](int fb) {
    if (j == -1 || j == ny) {
      const int d = (j == -1) ? 1 : -1;
#pragma unroll
      for (int o = 0; o < NB; ++o)
#pragma unroll
        for (int k = 0; k < C; ++k) {
          float* f = &sm.fy[fb][o][R][z0 + ZP * k];
          st4(f, PROD ? ext3(ld4(f + d * ZMAX), ld4(f + 2 * d * ZMAX), ld4(f + 3 * d * ZMAX)) : zero);
        }
    }
    __syncthreads();
  };

  // One march step for plane s = base + Q (relative slots are compile-time):
  // fluxes of plane s (F^y to buffer FB), output of plane s-1 (its F^y from
  // the other buffer), partial divergence of plane s.
  auto step = [&](auto qc, int base) {
    constexpr int Q = decltype(qc)::value;
    constexpr int QM = Q & 3, Q0 = (Q + 1) & 3, Q1 = (Q + 2) & 3, Q2 = (Q + 3) & 3, FB = Q & 1;
    const int s = base + Q;
    // Krylov dot operand of the plane emitted in this step, loaded with the geometry
    float4 yv[C];
#pragma unroll
    for (int k = 0; k < C; ++k) yv[k] = zero;
    if constexpr (KRY) {
      if (a.dot_y && emit && s - 1 >= x0 && s - 1 < x1 && s - 1 >= 1)
#pragma unroll
        for (int k = 0; k < C; ++k) yv[k] = ldg4(a.dot_y + (long long)(s - 1) * plane + col + ZP * k);
    }
    Geo4 g[C];
    if constexpr (REGPF) {
      g[0] = gn;
      gn = load_geo4(coeffs, veff, a.n, (long long)min(s + 1, nx - 1) * plane + col, hasv);
    } else {
      if (s + PF < nx) prefetch_geo(s + PF);
#pragma unroll
      for (int k = 0; k < C; ++k) g[k] = load_geo4(coeffs, veff, a.n, (long long)s * plane + col + ZP * k, hasv);
    }
    if (s + 1 == nx) {
      ghost_plane<NB, C, PROD>(sm, Q1, Q0, QM, Q2);
      __syncthreads();
    } else if (s + 1 >= sb + 3) {
      mbar_wait(&sm.bar[Q1], (ph >> Q1) & 1u, err);
      ph ^= 1u << Q1;
      if (PROD && yghost) {
        __syncthreads();
        ghost_rows<NB, C>(sm, Q1, ny, nz, j0);
        __syncthreads();
      }
    }
    if (yface && s > sb) fix_fy(1 - FB);  // F^y of plane s-1 is complete since the last barrier
    const int op = s - 1;
    const bool do_out = emit && op >= x0 && op < x1;
    float* const dst = outb + (long long)op * plane;
    if (PROD && op == 0)
#pragma unroll
      for (int k = 0; k < C; ++k) kij0[k] = kij_prev[k];
#pragma unroll
    for (int o = 0; o < NB; ++o) {
      float4 c[C], pp[C], fx[C], fz[C], gx[C], gy[C];
#pragma unroll
      for (int k = 0; k < C; ++k) {
        const float* pc = &sm.psi[Q0].v[o][yy0][z0 + ZP * k];
        c[k] = ld4(pc);
        gy[k] = ld4(pc + ZMAX) - ld4(pc - ZMAX);
        pp[k] = ld4(&sm.psi[QM].v[o][yy0][z0 + ZP * k]);  // psi(s-1) at the own points
        gx[k] = ld4(&sm.psi[Q1].v[o][yy0][z0 + ZP * k]) - pp[k];
      }
      // z neighbours of psi: lanes on either side, ghosts at the z faces
      float zl = __shfl_up_sync(FM, c[C - 1].w, 1), zr = __shfl_down_sync(FM, c[0].x, 1);
      if (zlo) zl = PROD ? 3.f * c[0].x - 3.f * c[0].y + c[0].z : 0.f;
      if (zhi) zr = PROD ? 3.f * c[C - 1].w - 3.f * c[C - 1].z + c[C - 1].y : 0.f;
#pragma unroll
      for (int k = 0; k < C; ++k) {
        const float L = k == 0 ? zl : c[k - 1].w, Rz = k == C - 1 ? zr : c[k + 1].x;
        const float4 gz = f4(c[k].y - L, c[k].z - c[k].x, c[k].w - c[k].y, Rz - c[k].z);
        fx[k] = flux(g[k].axx, gx[k], g[k].axy, gy[k], g[k].axz, gz);
        st4(&sm.fy[FB][o][R][z0 + ZP * k], flux(g[k].axy, gx[k], g[k].ayy, gy[k], g[k].ayz, gz));
        fz[k] = flux(g[k].axz, gx[k], g[k].ayz, gy[k], g[k].azz, gz);
      }
      float fl = __shfl_up_sync(FM, fz[C - 1].w, 1), fr = __shfl_down_sync(FM, fz[0].x, 1);
      if (zlo) fl = PROD ? 3.f * fz[0].x - 3.f * fz[0].y + fz[0].z : 0.f;
      if (zhi) fr = PROD ? 3.f * fz[C - 1].w - 3.f * fz[C - 1].z + fz[C - 1].y : 0.f;
#pragma unroll
      for (int k = 0; k < C; ++k) {
        const float L = k == 0 ? fl : fz[k - 1].w, Rz = k == C - 1 ? fr : fz[k + 1].x;
        const float4 zd = f4(fz[k].y - L, fz[k].z - fz[k].x, fz[k].w - fz[k].y, Rz - fz[k].z);
        // ---- output of plane s-1: its partial divergence, its F^y difference, F^x(s)
        if (do_out && (FULL || o < nvalid_o)) {
          const float* f = &sm.fy[1 - FB][o][R][z0 + ZP * k];
          float4 val = fma4(vv_prev[k], pp[k], kij_prev[k] * (part[o][k] + (ld4(f + ZMAX) - ld4(f - ZMAX)) + fx[k]));
          if constexpr (KRY) {
            // faces of a Krylov vector stay zero; the dots then cover interior points only
            if (j == 0 || j == ny - 1) val = zero;
            if (z0 + ZP * k == 0) val.x = 0.f;
            if (z0 + ZP * k + 3 == nz - 1) val.w = 0.f;
            if (op >= 1 && j >= tile * OY) {  // the shifted last tile re-emits rows of the one before
              d0.add4(val, a.dot_y ? yv[k] : pp[k]);
              d1.add4(val, val);
            }
          }
          if (PROD && op == 0)
            slot_b(o, k) = val;  // F^x ghost below the lower face needs F^x(0..2)
          else
            st4(dst + o * ostr + ZP * k, val);
        }
        if constexpr (PROD) {
          // fxp holds F^x(s-1) here and slot A F^x(s-2) in the steps that read it
          if (s == 0) slot_a(o, k) = fx[k];
          if (s == 2 && x0 == 0 && emit && (FULL || o < nvalid_o))
            st4(outb + o * ostr + ZP * k,
                KRY ? zero : slot_b(o, k) - kij0[k] * ext3(slot_a(o, k), fxp[o][k], fx[k]));
          if (s == nx - 3 && s >= 2) slot_a(o, k) = fx[k];
          if (nx == 4 && s == 2) slot_a(o, k) = fxp[o][k];  // F^x(1) = F^x(nx-3), after the read above
          if (s == nx - 1) slot_b(o, k) = ext3(fx[k], fxp[o][k], slot_a(o, k));  // F^x ghost above the upper face
        }
        part[o][k] = zd - fxp[o][k];
        fxp[o][k] = fx[k];
      }
    }
    __syncthreads();
    // the slot of plane s-1 is no longer read: refill it with plane s+3
    if (tid == 0 && s + 3 <= last) issue<NB, C>(sm, QM, s + 3, mpsi, j0, o0);
#pragma unroll
    for (int k = 0; k < C; ++k) {
      kij_prev[k] = kscale * g[k].ij;
      vv_prev[k] = vscale * g[k].v;
    }
  };

  for (int base = sb; base <= se; base += RING) {
    step(std::integral_constant<int, 0>{}, base);
    if (base + 1 > se) break;
    step(std::integral_constant<int, 1>{}, base);
    if (base + 2 > se) break;
    step(std::integral_constant<int, 2>{}, base);
    if (base + 3 > se) break;
    step(std::integral_constant<int, 3>{}, base);
  }

  // ---- epilogue: plane nx-1 (F^x ghost beyond the last face)
  if (x1 == nx) {
    const int fbl = (se - sb) & 1;  // F^y buffer of the last step (plane nx-1)
    if (yface) fix_fy(fbl);
    if (emit) {
      const int q = slot(nx - 1);
#pragma unroll
      for (int o = 0; o < NB; ++o) {
        if (FULL || o < nvalid_o) {
#pragma unroll
          for (int k = 0; k < C; ++k) {
            const float4 ghost = PROD ? slot_b(o, k) : zero;
            const float* f = &sm.fy[fbl][o][R][z0 + ZP * k];
            st4(outb + o * ostr + (long long)(nx - 1) * plane + ZP * k,
                KRY ? zero
                    : fma4(vv_prev[k], ld4(&sm.psi[q].v[o][yy0][z0 + ZP * k]),
                           kij_prev[k] * (part[o][k] + (ld4(f + ZMAX) - ld4(f - ZMAX)) + ghost)));
          }
        }
      }
    }
  }
}

// Start of share b of a (tile, plane) work list, moved back to the start of
// its tile when it would fall on plane 1 or 2 (the production closure's
// lower-face output needs the march through plane 2 in one segment).
__device__ __forceinline__ long long work_bound(long long b, long long total, long long shares, int nx) {
  long long w = b * total / shares;
  const int x = (int)(w % nx);
  if (x == 1 || x == 2) w -= x;
  return w;
}

// Persistent: the CTAs form sets of one CTA per orbital group; every set
// marches the segments of its contiguous share of the (tile, plane) work list,
// the CTAs of a set side by side, so each geometry plane is read from DRAM once
// and by the other groups from L2.
template <int NB, int C, bool PROD, bool FULL, bool KRY>
__global__ void __launch_bounds__(NT, 1)
    hpsi_agrid_zvec_kernel(const __grid_constant__ CUtensorMap mpsi, const float* __restrict__ coeffs,
                           const float* __restrict__ veff, float* __restrict__ out, ZArgs a, float kscale,
                           float vscale, unsigned* err) {
  if constexpr (KRY) {
    if (a.skip && *a.skip) return;  // the Krylov solve has stopped: uniform for the whole launch
  }
  extern __shared__ __align__(128) unsigned char smem_raw[];
  ZSmem<NB, C>& sm = *reinterpret_cast<ZSmem<NB, C>*>(smem_raw);
  if (threadIdx.x == 0) {
    for (int q = 0; q < RING; ++q) mbar_init(&sm.bar[q], 1);
    mbar_fence_init();
  }
  __syncthreads();
  const int nx = a.nx, groups = a.groups;
  const int sets = gridDim.x / groups, set = blockIdx.x / groups, grp = blockIdx.x % groups;
  const long long total = (long long)a.tiles * nx;
  const long long end = work_bound(set + 1, total, sets, nx);
  unsigned ph = 0;  // per-slot mbarrier parity, identical in every thread
  DotF d0, d1;
  for (long long pos = work_bound(set, total, sets, nx); pos < end;) {
    const int tile = (int)(pos / nx), x0 = (int)(pos % nx);
    const int x1 = (int)min((long long)nx, x0 + (end - pos));
    march<NB, C, PROD, FULL, KRY>(sm, &mpsi, coeffs, veff, out, a, kscale, vscale, err, tile * groups + grp, x0, x1,
                                  ph, d0, d1);
    pos += x1 - x0;
    __syncthreads();  // slots and F^y buffers are reused by the next segment
  }
  if constexpr (KRY) {
    __shared__ double dscratch[2 * (NT / 32)];
    double v2[2] = {(double)d0.s, (double)d1.s};
    block_sum<2, NT>(v2, dscratch);
    if (threadIdx.x == 0) {
      atomicAdd(a.dot_acc, v2[0]);
      atomicAdd(a.dot_acc + 1, v2[1]);
    }
  }
}

int zvec_sm_count() { return device_sm_count(); }

// Row chunks per lane for a row of nz points: 1 up to 128 points, 2 up to 256.
int zvec_chunks(int nz) { return nz <= 32 * ZP ? 1 : 2; }

template <int NB, int C, bool PROD, bool FULL, bool KRY = false>
int launch_zvec(const float* coeffs, const float* veff, const float* psi, float* out, int nx, int ny, int nz, int nb,
                long long ostride, double kscale, double vscale, cudaStream_t st, const float* dot_y = nullptr,
                double* dot_acc = nullptr, const int* skip = nullptr) {
  const unsigned long long es = sizeof(float), n = (unsigned long long)nx * ny * nz;
  const long long os = nb > 1 ? ostride : (long long)n;
  CUtensorMap mpsi;
  {
    const unsigned long long dims[4] = {(unsigned long long)nz, (unsigned long long)ny, (unsigned long long)nx,
                                        (unsigned long long)nb};
    const unsigned long long strides[3] = {nz * es, (unsigned long long)ny * nz * es, (unsigned long long)os * es};
    const unsigned box[4] = {(unsigned)zmax<C>(), PYT, 1, NB};
    if (!encode_tensor_map(&mpsi, false, 4, psi, dims, strides, box)) return -1;
  }
  unsigned* err = device_error_word();
  if (!err) return IGD_ERR_CUDA;
  auto kern = hpsi_agrid_zvec_kernel<NB, C, PROD, FULL, KRY>;
  // the production closure's two x-face slots per (orbital, chunk, thread)
  const size_t smem = sizeof(ZSmem<NB, C>) + (PROD ? 2 * NB * C * NT * sizeof(float4) : 0);
  if (ensure_dynamic_smem(reinterpret_cast<const void*>(kern), smem) != IGD_OK) return IGD_ERR_CUDA;
  const int per_sm = blocks_per_sm(reinterpret_cast<const void*>(kern), NT, smem);
  const int tiles_y = (ny + OY - 1) / OY, groups = (nb + NB - 1) / NB;
  const long long slots = (long long)zvec_sm_count() * per_sm;
  // sets of one CTA per orbital group, one wave when the groups fit, each set
  // with at least ~8 planes of work
  const long long sets = std::max(1LL, std::min(slots / groups, (long long)tiles_y * nx / 8));
  const long long ctas = sets * groups;
  ZArgs a;
  a.nx = nx; a.ny = ny; a.nz = nz; a.nb = nb; a.ostride = os;
  a.n = (long long)n;
  a.tiles = tiles_y;
  a.hasv = veff ? 1 : 0;
  a.groups = groups;
  a.lanes = nz / (ZP * C);
  a.dot_y = dot_y;
  a.dot_acc = dot_acc;
  a.skip = skip;
  dim3 grid((unsigned)ctas, 1, 1);
  kern<<<grid, NT, smem, st>>>(mpsi, coeffs, veff, out, a, (float)kscale, (float)vscale, err);
  return launch_status();
}

template <int NB, int C, bool PROD>
int zvec_nb(const float* c, const float* v, const float* p, float* o, int nx, int ny, int nz, int nb,
            long long ostride, double kscale, double vscale, cudaStream_t st) {
  if (nb % NB == 0) return launch_zvec<NB, C, PROD, true>(c, v, p, o, nx, ny, nz, nb, ostride, kscale, vscale, st);
  return launch_zvec<NB, C, PROD, false>(c, v, p, o, nx, ny, nz, nb, ostride, kscale, vscale, st);
}

bool al16(const void* p) { return (reinterpret_cast<uintptr_t>(p) & 15u) == 0; }

// Row lengths the whole-row kernel takes: multiples of 4 up to 128 points,
// multiples of 8 up to 256.
bool zvec_row_ok(int nz) {
  return zvec_chunks(nz) == 1 ? (nz % ZP == 0 && nz >= ZP) : (nz % (2 * ZP) == 0 && nz <= zmax<2>());
}

}  // namespace

bool hpsi_agrid_krylov_applies(int nz, const void* coeffs) {
  return zvec_row_ok(nz) && nz >= 2 * ZP && al16(coeffs);
}

int hpsi_agrid_krylov(int nx, int ny, int nz, const float* coeffs, const float* psi, float* out, double kscale,
                      const float* dot_y, double* dot_acc, const int* skip, cudaStream_t st) {
  if (!hpsi_agrid_krylov_applies(nz, coeffs) || !al16(psi) || !al16(out) || (dot_y && !al16(dot_y)) || !dot_acc)
    return -1;
  const long long n = (long long)nx * ny * nz;
  if (zvec_chunks(nz) == 1)
    return launch_zvec<1, 1, true, true, true>(coeffs, nullptr, psi, out, nx, ny, nz, 1, n, kscale, 0.0, st, dot_y,
                                               dot_acc, skip);
  return launch_zvec<1, 2, true, true, true>(coeffs, nullptr, psi, out, nx, ny, nz, 1, n, kscale, 0.0, st, dot_y,
                                             dot_acc, skip);
}

// ---------------------------------------------------------------- autotuner
// Orbitals per CTA (1, 2 or 4) of the whole-row kernel, picked per (device,
// closure, grid shape, orbital count, v_eff present) by timing every candidate
// on the caller's stream the first time that key is seen outside a stream
// capture (one warm-up and the fastest of three timed launches each; the fixed
// rule is kept unless another candidate is at least 20 % faster, so kernels of
// other streams timed alongside rarely move the pick; the candidates compute
// the same values, so the output is the same whichever runs last).  Inside a
// capture, or with the tuner off, the fixed rule applies: 4 orbitals per CTA
// where the count allows.
namespace {
using TuneKey = std::tuple<int, int, int, int, int, int, int>;
std::mutex g_tune_mu;
std::map<TuneKey, std::pair<int, float>> g_tune;  // key -> (orbitals per CTA, us per launch)
int g_tune_mode = 1;                               // igd_hpsi_autotune

int zvec_run(int NB, int closure, const float* c, const float* v, const float* p, float* o, int nx, int ny, int nz,
             int nb, long long ostride, double kscale, double vscale, cudaStream_t st) {
  if (zvec_chunks(nz) == 2) {
    if (nb != 1) return -1;
    return closure == IGD_CLOSURE_PRODUCTION
               ? launch_zvec<1, 2, true, true>(c, v, p, o, nx, ny, nz, nb, ostride, kscale, vscale, st)
               : launch_zvec<1, 2, false, true>(c, v, p, o, nx, ny, nz, nb, ostride, kscale, vscale, st);
  }
  if (closure == IGD_CLOSURE_PRODUCTION) {
    if (NB >= 4) return zvec_nb<4, 1, true>(c, v, p, o, nx, ny, nz, nb, ostride, kscale, vscale, st);
    if (NB >= 2) return zvec_nb<2, 1, true>(c, v, p, o, nx, ny, nz, nb, ostride, kscale, vscale, st);
    return zvec_nb<1, 1, true>(c, v, p, o, nx, ny, nz, nb, ostride, kscale, vscale, st);
  }
  if (NB >= 4) return zvec_nb<4, 1, false>(c, v, p, o, nx, ny, nz, nb, ostride, kscale, vscale, st);
  if (NB >= 2) return zvec_nb<2, 1, false>(c, v, p, o, nx, ny, nz, nb, ostride, kscale, vscale, st);
  return zvec_nb<1, 1, false>(c, v, p, o, nx, ny, nz, nb, ostride, kscale, vscale, st);
}

// Largest orbitals per CTA for the closure and row length.
int max_nb(int closure, int nz) {
  if (zvec_chunks(nz) == 2) return 1;
  if (closure == IGD_CLOSURE_PRODUCTION) return IGD_ZVEC_NB_PROD >= 4 ? 4 : (IGD_ZVEC_NB_PROD >= 2 ? 2 : 1);
  return IGD_ZVEC_NB_TRIAL >= 4 ? 4 : 2;
}

int fixed_rule(int closure, int nz, int nb) {
  const int m = max_nb(closure, nz);
  return (m >= 4 && nb >= 4) ? 4 : (m >= 2 && nb >= 2 ? 2 : 1);
}

// Times the candidates; returns the pick (or -1 if timing was not possible).
int tune(int closure, const float* c, const float* v, const float* p, float* o, int nx, int ny, int nz, int nb,
         long long ostride, double kscale, double vscale, cudaStream_t st, float* best_us) {
  int cands[3], nc = 0;
  const int m = max_nb(closure, nz);
  if (m >= 4 && nb >= 4) cands[nc++] = 4;
  if (m >= 2 && nb >= 2) cands[nc++] = 2;
  cands[nc++] = 1;
  const int fixed = fixed_rule(closure, nz, nb);
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess) return -1;
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return -1;
  }
  // each candidate: one warm-up launch, then the fastest of three timed launches (the
  // minimum is robust against other streams' kernels sharing the GPU during the timing)
  float t[3] = {0.f, 0.f, 0.f};
  bool have[3] = {false, false, false};
  for (int i = 0; i < nc; ++i) {
    if (zvec_run(cands[i], closure, c, v, p, o, nx, ny, nz, nb, ostride, kscale, vscale, st) != IGD_OK) continue;
    for (int r = 0; r < 3; ++r) {
      float ms = 0.f;
      if (cudaEventRecord(e0, st) != cudaSuccess ||
          zvec_run(cands[i], closure, c, v, p, o, nx, ny, nz, nb, ostride, kscale, vscale, st) != IGD_OK ||
          cudaEventRecord(e1, st) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess ||
          cudaEventElapsedTime(&ms, e0, e1) != cudaSuccess)
        break;
      if (!have[i] || ms < t[i]) t[i] = ms;
      have[i] = true;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaGetLastError();
  // the fixed rule stays unless another candidate is at least 20 % faster
  int pick = -1;
  float best = 0.f;
  for (int i = 0; i < nc; ++i)
    if (have[i] && cands[i] == fixed) {
      pick = fixed;
      best = t[i];
    }
  for (int i = 0; i < nc; ++i)
    if (have[i] && (pick < 0 || t[i] < 0.8f * best)) {
      pick = cands[i];
      best = t[i];
    }
  *best_us = best * 1000.f;
  return pick;
}
}  // namespace

// Returns -1 when the whole-row kernel does not apply (dtype, row length,
// alignment), else a status.
int hpsi_agrid_zvec_launch(int dtype, int closure, int nx, int ny, int nz, const void* coeffs, const void* veff,
                           const void* psi, void* out, int nb, long long ostride, double kscale, double vscale,
                           cudaStream_t st) {
  // rows of more than 128 points: one orbital only (the Poisson operator and its
  // Krylov form); blocks of such rows run faster on the tiled kernel (at 192^3 and
  // 16 orbitals 0.37 ms against 0.64 ms with two orbitals of two chunks per CTA,
  // whose march state does not fit the register budget without spills)
  if (dtype != IGD_F32 || !zvec_row_ok(nz) || (zvec_chunks(nz) == 2 && nb != 1)) return -1;
  if (nb > 1 && ostride % 4 != 0) return -1;
  if (!al16(psi) || !al16(out) || !al16(coeffs) || (veff && !al16(veff))) return -1;
  const float *c = static_cast<const float*>(coeffs), *v = static_cast<const float*>(veff),
              *p = static_cast<const float*>(psi);
  float* o = static_cast<float*>(out);
  int NB = fixed_rule(closure, nz, nb);
  if (g_tune_mode && nb > 1) {
    int dev = 0;
    cudaGetDevice(&dev);
    const TuneKey key{dev, closure, nx, ny, nz, nb, veff ? 1 : 0};
    bool have = false;
    {
      std::lock_guard<std::mutex> lk(g_tune_mu);
      auto it = g_tune.find(key);
      if (it != g_tune.end()) {
        NB = it->second.first;
        have = true;
      }
    }
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (!have && cudaStreamIsCapturing(st, &cap) == cudaSuccess && cap == cudaStreamCaptureStatusNone) {
      float us = 0.f;
      const int pick = tune(closure, c, v, p, o, nx, ny, nz, nb, ostride, kscale, vscale, st, &us);
      if (pick > 0) {
        NB = pick;
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune[key] = {pick, us};
      }
    }
    cudaGetLastError();
  }
  return zvec_run(NB, closure, c, v, p, o, nx, ny, nz, nb, ostride, kscale, vscale, st);
}

}  // namespace igd

using namespace igd;

// Tuner switch (process-wide): 1 = pick the whole-row kernel's orbitals per CTA
// by timing on first use of a shape (default), 0 = the fixed rule.
extern "C" int igd_hpsi_autotune(int mode) {
  if (mode < 0 || mode > 1) return IGD_ERR_ARG;
  g_tune_mode = mode;
  return IGD_OK;
}

// The tuner's picks as text, one line per key: "closure nx ny nz nb veff -> NB (us)";
// returns the length written (truncated to len - 1), or the full length when buf
// is null or len < 1.
extern "C" int igd_hpsi_autotune_report(char* buf, int len) {
  std::string sbuf;
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    for (const auto& kv : g_tune) {
      char line[160];
      const TuneKey& k = kv.first;
      std::snprintf(line, sizeof(line), "%s %d %d %d %d %d -> %d (%.2f us)\n",
                    std::get<1>(k) == IGD_CLOSURE_PRODUCTION ? "production" : "trial_fix", std::get<2>(k),
                    std::get<3>(k), std::get<4>(k), std::get<5>(k), std::get<6>(k), kv.second.first,
                    (double)kv.second.second);
      sbuf += line;
    }
  }
  if (!buf || len < 1) return (int)sbuf.size();
  const int n = std::min<int>((int)sbuf.size(), len - 1);
  std::memcpy(buf, sbuf.data(), n);
  buf[n] = 0;
  return n;
}
