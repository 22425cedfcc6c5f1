// K6 on the tensor pipe: tall-skinny weighted Gram G = A W B^T with tcgen05.
//
// Reference: _weighted_overlap_columns (ks/eigensolver_jax.py:105) and
// weighted_overlap_matrix (ks/eigensolver.py:246-272): G[i][j] = sum_p A_i[p] w[p] B_j[p].
//
// The contraction dimension is the grid (millions of points) and the outputs
// are small (a, b <= 64), so a plain M = a, N = b MMA would leave most of a
// 128-row tensor-core tile empty and read it from shared memory every step.
// Instead each pipeline stage stacks s = 128 / a_pad point chunks of 32 points:
// the M = 128 operand is [A_c0; A_c1; ...] (chunk c's a rows at rows c*a_pad)
// and the N = s*b_pad operand is [B_c0; B_c1; ...].  The s diagonal blocks of
// the accumulator are the chunk Grams A_c B_c^T; the off-diagonal blocks are
// ignored.  Tensor work grows s-fold but the operand bytes read per point stay
// close to the bytes that arrive from HBM, and the kernel remains HBM-bound.
//
// Precision (3xTF32): x = hi + lo with hi = x rounded to the nearest TF32
// value and lo = x - hi (exact in FP32, |lo| <= 2^-11 |x|); A_c B_c^T ~
// A_hi B_hi^T + A_hi B_lo^T + A_lo B_hi^T, about 2^-21 relative per product.
// The tensor core's FP32 accumulation does not round to nearest: each step
// into an accumulator can lose a fraction of an ulp of the running sum, and on
// sums of one sign (a self-Gram's diagonal) these losses add up instead of
// averaging out.  The hi*hi products therefore go to their own accumulator
// (4 MMAs per stage, FLUSH stages per window) and the much smaller cross terms
// to a second one, whose losses are 2^-11 smaller; both are read out every
// FLUSH stages into compensated (Kahan) FP32 sums in registers (GB300's FP64
// pipe is too slow to take one FP64 add per value and window), which become
// FP64 once per CTA and are summed in FP64 across blocks (deterministic
// per-block partials reduced by gram_reduce_kernel).
//
// Roles (128 + NW threads, one CTA per SM, persistent over stages):
//   warp 0 lane 0: TMA producer (FP32 tiles of A and B with 128-byte swizzle,
//                  w by a 1-D tensor copy) into an S-slot ring;
//   warp 1       : TMEM allocation; lane 0 issues the MMAs (12 per stage);
//   warps 4..    : NW worker threads for the split pass (B *= w, hi in place,
//                  lo to a second tile, proxy fence); warps 4-7 (one per TMEM
//                  lane quarter) also run the epilogue (TMEM -> FP64 sums).
// Two TMEM accumulator pairs alternate between windows so MMAs continue while
// the previous window is read out.  Every wait is bounded: on a timeout the error
// word is set, all roles leave their loops, TMEM is freed.
#include "gram_tc.cuh"
#include "tc.cuh"

namespace igd {
namespace {

constexpr int TC_ROLES = 128;  // warps 0-3: producer, MMA issuer, two idle
constexpr int TC_FLUSH = 4;    // stages per accumulation window (see the precision note)
constexpr int TC_MAX_SLOTS = 4;

struct GramTcPlan {
  int a, b, a_pad, b_pad, s, N, slots, tmem_cols;
  size_t slot_bytes, a_bytes, b_bytes, w_bytes, smem;
};

__host__ __device__ inline int pad_rows(int r) { return r <= 8 ? 8 : r <= 16 ? 16 : r <= 32 ? 32 : 64; }

bool plan_gram_tc(int a, int b, GramTcPlan* p) {
  if (a < 1 || b < 1 || a > 64 || b > 64) return false;
  p->a = a;
  p->b = b;
  p->a_pad = pad_rows(a);
  p->b_pad = pad_rows(b);
  p->s = std::min(128 / p->a_pad, 128 / p->b_pad);  // N <= 128: two accumulator pairs fit 512 columns
  p->N = p->s * p->b_pad;
  if (p->N % 16 != 0 || p->N > 128) return false;
  p->a_bytes = 128 * 128;  // 128 rows x 32 FP32 points
  p->b_bytes = (size_t)p->N * 128;
  p->w_bytes = (size_t)32 * p->s * 8;
  size_t slot = 2 * p->a_bytes + 2 * p->b_bytes + p->w_bytes;
  slot = (slot + 1023) & ~(size_t)1023;
  p->slot_bytes = slot;
  const size_t budget = 220 * 1024;
  p->slots = (int)std::min<size_t>(TC_MAX_SLOTS, budget / slot);
  if (p->slots < 2) return false;
  p->smem = p->slots * slot + 1024;  // + alignment slack
  int cols = 32;
  while (cols < 4 * p->N) cols <<= 1;
  p->tmem_cols = cols;
  return true;
}

struct GramTcArgs {
  long long n;
  int a, b, a_pad, b_pad, s, N, slots;
  unsigned slot_bytes, a_bytes, b_bytes;
  int has_w;
  long long stages;
  double* part;
  unsigned* err;
};

template <int NW, int BMAX>
__global__ void __launch_bounds__(TC_ROLES + NW, 1)
    gram_tc_kernel(const __grid_constant__ CUtensorMap mapA, const __grid_constant__ CUtensorMap mapB,
                   const __grid_constant__ CUtensorMap mapW, const GramTcArgs g, uint32_t tmem_cols) {
  constexpr int TC_THREADS = TC_ROLES + NW;
  extern __shared__ unsigned char tc_smem_raw[];
  __shared__ __align__(8) uint64_t full_bar[TC_MAX_SLOTS], ready_bar[TC_MAX_SLOTS], empty_bar[TC_MAX_SLOTS];
  __shared__ __align__(8) uint64_t accf_bar[2], acce_bar[2], done_bar;
  __shared__ uint32_t tmem_holder;
  __shared__ int abort_flag;
  unsigned char* base =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(tc_smem_raw) + 1023) & ~(uintptr_t)1023);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int S = g.slots;
  const long long G = gridDim.x;
  const long long J = g.stages > blockIdx.x ? (g.stages - blockIdx.x + G - 1) / G : 0;  // stages of this CTA

  auto slotA = [&](int q) { return base + (size_t)q * g.slot_bytes; };
  auto slotAlo = [&](int q) { return slotA(q) + g.a_bytes; };
  auto slotB = [&](int q) { return slotA(q) + 2 * g.a_bytes; };
  auto slotBlo = [&](int q) { return slotB(q) + g.b_bytes; };
  auto slotW = [&](int q) { return reinterpret_cast<double*>(slotB(q) + 2 * g.b_bytes); };

  if (tid == 0) {
    for (int q = 0; q < S; ++q) {
      mbar_init(&full_bar[q], 1);
      mbar_init(&ready_bar[q], NW);
      mbar_init(&empty_bar[q], 1);
    }
    for (int k = 0; k < 2; ++k) {
      mbar_init(&accf_bar[k], 1);
      mbar_init(&acce_bar[k], 128);  // the four epilogue warps
    }
    mbar_init(&done_bar, 1);
    abort_flag = 0;
    mbar_fence_init();
  }
  // zero every slot once: A rows past s * a_pad are never written by the
  // copies and must read as zero; w stays finite where no copy lands
  for (size_t e = tid; e < (size_t)S * g.slot_bytes / 16; e += TC_THREADS)
    reinterpret_cast<uint4*>(base)[e] = make_uint4(0u, 0u, 0u, 0u);
  if (warp == 1) tmem_alloc(&tmem_holder, tmem_cols);
  fence_proxy_async();  // the zero fill is visible to the tensor core and to later copies
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_holder;
  const unsigned tx_bytes = (unsigned)(g.s * (g.a_pad + g.b_pad) * 128 + (g.has_w ? 32 * g.s * 8 : 0));

  if (warp == 0 && lane == 0) {
    // ------------------------------------------------ producer
    long long issued = 0;
    for (long long j = 0; j < J; ++j) {
      const int q = (int)(j % S);
      if (j >= S && !mbar_wait_or_abort(&empty_bar[q], (unsigned)((j / S - 1) & 1), g.err, &abort_flag)) break;
      const long long t = blockIdx.x + j * G;
      const int p0 = (int)(t * 32 * g.s);
      mbar_arrive_expect_tx(&full_bar[q], tx_bytes);
      for (int c = 0; c < g.s; ++c) {
        tma_load_2d(slotA(q) + (size_t)c * g.a_pad * 128, &mapA, p0 + 32 * c, 0, &full_bar[q]);
        tma_load_2d(slotB(q) + (size_t)c * g.b_pad * 128, &mapB, p0 + 32 * c, 0, &full_bar[q]);
      }
      if (g.has_w)
        for (int o = 0; o < 32 * g.s; o += 256) tma_load_1d(slotW(q) + o, &mapW, p0 + o, &full_bar[q]);
      issued = j + 1;
    }
    // copies still in flight (after an abort) land before the CTA leaves
    for (long long j = std::max(0LL, issued - S); j < issued; ++j)
      mbar_wait(&full_bar[j % S], (unsigned)((j / S) & 1), g.err);
  } else if (warp == 1 && lane == 0) {
    // ------------------------------------------------ MMA issuer
    const uint32_t idesc = umma_idesc_tf32(128, g.N);
    for (long long j = 0; j < J; ++j) {
      const int q = (int)(j % S);
      const long long win = j / TC_FLUSH;
      const int buf = (int)(win & 1);
      if (j % TC_FLUSH == 0 && win >= 2) {
        if (!mbar_wait_or_abort(&acce_bar[buf], (unsigned)((win / 2 - 1) & 1), g.err, &abort_flag)) break;
      }
      if (!mbar_wait_or_abort(&ready_bar[q], (unsigned)((j / S) & 1), g.err, &abort_flag)) break;
      tc_fence_after();
      const uint32_t d0 = tmem + (uint32_t)(2 * buf * g.N), d1 = d0 + (uint32_t)g.N;  // hi*hi, cross terms
      const uint32_t aH = smem_u32(slotA(q)), aL = smem_u32(slotAlo(q));
      const uint32_t bH = smem_u32(slotB(q)), bL = smem_u32(slotBlo(q));
#pragma unroll
      for (int kk = 0; kk < 4; ++kk) {
        const uint32_t off = kk * 32;  // 8 TF32 values along K
        const uint32_t first = (j % TC_FLUSH == 0 && kk == 0) ? 0u : 1u;
        umma_tf32(d0, umma_desc_sw128(aH + off), umma_desc_sw128(bH + off), idesc, first);
        umma_tf32(d1, umma_desc_sw128(aH + off), umma_desc_sw128(bL + off), idesc, first);
        umma_tf32(d1, umma_desc_sw128(aL + off), umma_desc_sw128(bH + off), idesc, 1u);
      }
      umma_commit(&empty_bar[q]);
      if (j % TC_FLUSH == TC_FLUSH - 1 || j == J - 1) umma_commit(&accf_bar[buf]);
    }
    // every MMA issued has completed before TMEM is released
    umma_commit(&done_bar);
    mbar_wait(&done_bar, 0u, g.err);
  } else if (warp >= 4) {
    // ------------------------------------------------ split pass + epilogue
    const int wt = tid - TC_ROLES;         // 0 .. NW-1
    const bool epi = warp < 8;             // warps 4-7: one per TMEM lane quarter
    const int m = (warp & 3) * 32 + lane;  // TMEM lane = accumulator row of this thread
    const int my_c = m / g.a_pad, my_i = m % g.a_pad;
    const bool owns_row = epi && my_c < g.s && my_i < g.a;
    float acc[BMAX], cmp[BMAX];  // Kahan sum and compensation per output column
#pragma unroll
    for (int j = 0; j < BMAX; ++j) acc[j] = cmp[j] = 0.f;
    auto kahan = [&](int j, float x) {
      const float y = x - cmp[j], t = acc[j] + y;
      cmp[j] = (t - acc[j]) - y;
      acc[j] = t;
    };
    const int a_chunks = g.s * g.a_pad * 8;  // 16-byte chunks of live A rows
    // B: thread -> one column group (stack chunk c, logical 16-byte chunk jl: 4 points)
    // and every (NW / G)-th row of it, so each weight is converted once per thread
    const int G = 8 * g.s;
    const int grp = wt % G, rstep = NW >= G ? NW / G : 1, r0 = NW >= G ? wt / G : 0;
    const int bc = grp >> 3, bjl = grp & 7;
    const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;
    // epilogue of window `win`: TMEM diagonal blocks -> FP64 registers
    auto flush = [&](long long win) -> bool {
      const int buf = (int)(win & 1);
      // lanes agree before the warp-collective TMEM loads (an abort may reach them unevenly)
      if (!__all_sync(0xffffffffu, mbar_wait_or_abort(&accf_bar[buf], (unsigned)((win / 2) & 1), g.err, &abort_flag)))
        return false;
      tc_fence_after();
      // the warp covers chunks c0 .. c0 + 32/a_pad - 1 (or one chunk when a_pad >= 32)
      const int wc0 = ((warp & 3) * 32) / g.a_pad;
      const int wcn = g.a_pad >= 32 ? 1 : 32 / g.a_pad;
      for (int cc = 0; cc < wcn; ++cc) {
        const int c = wc0 + cc;
        if (c >= g.s) break;  // warp-uniform
#pragma unroll
        for (int j0 = 0; j0 < BMAX; j0 += 8) {  // compile-time indices keep acc in registers
          if (j0 < g.b_pad) {
            float v0[8], v1[8];
            const uint32_t col = lane_base + (uint32_t)(2 * buf * g.N + c * g.b_pad + j0);
            tmem_ld8(tmem + col, v0);
            tmem_ld8(tmem + col + (uint32_t)g.N, v1);
            tmem_ld_wait();
            if (owns_row && my_c == c) {
#pragma unroll
              for (int u = 0; u < 8; ++u) {
                kahan(j0 + u, v0[u]);
                kahan(j0 + u, v1[u]);
              }
            }
          }
        }
      }
      tc_fence_before();
      mbar_arrive(&acce_bar[buf]);
      return true;
    };
    // hi = x rounded to the nearest TF32 value (low 13 mantissa bits cleared), lo = x - hi
    auto split4 = [](float4 x, float4& h, float4& l) {
      h.x = __uint_as_float((__float_as_uint(x.x) + 0x1000u) & 0xFFFFE000u);
      h.y = __uint_as_float((__float_as_uint(x.y) + 0x1000u) & 0xFFFFE000u);
      h.z = __uint_as_float((__float_as_uint(x.z) + 0x1000u) & 0xFFFFE000u);
      h.w = __uint_as_float((__float_as_uint(x.w) + 0x1000u) & 0xFFFFE000u);
      l.x = x.x - h.x;
      l.y = x.y - h.y;
      l.z = x.z - h.z;
      l.w = x.w - h.w;
    };
    bool ok = true;
    for (long long j = 0; j < J && ok; ++j) {
      const int q = (int)(j % S);
      // warp-uniform: every lane of a worker warp leaves the loop in the same stage
      if (!__all_sync(0xffffffffu, mbar_wait_or_abort(&full_bar[q], (unsigned)((j / S) & 1), g.err, &abort_flag))) {
        ok = false;
        break;
      }
      float4* A4 = reinterpret_cast<float4*>(slotA(q));
      float4* AL4 = reinterpret_cast<float4*>(slotAlo(q));
#pragma unroll 4
      for (int e = wt; e < a_chunks; e += NW) {
        float4 h, l;
        split4(A4[e], h, l);
        A4[e] = h;
        AL4[e] = l;
      }
      float4* B4 = reinterpret_cast<float4*>(slotB(q));
      float4* BL4 = reinterpret_cast<float4*>(slotBlo(q));
      if (wt < G * rstep) {
        float4 wv = make_float4(1.f, 1.f, 1.f, 1.f);
        if (g.has_w) {
          const double* wq = slotW(q) + bc * 32 + bjl * 4;
          wv = make_float4((float)wq[0], (float)wq[1], (float)wq[2], (float)wq[3]);
        }
#pragma unroll 4
        for (int r = r0; r < g.b_pad; r += rstep) {
          const int ra = bc * g.b_pad + r;
          const int e = ra * 8 + (bjl ^ (ra & 7));  // physical 16-byte chunk (128-byte swizzle)
          float4 x = B4[e];
          x.x *= wv.x;
          x.y *= wv.y;
          x.z *= wv.z;
          x.w *= wv.w;
          float4 h, l;
          split4(x, h, l);
          B4[e] = h;
          BL4[e] = l;
        }
      }
      fence_proxy_async();  // generic-proxy writes -> visible to the tensor core
      mbar_arrive(&ready_bar[q]);
      // read out the previous window once this window's first stage is handed over
      if (epi && j % TC_FLUSH == 0 && j > 0) ok = flush(j / TC_FLUSH - 1);
    }
    if (epi && ok && J > 0) ok = flush((J - 1) / TC_FLUSH);
    // cross-chunk sum in shared memory (reuses the slots; every MMA has completed)
    named_bar_sync(1, NW);
    double* red = reinterpret_cast<double*>(base);
    if (owns_row) {
      double* row = red + ((size_t)my_c * g.a + my_i) * g.b;
#pragma unroll
      for (int x = 0; x < BMAX; ++x)
        if (x < g.b) row[x] = (double)acc[x] - (double)cmp[x];
    }
    named_bar_sync(1, NW);
    double* pb = g.part + (long long)blockIdx.x * g.a * g.b;
    for (int e = wt; e < g.a * g.b; e += NW) {
      double v = 0.0;
      for (int c = 0; c < g.s; ++c) v += red[(size_t)c * g.a * g.b + e];
      pb[e] = abort_flag ? 0.0 : v;
    }
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    __syncwarp();
    tc_fence_after();
    tmem_dealloc(tmem, tmem_cols);
  }
}

}  // namespace

int gram_tc_launch(long long n, int a, int b, const float* A, long long sa, const float* B, long long sb,
                   const double* w, double* part, int max_blocks, unsigned* err, cudaStream_t st) {
  GramTcPlan p;
  if (!plan_gram_tc(a, b, &p)) return -1;
  auto al16 = [](const void* q) { return (reinterpret_cast<uintptr_t>(q) & 15u) == 0; };
  if (!al16(A) || !al16(B) || (w && !al16(w)) || (sa * 4) % 16 != 0 || (sb * 4) % 16 != 0) return -1;
  if (n < 32 || n >= (1LL << 31) - 4096) return -1;
  if (!err) return IGD_ERR_CUDA;
  CUtensorMap mA, mB, mW;
  {
    const unsigned long long dims[2] = {(unsigned long long)n, (unsigned long long)a};
    const unsigned long long strides[1] = {(unsigned long long)sa * 4};
    const unsigned box[2] = {32, (unsigned)p.a_pad};
    if (!encode_tensor_map_ex(&mA, false, 2, A, dims, strides, box, true)) return -1;
  }
  {
    const unsigned long long dims[2] = {(unsigned long long)n, (unsigned long long)b};
    const unsigned long long strides[1] = {(unsigned long long)sb * 4};
    const unsigned box[2] = {32, (unsigned)p.b_pad};
    if (!encode_tensor_map_ex(&mB, false, 2, B, dims, strides, box, true)) return -1;
  }
  if (w) {
    const unsigned long long dims[1] = {(unsigned long long)n};
    const unsigned box[1] = {(unsigned)std::min(256, 32 * p.s)};
    if (!encode_tensor_map_ex(&mW, true, 1, w, dims, nullptr, box, false)) return -1;
  } else {
    mW = mA;  // unused
  }
  const int sms = device_sm_count();
  // up to 32 output columns: 8 worker warps (32 FP64 sums per epilogue thread);
  // 64 columns: 4 worker warps (64 sums, register budget of 256 threads)
  const bool wide = p.b_pad > 32;
  auto kern = wide ? gram_tc_kernel<128, 64> : gram_tc_kernel<256, 32>;
  const int threads = wide ? TC_ROLES + 128 : TC_ROLES + 256;
  if (ensure_dynamic_smem(reinterpret_cast<const void*>(kern), p.smem) != IGD_OK) return IGD_ERR_CUDA;
  GramTcArgs g;
  g.n = n;
  g.a = a;
  g.b = b;
  g.a_pad = p.a_pad;
  g.b_pad = p.b_pad;
  g.s = p.s;
  g.N = p.N;
  g.slots = p.slots;
  g.slot_bytes = (unsigned)p.slot_bytes;
  g.a_bytes = (unsigned)p.a_bytes;
  g.b_bytes = (unsigned)p.b_bytes;
  g.has_w = w ? 1 : 0;
  g.stages = (n + 32LL * p.s - 1) / (32LL * p.s);
  g.part = part;
  g.err = err;
  const int grid = (int)std::max<long long>(1, std::min<long long>({(long long)sms, g.stages, (long long)max_blocks}));
  kern<<<grid, threads, p.smem, st>>>(mA, mB, mW, g, (uint32_t)p.tmem_cols);
  return grid;
}

}  // namespace igd
