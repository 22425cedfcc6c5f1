// Device-side monitor A-grid generator (FP64).
//
// Restates grid/monitor_geometry.py on the GPU: monitor field :51-113,
// 7-point smoothing :116-135, damped-Jacobi sweeps of div(M grad X) = 0 with
// Dirichlet faces :268-321, covariant basis by np.gradient(edge_order=2),
// metric, inverse metric, Jacobian, cell volumes and spacings :324-373, and
// the Jacobian floor test of the backtracking update :376-396.  The host
// drives the outer loop (isogriddft_gb300/grid_device.py).  Coordinates are
// three SoA fields X, Y, Z of n = nx*ny*nz doubles.
#include <atomic>

#include "common.cuh"

namespace igd {
namespace {

constexpr int GB = 256;

// Monotone map double -> uint64 so unsigned atomics give min / max of doubles.
__device__ __forceinline__ unsigned long long ord64(double v) {
  unsigned long long u = __double_as_longlong(v);
  return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}

__global__ void monitor_field_kernel(long long n, const double* __restrict__ X, const double* __restrict__ Y,
                                     const double* __restrict__ Z, int natoms, const double* __restrict__ atoms,
                                     double* __restrict__ val, double* __restrict__ raw) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double v = 1.0, r0 = 1.0;
    for (int a = 0; a < natoms; ++a) {
      const double* p = atoms + 13 * a;  // px py pz kw ncr kexp lw lr lexp pw pr pexp cap
      const double dx = X[i] - p[0], dy = Y[i] - p[1], dz = Z[i] - p[2];
      const double r = sqrt(dx * dx + dy * dy + dz * dz);
      const double kin = p[3] * exp(-pow(r / p[4], p[5]));
      const double loc = p[6] / (1.0 + pow(r / p[7], p[8]));
      const double prj = p[9] > 0.0 ? p[9] * exp(-pow(r / p[10], p[11])) : 0.0;
      const double ra = kin + loc + prj;
      r0 += ra;
      v += p[12] * (1.0 - exp(-ra / p[12]));
    }
    val[i] = v;
    if (raw) raw[i] = r0;
  }
}

__global__ void smooth_kernel(int nx, int ny, int nz, const double* __restrict__ m, double* __restrict__ out,
                              double s) {
  const long long n = (long long)nx * ny * nz, pl = (long long)ny * nz;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i / pl), y = (int)((i / nz) % ny), z = (int)(i % nz);
    double v = m[i];
    if (x > 0 && x < nx - 1 && y > 0 && y < ny - 1 && z > 0 && z < nz - 1) {
      const double avg = (m[i] + m[i - pl] + m[i + pl] + m[i - nz] + m[i + nz] + m[i - 1] + m[i + 1]) / 7.0;
      v = (1.0 - s) * m[i] + s * avg;
    }
    out[i] = fmax(v, 1.0);
  }
}

struct SweepState {
  unsigned long long maxchange;  // ord64 of the running max |change|
  int done;                      // converged flag
  int conv_sweep;                // index of the sweep that converged (-1 = none)
};

// One damped-Jacobi sweep: Xo = (1-w) Xi + w * (sum_faces c_f X_f) / sum c_f on
// the interior, faces copied; skipped once converged.
__global__ void sweep_kernel(int nx, int ny, int nz, const double* __restrict__ m, const double* __restrict__ Xi,
                             double* __restrict__ Xo, double ihx2, double ihy2, double ihz2, double w,
                             SweepState* st) {
  if (st->done) return;
  const long long n = (long long)nx * ny * nz, pl = (long long)ny * nz;
  double local = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i / pl), y = (int)((i / nz) % ny), z = (int)(i % nz);
    const bool in = x > 0 && x < nx - 1 && y > 0 && y < ny - 1 && z > 0 && z < nz - 1;
    if (!in) {
#pragma unroll
      for (int c = 0; c < 3; ++c) Xo[c * n + i] = Xi[c * n + i];
      continue;
    }
    const double mc = m[i];
    const double axm = 0.5 * (mc + m[i - pl]) * ihx2, axp = 0.5 * (mc + m[i + pl]) * ihx2;
    const double aym = 0.5 * (mc + m[i - nz]) * ihy2, ayp = 0.5 * (mc + m[i + nz]) * ihy2;
    const double azm = 0.5 * (mc + m[i - 1]) * ihz2, azp = 0.5 * (mc + m[i + 1]) * ihz2;
    // one FP64 division per point rather than one per component (GB300's FP64 pipe is slow)
    const double idiag = 1.0 / (axm + axp + aym + ayp + azm + azp);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const double* A = Xi + c * n;
      const double cand = (axm * A[i - pl] + axp * A[i + pl] + aym * A[i - nz] + ayp * A[i + nz] + azm * A[i - 1] +
                           azp * A[i + 1]) * idiag;
      const double u = (1.0 - w) * A[i] + w * cand;
      Xo[c * n + i] = u;
      local = fmax(local, fabs(u - A[i]));
    }
  }
  local = warp_max(local);
  if ((threadIdx.x & 31) == 0) atomicMax(&st->maxchange, ord64(local));
}

__global__ void sweep_check_kernel(SweepState* st, double tol, int sweep) {
  if (st->done) return;
  const unsigned long long t = ord64(tol);
  if (st->maxchange < t) {
    st->done = 1;
    st->conv_sweep = sweep;
  }
  st->maxchange = ord64(0.0);
}

// Trial coordinates X + alpha (S - X) evaluated on the fly (alpha < 0: use X itself).
struct Coords {
  const double* X;
  const double* S;
  double alpha;
  long long n;
  __device__ __forceinline__ double at(int c, long long i) const {
    const double x = X[c * n + i];
    return alpha < 0.0 ? x : x + alpha * (S[c * n + i] - x);
  }
};

// i2h = 1 / (2 h), formed once (FP64 divisions are slow on GB300)
__device__ __forceinline__ double grad1c(const Coords& P, int c, long long i, long long stride, int idx, int n,
                                         double i2h) {
  if (idx == 0) return (-3.0 * P.at(c, i) + 4.0 * P.at(c, i + stride) - P.at(c, i + 2 * stride)) * i2h;
  if (idx == n - 1) return (3.0 * P.at(c, i) - 4.0 * P.at(c, i - stride) + P.at(c, i - 2 * stride)) * i2h;
  return (P.at(c, i + stride) - P.at(c, i - stride)) * i2h;
}

__device__ __forceinline__ void basis_at(const Coords& P, int nx, int ny, int nz, long long i, double hx, double hy,
                                         double hz, double B[3][3]) {
  const long long pl = (long long)ny * nz;
  const int x = (int)(i / pl), y = (int)((i / nz) % ny), z = (int)(i % nz);
  const double ix = 0.5 / hx, iy = 0.5 / hy, iz = 0.5 / hz;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    B[0][c] = grad1c(P, c, i, pl, x, nx, ix);
    B[1][c] = grad1c(P, c, i, nz, y, ny, iy);
    B[2][c] = grad1c(P, c, i, 1, z, nz, iz);
  }
}

__device__ __forceinline__ double det3(const double B[3][3]) {
  return B[0][0] * (B[1][1] * B[2][2] - B[1][2] * B[2][1]) - B[0][1] * (B[1][0] * B[2][2] - B[1][2] * B[2][0]) +
         B[0][2] * (B[1][0] * B[2][1] - B[1][1] * B[2][0]);
}

__global__ void min_jacobian_kernel(int nx, int ny, int nz, Coords P, double hx, double hy, double hz,
                                    unsigned long long* out_min) {
  const long long n = (long long)nx * ny * nz;
  double local = 1e300;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double B[3][3];
    basis_at(P, nx, ny, nz, i, hx, hy, hz, B);
    local = fmin(local, det3(B));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) local = fmin(local, __shfl_xor_sync(0xffffffffu, local, o));
  if ((threadIdx.x & 31) == 0) atomicMin(out_min, ord64(local));
}

// X <- X + alpha (S - X); running max |update - X|.
__global__ void relax_update_kernel(long long n3, double* __restrict__ X, const double* __restrict__ S, double alpha,
                                    unsigned long long* out_max) {
  double local = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n3; i += (long long)gridDim.x * blockDim.x) {
    const double x = X[i];
    const double t = x + alpha * (S[i] - x);
    local = fmax(local, fabs(t - x));
    X[i] = t;
  }
  local = warp_max(local);
  if ((threadIdx.x & 31) == 0) atomicMax(out_max, ord64(local));
}

// Final geometry: covariant basis (n,3,3), metric, inverse metric, Jacobian,
// cell volumes and the three point spacings (AoS as the reference arrays).
__global__ void geometry_kernel(int nx, int ny, int nz, Coords P, double hx, double hy, double hz,
                                double* __restrict__ basis, double* __restrict__ metric, double* __restrict__ inv,
                                double* __restrict__ jac, double* __restrict__ vol, double* __restrict__ spacing) {
  const long long n = (long long)nx * ny * nz;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    double B[3][3], G[3][3];
    basis_at(P, nx, ny, nz, i, hx, hy, hz, B);
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b) G[a][b] = B[a][0] * B[b][0] + B[a][1] * B[b][1] + B[a][2] * B[b][2];
    const double idg = 1.0 / det3(G);  // one FP64 division per point
    const double I00 = (G[1][1] * G[2][2] - G[1][2] * G[2][1]) * idg, I01 = (G[0][2] * G[2][1] - G[0][1] * G[2][2]) * idg,
                 I02 = (G[0][1] * G[1][2] - G[0][2] * G[1][1]) * idg, I10 = (G[1][2] * G[2][0] - G[1][0] * G[2][2]) * idg,
                 I11 = (G[0][0] * G[2][2] - G[0][2] * G[2][0]) * idg, I12 = (G[0][2] * G[1][0] - G[0][0] * G[1][2]) * idg,
                 I20 = (G[1][0] * G[2][1] - G[1][1] * G[2][0]) * idg, I21 = (G[0][1] * G[2][0] - G[0][0] * G[2][1]) * idg,
                 I22 = (G[0][0] * G[1][1] - G[0][1] * G[1][0]) * idg;
    const double Iv[9] = {I00, I01, I02, I10, I11, I12, I20, I21, I22};
#pragma unroll
    for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = 0; b < 3; ++b) {
        basis[9 * i + 3 * a + b] = B[a][b];
        metric[9 * i + 3 * a + b] = G[a][b];
        inv[9 * i + 3 * a + b] = Iv[3 * a + b];
      }
    const double J = det3(B);
    jac[i] = J;
    vol[i] = J * hx * hy * hz;
    const double h3[3] = {hx, hy, hz};
#pragma unroll
    for (int a = 0; a < 3; ++a)
      spacing[3 * i + a] = sqrt(B[a][0] * B[a][0] + B[a][1] * B[a][1] + B[a][2] * B[a][2]) * h3[a];
  }
}

inline int grid_blocks(long long n) { return (int)std::min<long long>((n + GB - 1) / GB, 152LL * 8); }

__global__ void ord_init_kernel(unsigned long long* u, double v) { *u = ord64(v); }
__global__ void ord_decode_kernel(const unsigned long long* u, double* out) {
  const unsigned long long w = *u;
  *out = __longlong_as_double((long long)((w >> 63) ? (w & 0x7fffffffffffffffull) : ~w));
}
__global__ void sweep_reset_kernel(SweepState* st) {
  st->maxchange = ord64(0.0);
  st->done = 0;
  st->conv_sweep = -1;
}

}  // namespace
}  // namespace igd

using namespace igd;

// atoms: 13 doubles per atom on the device (x, y, z, kinetic weight, near-core
// radius, kinetic exponent, local weight, local radius, local exponent,
// projector weight, projector radius, projector exponent, monitor cap).
extern "C" int igd_grid_monitor_field(long long n, const double* X, const double* Y, const double* Z, int natoms,
                                      const double* atoms, double* values, double* raw, void* stream) {
  if (n <= 0 || natoms < 0 || !X || !Y || !Z || !values || (natoms > 0 && !atoms)) return IGD_ERR_ARG;
  monitor_field_kernel<<<grid_blocks(n), GB, 0, as_stream(stream)>>>(n, X, Y, Z, natoms, atoms, values, raw);
  return launch_status();
}

extern "C" int igd_grid_smooth(int nx, int ny, int nz, const double* monitor, double* out, double smoothing,
                               void* stream) {
  if (nx < 3 || ny < 3 || nz < 3 || !monitor || !out || monitor == out) return IGD_ERR_ARG;
  smooth_kernel<<<grid_blocks((long long)nx * ny * nz), GB, 0, as_stream(stream)>>>(nx, ny, nz, monitor, out,
                                                                                    smoothing);
  return launch_status();
}

// Enqueue up to `sweeps` damped-Jacobi sweeps ping-ponging buf0 -> buf1 -> buf0
// (each 3n doubles; buf0 holds the start with the fixed faces).  state is a
// 16-byte device workspace; after the stream completes, state[3] (int) is the
// index of the sweep whose max |change| fell below tol (-1: none), so the result
// sits in buf[(c+1) % 2] (or buf[sweeps % 2] without convergence).
extern "C" int igd_grid_harmonic_sweeps(int nx, int ny, int nz, const double* monitor, double* buf0, double* buf1,
                                        double hx, double hy, double hz, double relaxation, double tol, int sweeps,
                                        void* state, void* stream) {
  if (nx < 3 || ny < 3 || nz < 3 || !monitor || !buf0 || !buf1 || !state || sweeps < 1) return IGD_ERR_ARG;
  cudaStream_t st = as_stream(stream);
  SweepState* s = static_cast<SweepState*>(state);
  sweep_reset_kernel<<<1, 1, 0, st>>>(s);
  const long long n = (long long)nx * ny * nz;
  for (int k = 0; k < sweeps; ++k) {
    const double* in = (k & 1) ? buf1 : buf0;
    double* out = (k & 1) ? buf0 : buf1;
    sweep_kernel<<<grid_blocks(n), GB, 0, st>>>(nx, ny, nz, monitor, in, out, 1.0 / (hx * hx), 1.0 / (hy * hy),
                                                1.0 / (hz * hz), relaxation, s);
    sweep_check_kernel<<<1, 1, 0, st>>>(s, tol, k);
  }
  return launch_status();
}

// Minimum Jacobian of X + alpha (S - X) (alpha < 0: of X); scratch = 8 bytes.
extern "C" int igd_grid_min_jacobian(int nx, int ny, int nz, const double* X, const double* S, double alpha,
                                     double hx, double hy, double hz, void* scratch, double* out_min, void* stream) {
  if (nx < 3 || ny < 3 || nz < 3 || !X || !scratch || !out_min || (alpha >= 0.0 && !S)) return IGD_ERR_ARG;
  cudaStream_t st = as_stream(stream);
  unsigned long long* u = static_cast<unsigned long long*>(scratch);
  ord_init_kernel<<<1, 1, 0, st>>>(u, 1e300);
  const long long n = (long long)nx * ny * nz;
  Coords P{X, S, alpha, n};
  min_jacobian_kernel<<<grid_blocks(n), GB, 0, st>>>(nx, ny, nz, P, hx, hy, hz, u);
  ord_decode_kernel<<<1, 1, 0, st>>>(u, out_min);
  return launch_status();
}

// X <- X + alpha (S - X) over 3n values; *out_max = max |update|.
extern "C" int igd_grid_relax_update(long long n3, double* X, const double* S, double alpha, void* scratch,
                                     double* out_max, void* stream) {
  if (n3 <= 0 || !X || !S || !scratch || !out_max) return IGD_ERR_ARG;
  cudaStream_t st = as_stream(stream);
  unsigned long long* u = static_cast<unsigned long long*>(scratch);
  ord_init_kernel<<<1, 1, 0, st>>>(u, 0.0);
  relax_update_kernel<<<grid_blocks(n3), GB, 0, st>>>(n3, X, S, alpha, u);
  ord_decode_kernel<<<1, 1, 0, st>>>(u, out_max);
  return launch_status();
}

extern "C" int igd_grid_geometry(int nx, int ny, int nz, const double* X, double hx, double hy, double hz,
                                 double* basis, double* metric, double* inverse_metric, double* jacobian,
                                 double* cell_volumes, double* spacing, void* stream) {
  if (nx < 3 || ny < 3 || nz < 3 || !X || !basis || !metric || !inverse_metric || !jacobian || !cell_volumes ||
      !spacing)
    return IGD_ERR_ARG;
  const long long n = (long long)nx * ny * nz;
  Coords P{X, nullptr, -1.0, n};
  geometry_kernel<<<grid_blocks(n), GB, 0, as_stream(stream)>>>(nx, ny, nz, P, hx, hy, hz, basis, metric,
                                                                inverse_metric, jacobian, cell_volumes, spacing);
  return launch_status();
}

// ---------------------------------------------------------------------------
// Zero-allocation variant of igd_grid_harmonic_sweeps.
//
// Some embedding hosts cannot let a library call cudaMalloc: for example an
// SCF driver inside a larger simulation code that reserves its whole device
// memory budget in one pool at start-up and treats any later allocation as a
// failure (cudaMalloc can also synchronise the device and stall their other
// streams).  For them the second coordinate buffer and the sweep state live in
// this fixed, library-owned array.  It is sized for grids of up to
// IGD_NOALLOC_MAX_POINTS points (3 doubles per point + the 16-byte state:
// 6 MiB), and every GPU that loads the library keeps it until the process
// exits.  All calls share it: calls that overlap on the GPU (two streams, two
// host threads) race and corrupt each other; serialise them.
namespace igd {
namespace {
constexpr long long kNoallocMaxPoints = IGD_NOALLOC_MAX_POINTS;
static __device__ __align__(256) double g_noalloc_scratch[3 * kNoallocMaxPoints + 2];
// Device address of the array, per device ordinal, resolved on the first call on
// that device.  Atomic so that first calls racing on several host threads are
// well defined (they store the same address).  The address belongs to the
// device's primary context: after cudaDeviceReset, or under another context
// made current by the driver API, it is stale (the header says so).
std::atomic<double*> g_noalloc_addr[64] = {};

__global__ void noalloc_finish_kernel(const SweepState* st, double* coords, const double* buf1, long long n3,
                                      int sweeps, int* conv_out) {
  const int c = st->conv_sweep;
  const int where = c >= 0 ? (c + 1) & 1 : sweeps & 1;  // 0: result already in coords, 1: in the scratch copy
  if (conv_out && blockIdx.x == 0 && threadIdx.x == 0) *conv_out = c;
  if (where == 0) return;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n3; i += (long long)gridDim.x * blockDim.x)
    coords[i] = buf1[i];
}
}  // namespace
}  // namespace igd

extern "C" int igd_grid_harmonic_sweeps_noalloc(int nx, int ny, int nz, const double* monitor, double* coords,
                                                double hx, double hy, double hz, double relaxation, double tol,
                                                int sweeps, int* conv_sweep_out, void* stream) {
  if (nx < 3 || ny < 3 || nz < 3 || !monitor || !coords || sweeps < 1) return IGD_ERR_ARG;
  const long long n = (long long)nx * ny * nz;
  if (n > kNoallocMaxPoints) return IGD_ERR_TOO_LARGE;
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return IGD_ERR_CUDA;
  double* buf1 = g_noalloc_addr[dev].load(std::memory_order_acquire);
  if (!buf1) {  // set-up, once per device, with that device current
    void* p = nullptr;
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return IGD_ERR_CUDA;
    buf1 = static_cast<double*>(p);
    g_noalloc_addr[dev].store(buf1, std::memory_order_release);
  }
  SweepState* state = reinterpret_cast<SweepState*>(buf1 + 3 * kNoallocMaxPoints);
  cudaStream_t st = as_stream(stream);
  sweep_reset_kernel<<<1, 1, 0, st>>>(state);  // the state must start cleared; the buffer is fully overwritten
  for (int k = 0; k < sweeps; ++k) {
    const double* in = (k & 1) ? buf1 : coords;
    double* out = (k & 1) ? coords : buf1;
    sweep_kernel<<<grid_blocks(n), GB, 0, st>>>(nx, ny, nz, monitor, in, out, 1.0 / (hx * hx), 1.0 / (hy * hy),
                                                1.0 / (hz * hz), relaxation, state);
    sweep_check_kernel<<<1, 1, 0, st>>>(state, tol, k);
  }
  noalloc_finish_kernel<<<grid_blocks(3 * n), GB, 0, st>>>(state, coords, buf1, 3 * n, sweeps, conv_sweep_out);
  return launch_status();
}
