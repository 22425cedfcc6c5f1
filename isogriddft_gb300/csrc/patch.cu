// Near-core local-GTH patch correction on the A-grid (pseudo/local.py:379-703):
// k-nearest-neighbour inverse-distance weights from the main grid to the
// points of an atom-centred Cartesian patch, and the gather that interpolates a
// field with them.
//
// The neighbour search is exhaustive over the main grid (one thread per patch
// point, a sorted list of the k closest kept in registers) and runs once per
// geometry; it finds the same neighbour sets as a k-d tree (ties at the k-th
// distance resolved towards the lower point index).  Weights follow
// _interpolate_field_to_patch_points: a patch point closer than 1e-12 to its
// nearest grid point copies that value; otherwise w_j = 1/max(d_j, 1e-12)^2,
// normalised to one.
#include "common.cuh"

namespace igd {
namespace {

constexpr int KMAX = 16;
constexpr int NB = 128;

__global__ void knn_kernel(int nq, const double* __restrict__ qx, const double* __restrict__ qy,
                           const double* __restrict__ qz, long long n, const double* __restrict__ X,
                           const double* __restrict__ Y, const double* __restrict__ Z, int k, int* __restrict__ oidx,
                           double* __restrict__ ow) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  double best[KMAX];
  int bi[KMAX];
#pragma unroll
  for (int j = 0; j < KMAX; ++j) {
    best[j] = 1e300;
    bi[j] = -1;
  }
  const double px = qx[q], py = qy[q], pz = qz[q];
  for (long long i = 0; i < n; ++i) {
    const double dx = X[i] - px, dy = Y[i] - py, dz = Z[i] - pz;
    const double d2 = dx * dx + dy * dy + dz * dz;
    if (d2 < best[k - 1]) {
      int j = k - 1;
      while (j > 0 && best[j - 1] > d2) {
        best[j] = best[j - 1];
        bi[j] = bi[j - 1];
        --j;
      }
      best[j] = d2;
      bi[j] = (int)i;
    }
  }
  int* io = oidx + (long long)q * k;
  double* wo = ow + (long long)q * k;
  const double d0 = sqrt(best[0]);
  if (d0 <= 1.0e-12) {
    for (int j = 0; j < k; ++j) {
      io[j] = bi[j];
      wo[j] = j == 0 ? 1.0 : 0.0;
    }
    return;
  }
  double s = 0.0;
  for (int j = 0; j < k; ++j) {
    const double d = fmax(sqrt(best[j]), 1.0e-12);
    const double w = 1.0 / (d * d);
    wo[j] = w;
    io[j] = bi[j];
    s += w;
  }
  for (int j = 0; j < k; ++j) wo[j] /= s;
}

__global__ void gather_kernel(int nq, int k, const int* __restrict__ idx, const double* __restrict__ w,
                              const double* __restrict__ field, double* __restrict__ out) {
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < nq; q += gridDim.x * blockDim.x) {
    double s = 0.0;
    for (int j = 0; j < k; ++j) s += w[(long long)q * k + j] * field[idx[(long long)q * k + j]];
    out[q] = s;
  }
}

}  // namespace
}  // namespace igd

using namespace igd;

// For nq query points, the k (<= 16) nearest of the n main-grid points and their
// normalised inverse-distance-squared weights (idx: nq*k int32, w: nq*k doubles).
extern "C" int igd_patch_knn(int nq, const double* qx, const double* qy, const double* qz, long long n,
                             const double* x, const double* y, const double* z, int k, int* idx, double* w,
                             void* stream) {
  if (nq <= 0 || n <= 0 || k < 1 || k > KMAX || k > n || !qx || !qy || !qz || !x || !y || !z || !idx || !w)
    return IGD_ERR_ARG;
  if (n >= (1LL << 31)) return IGD_ERR_TOO_LARGE;
  knn_kernel<<<(nq + NB - 1) / NB, NB, 0, as_stream(stream)>>>(nq, qx, qy, qz, n, x, y, z, k, idx, w);
  return launch_status();
}

// out[q] = sum_j w[q][j] field[idx[q][j]].
extern "C" int igd_patch_gather(int nq, int k, const int* idx, const double* w, const double* field, double* out,
                                void* stream) {
  if (nq <= 0 || k < 1 || !idx || !w || !field || !out) return IGD_ERR_ARG;
  gather_kernel<<<std::min((nq + 255) / 256, 152 * 8), 256, 0, as_stream(stream)>>>(nq, k, idx, w, field, out);
  return launch_status();
}
