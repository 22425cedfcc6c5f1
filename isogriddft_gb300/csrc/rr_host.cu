// Host half of one fused block-eigensolver iteration (no device code).
//
// The fused iteration of ks.py (`_block_subspace_iteration_fused`, the block
// iteration of ks/eigensolver_jax.py:417-524 reordered) brings two FP64 Gram
// matrices of the (m + k)-column block [B; R] to the host each iteration and
// turns them into the next rotation coefficients through a dozen small dense
// operations (projection, rank-revealing whitening, trial Rayleigh-Ritz,
// re-whitening).  This file does that algebra in one call: no interpreter
// overhead between the steps and no global interpreter lock held while it
// runs, so concurrent solves on several host threads overlap.
//
// Dense kernels are written here from the textbook methods: symmetric
// eigenpairs by the cyclic Jacobi method (Jacobi 1846; Golub & Van Loan,
// Matrix Computations, sec. 8.5), Cholesky factorisation, triangular
// inversion and Gaussian elimination with partial pivoting.  Sizes are small
// (m + k <= 64); matrices are row-major.
#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"

namespace igd {
namespace {

using Mat = std::vector<double>;

inline double& at(Mat& a, int ld, int i, int j) { return a[(size_t)i * ld + j]; }
inline double at(const Mat& a, int ld, int i, int j) { return a[(size_t)i * ld + j]; }

// c (r x s) = a (r x t) b (t x s), with optional transposes of a / b as stored.
void matmul(const Mat& a, bool ta, const Mat& b, bool tb, int r, int t, int s, Mat& c) {
  c.assign((size_t)r * s, 0.0);
  for (int i = 0; i < r; ++i)
    for (int l = 0; l < t; ++l) {
      const double ail = ta ? a[(size_t)l * r + i] : a[(size_t)i * t + l];
      if (ail == 0.0) continue;
      for (int j = 0; j < s; ++j) c[(size_t)i * s + j] += ail * (tb ? b[(size_t)j * t + l] : b[(size_t)l * s + j]);
    }
}

void symmetrize(Mat& a, int n) {
  for (int i = 0; i < n; ++i)
    for (int j = i + 1; j < n; ++j) {
      const double v = 0.5 * (at(a, n, i, j) + at(a, n, j, i));
      at(a, n, i, j) = v;
      at(a, n, j, i) = v;
    }
}

// Eigenpairs of the symmetric n x n matrix a by cyclic Jacobi rotations;
// w ascending, z columns = eigenvectors.  Returns false if not converged.
bool sym_eig(Mat a, int n, std::vector<double>& w, Mat& z) {
  z.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i) at(z, n, i, i) = 1.0;
  bool done = n <= 1;
  for (int sweep = 0; sweep < 100 && !done; ++sweep) {
    double off = 0.0, diag = 0.0;
    for (int i = 0; i < n; ++i) {
      diag += at(a, n, i, i) * at(a, n, i, i);
      for (int j = i + 1; j < n; ++j) off += at(a, n, i, j) * at(a, n, i, j);
    }
    if (!std::isfinite(off) || !std::isfinite(diag)) return false;
    if (off <= 1e-32 * diag || off == 0.0) {
      done = true;
      break;
    }
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = at(a, n, p, q);
        if (apq == 0.0) continue;
        const double app = at(a, n, p, p), aqq = at(a, n, q, q);
        // rotation angle: cot(2 phi) = (aqq - app) / (2 apq), t = tan(phi) of the smaller root
        const double theta = (aqq - app) / (2.0 * apq);
        const double t = (theta >= 0.0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int r = 0; r < n; ++r) {  // columns p, q
          const double arp = at(a, n, r, p), arq = at(a, n, r, q);
          at(a, n, r, p) = c * arp - s * arq;
          at(a, n, r, q) = s * arp + c * arq;
        }
        for (int r = 0; r < n; ++r) {  // rows p, q
          const double apr = at(a, n, p, r), aqr = at(a, n, q, r);
          at(a, n, p, r) = c * apr - s * aqr;
          at(a, n, q, r) = s * apr + c * aqr;
        }
        at(a, n, p, q) = at(a, n, q, p) = 0.0;
        for (int r = 0; r < n; ++r) {
          const double zrp = at(z, n, r, p), zrq = at(z, n, r, q);
          at(z, n, r, p) = c * zrp - s * zrq;
          at(z, n, r, q) = s * zrp + c * zrq;
        }
      }
  }
  if (!done) return false;
  std::vector<int> idx(n);
  for (int i = 0; i < n; ++i) idx[i] = i;
  std::stable_sort(idx.begin(), idx.end(), [&](int x, int y) { return at(a, n, x, x) < at(a, n, y, y); });
  w.resize(n);
  Mat zs((size_t)n * n);
  for (int j = 0; j < n; ++j) {
    w[j] = at(a, n, idx[j], idx[j]);
    for (int r = 0; r < n; ++r) at(zs, n, r, j) = at(z, n, r, idx[j]);
  }
  z.swap(zs);
  return true;
}

// Lower Cholesky factor of the symmetric positive definite a; false if not SPD.
bool cholesky(const Mat& a, int n, Mat& l) {
  l.assign((size_t)n * n, 0.0);
  for (int j = 0; j < n; ++j) {
    double d = at(a, n, j, j);
    for (int s = 0; s < j; ++s) d -= at(l, n, j, s) * at(l, n, j, s);
    if (!(d > 0.0) || !std::isfinite(d)) return false;
    const double ljj = std::sqrt(d);
    at(l, n, j, j) = ljj;
    for (int i = j + 1; i < n; ++i) {
      double v = at(a, n, i, j);
      for (int s = 0; s < j; ++s) v -= at(l, n, i, s) * at(l, n, j, s);
      at(l, n, i, j) = v / ljj;
    }
  }
  return true;
}

// (L^-1)^T of a lower-triangular L (upper triangular result).
void inv_lower_transposed(const Mat& l, int n, Mat& out) {
  Mat inv((size_t)n * n, 0.0);
  for (int j = 0; j < n; ++j) {
    at(inv, n, j, j) = 1.0 / at(l, n, j, j);
    for (int i = j + 1; i < n; ++i) {
      double v = 0.0;
      for (int s = j; s < i; ++s) v -= at(l, n, i, s) * at(inv, n, s, j);
      at(inv, n, i, j) = v / at(l, n, i, i);
    }
  }
  out.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) at(out, n, i, j) = at(inv, n, j, i);
}

// x (n x s) = a^-1 b by Gaussian elimination with partial pivoting; false if singular.
bool solve(Mat a, int n, Mat b, int s, Mat& x) {
  for (int c = 0; c < n; ++c) {
    int piv = c;
    for (int r = c + 1; r < n; ++r)
      if (std::fabs(at(a, n, r, c)) > std::fabs(at(a, n, piv, c))) piv = r;
    if (at(a, n, piv, c) == 0.0 || !std::isfinite(at(a, n, piv, c))) return false;
    if (piv != c) {
      for (int j = 0; j < n; ++j) std::swap(at(a, n, c, j), at(a, n, piv, j));
      for (int j = 0; j < s; ++j) std::swap(at(b, s, c, j), at(b, s, piv, j));
    }
    for (int r = c + 1; r < n; ++r) {
      const double f = at(a, n, r, c) / at(a, n, c, c);
      if (f == 0.0) continue;
      for (int j = c; j < n; ++j) at(a, n, r, j) -= f * at(a, n, c, j);
      for (int j = 0; j < s; ++j) at(b, s, r, j) -= f * at(b, s, c, j);
    }
  }
  x.assign((size_t)n * s, 0.0);
  for (int r = n - 1; r >= 0; --r)
    for (int j = 0; j < s; ++j) {
      double v = at(b, s, r, j);
      for (int c = r + 1; c < n; ++c) v -= at(a, n, r, c) * at(x, s, c, j);
      at(x, s, r, j) = v / at(a, n, r, r);
    }
  return true;
}

// Inverse square root of the symmetric Gram matrix g, or an inverse-Cholesky
// fallback (jittered when rank deficient) when its smallest eigenvalue is <= 1e-10.
bool whitening(Mat g, int n, Mat& out) {
  symmetrize(g, n);
  std::vector<double> ev;
  Mat v;
  if (!sym_eig(g, n, ev, v)) return false;
  auto isqrt = [&]() {
    out.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        double s = 0.0;
        for (int l = 0; l < n; ++l) s += at(v, n, i, l) * at(v, n, j, l) / std::sqrt(std::max(ev[l], 1e-14));
        at(out, n, i, j) = s;
      }
  };
  bool finite = true;
  double emin = INFINITY, dmax = 0.0;
  for (int i = 0; i < n; ++i) {
    finite = finite && std::isfinite(ev[i]);
    emin = std::min(emin, ev[i]);
    dmax = std::max(dmax, std::fabs(at(g, n, i, i)));
  }
  if (finite && emin > 1e-10) {
    isqrt();
    return true;
  }
  double jitter = 0.0;
  for (int attempt = 0; attempt < 8; ++attempt) {
    Mat gj = g, l;
    for (int i = 0; i < n; ++i) at(gj, n, i, i) += jitter;
    if (cholesky(gj, n, l)) {
      inv_lower_transposed(l, n, out);
      return true;
    }
    jitter = std::max(1e-14, 10.0 * jitter) * std::max(1.0, dmax);
  }
  isqrt();
  return true;
}

}  // namespace
}  // namespace igd

using namespace igd;

// One host step of the fused block iteration.  G0 = [B;R]^T W [HB;HR] and
// G1 = [B;R]^T W [B;R], both (m+k) x (m+k) row-major.  Writes
//   coeff = [CB (m x m); CR (k x m); V_k (m x k); -V_k diag(lam_k) (m x k)]
// (the two-part rotation of B and R, then the residual coefficients of the next
// iteration), P (m x m, the compressed Rayleigh-Ritz matrix), its eigenpairs
// lam (m, ascending) and V (m x m, columns), and rank_out = the number of
// residual directions kept by the whitening.  Mirrors the host algebra of
// ks.py `_block_subspace_iteration_fused`: W-projection of R against B,
// rank-revealing whitening (eigenvalues > cut * max diag(R^T W R)), trial
// Rayleigh-Ritz on [B R'], compression to m columns and re-whitening.
extern "C" int igd_subspace_step_host(int m, int k, const double* G0, const double* G1, double cut, double* coeff,
                                      double* P, double* lam, double* V, int* rank_out) {
  if (m < 1 || k < 1 || m + k > 64 || !G0 || !G1 || !coeff || !P || !lam || !V || !(cut > 0.0)) return IGD_ERR_ARG;
  const int mk = m + k;
  auto block = [&](const double* g, int r0, int c0, int r, int c) {
    Mat b((size_t)r * c);
    for (int i = 0; i < r; ++i)
      for (int j = 0; j < c; ++j) b[(size_t)i * c + j] = g[(size_t)(r0 + i) * mk + c0 + j];
    return b;
  };
  const Mat BHB = block(G0, 0, 0, m, m), BHR = block(G0, 0, m, m, k), RHB = block(G0, m, 0, k, m),
            RHR = block(G0, m, m, k, k);
  Mat GB = block(G1, 0, 0, m, m);
  const Mat BR = block(G1, 0, m, m, k), RR = block(G1, m, m, k, k);
  symmetrize(GB, m);
  // W-projection of R against B: G1m = GB^-1 BR
  Mat G1m, t1, t2;
  if (!solve(GB, m, BR, k, G1m)) return IGD_ERR_NONFINITE;
  // whitening of the projected residual Gram RR - BR^T G1m, dropping lost directions
  matmul(BR, true, G1m, false, k, m, k, t1);
  Mat M((size_t)k * k);
  double scale = 0.0;
  for (int i = 0; i < k; ++i) scale = std::max(scale, at(RR, k, i, i));
  for (size_t i = 0; i < M.size(); ++i) M[i] = RR[i] - t1[i];
  symmetrize(M, k);
  std::vector<double> ev;
  Mat vm;
  if (!sym_eig(M, k, ev, vm)) return IGD_ERR_NONFINITE;
  std::vector<int> keep;
  for (int i = 0; i < k; ++i)
    if (ev[i] > cut * std::max(scale, 1e-300)) keep.push_back(i);
  const int r = (int)keep.size();
  Mat T((size_t)k * std::max(r, 1), 0.0);
  for (int i = 0; i < k; ++i)
    for (int j = 0; j < r; ++j) at(T, r, i, j) = at(vm, k, i, keep[j]) / std::sqrt(ev[keep[j]]);
  // trial Rayleigh-Ritz on [B R'] with H[B R'] = [HB (HR - HB G1m) T]
  const int n = m + r;
  Mat Tns((size_t)n * n, 0.0);
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < m; ++j) at(Tns, n, i, j) = at(BHB, m, i, j);
  if (r > 0) {
    Mat X1 = BHR;  // BHR - BHB G1m  (m x k)
    matmul(BHB, false, G1m, false, m, m, k, t1);
    for (size_t i = 0; i < X1.size(); ++i) X1[i] -= t1[i];
    Mat X2 = RHB;  // RHB - G1m^T BHB  (k x m)
    matmul(G1m, true, BHB, false, k, m, m, t1);
    for (size_t i = 0; i < X2.size(); ++i) X2[i] -= t1[i];
    // X3 = RHR - RHB G1m - G1m^T BHR + G1m^T BHB G1m  (k x k)
    Mat X3 = RHR, t3;
    matmul(RHB, false, G1m, false, k, m, k, t1);
    matmul(G1m, true, BHR, false, k, m, k, t2);
    matmul(BHB, false, G1m, false, m, m, k, t3);
    Mat t4;
    matmul(G1m, true, t3, false, k, m, k, t4);
    for (size_t i = 0; i < X3.size(); ++i) X3[i] = X3[i] - t1[i] - t2[i] + t4[i];
    Mat BHRp, RpHB, RpHRp;
    matmul(X1, false, T, false, m, k, r, BHRp);
    matmul(T, true, X2, false, r, k, m, RpHB);
    matmul(X3, false, T, false, k, k, r, t1);
    matmul(T, true, t1, false, r, k, r, RpHRp);
    for (int i = 0; i < m; ++i)
      for (int j = 0; j < r; ++j) at(Tns, n, i, m + j) = at(BHRp, r, i, j);
    for (int i = 0; i < r; ++i) {
      for (int j = 0; j < m; ++j) at(Tns, n, m + i, j) = at(RpHB, m, i, j);
      for (int j = 0; j < r; ++j) at(Tns, n, m + i, m + j) = at(RpHRp, r, i, j);
    }
  }
  Mat Ts = Tns, Wt;
  symmetrize(Ts, n);
  std::vector<double> wt;
  if (!sym_eig(Ts, n, wt, Wt)) return IGD_ERR_NONFINITE;
  Mat W1((size_t)n * m);  // lowest m trial Ritz vectors
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < m; ++j) at(W1, m, i, j) = at(Wt, n, i, j);
  // re-whitening of the compressed basis: its Gram from the fresh B^T W B
  Mat S((size_t)n * n, 0.0);
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < m; ++j) at(S, n, i, j) = at(GB, m, i, j);
  for (int i = m; i < n; ++i) at(S, n, i, i) = 1.0;
  Mat SW, X, Tb, L;
  matmul(S, false, W1, false, n, n, m, SW);
  matmul(W1, true, SW, false, m, n, m, X);
  symmetrize(X, m);
  if (cholesky(X, m, L))
    inv_lower_transposed(L, m, Tb);
  else if (!whitening(X, m, Tb))
    return IGD_ERR_NONFINITE;
  // CB = (W1[:m] - G1m T W1[m:]) Tb, CR = (T W1[m:]) Tb
  Mat Wb((size_t)m * m), Wr((size_t)std::max(r, 1) * m, 0.0);
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < m; ++j) at(Wb, m, i, j) = at(W1, m, i, j);
  for (int i = 0; i < r; ++i)
    for (int j = 0; j < m; ++j) at(Wr, m, i, j) = at(W1, m, m + i, j);
  Mat TWr((size_t)k * m, 0.0), CB, CR;
  if (r > 0) matmul(T, false, Wr, false, k, r, m, TWr);
  matmul(G1m, false, TWr, false, m, k, m, t1);
  for (size_t i = 0; i < Wb.size(); ++i) Wb[i] -= t1[i];
  matmul(Wb, false, Tb, false, m, m, m, CB);
  matmul(TWr, false, Tb, false, k, m, m, CR);
  // P = sym(Tb^T (W1^T Tns W1) Tb), eigenpairs
  Mat TW, R1, R2, Pm;
  matmul(Tns, false, W1, false, n, n, m, TW);
  matmul(W1, true, TW, false, m, n, m, R1);
  matmul(R1, false, Tb, false, m, m, m, R2);
  matmul(Tb, true, R2, false, m, m, m, Pm);
  symmetrize(Pm, m);
  std::vector<double> lv;
  Mat Vm;
  if (!sym_eig(Pm, m, lv, Vm)) return IGD_ERR_NONFINITE;
  for (size_t i = 0; i < Pm.size(); ++i) {
    if (!std::isfinite(Pm[i]) || !std::isfinite(Vm[i])) return IGD_ERR_NONFINITE;
    P[i] = Pm[i];
    V[i] = Vm[i];
  }
  for (int i = 0; i < m; ++i) lam[i] = lv[i];
  double* o = coeff;
  for (double x : CB) *o++ = x;
  for (double x : CR) *o++ = x;
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < k; ++j) *o++ = at(Vm, m, i, j);
  for (int i = 0; i < m; ++i)
    for (int j = 0; j < k; ++j) *o++ = -at(Vm, m, i, j) * lv[j];
  if (rank_out) *rank_out = r;
  return IGD_OK;
}
