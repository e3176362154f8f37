// sym_eig.h -- dense symmetric eigensolver for the small projected matrix of
// the Lanczos restarts (host, FP64, m up to a few hundred).
//
// Written from the algorithm descriptions in Golub & Van Loan, "Matrix
// Computations", 4th ed.:
//  * §5.1.2 / §8.3.1: Householder tridiagonalisation, working forward over
//    the columns k = 0 .. m-3. Each reflector P = I - beta v v^T maps the
//    sub-column A[k+1:, k] to a multiple of e_1, and the trailing block is
//    updated as A22 -= v w^T + w v^T with p = beta A22 v and
//    w = p - (beta p^T v / 2) v.
//  * §5.1.6: the orthogonal factor Q = P_0 P_1 ... is accumulated backward.
//  * Algorithm 8.3.2 / §8.3.3: the implicit symmetric QR step with a
//    Wilkinson shift, performed as a chase of one bulge down the unreduced
//    block with Givens rotations, and deflation when an off-diagonal drops
//    below eps * (|d_i| + |d_i+1|).
// The eigenvector matrix is Q times the product of the rotations.
#pragma once

#include <algorithm>
#include <cmath>
#include <limits>
#include <vector>

namespace mds_symeig {

// Reduce the symmetric matrix a (row-major m x m, both triangles stored) to
// tridiagonal form. On return diag[0..m-1] and off[0..m-2] (off[i] couples i
// and i+1) hold T, and q (row-major m x m) holds Q with A = Q T Q^T.
inline void tridiagonalise(std::vector<double> a, int m, std::vector<double>& diag, std::vector<double>& off,
                           std::vector<double>& q) {
  diag.assign(m, 0.0);
  off.assign(std::max(m - 1, 0), 0.0);
  // reflectors: vecs[k] holds v (length m-k-1, v[0] = 1), betas[k] its beta
  std::vector<std::vector<double>> vecs(std::max(m - 2, 0));
  std::vector<double> betas(std::max(m - 2, 0), 0.0);
  std::vector<double> p(m), w(m);
  for (int k = 0; k + 2 < m; ++k) {
    const int len = m - k - 1, b0 = k + 1;
    // x = A[b0:, k]
    double tail = 0.0, amax = 0.0;
    for (int i = 0; i < len; ++i) amax = std::max(amax, std::fabs(a[(size_t)(b0 + i) * m + k]));
    std::vector<double>& v = vecs[k];
    v.assign(len, 0.0);
    if (amax == 0.0) {
      off[k] = 0.0;
      continue;
    }
    // scaled copy avoids overflow / underflow in the norm
    for (int i = 0; i < len; ++i) v[i] = a[(size_t)(b0 + i) * m + k] / amax;
    for (int i = 1; i < len; ++i) tail += v[i] * v[i];
    const double x0 = v[0];
    const double nrm = std::sqrt(x0 * x0 + tail);
    // P x = alpha e_1 with alpha = -sign(x0) ||x||; v = x - alpha e_1, then v[0] = 1
    const double alpha = (x0 >= 0.0) ? -nrm : nrm;
    const double v0 = x0 - alpha;
    if (tail == 0.0) {
      // x is already a multiple of e_1: no reflection needed
      off[k] = a[(size_t)b0 * m + k];
      v.assign(len, 0.0);
      continue;
    }
    for (int i = 1; i < len; ++i) v[i] /= v0;
    v[0] = 1.0;
    double vtv = 1.0;
    for (int i = 1; i < len; ++i) vtv += v[i] * v[i];
    const double beta = 2.0 / vtv;
    betas[k] = beta;
    off[k] = alpha * amax;
    // p = beta * A22 v
    for (int i = 0; i < len; ++i) {
      double acc = 0.0;
      const double* row = &a[(size_t)(b0 + i) * m + b0];
      for (int j = 0; j < len; ++j) acc += row[j] * v[j];
      p[i] = beta * acc;
    }
    double ptv = 0.0;
    for (int i = 0; i < len; ++i) ptv += p[i] * v[i];
    const double half = 0.5 * beta * ptv;
    for (int i = 0; i < len; ++i) w[i] = p[i] - half * v[i];
    // A22 -= v w^T + w v^T
    for (int i = 0; i < len; ++i) {
      double* row = &a[(size_t)(b0 + i) * m + b0];
      const double vi = v[i], wi = w[i];
      for (int j = 0; j < len; ++j) row[j] -= vi * w[j] + wi * v[j];
    }
  }
  for (int i = 0; i < m; ++i) diag[i] = a[(size_t)i * m + i];
  if (m >= 2) off[m - 2] = a[(size_t)(m - 1) * m + (m - 2)];
  // Q = P_0 P_1 ... P_{m-3}, accumulated backward: Q <- P_k Q on the block
  // of rows and columns k+1 .. m-1
  q.assign((size_t)m * m, 0.0);
  for (int i = 0; i < m; ++i) q[(size_t)i * m + i] = 1.0;
  for (int k = m - 3; k >= 0; --k) {
    if (betas[k] == 0.0) continue;
    const std::vector<double>& v = vecs[k];
    const int len = m - k - 1, b0 = k + 1;
    // s_j = beta * sum_i v_i Q[b0+i][b0+j]
    for (int j = 0; j < len; ++j) w[j] = 0.0;
    for (int i = 0; i < len; ++i) {
      const double* row = &q[(size_t)(b0 + i) * m + b0];
      const double vi = v[i];
      for (int j = 0; j < len; ++j) w[j] += vi * row[j];
    }
    for (int j = 0; j < len; ++j) w[j] *= betas[k];
    for (int i = 0; i < len; ++i) {
      double* row = &q[(size_t)(b0 + i) * m + b0];
      const double vi = v[i];
      for (int j = 0; j < len; ++j) row[j] -= vi * w[j];
    }
  }
}

// One implicit QR step with a Wilkinson shift on the unreduced block
// [lo, hi] of (diag, off), the rotations applied to the columns of z.
inline void qr_step(std::vector<double>& diag, std::vector<double>& off, int lo, int hi, std::vector<double>& z,
                    int m) {
  // shift: the eigenvalue of the trailing 2x2 block closer to diag[hi]
  const double t = off[hi - 1];
  const double delta = 0.5 * (diag[hi - 1] - diag[hi]);
  const double root = std::hypot(delta, t);
  const double mu = diag[hi] - t * t / (delta + (delta >= 0.0 ? root : -root));
  double x = diag[lo] - mu, y = off[lo];
  double bulge = 0.0;
  for (int k = lo; k < hi; ++k) {
    // rotation R on (k, k+1) with R (x, y)^T = (r, 0)^T
    const double r = std::hypot(x, y);
    double c = 1.0, s = 0.0;
    if (r != 0.0) {
      c = x / r;
      s = y / r;
    }
    if (k > lo) off[k - 1] = r;  // (k-1, k) after the bulge is removed
    const double a = diag[k], b = off[k], cc = diag[k + 1];
    diag[k] = c * c * a + 2.0 * c * s * b + s * s * cc;
    diag[k + 1] = s * s * a - 2.0 * c * s * b + c * c * cc;
    off[k] = c * s * (cc - a) + (c * c - s * s) * b;
    if (k + 1 < hi) {
      // row k+2 couples to k+1 only; the rotation moves part of it to (k, k+2)
      bulge = s * off[k + 1];
      off[k + 1] = c * off[k + 1];
      x = off[k];
      y = bulge;
    }
    // Z <- Z R^T on columns k, k+1
    for (int i = 0; i < m; ++i) {
      double* row = &z[(size_t)i * m];
      const double zk = row[k], zk1 = row[k + 1];
      row[k] = c * zk + s * zk1;
      row[k + 1] = -s * zk + c * zk1;
    }
  }
}

// Eigen-decomposition of the symmetric matrix a (row-major m x m): ascending
// eigenvalues in w, the matching orthonormal eigenvectors as the columns of
// z (row-major m x m). Returns false if some eigenvalue needs more than 60
// QR steps (never seen on projected Lanczos matrices).
inline bool sym_eig(const std::vector<double>& a, int m, std::vector<double>& w, std::vector<double>& z) {
  std::vector<double> diag, off;
  tridiagonalise(a, m, diag, off, z);
  const double eps = std::numeric_limits<double>::epsilon();
  const double tiny = std::numeric_limits<double>::min();
  int hi = m - 1, steps = 0;
  while (hi > 0) {
    // deflate negligible couplings at the bottom of the active block
    if (std::fabs(off[hi - 1]) <= eps * (std::fabs(diag[hi - 1]) + std::fabs(diag[hi])) + tiny) {
      off[hi - 1] = 0.0;
      --hi;
      steps = 0;
      continue;
    }
    int lo = hi - 1;
    while (lo > 0 && std::fabs(off[lo - 1]) > eps * (std::fabs(diag[lo - 1]) + std::fabs(diag[lo])) + tiny) --lo;
    if (lo > 0) off[lo - 1] = 0.0;
    if (++steps > 60) return false;
    qr_step(diag, off, lo, hi, z, m);
  }
  std::vector<int> ord(m);
  for (int i = 0; i < m; ++i) ord[i] = i;
  std::sort(ord.begin(), ord.end(), [&](int x, int y) { return diag[x] < diag[y]; });
  w.resize(m);
  std::vector<double> z2((size_t)m * m);
  for (int c = 0; c < m; ++c) {
    w[c] = diag[ord[c]];
    for (int r = 0; r < m; ++r) z2[(size_t)r * m + c] = z[(size_t)r * m + ord[c]];
  }
  z.swap(z2);
  return true;
}

}  // namespace mds_symeig
