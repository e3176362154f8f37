// qcp.cuh -- optimal-superposition arithmetic shared by the kNN-RMSD kernels.
//
// Quaternion key-matrix formulation (Horn 1987; Theobald 2005, Acta Cryst.
// A61:478; Liu, Agrafiotis & Theobald 2010): for centred frames x, y and
// S = sum_a x_a y_a^T, the optimal rotation R (R x ~ y) is the quaternion of
// the largest eigenvalue lambda of the symmetric traceless 4x4 key matrix
// K(S), and min RMSD^2 = (|x|^2 + |y|^2 - 2 lambda) / M.
//
// Two solvers live here:
//  * qcp_rotation_fp64: lambda by Newton on the characteristic quartic and
//    the quaternion from the adjugate of (K - lambda I), all in FP64. Used
//    once per frame (superposition onto the template) and once per
//    candidate pair (the recheck).
//  * screen_shifted_f32: the candidate screen. Frames are pre-superposed onto
//    a template mu, x_i = mu + a_i, so S_ij = P_i + Q_j + G_ij with the small
//    deviation Gram G_ij = sum a_i a_j^T. With K' = K - tr(S) I the wanted
//    eigenvalue nu = lambda - tr(S) lies in [0, D/2], D = |a_i - a_j|^2, and
//    RMSD^2 = D - 2 nu. The quartic in nu has coefficients built from the
//    small antisymmetric part b of S and the 3x3 block D' of K', so FP32
//    keeps relative accuracy in nu and D; E0 - 2 lambda never cancels.
//    Newton from nu = D/2 stays above the root, so the result never exceeds
//    the exact RMSD^2 (a lower bound, as the top-k guard needs); pairs below
//    the threshold are iterated to convergence, so their bounds are tight.
#pragma once

__device__ __forceinline__ double det3d(double a, double b, double c, double d, double e, double f,
                                        double g, double h, double i) {
  return a * (e * i - f * h) - b * (d * i - f * g) + c * (d * h - e * g);
}

// Build the key matrix from S (row-major S[3*c+d] = sum x_c y_d).
__device__ __forceinline__ void key_matrix(const double* S, double K[16]) {
  const double sxx = S[0], sxy = S[1], sxz = S[2], syx = S[3], syy = S[4], syz = S[5], szx = S[6],
               szy = S[7], szz = S[8];
  K[0] = sxx + syy + szz; K[1] = syz - szy;        K[2] = szx - sxz;         K[3] = sxy - syx;
  K[4] = K[1];            K[5] = sxx - syy - szz;  K[6] = sxy + syx;         K[7] = szx + sxz;
  K[8] = K[2];            K[9] = K[6];             K[10] = -sxx + syy - szz; K[11] = syz + szy;
  K[12] = K[3];           K[13] = K[7];            K[14] = K[11];            K[15] = -sxx - syy + szz;
}

__device__ __forceinline__ double det4d(const double* a) {
  double s0 = a[0] * a[5] - a[4] * a[1], s1 = a[0] * a[6] - a[4] * a[2];
  double s2 = a[0] * a[7] - a[4] * a[3], s3 = a[1] * a[6] - a[5] * a[2];
  double s4 = a[1] * a[7] - a[5] * a[3], s5 = a[2] * a[7] - a[6] * a[3];
  double c5 = a[10] * a[15] - a[14] * a[11], c4 = a[9] * a[15] - a[13] * a[11];
  double c3 = a[9] * a[14] - a[13] * a[10], c2 = a[8] * a[15] - a[12] * a[11];
  double c1 = a[8] * a[14] - a[12] * a[10], c0 = a[8] * a[13] - a[12] * a[9];
  return s0 * c5 - s1 * c4 + s2 * c3 + s3 * c2 - s4 * c1 + s5 * c0;
}

// Cofactor (i,j) of a 4x4 matrix (row-major).
__device__ __forceinline__ double cofactor4(const double* a, int i, int j) {
  double m[9];
  int t = 0;
  for (int r = 0; r < 4; ++r) {
    if (r == i) continue;
    for (int c = 0; c < 4; ++c) {
      if (c == j) continue;
      m[t++] = a[4 * r + c];
    }
  }
  double d = det3d(m[0], m[1], m[2], m[3], m[4], m[5], m[6], m[7], m[8]);
  return ((i + j) & 1) ? -d : d;
}

// Largest-eigenvector fallback for a degenerate top eigenvalue: cyclic
// Jacobi on the 4x4 key matrix.
__device__ inline void jacobi4_top(const double* Kin, double q[4]) {
  double a[16], v[16];
  for (int i = 0; i < 16; ++i) { a[i] = Kin[i]; v[i] = (i % 5 == 0) ? 1.0 : 0.0; }
  for (int sweep = 0; sweep < 30; ++sweep) {
    double off = 0;
    for (int p = 0; p < 4; ++p)
      for (int r = p + 1; r < 4; ++r) off += a[4 * p + r] * a[4 * p + r];
    if (off < 1e-60) break;
    for (int p = 0; p < 3; ++p)
      for (int r = p + 1; r < 4; ++r) {
        double apq = a[4 * p + r];
        if (apq == 0.0) continue;
        double theta = (a[4 * r + r] - a[4 * p + p]) / (2.0 * apq);
        double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
        double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < 4; ++k) {
          double akp = a[4 * k + p], akq = a[4 * k + r];
          a[4 * k + p] = c * akp - s * akq;
          a[4 * k + r] = s * akp + c * akq;
        }
        for (int k = 0; k < 4; ++k) {
          double apk = a[4 * p + k], aqk = a[4 * r + k];
          a[4 * p + k] = c * apk - s * aqk;
          a[4 * r + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < 4; ++k) {
          double vkp = v[4 * k + p], vkq = v[4 * k + r];
          v[4 * k + p] = c * vkp - s * vkq;
          v[4 * k + r] = s * vkp + c * vkq;
        }
      }
  }
  int best = 0;
  for (int i = 1; i < 4; ++i)
    if (a[5 * i] > a[5 * best]) best = i;
  for (int i = 0; i < 4; ++i) q[i] = v[4 * i + best];
}

// Optimal rotation R (row-major, R x ~ y) for S = sum x y^T. e0half =
// (|x|^2 + |y|^2) / 2, an upper bound of lambda_max. Returns lambda_max.
__device__ inline double qcp_rotation_fp64(const double* S, double e0half, double R[9]) {
  double K[16];
  key_matrix(S, K);
  double c2 = 0;
  for (int i = 0; i < 9; ++i) c2 += S[i] * S[i];
  c2 *= -2.0;
  double c1 = -8.0 * det3d(S[0], S[1], S[2], S[3], S[4], S[5], S[6], S[7], S[8]);
  double c0 = det4d(K);
  double lam = e0half;
  for (int it = 0; it < 60; ++it) {
    double l2 = lam * lam;
    double p = (l2 + c2) * l2 + c1 * lam + c0;
    double dp = 4.0 * l2 * lam + 2.0 * c2 * lam + c1;
    if (dp == 0.0) break;
    double nl = lam - p / dp;
    bool done = fabs(nl - lam) <= 1e-15 * fabs(nl) + 1e-300;
    lam = nl;
    if (done) break;
  }
  double A[16];
  for (int i = 0; i < 16; ++i) A[i] = K[i];
  for (int i = 0; i < 4; ++i) A[5 * i] -= lam;
  // adj(A) ~ c q q^T: take the column with the largest diagonal cofactor.
  double dg[4];
  int best = 0;
  for (int i = 0; i < 4; ++i) {
    dg[i] = cofactor4(A, i, i);
    if (fabs(dg[i]) > fabs(dg[best])) best = i;
  }
  double q[4];
  double scale = fabs(K[0]) + fabs(K[5]) + fabs(K[10]) + fabs(K[15]) + fabs(lam) + 1e-300;
  if (fabs(dg[best]) > 1e-13 * scale * scale * scale) {
    for (int i = 0; i < 4; ++i) q[i] = (i == best) ? dg[best] : cofactor4(A, i, best);
  } else {
    jacobi4_top(K, q);
  }
  double nq = sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
  double w = q[0] / nq, x = q[1] / nq, y = q[2] / nq, z = q[3] / nq;
  R[0] = w * w + x * x - y * y - z * z; R[1] = 2 * (x * y - w * z);         R[2] = 2 * (x * z + w * y);
  R[3] = 2 * (x * y + w * z);         R[4] = w * w - x * x + y * y - z * z; R[5] = 2 * (y * z - w * x);
  R[6] = 2 * (x * z - w * y);         R[7] = 2 * (y * z + w * x);         R[8] = w * w - x * x - y * y + z * z;
  return lam;
}

// Per-frame record used by the screen (all values per unit total mass):
//   rec[0..5]  M0 + sym(U_i)  as xx, yy, zz, xy, xz, yz   (row side)
//   rec[6..11] sym(U_j)       as xx, yy, zz, xy, xz, yz   (column side)
//   rec[12..14] antisymmetric part of U: (U_yz-U_zy, U_zx-U_xz, U_xy-U_yx)
//   rec[15]    Ea = |a|^2
// with U = sum a mu^T and M0 = sum mu mu^T.
#define MDS_REC 16

// Screen value (lower bound of RMSD^2, nm^2) from the deviation Gram
// G[3*c+d] = sum a_i^c a_j^d of fit frame i (row record r) and reference
// frame j (column record q). nofit: plain |a_i - a_j|^2.
//
// `guard` is subtracted from the result (the rounding margin of the caller's
// Gram). When a cheap lower bound already reaches `thr`, that bound is
// returned without the quartic solve (the caller rejects such pairs anyway):
// with g >= lambda_max(D') (Gershgorin), nu <= (g + sqrt(g^2 + 4|b|^2)) / 2,
// the largest eigenvalue of [[0, |b|], [|b|, g]], which dominates K'.
__device__ __forceinline__ float screen_shifted_f32(const float* G, const float* r, const float* q,
                                                    bool nofit, float guard = 0.0f,
                                                    float thr = __builtin_huge_valf(), bool refine = true) {
  float D = r[15] + q[15] - 2.0f * (G[0] + G[4] + G[8]);
  if (nofit) return fmaxf(D - guard, 0.0f);
  // symmetric part of S
  float sxx = r[0] + q[6] + G[0];
  float syy = r[1] + q[7] + G[4];
  float szz = r[2] + q[8] + G[8];
  float sxy = r[3] + q[9] + 0.5f * (G[1] + G[3]);
  float sxz = r[4] + q[10] + 0.5f * (G[2] + G[6]);
  float syz = r[5] + q[11] + 0.5f * (G[5] + G[7]);
  // antisymmetric part b = (Syz-Szy, Szx-Sxz, Sxy-Syx)
  float b0 = r[12] - q[12] + (G[5] - G[7]);
  float b1 = r[13] - q[13] + (G[6] - G[2]);
  float b2 = r[14] - q[14] + (G[1] - G[3]);
  // D' = lower-right block of K - tr(S) I
  float d00 = -2.0f * (syy + szz), d11 = -2.0f * (sxx + szz), d22 = -2.0f * (sxx + syy);
  float d01 = 2.0f * sxy, d02 = 2.0f * sxz, d12 = 2.0f * syz;
  float beta0 = b0 * b0 + b1 * b1 + b2 * b2;
  {
    float g = fmaxf(fmaxf(d00 + fabsf(d01) + fabsf(d02), d11 + fabsf(d01) + fabsf(d12)),
                    d22 + fabsf(d02) + fabsf(d12));
    float nu_up = 0.5f * (g + sqrtf(fmaf(g, g, 4.0f * beta0)));
    float lb = D - 2.0f * fmaxf(nu_up, 0.0f) - guard;
    if (lb >= thr) return lb;
  }
  // adjugate of D' (symmetric)
  float a00 = d11 * d22 - d12 * d12, a11 = d00 * d22 - d02 * d02, a22 = d00 * d11 - d01 * d01;
  float a01 = d02 * d12 - d01 * d22, a02 = d01 * d12 - d02 * d11, a12 = d01 * d02 - d00 * d12;
  float t = d00 + d11 + d22;
  float m2 = a00 + a11 + a22;
  float det = d00 * a00 + d01 * a01 + d02 * a02;
  float Db0 = d00 * b0 + d01 * b1 + d02 * b2;
  float Db1 = d01 * b0 + d11 * b1 + d12 * b2;
  float Db2 = d02 * b0 + d12 * b1 + d22 * b2;
  float beta1 = b0 * Db0 + b1 * Db1 + b2 * Db2;
  float badjb = b0 * (a00 * b0 + a01 * b1 + a02 * b2) + b1 * (a01 * b0 + a11 * b1 + a12 * b2) +
                b2 * (a02 * b0 + a12 * b1 + a22 * b2);
  // Q(nu) = nu^4 + k3 nu^3 + k2 nu^2 + k1 nu + k0
  float k3 = -t, k2 = m2 - beta0, k1 = -(det + beta1 - t * beta0), k0 = -badjb;
  float nu = 0.5f * fmaxf(D, 0.0f);
#pragma unroll
  for (int it = 0; it < 4; ++it) {
    float qv = (((nu + k3) * nu + k2) * nu + k1) * nu + k0;
    float qd = ((4.0f * nu + 3.0f * k3) * nu + 2.0f * k2) * nu + k1;
    float step = (qd > 0.0f) ? qv / qd : 0.0f;
    nu = fmaxf(nu - fmaxf(step, 0.0f), 0.0f);
  }
  float res = D - 2.0f * nu - guard;
  if (refine && res < thr) {
    // A candidate: far above the root Newton on the quartic removes only about
    // a quarter of the gap per step, so iterate on until the step is at
    // rounding level; the bound of a kept pair is then within the guard of
    // its exact value (the (k+1)-th bound threshold relies on that). From
    // above, every step keeps nu above the root.
#pragma unroll 1
    for (int it = 0; it < 16; ++it) {
      float qv = (((nu + k3) * nu + k2) * nu + k1) * nu + k0;
      float qd = ((4.0f * nu + 3.0f * k3) * nu + 2.0f * k2) * nu + k1;
      float step = (qd > 0.0f) ? qv / qd : 0.0f;
      if (!(step > 1e-7f * nu)) break;
      nu = fmaxf(nu - step, 0.0f);
    }
    res = D - 2.0f * nu - guard;
  }
  return fmaxf(res, 0.0f);
}

// Exact RMSD^2 (per unit mass) of a frame pair from the shifted key matrix:
// RMSD^2 = D - 2 nu, nu the largest eigenvalue of K - tr(S) I, whose lower
// right block is D' = [[-2(Syy+Szz), Sxy2, Sxz2], [Sxy2, -2(Sxx+Szz), Syz2],
// [Sxz2, Syz2, -2(Sxx+Syy)]] (Sab2 = Sab + Sba) and whose first row is
// (0, b). nu is found by Newton from D/2 (an upper bound) to convergence.
// Every input is well scaled (D = |x_i - x_j|^2 directly, b and D' at the
// scale of S), so FP32 gives nu, and hence RMSD^2, to ~1e-6 relative.
__device__ __forceinline__ float shifted_rmsd2_f32(float D, float Sxx, float Syy, float Szz, float Sxy2, float Sxz2,
                                                   float Syz2, float b0, float b1, float b2) {
  const float d00 = -2.0f * (Syy + Szz), d11 = -2.0f * (Sxx + Szz), d22 = -2.0f * (Sxx + Syy);
  const float d01 = Sxy2, d02 = Sxz2, d12 = Syz2;
  const float beta0 = b0 * b0 + b1 * b1 + b2 * b2;
  const float a00 = d11 * d22 - d12 * d12, a11 = d00 * d22 - d02 * d02, a22 = d00 * d11 - d01 * d01;
  const float a01 = d02 * d12 - d01 * d22, a02 = d01 * d12 - d02 * d11, a12 = d01 * d02 - d00 * d12;
  const float t = d00 + d11 + d22;
  const float m2 = a00 + a11 + a22;
  const float det = d00 * a00 + d01 * a01 + d02 * a02;
  const float Db0 = d00 * b0 + d01 * b1 + d02 * b2;
  const float Db1 = d01 * b0 + d11 * b1 + d12 * b2;
  const float Db2 = d02 * b0 + d12 * b1 + d22 * b2;
  const float beta1 = b0 * Db0 + b1 * Db1 + b2 * Db2;
  const float badjb = b0 * (a00 * b0 + a01 * b1 + a02 * b2) + b1 * (a01 * b0 + a11 * b1 + a12 * b2) +
                      b2 * (a02 * b0 + a12 * b1 + a22 * b2);
  const float k3 = -t, k2 = m2 - beta0, k1 = -(det + beta1 - t * beta0), k0 = -badjb;
  float nu = 0.5f * fmaxf(D, 0.0f);
  for (int it = 0; it < 40; ++it) {
    const float qv = (((nu + k3) * nu + k2) * nu + k1) * nu + k0;
    const float qd = ((4.0f * nu + 3.0f * k3) * nu + 2.0f * k2) * nu + k1;
    const float step = (qd > 0.0f) ? qv / qd : 0.0f;
    if (!(step > 1e-8f * nu)) break;  // converged (or at the rounding floor)
    nu = fmaxf(nu - step, 0.0f);
  }
  return D - 2.0f * nu;
}

