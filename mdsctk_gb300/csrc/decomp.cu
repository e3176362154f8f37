// decomp.cu -- spectral decomposition of the normalised Gaussian affinity
// (decomp_sparse, decomp_sparse_nystrom) on sm_103a, FP64.
//
// Replaces decomp_sparse.cpp:138-277 and decomp_sparse_nystrom.cpp:173-312:
//  1. symmetrise + kernelise: the stored triangle (CSC, one entry per
//     undirected edge, values are distances) is expanded into a symmetric CSR
//     holding both triangles: each stored off-diagonal entry gives (r,c) and
//     (c,r); a diagonal entry keeps the weight sp_dsymv gives it (once when it
//     is its column's first entry, twice otherwise, mdsctk.cpp:293-313). A
//     stable radix sort by (row, col) makes every row's order deterministic.
//     w = exp(-d^2 / 2 sigma^2); degrees as decomp_sparse.cpp:162-169 (each
//     stored entry adds w to both its row and its column, a diagonal entry
//     twice); entries scaled by d_r^-1/2 d_c^-1/2.
//  2. SpMV: FP64, one warp per row of the expanded CSR.
//  3. Thick-restart Lanczos (Wu & Simon 2000; equivalent to ARPACK's
//     implicitly restarted Lanczos for symmetric matrices) keeping ARPACK's
//     contract: which='LA', nev, ncv, tol (0 = machine epsilon, converged
//     when the Ritz estimate <= tol * max(eps^(2/3), |theta|)), maxiter
//     restarts, start vector from a fixed seed. Full reorthogonalisation
//     (classical Gram-Schmidt applied twice) by FP64 GEMV kernels; the
//     projected matrix (ncv x ncv, arrowhead + tridiagonal) is solved on the
//     host by Householder tridiagonalisation and implicit symmetric QR steps
//     with Wilkinson shifts (sym_eig.h).
//  4. Eigenvalues descending, eigenvectors in the same order, residuals
//     ||A z - lambda z||_2 / |lambda| (decomp_sparse.cpp:242-270).
//  5. Nystrom: B (general CSC, columns = queries) kernelised with the
//     landmark degrees d_a and its own column sums (decomp_sparse_nystrom.cpp:
//     181-219); extension ext[x] = B^T (z_x / lambda_x) for all nev vectors
//     in one pass (:301-312).
#include <algorithm>
#include <map>
#include <cmath>
#include <cstring>
#include <vector>

#include "mds_common.cuh"
#include "sym_eig.h"

// ---------------------------------------------------------------------------
// 1. symmetrise + kernelise
// ---------------------------------------------------------------------------
// half-entries: key = (row << 32 | col) (both non-negative), value = stored
// position p << 2 | kind; kind 0 off-diagonal, 1 diagonal first-in-column
// (matvec weight 1), 2 diagonal elsewhere (matvec weight 2).
__global__ void k_sym_expand(const int* __restrict__ pcol, const int* __restrict__ irow, int n,
                             unsigned long long* __restrict__ keys, int64_t* __restrict__ vals,
                             const int64_t* __restrict__ pos, int* __restrict__ bad) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  int64_t o = pos[c];
  for (int p = pcol[c]; p < pcol[c + 1]; ++p) {
    int r = irow[p];
    if (r < 0 || r >= n) {
      atomicExch(bad, 1);
      continue;
    }
    if (r == c) {
      keys[o] = ((unsigned long long)r << 32) | (unsigned)c;
      vals[o++] = ((int64_t)p << 2) | (p == pcol[c] ? 1 : 2);
    } else {
      keys[o] = ((unsigned long long)r << 32) | (unsigned)c;
      vals[o++] = ((int64_t)p << 2);
      keys[o] = ((unsigned long long)c << 32) | (unsigned)r;
      vals[o++] = ((int64_t)p << 2);
    }
  }
}

__global__ void k_sym_count(const int* __restrict__ pcol, const int* __restrict__ irow, int n,
                            int* __restrict__ cnt) {
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  int m = 0;
  for (int p = pcol[c]; p < pcol[c + 1]; ++p) m += (irow[p] == c) ? 1 : 2;
  cnt[c] = m;
}

__global__ void k_scan_i64(const int* __restrict__ in, int n, int64_t* __restrict__ out) {
  __shared__ long long part[1024];
  int per = (n + blockDim.x - 1) / blockDim.x;
  int b = threadIdx.x * per, e = min(n, b + per);
  long long s = 0;
  for (int i = b; i < e; ++i) s += in[i];
  part[threadIdx.x] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    long long acc = 0;
    for (int i = 0; i < (int)blockDim.x; ++i) {
      long long v = part[i];
      part[i] = acc;
      acc += v;
    }
  }
  __syncthreads();
  long long acc = part[threadIdx.x];
  for (int i = b; i < e; ++i) {
    out[i] = acc;
    acc += in[i];
  }
  if (threadIdx.x == blockDim.x - 1) out[n] = acc;
}

// sorted half-entries -> CSR row pointers (lower_bound per row)
__global__ void k_rowptr(const unsigned long long* __restrict__ keys, int64_t m, int n, int64_t* __restrict__ rp) {
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r > n) return;
  unsigned long long t = (unsigned long long)r << 32;
  int64_t lo = 0, hi = m;
  while (lo < hi) {
    int64_t mid = (lo + hi) / 2;
    if (keys[mid] < t) lo = mid + 1; else hi = mid;
  }
  rp[r] = lo;
}

// affinity weight of every half-entry, degree of every row (column order:
// deterministic), then d^-1/2. One warp per row.
// den = 2 sigma^2 (decomp_sparse.cpp:159), or with per-landmark sigmas
// (auto_decomp_sparse.cpp:182) 2 s_c s_r of the stored entry's column c and
// row r (the smaller and the larger index of a strictly lower-triangle entry).
__global__ void k_sym_degree(const unsigned long long* __restrict__ keys, const int64_t* __restrict__ vals,
                             const int64_t* __restrict__ rp, const double* __restrict__ dist, int n,
                             double den, const double* __restrict__ sig, int* __restrict__ col,
                             double* __restrict__ w, double* __restrict__ dinv) {
  int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (row >= n) return;
  double s = 0.0;
  for (int64_t e = rp[row] + lane; e < rp[row + 1]; e += 32) {
    int64_t v = vals[e];
    int kind = (int)(v & 3);
    double d = dist[v >> 2];
    int c = (int)(keys[e] & 0xffffffffu);
    double dn = den;
    if (sig) dn = 2.0 * sig[min(row, c)] * sig[max(row, c)];
    double a = exp(-(d * d) / dn);
    col[e] = c;
    w[e] = a * (kind == 2 ? 2.0 : 1.0);  // the weight sp_dsymv gives it
    s += (kind == 0) ? a : 2.0 * a;      // the reference's degree sum
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) dinv[row] = 1.0 / sqrt(s);
}

__global__ void k_sym_normalise(const int64_t* __restrict__ rp, const int* __restrict__ col,
                                const double* __restrict__ dinv, int n, double* __restrict__ w) {
  int row = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (row >= n) return;
  double dr = dinv[row];
  for (int64_t e = rp[row] + lane; e < rp[row + 1]; e += 32) w[e] *= dr * dinv[col[e]];
}

// ---------------------------------------------------------------------------
// 1b. per-landmark sigmas (auto_decomp_sparse.cpp:153-178, mdsctk.cpp:388-565)
// ---------------------------------------------------------------------------
// The landmark's list is its stored distances in neighbour-index order (the
// sorted symmetric rows give exactly that order; a diagonal entry counts
// twice), cut to the first ka entries, then sorted ascending:
// sigma = (sum in ascending order) / ka. One warp per landmark; the list is
// sorted in shared memory (P2 = next power of two >= ka doubles per warp).
// `lists` (n x ka, +inf past the list's end) keeps the sorted lists for the
// entropic step; *short_list is set if a list has fewer than ka entries.
__global__ void k_auto_sigma_mean(const int64_t* __restrict__ vals, const int64_t* __restrict__ rp,
                                  const double* __restrict__ dist, int n, int ka, int P2, double* __restrict__ sig,
                                  double* __restrict__ lists, int* __restrict__ short_list) {
  extern __shared__ double sl[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int row = blockIdx.x * (blockDim.x >> 5) + warp;
  if (row >= n) return;
  double* L = sl + (size_t)warp * P2;
  int base = 0;
  for (int64_t e0 = rp[row]; e0 < rp[row + 1] && base < ka; e0 += 32) {
    int64_t e = e0 + lane;
    int mult = 0;
    double dv = 0.0;
    if (e < rp[row + 1]) {
      int64_t v = vals[e];
      mult = ((v & 3) == 0) ? 1 : 2;
      dv = dist[v >> 2];
    }
    int inc = mult;
    for (int o = 1; o < 32; o <<= 1) {
      int t = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += t;
    }
    int pos = base + inc - mult;
    for (int r = 0; r < mult; ++r)
      if (pos + r < ka) L[pos + r] = dv;
    base += __shfl_sync(0xffffffffu, inc, 31);
  }
  const int cnt = min(base, ka);
  for (int t = cnt + lane; t < P2; t += 32) L[t] = __longlong_as_double(0x7ff0000000000000ll);
  __syncwarp();
  for (int size = 2; size <= P2; size <<= 1)
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int t = lane; t < P2 / 2; t += 32) {
        int i = 2 * t - (t & (stride - 1)), j = i + stride;
        double a = L[i], b = L[j];
        if ((a > b) == ((i & size) == 0)) {
          L[i] = b;
          L[j] = a;
        }
      }
      __syncwarp();
    }
  if (lane == 0) {
    double acc = 0.0;
    for (int t = 0; t < cnt; ++t) acc += L[t];
    sig[row] = acc / (double)ka;
    if (cnt < ka) atomicExch(short_list, 1);
  }
  if (lists)
    for (int t = lane; t < ka; t += 32) lists[(int64_t)row * ka + t] = L[t];
}

// Entropic sigma of one landmark: the log-precision b at which the entropy of
// p_x ~ exp(-d_x^2 e^b) over the ka sorted distances equals log K, by Newton
// steps kept inside a shrinking bracket [lo, hi] and bisection whenever the
// value or the slope is unusable (mdsctk.cpp:388-486); sigma = 1/sqrt(2 e^b).
// The bracket comes from mdsctk.cpp:517-530. The reference solves landmarks
// one after another, each started from its predecessor's b; here each starts
// at its own bracket's midpoint and all run in parallel, so sigmas agree to
// the root-finding tolerance (|entropy - log K| < 1e-10), not bit for bit.
// At most `cap` iterations (*capped set if reached).
__global__ void k_auto_sigma_entropic(const double* __restrict__ lists, int n, int ka, double K, double p1, int cap,
                                      double* __restrict__ sig, int* __restrict__ capped) {
  int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= n) return;
  const double* d = lists + (int64_t)x * ka;
  const double N = (double)ka, logK = log(K), logN = log(N), logNK = logN - logK;
  const double realmin = 2.225074e-308, tol = 1e-10, sq_eps = 1.4901161193847656e-08;  // 2^-26
  const double a0 = d[0] * d[0], a1 = d[1] * d[1], ak = d[ka - 1] * d[ka - 1];
  double hi = log((2.0 * log(p1 * (N - 1.0) / (1.0 - p1))) / (a1 - a0));
  double l1 = log((2.0 * logNK / (1.0 - (1.0 / N))) / (ak - a0));
  double l2 = log((2.0 * sqrt(logNK)) / sqrt((ak * ak) - (a0 * a0)));
  double lo = (l1 > l2) ? l1 : l2;
  double b = (lo + hi) / 2.0;
  int it = 1, total = 0;
  for (;;) {
    if (++total > cap) {
      atomicExch(capped, 1);
      break;
    }
    const double eb = exp(b);
    bool trouble = false;
    double z = 0.0, e, mean = 0.0, m2 = 0.0;
    for (int t = 0; t < ka; ++t) z += exp(-(d[t] * d[t]) * eb);
    if (z < realmin) {
      e = -logK;
      trouble = true;
    } else {
      for (int t = 0; t < ka; ++t) {
        double q = exp(-(d[t] * d[t]) * eb) * ((d[t] * d[t]) / z);
        mean += q;
        m2 += q * (d[t] * d[t]);
      }
      e = eb * mean + log(z) - logK;
    }
    if (fabs(e) < tol) break;
    if (hi - lo < 10.0 * sq_eps) break;
    if (e < 0.0 && b <= hi) hi = b;
    else if (e > 0.0 && b >= lo) lo = b;
    trouble = trouble || e < -logK || e > logN - logK;
    double g = 0.0;
    if (!trouble) {
      if (it == 20) {
        b = (lo + hi) / 2.0;
        it = 1;
        continue;
      }
      g = (eb * eb) * ((mean * mean) - m2);
      if (g == 0) trouble = true;
    }
    if (trouble) {
      double t2 = 0.0;
      const double elo = exp(lo), ehi = exp(hi);
      for (int t = 0; t < ka; ++t) t2 += exp(-(d[t] * d[t]) * elo) + exp(-(d[t] * d[t]) * ehi);
      if (t2 < 2.0 * sqrt(realmin)) break;
      b = (lo + hi) / 2.0;
      it = 1;
      continue;
    }
    b += -e / g;
    if (b < lo || b > hi) {
      b = (lo + hi) / 2.0;
      it = 0;
    }
    ++it;
  }
  sig[x] = 1.0 / sqrt(2.0 * exp(b));
}

// ---------------------------------------------------------------------------
// 2. SpMV and dense vector kernels
// ---------------------------------------------------------------------------
// y = A x, two rows per warp (a half-warp each), four elements per lane in
// flight; each row's sum in a fixed order (lane partials, then the
// half-warp's shuffle tree).
__global__ void k_spmv(const int64_t* __restrict__ rp, const int* __restrict__ col, const double* __restrict__ w,
                       const double* __restrict__ x, int n, double* __restrict__ y) {
  const int lane = threadIdx.x & 31, hl = lane & 15;
  const int row = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) * 2 + (lane >> 4);
  double s0 = 0.0, s1 = 0.0;
  if (row < n) {
    const int64_t e1 = rp[row + 1];
    int64_t e = rp[row] + hl;
    for (; e + 48 < e1; e += 64) {
      const int c0 = col[e], c1 = col[e + 16], c2 = col[e + 32], c3 = col[e + 48];
      const double w0 = w[e], w1 = w[e + 16], w2 = w[e + 32], w3 = w[e + 48];
      s0 += w0 * __ldg(x + c0);
      s1 += w1 * __ldg(x + c1);
      s0 += w2 * __ldg(x + c2);
      s1 += w3 * __ldg(x + c3);
    }
    for (; e < e1; e += 16) s0 += w[e] * __ldg(x + col[e]);
  }
  double s = s0 + s1;
  for (int o = 8; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);  // within each half
  if (hl == 0 && row < n) y[row] = s;
}
static inline int spmv_blocks(int n) { return (int)(((int64_t)(n + 1) / 2 * 32 + 255) / 256); }

// h[j] = sum_i V[i + j*ld] * w[i], j < ncols; partial sums per block then a
// second kernel reduces them (deterministic order).
#define GV_ROWS 256
//
// The second pass of the reorthogonalisation runs only where ARPACK's test
// (dsaitr, after Daniel, Gragg, Kaufman and Stewart) asks for it: when the
// first pass left ||w|| <= 0.717 of its norm before the projection. Its
// kernels then get `gate`: the first pass's partial sums of the new w_i^2
// (gnpart, gnparts of them) and ||w||^2 before it (gh[0]); every block of
// this kernel decides the same way (one warp, fixed order) and block 0
// stores the decision in *flag, which the pass's other kernels read. A
// skipped pass writes no partial sums.
// With with_wnorm also column ncols of part: the block's sum of w_i^2.
__global__ void k_gemv_t_part(const double* __restrict__ V, int64_t ld, int n, int ncols,
                              const double* __restrict__ w, double* __restrict__ part, int with_wnorm,
                              const double* __restrict__ gnpart, int gnparts, const double* __restrict__ gh,
                              int* __restrict__ flag) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  if (gnpart) {
    __shared__ int s_need;
    if (warp == 0) {
      double q = 0.0;
      for (int b = lane; b < gnparts; b += 32) q += gnpart[b];
      for (int o = 16; o > 0; o >>= 1) q += __shfl_xor_sync(0xffffffffu, q, o);
      if (lane == 0) {
        const int need = !(q > 0.514089 * gh[0]);  // 0.717^2
        s_need = need;
        if (blockIdx.x == 0) *flag = need;
      }
    }
    __syncthreads();
    if (!s_need) return;
  }
  const int r0 = blockIdx.x * GV_ROWS, r1 = min(n, r0 + GV_ROWS);
  const int nout = ncols + (with_wnorm ? 1 : 0);
  for (int j = warp; j < nout; j += nw) {
    double s = 0.0;
    if (j < ncols)
      for (int i = r0 + lane; i < r1; i += 32) s += V[i + j * ld] * w[i];
    else
      for (int i = r0 + lane; i < r1; i += 32) s += w[i] * w[i];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) part[(int64_t)blockIdx.x * nout + j] = s;
  }
}
// h[j] = sum over blocks of part[b][j]: one warp per column (lanes take
// blocks b = lane, lane + 32, ...; fixed shuffle tree, deterministic). A
// skipped pass (flag 0) gives h = 0.
__global__ void k_reduce_part(const double* __restrict__ part, int nparts, int ncols, double* __restrict__ h,
                              const int* __restrict__ flag) {
  const int j = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  if (j >= ncols) return;
  if (flag && !*flag) {
    if (lane == 0) h[j] = 0.0;
    return;
  }
  double s = 0.0;
  for (int b = lane; b < nparts; b += 32) s += part[(int64_t)b * ncols + j];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) h[j] = s;
}
// w -= V[:, 0:ncols] h. With npart (blockDim.x = 256) also each block's sum
// of the new w_i^2, in a fixed order, into npart[blockIdx.x] (the norm of w
// without another pass over it). A skipped pass (flag 0) leaves w and takes
// the partial sums of the pass before (npart_in).
__global__ void k_gemv_sub(const double* __restrict__ V, int64_t ld, int n, int ncols,
                           const double* __restrict__ h, double* __restrict__ w, double* __restrict__ npart,
                           const int* __restrict__ flag, const double* __restrict__ npart_in) {
  extern __shared__ double hs[];
  __shared__ double red[8];
  if (flag && !*flag) {
    if (npart && threadIdx.x == 0) npart[blockIdx.x] = npart_in[blockIdx.x];
    return;
  }
  for (int j = threadIdx.x; j < ncols; j += blockDim.x) hs[j] = h[j];
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double q = 0.0;
  if (i < n) {
    double s = 0.0;
    for (int j = 0; j < ncols; ++j) s += V[i + j * ld] * hs[j];
    const double wi = w[i] - s;
    w[i] = wi;
    q = wi * wi;
  }
  if (!npart) return;
  for (int o = 16; o > 0; o >>= 1) q += __shfl_xor_sync(0xffffffffu, q, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = q;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int x = 0; x < (int)(blockDim.x >> 5); ++x) t += red[x];
    npart[blockIdx.x] = t;
  }
}
// The end of a Lanczos step in one launch: alpha_j = both projections onto
// v_j; beta_j = ||w|| from the per-block partial sums of w_i^2, which every
// block reduces itself in the same fixed order (one warp), so all blocks use
// the same beta_j; breakdown when beta_j <= tol * max(|alpha_j|, 1); then
// v_{j+1} = w / beta_j (zeros after a breakdown; those steps are redone).
// Block 0 records alpha_j, beta_j and the flag. (A separate one-warp kernel
// for alpha/beta cost one launch more per step.)
__global__ void k_lz_finish_scale(const double* __restrict__ h1, const double* __restrict__ h2,
                                  const double* __restrict__ npart, int nparts, int idx, int j, double tol,
                                  double* __restrict__ alpha, double* __restrict__ beta, int* __restrict__ brk,
                                  const double* __restrict__ w, int n, double* __restrict__ out) {
  __shared__ double s_scale;
  __shared__ int s_brk;
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    double q = 0.0;
    for (int b = lane; b < nparts; b += 32) q += npart[b];
    for (int o = 16; o > 0; o >>= 1) q += __shfl_xor_sync(0xffffffffu, q, o);
    if (lane == 0) {
      const double a = h1[idx] + h2[idx];
      const double bt = sqrt(fmax(q, 0.0));
      const int bk = (bt <= tol * fmax(fabs(a), 1.0)) ? 1 : 0;
      s_scale = 1.0 / bt;
      s_brk = bk;
      if (blockIdx.x == 0) {
        alpha[j] = a;
        beta[j] = bt;
        brk[j] = bk;
      }
    }
  }
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = s_brk ? 0.0 : w[i] * s_scale;
}
__global__ void k_scale_copy(const double* __restrict__ w, double a, int n, double* __restrict__ out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = w[i] * a;
}
// X[:, 0:nout] = V[:, 0:m] * Y (Y: m x nout, column-major on device). One
// thread per row and GV_CB output columns per block (grid.y); Y is staged in
// shared memory GV_JT rows at a time, so every V element is read once per
// GV_CB outputs. Each output is a sequential sum over j (deterministic).
#define GV_CB 8
#define GV_JT 64
__global__ void k_gemm_vy(const double* __restrict__ V, int64_t ld, int n, int m, const double* __restrict__ Y,
                          int nout, double* __restrict__ X, int64_t ldx) {
  __shared__ double ys[GV_JT][GV_CB];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int c0 = blockIdx.y * GV_CB;
  double acc[GV_CB];
#pragma unroll
  for (int c = 0; c < GV_CB; ++c) acc[c] = 0.0;
  for (int j0 = 0; j0 < m; j0 += GV_JT) {
    const int jn = min(GV_JT, m - j0);
    __syncthreads();
    for (int e = threadIdx.x; e < GV_JT * GV_CB; e += blockDim.x) {
      const int jj = e / GV_CB, cc = e % GV_CB;
      ys[jj][cc] = (jj < jn && c0 + cc < nout) ? Y[(j0 + jj) + (int64_t)(c0 + cc) * m] : 0.0;
    }
    __syncthreads();
    if (i < n)
      for (int jj = 0; jj < jn; ++jj) {
        const double v = V[i + (int64_t)(j0 + jj) * ld];
#pragma unroll
        for (int c = 0; c < GV_CB; ++c) acc[c] += v * ys[jj][c];
      }
  }
  if (i < n)
#pragma unroll
    for (int c = 0; c < GV_CB; ++c)
      if (c0 + c < nout) X[i + (int64_t)(c0 + c) * ldx] = acc[c];
}


// ---------------------------------------------------------------------------
// device-resident symmetric operator
// ---------------------------------------------------------------------------
// Largest k-sigma the per-landmark sigma kernel takes (its sorted list lives
// in 32 KB of shared memory).
#define MDS_MAX_KSIGMA 4096

// Per-landmark sigmas into `sig` (n doubles), from the sorted symmetric rows.
static int auto_sigmas(mds_ctx* ctx, int n, const int64_t* vals, const int64_t* rp, const double* ddist, int ka,
                       double K, DevBuf& sig) {
  cudaStream_t s = ctx->stream;
  if (ka < 1 || ka > MDS_MAX_KSIGMA) return mds_fail(ctx, MDS_ERR_UNSUPPORTED, "k-sigma %d outside [1, %d]", ka,
                                                     MDS_MAX_KSIGMA);
  const bool entropic = K > 0.0;
  if (entropic && (ka < 2 || (int)std::ceil(K) > ka))
    return mds_fail(ctx, MDS_ERR_ARG, "perplexity %g needs 2 <= ceil(K) <= k-sigma (%d)", K, ka);
  int P2 = 1;
  while (P2 < ka) P2 <<= 1;
  const int wpb = std::max(1, std::min(8, 1024 / P2));  // warps per block, <= 32 KB of lists
  DevBuf lists(ctx), flags(ctx);
  MDS_TRY(sig.alloc(ctx, sizeof(double) * std::max(n, 1)));
  MDS_TRY(flags.alloc(ctx, 2 * sizeof(int)));
  MDS_CUDA(ctx, cudaMemsetAsync(flags.p, 0, 2 * sizeof(int), s));
  if (entropic) MDS_TRY(lists.alloc(ctx, sizeof(double) * (size_t)n * ka));
  ctx->stats.launches++;
  k_auto_sigma_mean<<<(n + wpb - 1) / wpb, 32 * wpb, sizeof(double) * P2 * wpb, s>>>(
      vals, rp, ddist, n, ka, P2, sig.as<double>(), entropic ? lists.as<double>() : nullptr, flags.as<int>());
  MDS_CUDA(ctx, cudaGetLastError());
  int hf[2] = {0, 0};
  if (entropic) {
    MDS_CUDA(ctx, cudaMemcpyAsync(hf, flags.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    MDS_CUDA(ctx, cudaStreamSynchronize(s));
    if (hf[0])
      return mds_fail(ctx, MDS_ERR_ARG, "a landmark has fewer than k-sigma=%d stored distances (the entropic "
                      "sigmas read past its list)", ka);
    // p1 (mdsctk.cpp:505-514): scalar, on the host
    const double N = (double)ka, logK = std::log(K);
    double p1;
    if (logK > std::log(std::sqrt(2.0 * N))) {
      p1 = 3.0 / 4.0;
    } else {
      p1 = 1.0 / 4.0;
      for (int it = 0; it < 100; ++it) p1 -= (-p1 * std::log(p1 / N) - logK) / (-std::log(p1 / N) + 1.0);
      p1 = 1.0 - (p1 / 2.0);
    }
    ctx->stats.launches++;
    k_auto_sigma_entropic<<<(n + 127) / 128, 128, 0, s>>>(lists.as<double>(), n, ka, K, p1, 10000,
                                                          sig.as<double>(), flags.as<int>() + 1);
    MDS_CUDA(ctx, cudaGetLastError());
    MDS_CUDA(ctx, cudaMemcpyAsync(hf + 1, flags.as<int>() + 1, sizeof(int), cudaMemcpyDeviceToHost, s));
    MDS_CUDA(ctx, cudaStreamSynchronize(s));
    if (hf[1]) return mds_fail(ctx, MDS_ERR_INTERNAL, "entropic sigma did not settle within 10000 iterations");
  }
  return MDS_OK;
}

struct SymOp {
  int n = 0;
  int64_t nnz = 0;
  DevBuf rp, col, w, dinv;
  DevBuf sig;  // per-landmark sigmas (auto mode only)
};

// ka > 0 selects per-landmark sigmas (mean of the ka-entry lists; entropic
// with perplexity K when K > 0) in place of the single sigma.
static int build_symop(mds_ctx* ctx, int n, const int* dpcol, const int* dirow, const double* ddist, double sigma,
                       SymOp& op, int ka = 0, double K = 0.0) {
  cudaStream_t s = ctx->stream;
  op.n = n;
  DevBuf cnt(ctx), pos(ctx), bad(ctx), k0(ctx), v0(ctx), k1(ctx), v1(ctx);
  MDS_TRY(cnt.alloc(ctx, sizeof(int) * std::max(n, 1)));
  MDS_TRY(pos.alloc(ctx, sizeof(int64_t) * (n + 1)));
  MDS_TRY(bad.alloc(ctx, sizeof(int)));
  MDS_CUDA(ctx, cudaMemsetAsync(bad.p, 0, sizeof(int), s));
  ctx->stats.launches += 2;
  k_sym_count<<<(n + 255) / 256, 256, 0, s>>>(dpcol, dirow, n, cnt.as<int>());
  k_scan_i64<<<1, 1024, 0, s>>>(cnt.as<int>(), n, pos.as<int64_t>());
  MDS_CUDA(ctx, cudaGetLastError());
  int64_t m = 0;
  MDS_CUDA(ctx, cudaMemcpyAsync(&m, pos.as<int64_t>() + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
  MDS_CUDA(ctx, cudaStreamSynchronize(s));
  op.nnz = m;
  MDS_TRY(k0.alloc(ctx, sizeof(unsigned long long) * std::max<int64_t>(m, 1)));
  MDS_TRY(v0.alloc(ctx, sizeof(int64_t) * std::max<int64_t>(m, 1)));
  MDS_TRY(k1.alloc(ctx, sizeof(unsigned long long) * std::max<int64_t>(m, 1)));
  MDS_TRY(v1.alloc(ctx, sizeof(int64_t) * std::max<int64_t>(m, 1)));
  ctx->stats.launches++;
  k_sym_expand<<<(n + 255) / 256, 256, 0, s>>>(dpcol, dirow, n, k0.as<unsigned long long>(), v0.as<int64_t>(),
                                               pos.as<int64_t>(), bad.as<int>());
  MDS_CUDA(ctx, cudaGetLastError());
  int hbad = 0;
  MDS_CUDA(ctx, cudaMemcpyAsync(&hbad, bad.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  MDS_CUDA(ctx, cudaStreamSynchronize(s));
  if (hbad) return mds_fail(ctx, MDS_ERR_ARG, "row index outside [0, n) in the sparse matrix");
  int bits = 0;
  while ((1ll << bits) < (int64_t)n) ++bits;
  unsigned long long mask = ((1ull << bits) - 1ull) | (((1ull << bits) - 1ull) << 32);
  int which = 0;
  MDS_TRY(radix_sort(ctx, k0.as<unsigned long long>(), v0.as<int64_t>(), k1.as<unsigned long long>(),
                     v1.as<int64_t>(), m, mask, &which));
  unsigned long long* keys = which ? k1.as<unsigned long long>() : k0.as<unsigned long long>();
  int64_t* vals = which ? v1.as<int64_t>() : v0.as<int64_t>();
  MDS_TRY(op.rp.alloc(ctx, sizeof(int64_t) * (n + 1)));
  MDS_TRY(op.col.alloc(ctx, sizeof(int) * std::max<int64_t>(m, 1)));
  MDS_TRY(op.w.alloc(ctx, sizeof(double) * std::max<int64_t>(m, 1)));
  MDS_TRY(op.dinv.alloc(ctx, sizeof(double) * std::max(n, 1)));
  const int wb = (int)(((int64_t)n * 32 + 255) / 256);
  ctx->stats.launches++;
  k_rowptr<<<(n + 1 + 255) / 256, 256, 0, s>>>(keys, m, n, op.rp.as<int64_t>());
  if (ka > 0) MDS_TRY(auto_sigmas(ctx, n, vals, op.rp.as<int64_t>(), ddist, ka, K, op.sig));
  ctx->stats.launches += 2;
  k_sym_degree<<<wb, 256, 0, s>>>(keys, vals, op.rp.as<int64_t>(), ddist, n, 2.0 * sigma * sigma,
                                  ka > 0 ? op.sig.as<double>() : nullptr, op.col.as<int>(), op.w.as<double>(),
                                  op.dinv.as<double>());
  k_sym_normalise<<<wb, 256, 0, s>>>(op.rp.as<int64_t>(), op.col.as<int>(), op.dinv.as<double>(), n,
                                     op.w.as<double>());
  MDS_CUDA(ctx, cudaGetLastError());
  return MDS_OK;
}

static void spmv(mds_ctx* ctx, const SymOp& op, const double* x, double* y) {
  ctx->stats.launches++;
  k_spmv<<<spmv_blocks(op.n), 256, 0, ctx->stream>>>(op.rp.as<int64_t>(), op.col.as<int>(),
                                                                           op.w.as<double>(), x, op.n, y);
}

// ---------------------------------------------------------------------------
// 3. thick-restart Lanczos
// ---------------------------------------------------------------------------
struct LanczosOut {
  std::vector<double> evals;  // descending
  int nconv = 0;
  int restarts = 0;
  int matvecs = 0;
};

// With nlock > 0 the sequence runs on the operator deflated by the nlock
// orthonormal columns dLock [nlock][n]: every new basis vector is
// orthogonalised against them as well as against the Lanczos basis.
static int lanczos(mds_ctx* ctx, const SymOp& op, int nev, int ncv, double tol, int maxiter, double* dX /*n*nev*/,
                   LanczosOut& out, const double* dLock = nullptr, int nlock = 0,
                   uint64_t seed = 0x9E3779B97F4A7C15ull) {
  cudaStream_t s = ctx->stream;
  const int n = op.n;
  const int m = ncv;
  const int64_t ld = n;
  DevBuf V(ctx), wv(ctx), h(ctx), part(ctx), Yd(ctx), tmp(ctx);
  MDS_TRY(V.alloc(ctx, sizeof(double) * (size_t)n * (nlock + m + 1)));
  MDS_TRY(wv.alloc(ctx, sizeof(double) * n));
  MDS_TRY(h.alloc(ctx, sizeof(double) * (nlock + m + 1)));
  const int nparts = (n + GV_ROWS - 1) / GV_ROWS;
  MDS_TRY(part.alloc(ctx, sizeof(double) * (size_t)nparts * (nlock + m + 1)));
  MDS_TRY(Yd.alloc(ctx, sizeof(double) * (size_t)m * m));
  MDS_TRY(tmp.alloc(ctx, sizeof(double) * (size_t)n * m));
  DevBuf h1(ctx), h2(ctx), ab(ctx), brk(ctx), npart(ctx), npart1(ctx), flag2(ctx);
  MDS_TRY(npart.alloc(ctx, sizeof(double) * (size_t)((n + 255) / 256)));
  MDS_TRY(npart1.alloc(ctx, sizeof(double) * (size_t)((n + 255) / 256)));
  MDS_TRY(flag2.alloc(ctx, sizeof(int)));
  // step graphs by first step of the cycle; destroyed on every return path
  struct Graphs : std::map<int, cudaGraphExec_t> {
    ~Graphs() {
      for (auto& g : *this) cudaGraphExecDestroy(g.second);
    }
  } graphs;
  MDS_TRY(h1.alloc(ctx, sizeof(double) * (nlock + m + 1)));
  MDS_TRY(h2.alloc(ctx, sizeof(double) * (nlock + m + 1)));
  MDS_TRY(ab.alloc(ctx, sizeof(double) * 2 * m));
  MDS_TRY(brk.alloc(ctx, sizeof(int) * m));
  double* Vl = V.as<double>();           // locked columns, then the Lanczos basis
  double* Vp = Vl + (int64_t)nlock * ld;  // Lanczos basis v_0..v_m
  if (nlock)
    MDS_CUDA(ctx, cudaMemcpyAsync(Vl, dLock, sizeof(double) * (size_t)n * nlock, cudaMemcpyDeviceToDevice, s));
  double* w = wv.as<double>();
  const double eps = std::numeric_limits<double>::epsilon();
  const double eps23 = std::pow(eps, 2.0 / 3.0);
  if (tol <= 0.0) tol = eps;

  // dots/subtract act on the first ncols columns of [locked | basis]
  auto dots = [&](int ncols, std::vector<double>& hh) -> int {
    ctx->stats.launches += 2;
    k_gemv_t_part<<<nparts, 256, 0, s>>>(Vl, ld, n, ncols, w, part.as<double>(), 0, nullptr, 0, nullptr, nullptr);
    k_reduce_part<<<(ncols + 3) / 4, 128, 0, s>>>(part.as<double>(), nparts, ncols, h.as<double>(), nullptr);
    MDS_CUDA(ctx, cudaGetLastError());
    hh.resize(ncols);
    MDS_CUDA(ctx, cudaMemcpyAsync(hh.data(), h.p, sizeof(double) * ncols, cudaMemcpyDeviceToHost, s));
    MDS_CUDA(ctx, cudaStreamSynchronize(s));
    return MDS_OK;
  };
  auto subtract = [&](int ncols, const std::vector<double>& hh) -> int {
    MDS_CUDA(ctx, cudaMemcpyAsync(h.p, hh.data(), sizeof(double) * ncols, cudaMemcpyHostToDevice, s));
    ctx->stats.launches++;
    k_gemv_sub<<<(n + 255) / 256, 256, sizeof(double) * ncols, s>>>(Vl, ld, n, ncols, h.as<double>(), w,
                                                                      nullptr, nullptr, nullptr);
    MDS_CUDA(ctx, cudaGetLastError());
    return MDS_OK;
  };
  std::vector<double> hh0;
  auto norm_w = [&](double* nr) -> int {
    // ||w|| through the same partial-sum kernels (V column = w itself)
    ctx->stats.launches += 2;
    k_gemv_t_part<<<nparts, 256, 0, s>>>(w, ld, n, 1, w, part.as<double>(), 0, nullptr, 0, nullptr, nullptr);
    k_reduce_part<<<1, 128, 0, s>>>(part.as<double>(), nparts, 1, h.as<double>(), nullptr);
    double v = 0;
    MDS_CUDA(ctx, cudaMemcpyAsync(&v, h.p, sizeof(double), cudaMemcpyDeviceToHost, s));
    MDS_CUDA(ctx, cudaStreamSynchronize(s));
    *nr = std::sqrt(std::max(v, 0.0));
    return MDS_OK;
  };
  // start vector: fixed-seed pseudo-random, orthogonalised and normalised
  {
    std::vector<double> v0(n);
    uint64_t st = seed;
    for (int i = 0; i < n; ++i) {
      st ^= st << 13; st ^= st >> 7; st ^= st << 17;
      v0[i] = (double)(st >> 11) * (1.0 / 9007199254740992.0) - 0.5;
    }
    MDS_CUDA(ctx, cudaMemcpyAsync(w, v0.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s));
    for (int rep = 0; rep < 2 && nlock; ++rep) {
      MDS_TRY(dots(nlock, hh0));
      MDS_TRY(subtract(nlock, hh0));
    }
    double nr = 0;
    MDS_TRY(norm_w(&nr));
    ctx->stats.launches++;
    k_scale_copy<<<(n + 255) / 256, 256, 0, s>>>(w, 1.0 / nr, n, Vp);
  }
  int k = 0;
  std::vector<double> theta_k, s_k;  // kept Ritz values and couplings
  std::vector<double> alpha(m, 0.0), beta(m, 0.0);
  std::vector<double> hh, hh2, T, Z, th;
  int restart = 0;
  for (;; ++restart) {
    // Lanczos steps k..m-1 run with no host round trip: the projections,
    // alpha_j, beta_j and the next basis vector are computed on the device;
    // alpha/beta/breakdown flags are read once afterwards. A breakdown
    // (invariant subspace, beta_j ~ 0) found then restarts the steps after
    // it from a fresh direction orthogonal to the basis.
    for (int j0 = k; j0 < m;) {
      // The steps j0..m-1 are one CUDA graph, captured the first time a cycle
      // starts at j0 (every pointer and size is fixed within this call) and
      // replayed afterwards: one launch instead of 9 per step.
      auto git = graphs.find(j0);
      if (git == graphs.end()) {
        MDS_CUDA(ctx, cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
        for (int j = j0; j < m; ++j) {
          const int nc = nlock + j + 1;  // full reorthogonalisation (twice)
          k_spmv<<<spmv_blocks(op.n), 256, 0, s>>>(op.rp.as<int64_t>(), op.col.as<int>(), op.w.as<double>(),
                                                   Vp + (int64_t)j * ld, op.n, w);
          // first pass, with ||w||^2 before it (h1[nc]) and the new w's
          // partial sums (npart1); the second pass only where ARPACK's test
          // asks for it (k_gemv_t_part)
          k_gemv_t_part<<<nparts, 256, 0, s>>>(Vl, ld, n, nc, w, part.as<double>(), 1, nullptr, 0, nullptr, nullptr);
          k_reduce_part<<<(nc + 4) / 4, 128, 0, s>>>(part.as<double>(), nparts, nc + 1, h1.as<double>(), nullptr);
          k_gemv_sub<<<(n + 255) / 256, 256, sizeof(double) * nc, s>>>(Vl, ld, n, nc, h1.as<double>(), w,
                                                                        npart1.as<double>(), nullptr, nullptr);
          k_gemv_t_part<<<nparts, 256, 0, s>>>(Vl, ld, n, nc, w, part.as<double>(), 0, npart1.as<double>(),
                                               (n + 255) / 256, h1.as<double>() + nc, flag2.as<int>());
          k_reduce_part<<<(nc + 3) / 4, 128, 0, s>>>(part.as<double>(), nparts, nc, h2.as<double>(), flag2.as<int>());
          k_gemv_sub<<<(n + 255) / 256, 256, sizeof(double) * nc, s>>>(Vl, ld, n, nc, h2.as<double>(), w,
                                                                       npart.as<double>(), flag2.as<int>(),
                                                                       npart1.as<double>());
          k_lz_finish_scale<<<(n + 255) / 256, 256, 0, s>>>(h1.as<double>(), h2.as<double>(), npart.as<double>(),
                                                             (n + 255) / 256, nlock + j, j, eps * 10.0,
                                                             ab.as<double>(), ab.as<double>() + m, brk.as<int>(), w,
                                                             n, Vp + (int64_t)(j + 1) * ld);
        }
        cudaGraph_t g = nullptr;
        cudaError_t ce = cudaStreamEndCapture(s, &g);
        if (ce != cudaSuccess) return mds_fail(ctx, MDS_ERR_CUDA, "Lanczos step capture: %s", cudaGetErrorString(ce));
        cudaGraphExec_t ge = nullptr;
        ce = cudaGraphInstantiate(&ge, g, 0);
        cudaGraphDestroy(g);
        if (ce != cudaSuccess) return mds_fail(ctx, MDS_ERR_CUDA, "Lanczos step graph: %s", cudaGetErrorString(ce));
        git = graphs.emplace(j0, ge).first;
      }
      MDS_CUDA(ctx, cudaGraphLaunch(git->second, s));
      out.matvecs += m - j0;
      ctx->stats.launches += 8 * (m - j0);
      MDS_CUDA(ctx, cudaGetLastError());
      std::vector<double> hab(2 * m);
      std::vector<int> hbrk(m);
      MDS_CUDA(ctx, cudaMemcpyAsync(hab.data(), ab.p, sizeof(double) * 2 * m, cudaMemcpyDeviceToHost, s));
      MDS_CUDA(ctx, cudaMemcpyAsync(hbrk.data(), brk.p, sizeof(int) * m, cudaMemcpyDeviceToHost, s));
      MDS_CUDA(ctx, cudaStreamSynchronize(s));
      int jb = -1;
      for (int j = j0; j < m; ++j) {
        alpha[j] = hab[j];
        beta[j] = hab[m + j];
        if (hbrk[j]) {
          jb = j;
          break;
        }
      }
      if (jb < 0) break;
      // invariant subspace at step jb: continue with a fresh direction orthogonal to V
      std::vector<double> v0(n);
      uint64_t st = 0xD1B54A32D192ED03ull + (seed - 0x9E3779B97F4A7C15ull) + 7919ull * (uint64_t)(jb + 1 + restart * m);
      for (int i = 0; i < n; ++i) {
        st ^= st << 13; st ^= st >> 7; st ^= st << 17;
        v0[i] = (double)(st >> 11) * (1.0 / 9007199254740992.0) - 0.5;
      }
      MDS_CUDA(ctx, cudaMemcpyAsync(w, v0.data(), sizeof(double) * n, cudaMemcpyHostToDevice, s));
      for (int rep = 0; rep < 2; ++rep) {
        MDS_TRY(dots(nlock + jb + 1, hh));
        MDS_TRY(subtract(nlock + jb + 1, hh));
      }
      double nr = 0;
      MDS_TRY(norm_w(&nr));
      beta[jb] = 0.0;
      ctx->stats.launches++;
      k_scale_copy<<<(n + 255) / 256, 256, 0, s>>>(w, 1.0 / nr, n, Vp + (int64_t)(jb + 1) * ld);
      j0 = jb + 1;
    }
    // projected matrix: arrowhead (kept Ritz pairs) + tridiagonal
    T.assign((size_t)m * m, 0.0);
    for (int i = 0; i < k; ++i) {
      T[i * m + i] = theta_k[i];
      T[i * m + k] = T[k * m + i] = s_k[i];
    }
    for (int j = k; j < m; ++j) {
      T[j * m + j] = alpha[j];
      if (j + 1 < m) T[j * m + j + 1] = T[(j + 1) * m + j] = beta[j];
    }
    if (!mds_symeig::sym_eig(T, m, th, Z)) return mds_fail(ctx, MDS_ERR_INTERNAL, "projected eigenproblem did not converge");
    const double bm = beta[m - 1];
    // wanted: the nev largest (ascending order -> last nev)
    int nconv = 0;
    for (int c = m - nev; c < m; ++c) {
      double est = std::fabs(bm * Z[(m - 1) * m + c]);
      if (est <= tol * std::max(eps23, std::fabs(th[c]))) ++nconv;
    }
    out.nconv = nconv;
    if (nconv >= nev || restart >= maxiter) {
      // Ritz vectors of the wanted values, descending
      std::vector<double> Y((size_t)m * nev);
      out.evals.resize(nev);
      for (int x = 0; x < nev; ++x) {
        int c = m - 1 - x;
        out.evals[x] = th[c];
        for (int r = 0; r < m; ++r) Y[r + (size_t)x * m] = Z[r * m + c];
      }
      MDS_CUDA(ctx, cudaMemcpyAsync(Yd.p, Y.data(), sizeof(double) * Y.size(), cudaMemcpyHostToDevice, s));
      ctx->stats.launches++;
      k_gemm_vy<<<dim3((n + 127) / 128, (nev + GV_CB - 1) / GV_CB), 128, 0, s>>>(Vp, ld, n, m, Yd.as<double>(), nev,
                                                                               dX, n);
      MDS_CUDA(ctx, cudaGetLastError());
      out.restarts = restart;
      return MDS_OK;
    }
    // thick restart with the kk largest Ritz pairs
    // ARPACK's rule (dsaup2): keep nev + min(nconv, np/2) Ritz pairs, np =
    // ncv - nev; with nev = 1 keep ncv/2 (ncv >= 6) or 2
    int kk = nev + std::min(nconv, (m - nev) / 2);
    if (kk == 1) kk = (m >= 6) ? m / 2 : (m > 2 ? 2 : 1);
    kk = std::max(nev, std::min(kk, m - 2));
    std::vector<double> Y((size_t)m * kk);
    theta_k.assign(kk, 0.0);
    s_k.assign(kk, 0.0);
    for (int x = 0; x < kk; ++x) {
      int c = m - kk + x;
      theta_k[x] = th[c];
      s_k[x] = bm * Z[(m - 1) * m + c];
      for (int r = 0; r < m; ++r) Y[r + (size_t)x * m] = Z[r * m + c];
    }
    MDS_CUDA(ctx, cudaMemcpyAsync(Yd.p, Y.data(), sizeof(double) * Y.size(), cudaMemcpyHostToDevice, s));
    ctx->stats.launches++;
    k_gemm_vy<<<dim3((n + 127) / 128, (kk + GV_CB - 1) / GV_CB), 128, 0, s>>>(Vp, ld, n, m, Yd.as<double>(), kk,
                                                                              tmp.as<double>(), n);
    MDS_CUDA(ctx, cudaGetLastError());
    MDS_CUDA(ctx, cudaMemcpyAsync(Vp, tmp.p, sizeof(double) * (size_t)n * kk, cudaMemcpyDeviceToDevice, s));
    MDS_CUDA(ctx, cudaMemcpyAsync(Vp + (int64_t)kk * ld, Vp + (int64_t)m * ld, sizeof(double) * n,
                                  cudaMemcpyDeviceToDevice, s));
    k = kk;
  }
}

// Lanczos from one start vector sees one direction of each eigenspace, so a
// wanted eigenvalue of multiplicity > 1 (e.g. 1.0 once per connected
// component of the kNN graph) can be missed. After convergence, run a
// sequence on the operator deflated by the nev converged vectors, its top
// Ritz value converged to 1e-8 (at most 30 restarts of 40 vectors): that
// value is a lower bound of the deflated spectrum's top, so a value more than
// 1e-10 (relative) above the nev-th eigenvalue proves a missed eigenpair. If
// it is a further copy of an eigenvalue already found (within 1e-9
// relative), it is converged to the requested tolerance, inserted in order
// (dropping the smallest) and the check repeats.
// Eigenvalues within 1e-10 of the nev-th are interchangeable with it.
static int lanczos_complete(mds_ctx* ctx, const SymOp& op, int nev, int ncv, double tol, int maxiter, double* dX,
                            LanczosOut& out) {
  MDS_TRY(lanczos(ctx, op, nev, ncv, tol, maxiter, dX, out));
  const int n = op.n;
  // The check runs until the deflated top Ritz value converges (to 1e-8, at
  // most 30 restarts of 40 vectors): crowded eigenvalues just below a missed
  // one slow its convergence, and a Ritz value stopped early can sit below
  // the nev-th eigenvalue although the missed one is above it (a graph of
  // three components, triple eigenvalue 1 with 0.9996 next, asked for nev = 3:
  // three restarts of 20 vectors reached 0.99977 < 0.99990; converged, 1.0).
  const int ncv2 = std::min(40, n - nev);
  if (ncv2 < 3) return MDS_OK;
  cudaStream_t s = ctx->stream;
  DevBuf y(ctx);
  MDS_TRY(y.alloc(ctx, sizeof(double) * n));
  const double eps = std::numeric_limits<double>::epsilon();
  (void)eps;
  for (int pass = 0; pass < nev; ++pass) {
    const uint64_t seed = 0x9E3779B97F4A7C15ull + 0x632BE59BD9B4E019ull * (uint64_t)(pass + 1);
    LanczosOut o2;
    MDS_TRY(lanczos(ctx, op, 1, ncv2, 1e-8, 30, y.as<double>(), o2, dX, nev, seed));
    out.matvecs += o2.matvecs;
    const double th = o2.evals[0], lo = out.evals[nev - 1];
    if (!(th > lo + 1e-10 * std::max(1.0, std::fabs(lo)))) break;
    // Only a further copy of an eigenvalue already found is inserted: a
    // multiple eigenvalue is what one start vector cannot see. A distinct
    // eigenvalue above the nev-th that the sequence left out (crowded
    // spectra near 1) is left out as ARPACK leaves it out.
    bool copy = false;
    for (int x = 0; x < nev && !copy; ++x)
      copy = std::fabs(th - out.evals[x]) <= 1e-9 * std::max(1.0, std::fabs(out.evals[x]));
    if (!copy) break;
    o2 = LanczosOut();  // converge the missed pair to the requested tolerance
    MDS_TRY(lanczos(ctx, op, 1, ncv2, tol, maxiter, y.as<double>(), o2, dX, nev, seed));
    out.matvecs += o2.matvecs;
    int p = nev - 1;
    while (p > 0 && out.evals[p - 1] < o2.evals[0]) --p;
    for (int c = nev - 1; c > p; --c) {
      out.evals[c] = out.evals[c - 1];
      MDS_CUDA(ctx, cudaMemcpyAsync(dX + (int64_t)c * n, dX + (int64_t)(c - 1) * n, sizeof(double) * n,
                                    cudaMemcpyDeviceToDevice, s));
    }
    out.evals[p] = o2.evals[0];
    MDS_CUDA(ctx, cudaMemcpyAsync(dX + (int64_t)p * n, y.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
  }
  return MDS_OK;
}

// residual ||A z - lambda z|| / |lambda| for each vector
__global__ void k_resid_part(const double* __restrict__ Az, const double* __restrict__ z, double lam, int n,
                             double* __restrict__ part) {
  __shared__ double sh[256];
  double s = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    double r = Az[i] - lam * z[i];
    s += r * r;
  }
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// ---------------------------------------------------------------------------
// 5. Nystrom
// ---------------------------------------------------------------------------
// B affinity: w = exp(-d^2/2s^2); d_b[q] = (sum of column q)^-1/2;
// B[l,q] = w * d_a[l] * d_b[q]   (one warp per column q)
// den = 2 sigma^2, or with per-landmark sigmas 2 s_l s_l of the entry's
// landmark l (auto_decomp_sparse_nystrom.cpp:171-173).
__global__ void k_nystrom_b(const int* __restrict__ pcol, const int* __restrict__ irow, const double* __restrict__ dist,
                            int m, int n, double den, const double* __restrict__ sig,
                            const double* __restrict__ dinv_a, double* __restrict__ B, int* __restrict__ bad) {
  int q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (q >= m) return;
  double s = 0.0;
  for (int p = pcol[q] + lane; p < pcol[q + 1]; p += 32) {
    double d = dist[p];
    double dn = den;
    if (sig) {
      int l = irow[p];
      dn = (l >= 0 && l < n) ? 2.0 * sig[l] * sig[l] : 1.0;
    }
    double a = exp(-(d * d) / dn);
    B[p] = a;
    s += a;
  }
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  double db = 1.0 / sqrt(s);
  for (int p = pcol[q] + lane; p < pcol[q + 1]; p += 32) {
    int l = irow[p];
    if (l < 0 || l >= n) {
      atomicExch(bad, 1);
      continue;
    }
    B[p] *= dinv_a[l] * db;
  }
}
// ext[x][q] = sum_{p in col q} B[p] z_x[irow[p]] / lambda_x, all x at once
__global__ void k_nystrom_ext(const int* __restrict__ pcol, const int* __restrict__ irow, const double* __restrict__ B,
                              int m, int n, const double* __restrict__ Z, const double* __restrict__ inv_lam, int nev,
                              double* __restrict__ ext) {
  int q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (q >= m) return;
  for (int x = 0; x < nev; ++x) {
    double s = 0.0;
    for (int p = pcol[q] + lane; p < pcol[q + 1]; p += 32) s += B[p] * Z[(int64_t)x * n + irow[p]];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if (lane == 0) ext[(int64_t)x * m + q] = s * inv_lam[x];
  }
}

// ---------------------------------------------------------------------------
// C ABI
// ---------------------------------------------------------------------------
// k_sigma > 0: per-landmark sigmas (auto_decomp_sparse), entropic when
// perplexity > 0; `sigma` is then unused and sig_out (n, may be null) gets
// the sigmas.
static int decomp_impl(mds_ctx* ctx, int n, const int32_t* pcol, const int32_t* irow, const double* dist, double sigma,
                       int nev, int ncv, double tol, int maxiter, unsigned flags, double* evals, double* evecs,
                       double* resid, int* nconv, int m, const int32_t* pcolB, const int32_t* irowB,
                       const double* distB, double* ext, int k_sigma = 0, double perplexity = 0.0,
                       double* sig_out = nullptr) {
  if (!ctx) return MDS_ERR_ARG;
  ctx->stats = mds_knn_stats{};
  if (!pcol || !irow || !dist || !evals || !evecs) return mds_fail(ctx, MDS_ERR_ARG, "null argument");
  if (n < 1 || nev < 1) return mds_fail(ctx, MDS_ERR_ARG, "invalid sizes n=%d nev=%d", n, nev);
  if (k_sigma > 0) sigma = 1.0;
  if (!(sigma > 0.0)) return mds_fail(ctx, MDS_ERR_ARG, "sigma must be positive");
  // decomp_sparse.cpp:199-205: ncv = min(10 nev + 1, n), maxiter = 100 nev
  if (ncv <= 0) ncv = std::min(10 * nev + 1, n);
  ncv = std::min(ncv, n);
  if (maxiter <= 0) maxiter = 100 * nev;
  if (nev >= ncv) return mds_fail(ctx, MDS_ERR_ARG, "need nev < ncv <= n (nev=%d ncv=%d n=%d)", nev, ncv, n);
  if (ncv > 4096) return mds_fail(ctx, MDS_ERR_UNSUPPORTED, "ncv=%d too large", ncv);
  cudaSetDevice(ctx->device);
  cudaStream_t s = ctx->stream;
  const bool dev = (flags & MDS_DEVICE_IO) != 0;
  std::vector<int> hp;
  const int* hpcol = pcol;
  if (dev) {
    hp.resize(n + 1);
    MDS_CUDA(ctx, cudaMemcpyAsync(hp.data(), pcol, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, s));
    MDS_CUDA(ctx, cudaStreamSynchronize(s));
    hpcol = hp.data();
  }
  const int64_t nnz = hpcol[n];
  if (nnz < 0 || hpcol[0] != 0) return mds_fail(ctx, MDS_ERR_ARG, "malformed column pointers");
  for (int c = 0; c < n; ++c)
    if (hpcol[c + 1] < hpcol[c]) return mds_fail(ctx, MDS_ERR_ARG, "column pointers not ascending at %d", c);
  DevBuf dp(ctx), dr(ctx), dd(ctx), dX(ctx);
  const int* ppcol = pcol;
  const int* pirow = irow;
  const double* pdist = dist;
  if (!dev) {
    MDS_TRY(dp.alloc(ctx, sizeof(int) * (n + 1)));
    MDS_TRY(dr.alloc(ctx, sizeof(int) * std::max<int64_t>(nnz, 1)));
    MDS_TRY(dd.alloc(ctx, sizeof(double) * std::max<int64_t>(nnz, 1)));
    MDS_CUDA(ctx, cudaMemcpyAsync(dp.p, pcol, sizeof(int) * (n + 1), cudaMemcpyHostToDevice, s));
    if (nnz) {
      MDS_CUDA(ctx, cudaMemcpyAsync(dr.p, irow, sizeof(int) * nnz, cudaMemcpyHostToDevice, s));
      MDS_CUDA(ctx, cudaMemcpyAsync(dd.p, dist, sizeof(double) * nnz, cudaMemcpyHostToDevice, s));
    }
    ppcol = dp.as<int>();
    pirow = dr.as<int>();
    pdist = dd.as<double>();
  }
  MDS_CUDA(ctx, cudaEventRecord(ctx->ev[0], s));
  SymOp op;
  MDS_TRY(build_symop(ctx, n, ppcol, pirow, pdist, sigma, op, k_sigma, perplexity));
  if (k_sigma > 0 && sig_out)
    MDS_CUDA(ctx, cudaMemcpyAsync(sig_out, op.sig.p, sizeof(double) * n,
                                  dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, s));
  MDS_CUDA(ctx, cudaEventRecord(ctx->ev[1], s));
  double* pX = evecs;
  if (!dev) {
    MDS_TRY(dX.alloc(ctx, sizeof(double) * (size_t)n * nev));
    pX = dX.as<double>();
  }
  LanczosOut lo;
  MDS_TRY(lanczos_complete(ctx, op, nev, ncv, tol, maxiter, pX, lo));
  MDS_CUDA(ctx, cudaEventRecord(ctx->ev[2], s));
  for (int x = 0; x < nev; ++x) evals[x] = lo.evals[x];
  if (nconv) *nconv = lo.nconv;
  // residuals
  if (resid) {
    DevBuf Az(ctx), part(ctx);
    MDS_TRY(Az.alloc(ctx, sizeof(double) * n));
    MDS_TRY(part.alloc(ctx, sizeof(double) * 256));
    for (int x = 0; x < nev; ++x) {
      spmv(ctx, op, pX + (int64_t)x * n, Az.as<double>());
      ctx->stats.launches++;
      k_resid_part<<<256, 256, 0, s>>>(Az.as<double>(), pX + (int64_t)x * n, lo.evals[x], n, part.as<double>());
      std::vector<double> hpart(256);
      MDS_CUDA(ctx, cudaMemcpyAsync(hpart.data(), part.p, sizeof(double) * 256, cudaMemcpyDeviceToHost, s));
      MDS_CUDA(ctx, cudaStreamSynchronize(s));
      double ss = 0;
      for (double v : hpart) ss += v;
      resid[x] = std::sqrt(ss) / std::fabs(lo.evals[x]);
    }
  }
  // Nystrom extension
  if (m > 0 && ext) {
    if (!pcolB || !irowB || !distB) return mds_fail(ctx, MDS_ERR_ARG, "null Nystrom argument");
    std::vector<int> hpB;
    const int* hpcolB = pcolB;
    if (dev) {
      hpB.resize(m + 1);
      MDS_CUDA(ctx, cudaMemcpyAsync(hpB.data(), pcolB, sizeof(int) * (m + 1), cudaMemcpyDeviceToHost, s));
      MDS_CUDA(ctx, cudaStreamSynchronize(s));
      hpcolB = hpB.data();
    }
    const int64_t nnzB = hpcolB[m];
    DevBuf bp(ctx), br(ctx), bd(ctx), B(ctx), il(ctx), de(ctx), bad(ctx);
    const int* qp = pcolB;
    const int* qr = irowB;
    const double* qd = distB;
    if (!dev) {
      MDS_TRY(bp.alloc(ctx, sizeof(int) * (m + 1)));
      MDS_TRY(br.alloc(ctx, sizeof(int) * std::max<int64_t>(nnzB, 1)));
      MDS_TRY(bd.alloc(ctx, sizeof(double) * std::max<int64_t>(nnzB, 1)));
      MDS_CUDA(ctx, cudaMemcpyAsync(bp.p, pcolB, sizeof(int) * (m + 1), cudaMemcpyHostToDevice, s));
      if (nnzB) {
        MDS_CUDA(ctx, cudaMemcpyAsync(br.p, irowB, sizeof(int) * nnzB, cudaMemcpyHostToDevice, s));
        MDS_CUDA(ctx, cudaMemcpyAsync(bd.p, distB, sizeof(double) * nnzB, cudaMemcpyHostToDevice, s));
      }
      qp = bp.as<int>();
      qr = br.as<int>();
      qd = bd.as<double>();
    }
    MDS_TRY(B.alloc(ctx, sizeof(double) * std::max<int64_t>(nnzB, 1)));
    MDS_TRY(il.alloc(ctx, sizeof(double) * nev));
    MDS_TRY(bad.alloc(ctx, sizeof(int)));
    MDS_CUDA(ctx, cudaMemsetAsync(bad.p, 0, sizeof(int), s));
    std::vector<double> inv(nev);
    for (int x = 0; x < nev; ++x) inv[x] = 1.0 / lo.evals[x];
    MDS_CUDA(ctx, cudaMemcpyAsync(il.p, inv.data(), sizeof(double) * nev, cudaMemcpyHostToDevice, s));
    double* pext = ext;
    if (!dev) {
      MDS_TRY(de.alloc(ctx, sizeof(double) * (size_t)m * nev));
      pext = de.as<double>();
    }
    const int wb = (int)(((int64_t)m * 32 + 255) / 256);
    ctx->stats.launches += 2;
    k_nystrom_b<<<wb, 256, 0, s>>>(qp, qr, qd, m, n, 2.0 * sigma * sigma,
                                   k_sigma > 0 ? op.sig.as<double>() : nullptr, op.dinv.as<double>(),
                                   B.as<double>(), bad.as<int>());
    k_nystrom_ext<<<wb, 256, 0, s>>>(qp, qr, B.as<double>(), m, n, pX, il.as<double>(), nev, pext);
    MDS_CUDA(ctx, cudaGetLastError());
    int hbad = 0;
    MDS_CUDA(ctx, cudaMemcpyAsync(&hbad, bad.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    if (!dev) MDS_CUDA(ctx, cudaMemcpyAsync(ext, pext, sizeof(double) * (size_t)m * nev, cudaMemcpyDeviceToHost, s));
    MDS_CUDA(ctx, cudaStreamSynchronize(s));
    if (hbad) return mds_fail(ctx, MDS_ERR_ARG, "landmark index outside [0, n) in the general sparse matrix");
  }
  if (!dev) MDS_CUDA(ctx, cudaMemcpyAsync(evecs, pX, sizeof(double) * (size_t)n * nev, cudaMemcpyDeviceToHost, s));
  MDS_CUDA(ctx, cudaStreamSynchronize(s));
  float a = 0, b = 0;
  cudaEventElapsedTime(&a, ctx->ev[0], ctx->ev[1]);
  cudaEventElapsedTime(&b, ctx->ev[1], ctx->ev[2]);
  ctx->stats.prep_ms = a;
  ctx->stats.screen_ms = b;  // eigensolve time
  ctx->stats.passes = lo.restarts;
  ctx->stats.pairs = lo.matvecs;
  return MDS_OK;
}

// Device-resident eigensolve for the serving model: the .ssm arrays on the
// device in, eigenvalues (host, descending), eigenvectors Z [nev][n] and the
// landmark inverse-square-root degrees d_a [n] (device) out.
int decomp_resident(mds_ctx* ctx, int n, const int* dpcol, const int* dirow, const double* ddist, double sigma,
                    int nev, int ncv, double tol, int maxiter, std::vector<double>& evals, double* dZ, double* ddinv,
                    int* nconv) {
  if (ncv <= 0) ncv = std::min(10 * nev + 1, n);
  ncv = std::min(ncv, n);
  if (maxiter <= 0) maxiter = 100 * nev;
  if (nev < 1 || nev >= ncv) return mds_fail(ctx, MDS_ERR_ARG, "need 0 < nev < ncv <= n");
  SymOp op;
  MDS_TRY(build_symop(ctx, n, dpcol, dirow, ddist, sigma, op));
  LanczosOut lo;
  MDS_TRY(lanczos_complete(ctx, op, nev, ncv, tol, maxiter, dZ, lo));
  MDS_CUDA(ctx, cudaMemcpyAsync(ddinv, op.dinv.p, sizeof(double) * n, cudaMemcpyDeviceToDevice, ctx->stream));
  MDS_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  evals = lo.evals;
  if (nconv) *nconv = lo.nconv;
  return MDS_OK;
}

extern "C" int mds_decomp_sparse(mds_ctx* ctx, int n, const int32_t* pcol, const int32_t* irow, const double* dist,
                                 double sigma, int nev, int ncv, double tol, int maxiter, unsigned flags,
                                 double* evals, double* evecs, double* resid, int* nconv) {
  return decomp_impl(ctx, n, pcol, irow, dist, sigma, nev, ncv, tol, maxiter, flags, evals, evecs, resid, nconv, 0,
                     nullptr, nullptr, nullptr, nullptr);
}

extern "C" int mds_decomp_sparse_nystrom(mds_ctx* ctx, int n, const int32_t* pcol, const int32_t* irow,
                                         const double* dist, int m, const int32_t* pcolB, const int32_t* irowB,
                                         const double* distB, double sigma, int nev, int ncv, double tol, int maxiter,
                                         unsigned flags, double* evals, double* evecs, double* ext, double* resid,
                                         int* nconv) {
  if (m < 0) return mds_fail(ctx, MDS_ERR_ARG, "m must be >= 0");
  return decomp_impl(ctx, n, pcol, irow, dist, sigma, nev, ncv, tol, maxiter, flags, evals, evecs, resid, nconv, m,
                     pcolB, irowB, distB, ext);
}

extern "C" int mds_auto_decomp_sparse(mds_ctx* ctx, int n, const int32_t* pcol, const int32_t* irow,
                                      const double* dist, int k_sigma, double perplexity, int nev, int ncv, double tol,
                                      int maxiter, unsigned flags, double* evals, double* evecs, double* resid,
                                      int* nconv, double* sigmas) {
  if (!ctx) return MDS_ERR_ARG;
  if (k_sigma < 1) return mds_fail(ctx, MDS_ERR_ARG, "k-sigma must be >= 1");
  return decomp_impl(ctx, n, pcol, irow, dist, 1.0, nev, ncv, tol, maxiter, flags, evals, evecs, resid, nconv, 0,
                     nullptr, nullptr, nullptr, nullptr, k_sigma, perplexity, sigmas);
}

extern "C" int mds_auto_decomp_sparse_nystrom(mds_ctx* ctx, int n, const int32_t* pcol, const int32_t* irow,
                                              const double* dist, int m, const int32_t* pcolB, const int32_t* irowB,
                                              const double* distB, int k_sigma, double perplexity, int nev, int ncv,
                                              double tol, int maxiter, unsigned flags, double* evals, double* evecs,
                                              double* ext, double* resid, int* nconv, double* sigmas) {
  if (!ctx) return MDS_ERR_ARG;
  if (k_sigma < 1) return mds_fail(ctx, MDS_ERR_ARG, "k-sigma must be >= 1");
  if (m < 0) return mds_fail(ctx, MDS_ERR_ARG, "m must be >= 0");
  return decomp_impl(ctx, n, pcol, irow, dist, 1.0, nev, ncv, tol, maxiter, flags, evals, evecs, resid, nconv, m,
                     pcolB, irowB, distB, ext, k_sigma, perplexity, sigmas);
}
