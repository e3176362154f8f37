// mds_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
//
// A CPU restatement, in FP64 where the reference's result depends on it, of
// the MDSCTK 1.2.5 hot path: knn_rms, knn_data, knn_data_sparse,
// contact_profile, make_sysparse, make_gesparse and the affinity / sparse
// mat-vec steps of decomp_sparse(_nystrom).
// Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
// load this library, and only as the checker or the timed CPU baseline.
// The product (libmdsgpu) never links or calls it.
//
// PARITY STATUS: parity unpinned. The reference cannot be compiled here.
// Every tool includes mdsctk.h, which pulls in GROMACS, Boost and Berkeley
// DB headers (mdsctk.h:53-79), and links ARPACK/BLAS. The reference ships no
// tests, golden vectors or expected outputs. The RMSD arithmetic of
// GROMACS do_fit/rmsdev/reset_x (third party, GROMACS 5.0-5.1) is restated
// from its published method: least-squares superposition by the 6x6
// "omega" eigenproblem (Kabsch), and a mass-weighted RMSD. It is
// cross-checked in the tests against an independent FP64 quaternion
// solver, a scipy SVD Kabsch and scipy's Rotation.align_vectors.
//
// Two knn_rms variants live here:
//   orc_knn_rms       FP64 minimum RMSD (the checker);
//   orc_knn_rms_port  the reference's per-pair work as the reference does it
//                     (float covariance, FP64 6x6 Jacobi, float rotation,
//                     float rmsdev), under the reference's OpenMP block loop.
//                     This is the timed CPU baseline.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <numeric>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------------------
// Cyclic Jacobi eigen-decomposition of a small dense symmetric matrix (FP64).
// a: n*n row-major, destroyed. d: eigenvalues. v: eigenvectors as columns
// (v[i*n+j] = component i of eigenvector j).
void jacobi_sym(double* a, int n, double* d, double* v) {
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) v[i * n + j] = (i == j) ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 64; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        tot += a[i * n + j] * a[i * n + j];
        if (i != j) off += a[i * n + j] * a[i * n + j];
      }
    if (off <= 1e-34 * tot || off == 0.0) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        double apq = a[p * n + q];
        if (apq == 0.0) continue;
        double app = a[p * n + p], aqq = a[q * n + q];
        double theta = (aqq - app) / (2.0 * apq);
        double t = (theta >= 0 ? 1.0 : -1.0) /
                   (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {  // rotate columns p,q
          double akp = a[k * n + p], akq = a[k * n + q];
          a[k * n + p] = c * akp - s * akq;
          a[k * n + q] = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {  // rotate rows p,q
          double apk = a[p * n + k], aqk = a[q * n + k];
          a[p * n + k] = c * apk - s * aqk;
          a[q * n + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          double vkp = v[k * n + p], vkq = v[k * n + q];
          v[k * n + p] = c * vkp - s * vkq;
          v[k * n + q] = s * vkp + c * vkq;
        }
      }
  }
  for (int i = 0; i < n; ++i) d[i] = a[i * n + i];
}

// Mass-weighted centring of one frame, in place, as GROMACS reset_x does
// (knn_rms.cpp:189,199): centre accumulated in double, total mass in float,
// coordinates shifted in double and stored back as float.
void center_frame(float* x, int natoms, const float* mass) {
  double xt[3] = {0, 0, 0};
  float tm = 0.0f;
  for (int i = 0; i < natoms; ++i) {
    float mm = mass[i];
    for (int m = 0; m < 3; ++m) xt[m] += (double)(mm * x[3 * i + m]);
    tm += mm;
  }
  for (int m = 0; m < 3; ++m) xt[m] /= (double)tm;
  for (int i = 0; i < natoms; ++i)
    for (int m = 0; m < 3; ++m) x[3 * i + m] = (float)((double)x[3 * i + m] - xt[m]);
}

// FP64 minimum mass-weighted RMSD (nm) over proper rotations between two
// centred frames, by the quaternion key-matrix method (Horn 1987; Theobald
// 2005): RMSD^2 = (Ga + Gb - 2*lambda_max(K)) / M, lambda_max from Jacobi.
double rmsd_fp64(const float* x, const float* y, int natoms, const float* mass,
                 bool fit) {
  double S[9] = {0}, ga = 0, gb = 0, M = 0;
  for (int a = 0; a < natoms; ++a) {
    double w = mass[a];
    double xa[3] = {x[3 * a], x[3 * a + 1], x[3 * a + 2]};
    double ya[3] = {y[3 * a], y[3 * a + 1], y[3 * a + 2]};
    for (int c = 0; c < 3; ++c)
      for (int d = 0; d < 3; ++d) S[3 * c + d] += w * xa[c] * ya[d];
    ga += w * (xa[0] * xa[0] + xa[1] * xa[1] + xa[2] * xa[2]);
    gb += w * (ya[0] * ya[0] + ya[1] * ya[1] + ya[2] * ya[2]);
    M += w;
  }
  double lam;
  if (!fit) {
    lam = S[0] + S[4] + S[8];
  } else {
    const double sxx = S[0], sxy = S[1], sxz = S[2], syx = S[3], syy = S[4],
                 syz = S[5], szx = S[6], szy = S[7], szz = S[8];
    double K[16] = {sxx + syy + szz, syz - szy,        szx - sxz,        sxy - syx,
                    syz - szy,       sxx - syy - szz,  sxy + syx,        szx + sxz,
                    szx - sxz,       sxy + syx,        -sxx + syy - szz, syz + szy,
                    sxy - syx,       szx + sxz,        syz + szy,        -sxx - syy + szz};
    double d[4], v[16];
    jacobi_sym(K, 4, d, v);
    lam = std::max(std::max(d[0], d[1]), std::max(d[2], d[3]));
  }
  double r2 = (ga + gb - 2.0 * lam) / M;
  return r2 > 0 ? std::sqrt(r2) : 0.0;
}

// ---- the reference's per-pair work (port of do_fit + rmsdev) --------------
// Rotation of `fit` onto `ref` from the 6x6 omega eigenproblem: the two
// leading eigenvectors give two singular-vector pairs, the third pair is
// their cross product, which makes the rotation proper.
void fit_onto(int natoms, const float* w, const float* ref, float* fit) {
  float u[3][3] = {{0}};
  for (int n = 0; n < natoms; ++n) {
    float mn = w[n];
    if (mn == 0.0f) continue;
    for (int c = 0; c < 3; ++c) {
      double xpc = ref[3 * n + c];
      for (int r = 0; r < 3; ++r) {
        double xnr = fit[3 * n + r];
        u[c][r] += (float)(mn * xnr * xpc);
      }
    }
  }
  double om[36] = {0}, d[6], V[36];
  for (int r = 3; r < 6; ++r)
    for (int c = 0; c < 3; ++c) {
      om[r * 6 + c] = u[r - 3][c];
      om[c * 6 + r] = u[r - 3][c];
    }
  jacobi_sym(om, 6, d, V);
  int idx[2];
  bool used[6] = {false};
  for (int j = 0; j < 2; ++j) {
    int best = -1;
    for (int i = 0; i < 6; ++i)
      if (!used[i] && (best < 0 || d[i] > d[best])) best = i;
    used[best] = true;
    idx[j] = best;
  }
  double vh[3][3], vk[3][3];
  for (int j = 0; j < 2; ++j)
    for (int i = 0; i < 3; ++i) {
      vh[j][i] = M_SQRT2 * V[i * 6 + idx[j]];
      vk[j][i] = M_SQRT2 * V[(i + 3) * 6 + idx[j]];
    }
  auto cross = [](const double* a, const double* b, double* c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
  };
  cross(vh[0], vh[1], vh[2]);
  cross(vk[0], vk[1], vk[2]);
  float R[3][3];
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 3; ++c) {
      double s = 0;
      for (int k = 0; k < 3; ++k) s += vk[k][r] * vh[k][c];
      R[r][c] = (float)s;
    }
  for (int j = 0; j < natoms; ++j) {
    float x0 = fit[3 * j], x1 = fit[3 * j + 1], x2 = fit[3 * j + 2];
    for (int r = 0; r < 3; ++r)
      fit[3 * j + r] = R[r][0] * x0 + R[r][1] * x1 + R[r][2] * x2;
  }
}

float rmsdev_f(int natoms, const float* w, const float* x, const float* xp) {
  float tm = 0, rs = 0;
  for (int j = 0; j < natoms; ++j) {
    float m = w[j];
    tm += m;
    for (int c = 0; c < 3; ++c) {
      float xd = x[3 * j + c] - xp[3 * j + c];
      rs += m * xd * xd;
    }
  }
  return std::sqrt(rs / tm);
}

// permutation<T>::sort(k) semantics (mdsctk.h:177-199): the k smallest
// values in ascending order. Ties are ordered by index here (the reference's
// std::partial_sort leaves tie order unspecified).
void select_k(const std::vector<double>& data, int k1, std::vector<int>& order) {
  int n = (int)data.size();
  order.resize(n);
  std::iota(order.begin(), order.end(), 0);
  auto cmp = [&](int a, int b) {
    return data[a] < data[b] || (data[a] == data[b] && a < b);
  };
  if (k1 > n) k1 = n;
  std::partial_sort(order.begin(), order.begin() + k1, order.end(), cmp);
}

// Shared driver: the reference's row loop (knn_rms.cpp:213-293 and
// knn_data.cpp:176-250). `dist(i, j)` gives fit row i vs ref j.
template <class F>
int knn_driver(int nref, int nfit, int k, int sort, int nthreads, F dist,
               double* out_d, int* out_i) {
  if (nref <= 0 || nfit < 0) return -1;
  if (nref - 1 < k) k = nref - 1;
  int k1 = k + 1;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel
  {
    std::vector<double> row(nref);
    std::vector<int> order;
#pragma omp for schedule(dynamic, 1)
    for (int i = 0; i < nfit; ++i) {
      for (int j = 0; j < nref; ++j) row[j] = dist(i, j);
      if (sort) {
        select_k(row, k1, order);
        for (int x = 1; x <= k; ++x) {
          out_d[(int64_t)i * k + x - 1] = row[order[x]];
          out_i[(int64_t)i * k + x - 1] = order[x];
        }
      } else {
        for (int j = 0; j < nref; ++j) {
          out_d[(int64_t)i * nref + j] = row[j];
          out_i[(int64_t)i * nref + j] = j;
        }
      }
    }
  }
  return k;
}

}  // namespace

extern "C" {

// reset_x restated for every frame (knn_rms.cpp:186-206).
void orc_center(float* xyz, int nframes, int natoms, const float* mass) {
  for (int f = 0; f < nframes; ++f) center_frame(xyz + (int64_t)f * natoms * 3, natoms, mass);
}

// FP64 minimum RMSD in nm of two already-centred frames.
double orc_rmsd(const float* x, const float* y, int natoms, const float* mass, int nofit) {
  return rmsd_fp64(x, y, natoms, mass, !nofit);
}

// RMSD in nm from the reference's own per-pair procedure (do_fit + rmsdev).
double orc_rmsd_port(const float* ref, const float* fit, int natoms, const float* mass, int nofit) {
  std::vector<float> f(fit, fit + 3 * natoms);
  if (!nofit) fit_onto(natoms, mass, ref, f.data());
  return rmsdev_f(natoms, mass, f.data(), ref);
}

// knn_rms (knn_rms.cpp:38-41,186-293). Inputs are raw (uncentred) float
// frames [n][natoms][3] in nm; they are centred internally like reset_x.
// Output: distances in Angstrom (RMSD x 10), k per row (k+1 found, position
// 0 dropped), or the full N_ref row when sort == 0. Returns the k used.
int orc_knn_rms(const float* ref, int nref, const float* fit, int nfit, int natoms,
                const float* mass, int k, int nofit, int sort, int nthreads,
                double* out_d, int* out_i) {
  std::vector<float> r(ref, ref + (int64_t)nref * natoms * 3);
  std::vector<float> f(fit, fit + (int64_t)nfit * natoms * 3);
  orc_center(r.data(), nref, natoms, mass);
  orc_center(f.data(), nfit, natoms, mass);
  const int64_t st = (int64_t)natoms * 3;
  return knn_driver(nref, nfit, k, sort, nthreads,
                    [&](int i, int j) {
                      return rmsd_fp64(f.data() + i * st, r.data() + j * st, natoms,
                                       mass, !nofit) * 10.0;
                    },
                    out_d, out_i);
}

// The timed CPU baseline: knn_rms.cpp's loop (blocks of `blksize` fit rows,
// OpenMP over rows, serial over refs; each row's fit copy is rotated in place
// onto every ref in turn, knn_rms.cpp:236-240) with the float per-pair fit
// and rmsdev, then the partial sort of k+1 and the position-0 drop.
int orc_knn_rms_port(const float* ref, int nref, const float* fit, int nfit, int natoms,
                     const float* mass, int k, int nofit, int blksize, int nthreads,
                     double* out_d, int* out_i) {
  std::vector<float> r(ref, ref + (int64_t)nref * natoms * 3);
  std::vector<float> f(fit, fit + (int64_t)nfit * natoms * 3);
  orc_center(r.data(), nref, natoms, mass);
  orc_center(f.data(), nfit, natoms, mass);
  if (nref - 1 < k) k = nref - 1;
  int k1 = k + 1;
  if (blksize > nfit) blksize = nfit;
  if (blksize < 1) blksize = 1;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
  const int64_t st = (int64_t)natoms * 3;
  int remainder = nfit % blksize;
  auto do_rows = [&](int first, int count) {
#pragma omp parallel for schedule(static)
    for (int fr = 0; fr < count; ++fr) {
      int i = first + fr;
      std::vector<float> fitc(f.data() + i * st, f.data() + (i + 1) * st);
      std::vector<float> refc(st);
      std::vector<double> row(nref);
      std::vector<int> order;
      for (int j = 0; j < nref; ++j) {
        std::memcpy(refc.data(), r.data() + j * st, sizeof(float) * st);
        if (!nofit) fit_onto(natoms, mass, refc.data(), fitc.data());
        row[j] = (double)rmsdev_f(natoms, mass, fitc.data(), refc.data()) * 10.0;
      }
      select_k(row, k1, order);
      for (int x = 1; x <= k; ++x) {
        out_d[(int64_t)i * k + x - 1] = row[order[x]];
        out_i[(int64_t)i * k + x - 1] = order[x];
      }
    }
  };
  do_rows(0, remainder);
  for (int b = remainder; b < nfit; b += blksize) do_rows(b, blksize);
  return k;
}

// knn_data (knn_data.cpp:141-250) with euclidean_distance
// (mdsctk.cpp:330-335) or correlation_distance (mdsctk.cpp:337-360), both
// restated operation for operation so the FP64 results are bit-identical.
int orc_knn_data(const double* ref, int nref, const double* fit, int nfit, int dim, int k,
                 int correlation, int sort, int nthreads, double* out_d, int* out_i) {
  auto eu = [&](int i, int j) {
    const double* a = fit + (int64_t)i * dim;  // knn_data passes (fit, ref)
    const double* b = ref + (int64_t)j * dim;
    double value = 0.0;
    for (int x = 0; x < dim; ++x) value += (a[x] - b[x]) * (a[x] - b[x]);
    return std::sqrt(value);
  };
  auto co = [&](int i, int j) {
    const double* reference = fit + (int64_t)i * dim;
    const double* fitting = ref + (int64_t)j * dim;
    double rvalue = 0.0, rsvalue = 0.0, fvalue = 0.0, fsvalue = 0.0;
    double dsize = (double)dim, value = 0.0;
    for (int x = 0; x < dim; ++x) {
      rvalue += reference[x];
      rsvalue += reference[x] * reference[x];
      fvalue += fitting[x];
      fsvalue += fitting[x] * fitting[x];
    }
    rsvalue = std::sqrt(((dsize * rsvalue) - (rvalue * rvalue)) / (dsize * (dsize - 1.0)));
    rvalue /= dsize;
    fsvalue = std::sqrt(((dsize * fsvalue) - (fvalue * fvalue)) / (dsize * (dsize - 1.0)));
    fvalue /= dsize;
    for (int x = 0; x < dim; ++x) value += (reference[x] - rvalue) * (fitting[x] - fvalue);
    value = (1.0 - (value / ((dsize - 1.0) * rsvalue * fsvalue))) / 2.0;
    if (value < 0.0) value = 0.0;
    return std::sqrt(value);
  };
  if (correlation) return knn_driver(nref, nfit, k, sort, nthreads, co, out_d, out_i);
  return knn_driver(nref, nfit, k, sort, nthreads, eu, out_d, out_i);
}

// knn_data_sparse (knn_data_sparse.cpp:141-260): k nearest sparse vectors by
// euclidean_distance_sparse (mdsctk.cpp:362-386), restated operation for
// operation: the merge walk over the reference vector's entries, fit-only
// entries before each reference entry, squares and differences in FP64 added
// in walk order. Vectors are CSR rows (off[n+1] int64, idx int32, val f64);
// the distance is called as distance(ref row, fit row).
int orc_knn_data_sparse(const int64_t* ref_off, const int* ref_idx, const double* ref_val, int nref,
                        const int64_t* fit_off, const int* fit_idx, const double* fit_val, int nfit, int k,
                        int sort, int nthreads, double* out_d, int* out_i) {
  auto sp = [&](int i, int j) {
    const int ref_size = (int)(ref_off[j + 1] - ref_off[j]), fit_size = (int)(fit_off[i + 1] - fit_off[i]);
    const int* ri = ref_idx + ref_off[j];
    const double* rd = ref_val + ref_off[j];
    const int* fi = fit_idx + fit_off[i];
    const double* fd = fit_val + fit_off[i];
    double value = 0.0;
    int f = 0;
    for (int r = 0; r < ref_size; r++) {
      while (f < fit_size && fi[f] < ri[r]) {
        value += fd[f] * fd[f];
        f++;
      }
      if (f < fit_size && ri[r] == fi[f]) {
        value += (rd[r] - fd[f]) * (rd[r] - fd[f]);
        f++;
      } else {
        value += rd[r] * rd[r];
      }
    }
    for (; f < fit_size; f++) value += fd[f] * fd[f];
    return std::sqrt(value);
  };
  return knn_driver(nref, nfit, k, sort, nthreads, sp, out_d, out_i);
}

// contact_profile (contact_profile.cpp:200-262): for every frame, atom pairs
// (g1[i], g2[j]) closer than eps Angstrom, as sparse binary vectors over the
// grid index i * n2 + j. Distance as the reference forms it: float
// differences and squares, summed into a double, sqrt, times 10. Coordinates
// [nframes][natoms][3] in nm. offsets[nframes+1] (int64) and, when idx is not
// null, the ascending grid indices of every frame's contacts.
void orc_contact_profile(const float* xyz, int nframes, int natoms, const int* g1, int n1, const int* g2, int n2,
                         double eps, int64_t* offsets, int* idx) {
  int64_t pos = 0;
  for (int f = 0; f < nframes; ++f) {
    offsets[f] = pos;
    const float* x = xyz + (int64_t)f * natoms * 3;
    for (int i = 0; i < n1; ++i)
      for (int j = 0; j < n2; ++j) {
        const float* a = x + 3 * (int64_t)g1[i];
        const float* b = x + 3 * (int64_t)g2[j];
        double d = 0.0;
        for (int c = 0; c < 3; ++c) {
          const float t = a[c] - b[c];
          const float t2 = t * t;
          d += (double)t2;
        }
        d = std::sqrt(d) * 10.0;
        if (d < eps) {
          if (idx) idx[pos] = i * n2 + j;
          ++pos;
        }
      }
  }
  offsets[nframes] = pos;
}

// make_sysparse (make_sysparse.cpp:225-329; compare_edge mdsctk.cpp:567-577;
// split_edges mdsctk.cpp:580-604). Rows of the kNN files are read in order;
// the first k of maxk entries give undirected keys (min,max) whose value is
// the distance; a later put overwrites. The cursor walk emits column c =
// keys with from == c; it stops at the first key whose `from` is not the
// current column, so a negative `from` blocks every column.
// Returns nnz, fills pcol[nrows+1], irow[nnz], val[nnz] (capacity nrows*k).
int64_t orc_sysparse(const double* dist, const int* idx, int nrows, int maxk, int k,
                     int* pcol, int* irow, double* val) {
  struct E { int from, to; int64_t seq; double d; };
  std::vector<E> e;
  e.reserve((size_t)nrows * k);
  for (int r = 0; r < nrows; ++r)
    for (int x = 0; x < k; ++x) {
      int j = idx[(int64_t)r * maxk + x];
      double d = dist[(int64_t)r * maxk + x];
      int64_t seq = (int64_t)r * maxk + x;
      if (r < j) e.push_back({r, j, seq, d});
      if (j < r) e.push_back({j, r, seq, d});
    }
  std::stable_sort(e.begin(), e.end(), [](const E& a, const E& b) {
    return a.from < b.from || (a.from == b.from && a.to < b.to);
  });
  std::vector<E> u;
  for (size_t p = 0; p < e.size(); ++p)
    if (p + 1 == e.size() || e[p + 1].from != e[p].from || e[p + 1].to != e[p].to)
      u.push_back(e[p]);  // last writer of each key
  size_t cur = 0;
  int64_t nnz = 0;
  for (int c = 0; c < nrows; ++c) {
    pcol[c] = (int)nnz;
    while (cur < u.size() && u[cur].from == c) {
      irow[nnz] = u[cur].to;
      val[nnz] = u[cur].d;
      ++nnz;
      ++cur;
    }
  }
  pcol[nrows] = (int)nnz;
  return nnz;
}

// make_gesparse (make_gesparse.cpp:246-335): key (query row, landmark) with
// put-overwrite; with `symmetric`, the transposed key is added only when it
// is absent at that moment (db.get == DB_NOTFOUND). Columns 0..nrows-1.
int64_t orc_gesparse(const double* dist, const int* idx, int nrows, int maxk, int k,
                     int symmetric, int* pcol, int* irow, double* val) {
  struct KeyCmp {
    bool operator()(const std::pair<int, int>& a, const std::pair<int, int>& b) const {
      return a.first < b.first || (a.first == b.first && a.second < b.second);
    }
  };
  // Ordered map emulated by a sorted vector (the B-tree of the reference).
  std::vector<std::pair<int, int>> mk;
  std::vector<double> mv;
  auto find = [&](std::pair<int, int> key) -> int64_t {
    auto it = std::lower_bound(mk.begin(), mk.end(), key, KeyCmp());
    if (it != mk.end() && *it == key) return it - mk.begin();
    return -1;
  };
  auto put = [&](std::pair<int, int> key, double d) {
    auto it = std::lower_bound(mk.begin(), mk.end(), key, KeyCmp());
    int64_t p = it - mk.begin();
    if (it != mk.end() && *it == key) {
      mv[p] = d;
    } else {
      mk.insert(it, key);
      mv.insert(mv.begin() + p, d);
    }
  };
  for (int r = 0; r < nrows; ++r)
    for (int x = 0; x < k; ++x) {
      int j = idx[(int64_t)r * maxk + x];
      double d = dist[(int64_t)r * maxk + x];
      put({r, j}, d);
      if (symmetric && find({j, r}) < 0) put({j, r}, d);
    }
  size_t cur = 0;
  int64_t nnz = 0;
  for (int c = 0; c < nrows; ++c) {
    pcol[c] = (int)nnz;
    while (cur < mk.size() && mk[cur].first == c) {
      irow[nnz] = mk[cur].second;
      val[nnz] = mv[cur];
      ++nnz;
      ++cur;
    }
  }
  pcol[nrows] = (int)nnz;
  return nnz;
}

// decomp_sparse affinity (decomp_sparse.cpp:158-178): val <- exp(-d^2/2s^2),
// degrees over both triangles, then val *= d_r^-1/2 d_c^-1/2. d_out (n) gets
// the inverse square-root degrees.
void orc_affinity(int n, const int* pcol, const int* irow, double* val, double sigma,
                  double* d_out) {
  int nnz = pcol[n];
  for (int x = 0; x < nnz; ++x) val[x] = std::exp(-(val[x] * val[x]) / (2.0 * sigma * sigma));
  std::vector<double> d(n, 0.0);
  for (int x = 0; x < n; ++x)
    for (int y = pcol[x]; y < pcol[x + 1]; ++y) {
      d[x] += val[y];
      d[irow[y]] += val[y];
    }
  for (int x = 0; x < n; ++x) d[x] = 1.0 / std::sqrt(d[x]);
  for (int x = 0; x < n; ++x)
    for (int y = pcol[x]; y < pcol[x + 1]; ++y) val[y] *= d[irow[y]] * d[x];
  if (d_out)
    for (int x = 0; x < n; ++x) d_out[x] = d[x];
}

// decomp_sparse_nystrom B normalisation (decomp_sparse_nystrom.cpp:181-219):
// valB <- exp(-d^2/2s^2); d_b[q] = (sum of column q)^-1/2; B[l,q] *= d_a[l] d_b[q].
void orc_affinity_nystrom(int m, const int* pcolB, const int* irowB, double* valB,
                          double sigma, const double* d_a) {
  int nnz = pcolB[m];
  for (int x = 0; x < nnz; ++x) valB[x] = std::exp(-(valB[x] * valB[x]) / (2.0 * sigma * sigma));
  std::vector<double> db(m, 0.0);
  for (int x = 0; x < m; ++x)
    for (int y = pcolB[x]; y < pcolB[x + 1]; ++y) db[x] += valB[y];
  for (int x = 0; x < m; ++x) db[x] = 1.0 / std::sqrt(db[x]);
  for (int x = 0; x < m; ++x)
    for (int y = pcolB[x]; y < pcolB[x + 1]; ++y) valB[y] *= d_a[irowB[y]] * db[x];
}

// ---------------------------------------------------------------------------
// auto_decomp_sparse per-landmark sigmas (auto_decomp_sparse.cpp:153-178,
// auto_decomp_sparse_nystrom.cpp:144-163, mdsctk.cpp:388-565).
// ---------------------------------------------------------------------------
// Entropic-affinity root finding for one landmark (mdsctk.cpp:388-486): find
// the log-precision b with entropy of exp(-d^2 e^b) (normalised) = log K, by
// Newton steps inside a shrinking bracket [lo, hi], bisecting on trouble;
// sigma = 1/sqrt(2 e^b). `d` holds the k smallest distances ascending.
static double entropic_sigma(const double* d, int k, double b0, double logK, double logN, double lo, double hi) {
  const int maxit = 20;
  const double tol = 1e-10, realmin = 2.225074e-308;
  const double sq_eps = std::ldexp(1.0, -26);  // sqrt of the machine epsilon loop's 2^-52
  double b = (b0 < lo || b0 > hi) ? (lo + hi) / 2.0 : b0;
  std::vector<double> p(k), q(k);
  int it = 1;
  for (;;) {
    const double eb = std::exp(b);
    bool trouble = false;
    double z = 0.0, e, mean = 0.0;
    for (int x = 0; x < k; ++x) p[x] = std::exp(-(d[x] * d[x]) * eb);
    for (int x = 0; x < k; ++x) z += p[x];
    if (z < realmin) {
      e = -logK;
      trouble = true;
    } else {
      for (int x = 0; x < k; ++x) q[x] = p[x] * ((d[x] * d[x]) / z);
      for (int x = 0; x < k; ++x) mean += q[x];
      e = eb * mean + std::log(z) - logK;
    }
    if (std::fabs(e) < tol) break;
    if (hi - lo < 10.0 * sq_eps) break;
    if (e < 0.0 && b <= hi) hi = b;
    else if (e > 0.0 && b >= lo) lo = b;
    trouble = trouble || e < -logK || e > logN - logK;
    double g = 0.0;
    if (!trouble) {
      if (it == maxit) {
        b = (lo + hi) / 2.0;
        it = 1;
        continue;
      }
      double m2 = 0.0;
      for (int x = 0; x < k; ++x) m2 += q[x] * (d[x] * d[x]);
      g = (eb * eb) * ((mean * mean) - m2);
      if (g == 0) trouble = true;
    }
    if (trouble) {
      double t = 0.0;
      for (int x = 0; x < k; ++x)
        t += std::exp(-(d[x] * d[x]) * std::exp(lo)) + std::exp(-(d[x] * d[x]) * std::exp(hi));
      if (t < 2.0 * std::sqrt(realmin)) break;
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
  return 1.0 / std::sqrt(2.0 * std::exp(b));
}

// Per-landmark sigmas. List of landmark x = its stored distances in
// neighbour-index order (entries of the columns before x that name x, then
// column x's own entries; a diagonal entry twice), cut to the first ka
// entries BEFORE sorting, then sorted ascending; sigma = sum / ka.
// With use_perplexity, sigmas are replaced by the entropic ones
// (mdsctk.cpp:488-565), solved landmark by landmark in ascending order of the
// ceil(K)-th list entry, each warm-started from the previous solution.
// Returns -1 if the entropic step would read past a list (fewer than ka
// entries, or ceil(K) > ka), which the reference leaves undefined.
int orc_auto_sigmas(int n, const int* pcol, const int* irow, const double* val, int ka, double K,
                    int use_perplexity, double* sig) {
  std::vector<std::vector<double>> L(n);
  for (int x = 0; x < n; ++x)
    for (int y = pcol[x]; y < pcol[x + 1]; ++y) {
      L[x].push_back(val[y]);
      L[irow[y]].push_back(val[y]);
    }
  for (int x = 0; x < n; ++x) {
    if ((int)L[x].size() > ka) L[x].resize(ka);
    std::sort(L[x].begin(), L[x].end());
    double s = 0.0;
    for (double v : L[x]) s += v;
    sig[x] = s / (double)ka;
  }
  if (!use_perplexity) return 0;
  const int Ki = (int)std::ceil(K);
  if (ka < 2 || Ki < 1 || Ki > ka) return -1;
  for (int x = 0; x < n; ++x)
    if ((int)L[x].size() < ka) return -1;
  const double N = (double)ka, logK = std::log(K), logN = std::log(N), logNK = logN - logK;
  double p1;
  if (logK > std::log(std::sqrt(2.0 * N))) {
    p1 = 3.0 / 4.0;
  } else {
    p1 = 1.0 / 4.0;
    for (int it = 0; it < 100; ++it) p1 -= (-p1 * std::log(p1 / N) - logK) / (-std::log(p1 / N) + 1.0);
    p1 = 1.0 - (p1 / 2.0);
  }
  std::vector<double> lo(n), hi(n), kth(n);
  for (int x = 0; x < n; ++x) {
    const double* a = L[x].data();
    hi[x] = std::log((2.0 * std::log(p1 * (N - 1.0) / (1.0 - p1))) / ((a[1] * a[1]) - (a[0] * a[0])));
    double l1 = std::log((2.0 * logNK / (1.0 - (1.0 / N))) / ((a[ka - 1] * a[ka - 1]) - (a[0] * a[0])));
    double l2 = std::log((2.0 * std::sqrt(logNK)) /
                         std::sqrt(((a[ka - 1] * a[ka - 1]) * (a[ka - 1] * a[ka - 1])) -
                                   ((a[0] * a[0]) * (a[0] * a[0]))));
    lo[x] = (l1 > l2) ? l1 : l2;
    kth[x] = a[Ki - 1];
  }
  // processing order: indices sorted by kth with std::sort (as permutation::sort)
  std::vector<int> order(n);
  for (int x = 0; x < n; ++x) order[x] = x;
  std::sort(order.begin(), order.end(), [&](int a, int b) { return kth[a] < kth[b]; });
  double b0 = (lo[order[0]] + hi[order[0]]) / 2.0;
  for (int j : order) {
    sig[j] = entropic_sigma(L[j].data(), ka, b0, logK, logN, lo[j], hi[j]);
    b0 = std::log((1.0 / sig[j]) * (1.0 / sig[j]) / 2.0);
  }
  return 0;
}

// auto_decomp_sparse affinity (auto_decomp_sparse.cpp:180-203): as
// orc_affinity with w = exp(-d^2 / (2 s_col s_row)).
void orc_affinity_auto(int n, const int* pcol, const int* irow, double* val, const double* sig, double* d_out) {
  for (int x = 0; x < n; ++x)
    for (int y = pcol[x]; y < pcol[x + 1]; ++y)
      val[y] = std::exp(-(val[y] * val[y]) / (2.0 * sig[x] * sig[irow[y]]));
  std::vector<double> d(n, 0.0);
  for (int x = 0; x < n; ++x)
    for (int y = pcol[x]; y < pcol[x + 1]; ++y) {
      d[x] += val[y];
      d[irow[y]] += val[y];
    }
  for (int x = 0; x < n; ++x) d[x] = 1.0 / std::sqrt(d[x]);
  for (int x = 0; x < n; ++x)
    for (int y = pcol[x]; y < pcol[x + 1]; ++y) val[y] *= d[irow[y]] * d[x];
  if (d_out)
    for (int x = 0; x < n; ++x) d_out[x] = d[x];
}

// auto_decomp_sparse_nystrom B (auto_decomp_sparse_nystrom.cpp:171-209):
// w = exp(-d^2 / (2 s_l s_l)) with the landmark's sigma, then as
// orc_affinity_nystrom.
void orc_affinity_nystrom_auto(int m, const int* pcolB, const int* irowB, double* valB, const double* sig,
                               const double* d_a) {
  for (int x = 0; x < m; ++x)
    for (int y = pcolB[x]; y < pcolB[x + 1]; ++y)
      valB[y] = std::exp(-(valB[y] * valB[y]) / (2.0 * sig[irowB[y]] * sig[irowB[y]]));
  std::vector<double> db(m, 0.0);
  for (int x = 0; x < m; ++x)
    for (int y = pcolB[x]; y < pcolB[x + 1]; ++y) db[x] += valB[y];
  for (int x = 0; x < m; ++x) db[x] = 1.0 / std::sqrt(db[x]);
  for (int x = 0; x < m; ++x)
    for (int y = pcolB[x]; y < pcolB[x + 1]; ++y) valB[y] *= d_a[irowB[y]] * db[x];
}

// sp_dsymv (mdsctk.cpp:293-313): y = A x, A symmetric stored as one triangle
// per column, a diagonal entry counted once only when it is the column's
// first stored entry.
void orc_sp_dsymv(int n, const int* irow, const int* pcol, const double* A, const double* v,
                  double* w) {
  for (int i = 0; i < n; ++i) w[i] = 0.0;
  for (int i = 0; i < n; ++i) {
    double t = v[i];
    int k = pcol[i];
    if ((k != pcol[i + 1]) && (irow[k] == i)) {
      w[i] += t * A[k];
      k++;
    }
    for (int j = k; j < pcol[i + 1]; ++j) {
      w[irow[j]] += t * A[j];
      w[i] += v[irow[j]] * A[j];
    }
  }
}

// sp_dgemv (mdsctk.cpp:315-328): w[i] = sum over column i of A[j] v[irow[j]]
// (that is, w = B^T v for the general CSC B with n columns).
void orc_sp_dgemv(int n, const int* irow, const int* pcol, const double* A, const double* v,
                  double* w) {
  for (int i = 0; i < n; ++i) {
    w[i] = 0.0;
    for (int j = pcol[i]; j < pcol[i + 1]; ++j) w[i] += v[irow[j]] * A[j];
  }
}

// ---------------------------------------------------------------------------
// .xtc decoding (GROMACS compressed coordinates; read through GROMACS by the
// reference, mdsctk.cpp:217-267). Restated from the published format with a
// plain bit-position reader and 128-bit mixed-radix arithmetic. Returns the
// number of frames decoded into xyz [frame][atom][3] (at most max_frames), or
// -1 on a malformed frame. *natoms receives the atom count.
// ---------------------------------------------------------------------------
static const int kXtcMagic[73] = {
    0, 0, 0, 0, 0, 0, 0, 0, 0, 8, 10, 12, 16, 20, 25, 32, 40, 50, 64, 80, 101, 128, 161, 203, 256, 322, 406,
    512, 645, 812, 1024, 1290, 1625, 2048, 2580, 3250, 4096, 5060, 6501, 8192, 10321, 13003, 16384, 20642,
    26007, 32768, 41285, 52015, 65536, 82570, 104031, 131072, 165140, 208063, 262144, 330280, 416127, 524287,
    660561, 832255, 1048576, 1321122, 1664510, 2097152, 2642245, 3329021, 4194304, 5284491, 6658042, 8388607,
    10568983, 13316085, 16777216};

static uint32_t xdr_u32(const unsigned char* p) {
  return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3];
}
static float xdr_f32(const unsigned char* p) {
  uint32_t u = xdr_u32(p);
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}

struct BitPos {
  const unsigned char* d;
  uint64_t nbits, at = 0;
  bool bad = false;
  uint64_t take(int n) {  // n <= 64 bits, most significant first
    uint64_t v = 0;
    for (int i = 0; i < n; ++i) {
      if (at >= nbits) {
        bad = true;
        return 0;
      }
      v = (v << 1) | ((d[at >> 3] >> (7 - (at & 7))) & 1u);
      ++at;
    }
    return v;
  }
  // nbits-bit number sent as little-endian 8-bit groups (the last one short)
  unsigned __int128 packed(int n) {
    unsigned __int128 v = 0;
    int shift = 0;
    while (n > 8) {
      v |= (unsigned __int128)take(8) << shift;
      shift += 8;
      n -= 8;
    }
    if (n > 0) v |= (unsigned __int128)take(n) << shift;
    return v;
  }
};

static int bits_needed(uint64_t size) {  // smallest b with 2^b > size
  int b = 0;
  while (b < 32 && (1ull << b) <= size) ++b;
  return b;
}

int orc_xtc_decode(const unsigned char* buf, size_t len, int max_frames, int* natoms_out, float* xyz, int* steps,
                   float* times) {
  size_t o = 0;
  int nf = 0, na = -1;
  while (o + 56 <= len && nf < max_frames) {
    const unsigned char* h = buf + o;
    if (xdr_u32(h) != 1995) return -1;
    int a = (int)xdr_u32(h + 4);
    if (na >= 0 && a != na) return -1;
    na = a;
    if (steps) steps[nf] = (int)xdr_u32(h + 8);
    if (times) times[nf] = xdr_f32(h + 12);
    float* out = xyz ? xyz + (size_t)nf * a * 3 : nullptr;
    if (a <= 9) {
      if (o + 56 + 12 * (size_t)a > len) break;
      if (out)
        for (int i = 0; i < 3 * a; ++i) out[i] = xdr_f32(h + 56 + 4 * i);
      o += 56 + 12 * (size_t)a;
      ++nf;
      continue;
    }
    if (o + 92 > len) break;
    float prec = xdr_f32(h + 56);
    long long mn[3], mx[3];
    for (int c = 0; c < 3; ++c) {
      mn[c] = (int)xdr_u32(h + 60 + 4 * c);
      mx[c] = (int)xdr_u32(h + 72 + 4 * c);
    }
    int sidx = (int)xdr_u32(h + 84);
    if (sidx < 9 || sidx > 72) return -1;
    size_t nbytes = xdr_u32(h + 88);
    if (o + 92 + nbytes > len) break;
    uint64_t sz[3];
    bool large = false;
    for (int c = 0; c < 3; ++c) {
      sz[c] = (uint64_t)(mx[c] - mn[c] + 1);
      if (sz[c] > 0xffffff) large = true;
    }
    // bits of sz0*sz1*sz2 (exact)
    unsigned __int128 prod = (unsigned __int128)sz[0] * sz[1] * sz[2];
    int pbits = 0;  // bit length of the product itself (not of product - 1)
    while (pbits < 128 && (prod >> pbits) != 0) ++pbits;
    BitPos br{h + 92, (uint64_t)nbytes * 8};
    const float inv = (float)(1.0 / (double)prec);
    int smaller = kXtcMagic[std::max(9, sidx - 1)] / 2, smallnum = kXtcMagic[sidx] / 2;
    long long prev[3] = {0, 0, 0};
    int run = 0, i = 0, w = 0;
    auto emit = [&](const long long* v) {
      if (out)
        for (int c = 0; c < 3; ++c) out[3 * w + c] = (float)(int)v[c] * inv;
      ++w;
    };
    while (i < a) {
      long long cur[3];
      if (large) {
        for (int c = 0; c < 3; ++c) cur[c] = (long long)(uint32_t)br.take(bits_needed(sz[c]));
      } else {
        unsigned __int128 v = br.packed(pbits);
        cur[2] = (long long)(v % sz[2]);
        v /= sz[2];
        cur[1] = (long long)(v % sz[1]);
        v /= sz[1];
        cur[0] = (long long)(int32_t)(uint32_t)v;
      }
      ++i;
      for (int c = 0; c < 3; ++c) {
        cur[c] = (long long)(int32_t)(uint32_t)(cur[c] + mn[c]);
        prev[c] = cur[c];
      }
      int dsmall = 0;
      if (br.take(1)) {
        int r = (int)br.take(5);
        dsmall = r % 3 - 1;
        run = r - r % 3;
      }
      if (run > 0) {
        if (i + run / 3 > a) return -1;
        const uint64_t m = (uint64_t)kXtcMagic[sidx];
        for (int k = 0; k < run; k += 3) {
          unsigned __int128 v = br.packed(sidx);
          long long t[3];
          t[2] = (long long)(v % m);
          v /= m;
          t[1] = (long long)(v % m);
          v /= m;
          t[0] = (long long)(int32_t)(uint32_t)v;
          ++i;
          for (int c = 0; c < 3; ++c) t[c] += prev[c] - smallnum;
          if (k == 0) {
            emit(t);      // the first atom of a run comes before the large one
            emit(prev);
            for (int c = 0; c < 3; ++c) prev[c] = t[c];
          } else {
            for (int c = 0; c < 3; ++c) prev[c] = t[c];
            emit(t);
          }
        }
      } else {
        emit(cur);
      }
      if (br.bad) return -1;
      sidx += dsmall;
      if (sidx < 9 || sidx > 72) return -1;
      if (dsmall < 0) {
        smallnum = smaller;
        smaller = sidx > 9 ? kXtcMagic[sidx - 1] / 2 : 0;
      } else if (dsmall > 0) {
        smaller = smallnum;
        smallnum = kXtcMagic[sidx] / 2;
      }
    }
    o += 92 + ((nbytes + 3) / 4) * 4;
    ++nf;
  }
  if (natoms_out) *natoms_out = na < 0 ? 0 : na;
  return nf;
}

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
