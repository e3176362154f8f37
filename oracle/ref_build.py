"""Builds oracle/_ref/libmds_ref.so from the reference's own source text --
TEST INFRASTRUCTURE ONLY (it pins the oracle; nothing in the product uses it).

The reference tools cannot be compiled whole here: every one includes
mdsctk.h, which needs GROMACS, Boost and Berkeley DB (mdsctk.h:53-79). Its
hot-path arithmetic, though, is in self-contained functions, which this
recipe takes verbatim from the checkout at build time (nothing of them is
stored in the repository) and compiles with g++ -ffp-contract=off, as the
reference's x86-64 build evaluates a*b+c:

  mdsctk.cpp   sp_dsymv, sp_dgemv, euclidean_distance, correlation_distance,
               euclidean_distance_sparse, entropic_affinity_sigma,
               entropic_affinity_sigmas
  mdsctk.h     the SQR and AVG macros and template struct permutation (the
               k+1 selection of every kNN tool)
  decomp_sparse.cpp  the affinity / degree / normalisation block of main()
               (from "// Make affinity matrix" to "delete [] d_a"), wrapped
               in a function whose parameters carry main()'s variable names

Each piece is located by its signature or marker, not by line number, and
the build fails if one is missing. The extern "C" wrappers below are this
repository's own code: the kNN drivers restate knn_data.cpp:195-250 and
knn_data_sparse.cpp:204-250 around the reference's distance functions and
permutation::sort(k1) (the distance pointer called with the fit row first,
as ::distance(vector_size, fit, ref) there).

Usage: python oracle/ref_build.py [REFERENCE_CHECKOUT]  (default
$MDS_REFERENCE, else /root/reference). Output: oracle/_ref/ only.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT, "libmds_ref.so")

FUNCTIONS = [
    "void sp_dsymv(",
    "void sp_dgemv(",
    "double euclidean_distance(",
    "double correlation_distance(",
    "double euclidean_distance_sparse(",
    "double entropic_affinity_sigma(",
    "void entropic_affinity_sigmas(",
]


def reference_dir(arg: str | None = None) -> str:
    return arg or os.environ.get("MDS_REFERENCE", "/root/reference")


def _block_from(lines, start):
    """Lines from `start` through the line closing the first brace opened."""
    depth, opened = 0, False
    for j in range(start, len(lines)):
        depth += lines[j].count("{") - lines[j].count("}")
        opened = opened or "{" in lines[j]
        if opened and depth == 0:
            return lines[start:j + 1]
    raise RuntimeError(f"unbalanced braces after line {start + 1}")


def _function(lines, sig):
    for i, ln in enumerate(lines):
        if ln.startswith(sig):
            return _block_from(lines, i)
    raise RuntimeError(f"reference function not found: {sig}")


def _between(lines, first_marker, stop_marker):
    i0 = next(i for i, ln in enumerate(lines) if first_marker in ln)
    i1 = next(i for i in range(i0, len(lines)) if stop_marker in lines[i])
    return lines[i0:i1]


WRAPPERS = r'''
// ---- this repository's wrappers (not reference code) ----------------------
extern "C" {

double ref_euclidean_distance(int size, double* reference, double* fitting) {
  return euclidean_distance(size, reference, fitting);
}
double ref_correlation_distance(int size, double* reference, double* fitting) {
  return correlation_distance(size, reference, fitting);
}
double ref_euclidean_distance_sparse(int rs, int* ri, double* rd, int fs, int* fi, double* fd) {
  return euclidean_distance_sparse(rs, ri, rd, fs, fi, fd);
}
void ref_sp_dsymv(int n, int* irow, int* pcol, double* A, double* v, double* w) { sp_dsymv(n, irow, pcol, A, v, w); }
void ref_sp_dgemv(int n, int* irow, int* pcol, double* A, double* v, double* w) { sp_dgemv(n, irow, pcol, A, v, w); }

// decomp_sparse.cpp's affinity block on (n, pcol, irow, A); A is overwritten
// with the normalised affinities, d_out receives D_A^(-1/2).
void ref_affinity(int n, int* pcol, int* irow, double* A, double sigma_a, double* d_out) {
  int nnz = pcol[n];
  double *d_a = new double[n];
@AFFINITY@
  for (int x = 0; x < n; x++) d_out[x] = d_a[x];
  delete [] d_a;
}

// entropic_affinity_sigmas on n lists of k sorted distances (row-major).
void ref_entropic_sigmas(int n, int k, double K, const double* lists, double* s) {
  std::vector<double>* A = new std::vector<double>[n];
  for (int x = 0; x < n; x++) A[x].assign(lists + (size_t)x * k, lists + (size_t)(x + 1) * k);
  entropic_affinity_sigmas(n, k, K, A, s);
  delete [] A;
}

// knn_data's row loop: distances of fit row `frame` to every reference row,
// permutation::sort(k + 1), entries [1..k] written (sort != 0), or the full
// row in reference order (sort == 0).
void ref_knn_data(double* ref, int nref, double* fit, int nfit, int dim, int k, int corr, int sort,
                  double* out_d, int* out_i) {
  double (*dist)(int, double*, double*) = corr ? correlation_distance : euclidean_distance;
  if (nref - 1 < k) k = nref - 1;
  int k1 = k + 1;
  for (int frame = 0; frame < nfit; frame++) {
    permutation<double> p;
    p.data.resize(nref);
    for (int r = 0; r < nref; r++) p.data[r] = dist(dim, fit + (size_t)frame * dim, ref + (size_t)r * dim);
    if (sort) {
      p.sort(k1);
      for (int x = 0; x < k; x++) {
        out_d[(size_t)frame * k + x] = p.data[x + 1];
        out_i[(size_t)frame * k + x] = p.indices[x + 1];
      }
    } else {
      for (int x = 0; x < nref; x++) out_d[(size_t)frame * nref + x] = p.data[x];
    }
  }
}

// knn_data_sparse's row loop over CSR vectors (ref_off / fit_off: n + 1
// offsets), the distance called as ::distance(ref..., fit...).
void ref_knn_data_sparse(const long long* ref_off, int* ref_idx, double* ref_val, int nref, const long long* fit_off,
                         int* fit_idx, double* fit_val, int nfit, int k, double* out_d, int* out_i) {
  if (nref - 1 < k) k = nref - 1;
  int k1 = k + 1;
  for (int frame = 0; frame < nfit; frame++) {
    permutation<double> p;
    p.data.resize(nref);
    for (int r = 0; r < nref; r++)
      p.data[r] = euclidean_distance_sparse((int)(ref_off[r + 1] - ref_off[r]), ref_idx + ref_off[r],
                                            ref_val + ref_off[r], (int)(fit_off[frame + 1] - fit_off[frame]),
                                            fit_idx + fit_off[frame], fit_val + fit_off[frame]);
    p.sort(k1);
    for (int x = 0; x < k; x++) {
      out_d[(size_t)frame * k + x] = p.data[x + 1];
      out_i[(size_t)frame * k + x] = p.indices[x + 1];
    }
  }
}

}  // extern "C"
'''


def build(ref: str | None = None, verbose: bool = False) -> str | None:
    """Build the library; returns its path, or None when no reference
    checkout is present (the tests that need it then skip)."""
    ref = reference_dir(ref)
    src_c = os.path.join(ref, "mdsctk.cpp")
    if not os.path.exists(src_c):
        return None
    os.makedirs(OUT, exist_ok=True)
    srcs = [src_c, os.path.join(ref, "mdsctk.h"), os.path.join(ref, "decomp_sparse.cpp"), __file__]
    if os.path.exists(LIB) and all(os.path.getmtime(LIB) >= os.path.getmtime(s) for s in srcs):
        return LIB
    with open(src_c) as f:
        c_lines = f.read().splitlines()
    with open(os.path.join(ref, "mdsctk.h")) as f:
        h_lines = f.read().splitlines()
    with open(os.path.join(ref, "decomp_sparse.cpp")) as f:
        d_lines = f.read().splitlines()
    macros = [ln for ln in h_lines if ln.startswith("#define SQR(") or ln.startswith("#define AVG(")]
    if len(macros) != 2:
        raise RuntimeError("SQR / AVG macros not found in mdsctk.h")
    perm = None
    for i, ln in enumerate(h_lines):
        if ln.startswith("template <class T> struct permutation"):
            perm = _block_from(h_lines, i)
            break
    if perm is None:
        raise RuntimeError("permutation template not found in mdsctk.h")
    funcs = []
    for sig in FUNCTIONS:
        funcs += _function(c_lines, sig) + [""]
    aff = _between(d_lines, "// Make affinity matrix", "delete [] d_a")
    unit = ["// Generated by oracle/ref_build.py from the reference checkout; not committed.",
            "#include <cmath>", "#include <cstddef>", "#include <algorithm>", "#include <vector>",
            "using namespace std;"] + macros + [""] + perm + [""] + funcs
    unit += WRAPPERS.replace("@AFFINITY@", "\n".join(aff)).splitlines()
    tu = os.path.join(OUT, "ref_extract.cpp")
    with open(tu, "w") as f:
        f.write("\n".join(unit) + "\n")
    cxx = shutil.which("g++") or "g++"
    cmd = [cxx, "-O2", "-std=c++14", "-fPIC", "-shared", "-ffp-contract=off", "-w", tu, "-o", LIB]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"reference extract did not compile:\n{r.stderr}")
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    p = build(sys.argv[1] if len(sys.argv) > 1 else None, verbose=True)
    if p is None:
        print("no reference checkout: nothing built")
