// decomp_common.h -- output writing shared by decomp_sparse and
// decomp_sparse_nystrom: text files with the default ostream format (six
// significant digits), eigenvalues descending one per line, each
// eigenvector on one line with a trailing space, residuals one per line
// (decomp_sparse.cpp:242-277), or raw doubles with --binary-out (the layout
// of the reference's DECOMP_WRITE_DOUBLE build).
#pragma once
#include <cfloat>
#include <cmath>

#include "cli.h"

namespace cli {

inline double sqrt_eps() {
  double eps = 1.0;
  do { eps /= 2.0; } while (1.0 + (eps / 2.0) != 1.0);
  return std::sqrt(eps);
}

// auto_decomp_sparse[_nystrom] take -k/-K (per-landmark sigmas) in place of -q.
inline void add_decomp_options(Parser& p, bool auto_sigma = false) {
  if (auto_sigma) {
    p.add("k-sigma", 'k', INT, "Input:  K-nn to average for sigmas (int)");
    p.add("k-perplexity", 'K', DOUBLE, "Input:  Desired perplexity within knn (real)");
  } else {
    p.add("sigma", 'q', DOUBLE, "Input:  Standard deviation of gaussian kernel (real)");
  }
  p.add("nevals", 'n', INT, "Input:  Number of eigenvalues/vectors (int)");
  p.add("ssm-file", 's', STRING, "Input:  Symmetric sparse matrix file (string:filename)", "distances.ssm");
  p.add("evals-file", 'v', STRING, "Output:  Eigenvalues file (string:filename)", "eigenvalues.dat");
  p.add("evecs-file", 'e', STRING, "Output: Eigenvectors file (string:filename)", "eigenvectors.dat");
  p.add("residuals-file", 'r', STRING, "Output: Residuals file (string:filename)", "residuals.dat");
  p.add("ncv", 0, INT, "Input:  Lanczos basis size (int; 0 = min(10*nev+1, n) as ARPACK is called)", "0");
  p.add("tol", 0, DOUBLE, "Input:  Convergence tolerance (real; 0 = machine precision)", "0");
  p.add("maxiter", 0, INT, "Input:  Maximum restarts (int; 0 = 100*nev)", "0");
  p.add("binary-out", 0, SWITCH, "Output: write raw doubles instead of text");
  p.add("device", 0, INT, "Input:  CUDA device (int)", "0");
}

// ext may be null (decomp_sparse); otherwise the m extension values follow
// the n eigenvector values on the same line / in the same record.
// max_style: auto_decomp_sparse's wording of the residual report
// (auto_decomp_sparse.cpp:244-248).
inline int write_decomp(const Parser& p, int n, int nev, const std::vector<double>& ev, const std::vector<double>& V,
                        const std::vector<double>* ext, int m, const std::vector<double>& res, int nconv,
                        bool max_style = false) {
  std::cout << "Number of converged eigenvalues/vectors found: " << nconv << std::endl;
  const bool bin = p.b("binary-out");
  std::ofstream fv(p.str("evals-file").c_str(), bin ? std::ios::binary : std::ios::out);
  std::ofstream fe(p.str("evecs-file").c_str(), bin ? std::ios::binary : std::ios::out);
  std::ofstream fr(p.str("residuals-file").c_str(), bin ? std::ios::binary : std::ios::out);
  double maxr = 0.0;
  for (int x = 0; x < nev; ++x) {
    if (bin) {
      fv.write(reinterpret_cast<const char*>(&ev[x]), sizeof(double));
      fe.write(reinterpret_cast<const char*>(&V[(size_t)x * n]), sizeof(double) * n);
      if (ext) fe.write(reinterpret_cast<const char*>(&(*ext)[(size_t)x * m]), sizeof(double) * m);
      fr.write(reinterpret_cast<const char*>(&res[x]), sizeof(double));
    } else {
      fv << ev[x] << std::endl;
      for (int y = 0; y < n; ++y) fe << V[(size_t)x * n + y] << " ";
      if (ext)
        for (int y = 0; y < m; ++y) fe << (*ext)[(size_t)x * m + y] << " ";
      fe << std::endl;
      fr << res[x] << std::endl;
    }
    maxr = std::max(maxr, res[x]);
  }
  const double eps = sqrt_eps();
  std::cout << (max_style ? "Maximum residual: " : "Max residual: ") << maxr << " (eps: " << eps << ")"
            << std::endl;
  if (maxr > eps) {
    std::cout << (max_style ? "*** Max residual too high (max_r > eps)!" : "*** Sum of residuals too high (max_r > eps)!")
              << std::endl;
    std::cout << "*** Please, check results manually..." << std::endl;
  }
  return 0;
}

// average sigma as the reference prints it (sequential sum / n)
inline void print_average_sigma(const std::vector<double>& sig) {
  double s = sig.empty() ? 0.0 : sig[0];
  for (size_t x = 1; x < sig.size(); ++x) s += sig[x];
  std::cout << "Average sigma: " << (s / (double)sig.size()) << std::endl << std::endl;
}

inline bool check_auto_args(const Parser& p) {
  bool ok = true;
  if (!p.is_set("k-sigma")) {
    std::cout << "ERROR: --k-sigma not supplied." << std::endl << std::endl;
    ok = false;
  }
  if (!p.is_set("nevals")) {
    std::cout << "ERROR: --nevals not supplied." << std::endl << std::endl;
    ok = false;
  }
  return ok;
}

inline bool check_decomp_args(const Parser& p) {
  bool ok = true;
  if (!p.is_set("sigma")) {
    std::cout << "ERROR: --sigma not supplied." << std::endl << std::endl;
    ok = false;
  }
  if (!p.is_set("nevals")) {
    std::cout << "ERROR: --nevals not supplied." << std::endl << std::endl;
    ok = false;
  }
  return ok;
}

}  // namespace cli
