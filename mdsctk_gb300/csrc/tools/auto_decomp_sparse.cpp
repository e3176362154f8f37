// auto_decomp_sparse -- drop-in for MDSCTK's auto_decomp_sparse
// (auto_decomp_sparse.cpp): decomp_sparse with a sigma per landmark, the mean
// of its first k-sigma stored distances, or (with -K) the entropic-affinity
// sigma of perplexity K; computed on the GPU by libmdsgpu.
#include <cmath>

#include "decomp_common.h"

int main(int argc, char** argv) {
  const char* prog = "auto_decomp_sparse";
  cli::banner(prog);
  std::cout << "   Reads the symmetric CSC format sparse matrix from" << std::endl
            << "   input-file, and computes the number of requested" << std::endl
            << "   eigenvalues/vectors of the normalized laplacian" << std::endl
            << "   using a gaussian kernel of width sigma," << std::endl
            << "   where sigma is calculated using the average of the" << std::endl
            << "   k-closest neighbor distances in each column." << std::endl
            << "   Note that k is normally smaller than the number of" << std::endl
            << "   neighbors used to construct the sparse CSC matrix." << std::endl << std::endl;
  cli::Parser p(prog);
  cli::add_decomp_options(p, true);
  int pr = p.parse(argc, argv);
  if (pr == 1) return 1;
  if (pr < 0) return -1;
  bool ok = cli::check_auto_args(p);
  const bool pset = p.is_set("k-perplexity");
  const int ka = ok ? p.i("k-sigma") : 0;
  const double K = pset ? p.d("k-perplexity") : 0.0;
  if (pset && std::ceil(K) > (double)ka)
    std::cout << "WARNING: --k-perplexity (" << K << ") is higher than --k-sigma (" << ka << ")" << std::endl;
  if (!ok) return -1;
  const int nev = p.i("nevals");
  std::cout << "Running with the following options:" << std::endl << "k-sigma =        " << ka << std::endl;
  if (pset) std::cout << "k-perplexity =   " << K << std::endl;
  std::cout << "nevals =         " << nev << std::endl
            << "ssm-file =       " << p.str("ssm-file") << std::endl
            << "residuals-file = " << p.str("residuals-file") << std::endl
            << "evals-file =     " << p.str("evals-file") << std::endl
            << "evecs-file =     " << p.str("evecs-file") << std::endl << std::endl;
  cli::Csc A;
  if (!cli::read_csc(p.str("ssm-file"), A)) {
    std::cout << "***ERROR*** could not read " << p.str("ssm-file") << std::endl;
    return -1;
  }
  mds_ctx* ctx = nullptr;
  int rc = mds_create(p.i("device"), 0, &ctx);
  if (rc) return cli::fail(ctx, rc);
  const int ne = std::max(nev, 0);
  std::vector<double> ev(ne), V((size_t)ne * A.n), res(ne), sig(A.n);
  int nconv = 0;
  rc = mds_auto_decomp_sparse(ctx, A.n, A.pcol.data(), A.irow.data(), A.val.data(), ka, K, nev, p.i("ncv"),
                              p.d("tol"), p.i("maxiter"), 0, ev.data(), V.data(), res.data(), &nconv, sig.data());
  if (rc) return cli::fail(ctx, rc);
  mds_destroy(ctx);
  cli::print_average_sigma(sig);
  return cli::write_decomp(p, A.n, nev, ev, V, nullptr, 0, res, nconv, true);
}
