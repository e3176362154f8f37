// decomp_sparse -- drop-in for MDSCTK's decomp_sparse (decomp_sparse.cpp):
// normalised Gaussian affinity of the .ssm matrix and its nev largest
// eigenpairs, computed on the GPU by libmdsgpu (thick-restart Lanczos with
// ARPACK's which/nev/ncv/tol semantics). New options --ncv, --tol,
// --maxiter and --binary-out leave the default outputs unchanged.
#include "decomp_common.h"

int main(int argc, char** argv) {
  const char* prog = "decomp_sparse";
  cli::banner(prog);
  std::cout << "   Reads the symmetric CSC format sparse matrix from" << std::endl
            << "   input-file, and computes the number of requested" << std::endl
            << "   eigenvalues/vectors of the normalized laplacian" << std::endl
            << "   using a gaussian kernel of width sigma." << std::endl << std::endl;
  cli::Parser p(prog);
  cli::add_decomp_options(p);
  int pr = p.parse(argc, argv);
  if (pr == 1) return 1;
  if (pr < 0 || !cli::check_decomp_args(p)) return -1;
  const double sigma = p.d("sigma");
  const int nev = p.i("nevals");
  std::cout << "Running with the following options:" << std::endl
            << "sigma =          " << sigma << std::endl
            << "nevals =         " << nev << std::endl
            << "ssm-file =       " << p.str("ssm-file") << std::endl
            << "evals-file =     " << p.str("evals-file") << std::endl
            << "evecs-file =     " << p.str("evecs-file") << std::endl
            << "residuals-file = " << p.str("residuals-file") << std::endl << std::endl;
  cli::Csc A;
  if (!cli::read_csc(p.str("ssm-file"), A)) {
    std::cout << "***ERROR*** could not read " << p.str("ssm-file") << std::endl;
    return -1;
  }
  mds_ctx* ctx = nullptr;
  int rc = mds_create(p.i("device"), 0, &ctx);
  if (rc) return cli::fail(ctx, rc);
  std::vector<double> ev(std::max(nev, 0)), V((size_t)std::max(nev, 0) * A.n), res(std::max(nev, 0));
  int nconv = 0;
  rc = mds_decomp_sparse(ctx, A.n, A.pcol.data(), A.irow.data(), A.val.data(), sigma, nev, p.i("ncv"), p.d("tol"),
                         p.i("maxiter"), 0, ev.data(), V.data(), res.data(), &nconv);
  if (rc) return cli::fail(ctx, rc);
  mds_destroy(ctx);
  return cli::write_decomp(p, A.n, nev, ev, V, nullptr, 0, res, nconv);
}
