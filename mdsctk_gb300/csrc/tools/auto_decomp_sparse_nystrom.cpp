// auto_decomp_sparse_nystrom -- drop-in for MDSCTK's
// auto_decomp_sparse_nystrom (auto_decomp_sparse_nystrom.cpp): per-landmark
// sigmas (mean of the first k-sigma stored distances) for the landmark graph
// and, squared, for the out-of-sample matrix, then the eigenpairs and their
// Nystrom extension. As in the reference, -K is accepted and not applied.
#include "decomp_common.h"

int main(int argc, char** argv) {
  const char* prog = "auto_decomp_sparse_nystrom";
  cli::banner(prog);
  cli::Parser p(prog);
  cli::add_decomp_options(p, true);
  p.add("gsm-file", 'g', cli::STRING, "Input:  General sparse matrix file (string:filename)", "distances.gsm");
  int pr = p.parse(argc, argv);
  if (pr == 1) return 1;
  if (pr < 0 || !cli::check_auto_args(p)) return -1;
  const int ka = p.i("k-sigma");
  const int nev = p.i("nevals");
  std::cout << "Running with the following options:" << std::endl
            << "k-sigma =    " << ka << std::endl
            << "nevals =     " << nev << std::endl
            << "ssm-file =   " << p.str("ssm-file") << std::endl
            << "gsm-file =   " << p.str("gsm-file") << std::endl
            << "evals-file = " << p.str("evals-file") << std::endl
            << "evecs-file = " << p.str("evecs-file") << std::endl << std::endl;
  cli::Csc A, B;
  if (!cli::read_csc(p.str("ssm-file"), A) || !cli::read_csc(p.str("gsm-file"), B)) {
    std::cout << "***ERROR*** could not read the sparse matrix files" << std::endl;
    return -1;
  }
  mds_ctx* ctx = nullptr;
  int rc = mds_create(p.i("device"), 0, &ctx);
  if (rc) return cli::fail(ctx, rc);
  const int ne = std::max(nev, 0);
  std::vector<double> ev(ne), V((size_t)ne * A.n), E((size_t)ne * B.n), res(ne), sig(A.n);
  int nconv = 0;
  rc = mds_auto_decomp_sparse_nystrom(ctx, A.n, A.pcol.data(), A.irow.data(), A.val.data(), B.n, B.pcol.data(),
                                      B.irow.data(), B.val.data(), ka, 0.0, nev, p.i("ncv"), p.d("tol"),
                                      p.i("maxiter"), 0, ev.data(), V.data(), E.data(), res.data(), &nconv,
                                      sig.data());
  if (rc) return cli::fail(ctx, rc);
  mds_destroy(ctx);
  cli::print_average_sigma(sig);
  return cli::write_decomp(p, A.n, nev, ev, V, &E, B.n, res, nconv);
}
