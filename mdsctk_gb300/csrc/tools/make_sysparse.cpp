// make_sysparse -- drop-in for MDSCTK's make_sysparse (make_sysparse.cpp):
// kNN files -> symmetric CSC holding one strict triangle of distances
// (distances.ssm: int n; int pcol[n+1]; int irow[nnz]; double val[nnz]),
// assembled on the GPU by libmdsgpu (sort-based; no on-disk B-tree).
#include "knn_files.h"

int main(int argc, char** argv) {
  const char* prog = "make_sysparse";
  cli::banner(prog);
  std::cout << "   Converts the results from knn_* into symmetric CSC format." << std::endl << std::endl;
  cli::Parser p(prog);
  p.add("knn", 'k', cli::INT, "Input:  K-nearest neighbors (int)");
  p.add("output-knn", 'n', cli::INT, "Input:  K-nn to keep in output (int)");
  p.add("index-file", 'i', cli::STRING, "Input:  Index file (string:filename)", "indices.dat");
  p.add("distance-file", 'd', cli::STRING, "Input:  Distances file (string:filename)", "distances.dat");
  p.add("output-file", 'o', cli::STRING, "Output: Symmetric sparse matrix file (string:filename)", "distances.ssm");
  p.add("device", 0, cli::INT, "Input:  CUDA device (int)", "0");
  int pr = p.parse(argc, argv);
  if (pr == 1) return 1;
  if (pr < 0) return -1;
  bool ok = true;
  if (!p.is_set("knn")) {
    std::cout << "ERROR: --knn not supplied." << std::endl << std::endl;
    ok = false;
  }
  int maxk = p.is_set("knn") ? p.i("knn") : 0;
  int k = p.is_set("output-knn") ? p.i("output-knn") : maxk;
  if (maxk < k) {
    std::cout << "ERROR: Output k (" << k << ") is not less than the input k (" << maxk << ")." << std::endl
              << std::endl;
    ok = false;
  }
  if (!ok) return -1;
  std::cout << "Running with the following options:" << std::endl
            << "knn =            " << maxk << std::endl
            << "output-knn =     " << k << std::endl
            << "index-file =     " << p.str("index-file") << std::endl
            << "distances-file = " << p.str("distance-file") << std::endl
            << "output-file =    " << p.str("output-file") << std::endl << std::endl;
  if (maxk < 1) {
    std::cout << "ERROR: --knn must be positive." << std::endl;
    return -1;
  }
  std::vector<double> dist;
  std::vector<int32_t> idx;
  int n = 0;
  if (!cli::read_knn_pair(p.str("distance-file"), p.str("index-file"), maxk, dist, idx, n)) {
    std::cout << "***ERROR***" << std::endl << "Could not open the input files" << std::endl << std::endl;
    return -1;
  }
  std::cout << "Creating sparse matrix..." << std::endl;
  mds_ctx* ctx = nullptr;
  int rc = mds_create(p.i("device"), 0, &ctx);
  if (rc) return cli::fail(ctx, rc);
  int64_t cap = std::max<int64_t>(1, (int64_t)n * std::max(k, 0));
  std::vector<int32_t> pcol(n + 1), irow(cap);
  std::vector<double> val(cap);
  int64_t nnz = 0;
  rc = mds_sysparse(ctx, dist.data(), idx.data(), n, maxk, std::max(k, 0), 0, pcol.data(), irow.data(), val.data(),
                    cap, &nnz);
  if (rc) return cli::fail(ctx, rc);
  mds_destroy(ctx);
  if (!cli::write_csc(p.str("output-file"), n, pcol.data(), irow.data(), val.data())) {
    std::cout << "Could not create symmetric CSC matrix file: " << p.str("output-file") << std::endl;
    return -1;
  }
  std::cout << std::endl << std::endl;
  return 0;
}
