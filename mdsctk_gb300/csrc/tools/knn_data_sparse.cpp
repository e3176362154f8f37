// knn_data_sparse -- drop-in for MDSCTK's knn_data_sparse (knn_data_sparse.cpp):
// k nearest neighbours of sparse vectors by Euclidean distance, computed by
// libmdsgpu on the GPU. Same options, inputs and outputs:
//   -R/-r  reference index file (records [int n][int idx[n]]) and data file
//          (records [double val[n]]), defaults reference.svi / reference.svd;
//   -F/-f  fit files (default: the reference files);
//   distances.dat double[n_fit][k], indices.dat int[n_fit][k]; with -s false
//   the full distance rows, and indices.dat holds 0..N_ref-1 per row.
// A record cut short by the end of either file is dropped.
#include "cli.h"

static bool read_sparse(const std::string& ipath, const std::string& dpath, std::vector<int64_t>& off,
                        std::vector<int32_t>& idx, std::vector<double>& val) {
  std::vector<char> ib, db;
  if (!cli::read_file(ipath, ib) || !cli::read_file(dpath, db)) return false;
  off.assign(1, 0);
  idx.clear();
  val.clear();
  size_t ip = 0, dp = 0;
  while (ip + sizeof(int32_t) <= ib.size()) {
    int32_t n = 0;
    std::memcpy(&n, ib.data() + ip, sizeof(n));
    if (n < 0) break;
    const size_t ibytes = sizeof(int32_t) * (size_t)n, dbytes = sizeof(double) * (size_t)n;
    if (ip + sizeof(n) + ibytes > ib.size() || dp + dbytes > db.size()) break;
    const size_t i0 = idx.size();
    idx.resize(i0 + n);
    val.resize(i0 + n);
    if (n) {
      std::memcpy(idx.data() + i0, ib.data() + ip + sizeof(n), ibytes);
      std::memcpy(val.data() + i0, db.data() + dp, dbytes);
    }
    ip += sizeof(n) + ibytes;
    dp += dbytes;
    off.push_back((int64_t)idx.size());
  }
  return true;
}

int main(int argc, char** argv) {
  const char* prog = "knn_data_sparse";
  cli::banner(prog);
  std::cout << "   Computes the k nearest neighbors of all pairs of" << std::endl
            << "   vectors in the given sparse binary data files." << std::endl << std::endl;
  cli::Parser p(prog);
  p.add("threads", 't', cli::INT, "Input:  Number of threads to start (int; accepted, the GPU is used)", "1");
  p.add("knn", 'k', cli::INT, "Input:  K-nearest neighbors (int)");
  p.add("sort", 's', cli::BOOL, "Input:  Find K-nn,false=full distance matix (bool)", "1");
  p.add("block-size", 'b', cli::INT, "Input:  Workgroup block size in # frames (int; accepted)", "128");
  p.add("reference-index-file", 'R', cli::STRING, "Input:  Reference index file (string:filename)", "reference.svi");
  p.add("reference-data-file", 'r', cli::STRING, "Input:  Reference data file (string:filename)", "reference.svd");
  p.add("fit-index-file", 'F', cli::STRING, "Input:  Fitting index file (string:filename)");
  p.add("fit-data-file", 'f', cli::STRING, "Input:  Fitting data file (string:filename)");
  p.add("distance-file", 'd', cli::STRING, "Output: K-nn distances file (string:filename)", "distances.dat");
  p.add("index-file", 'i', cli::STRING, "Output: K-nn indices file (string:filename)", "indices.dat");
  p.add("device", 0, cli::INT, "Input:  CUDA device (int)", "0");
  int pr = p.parse(argc, argv);
  if (pr == 1) return 1;
  if (pr < 0) return -1;
  const bool sort = p.b("sort");
  if (!p.is_set("knn") && sort) {
    std::cout << "ERROR: --knn not supplied." << std::endl << std::endl;
    return -1;
  }
  const std::string rif = p.str("reference-index-file"), rdf = p.str("reference-data-file");
  const std::string fif = p.is_set("fit-index-file") ? p.str("fit-index-file") : rif;
  const std::string fdf = p.is_set("fit-data-file") ? p.str("fit-data-file") : rdf;
  const int k = p.is_set("knn") ? p.i("knn") : 0;
  std::cout << "Running with the following options:" << std::endl
            << "knn =                  " << k << std::endl
            << "sort =                 " << sort << std::endl
            << "reference-index-file = " << rif << std::endl
            << "reference-file =       " << rdf << std::endl
            << "fit-index-file =       " << fif << std::endl
            << "fit-file =             " << fdf << std::endl
            << "distance-file =        " << p.str("distance-file") << std::endl
            << "index-file =           " << p.str("index-file") << std::endl << std::endl;
  std::vector<int64_t> ro, fo;
  std::vector<int32_t> ri, fi;
  std::vector<double> rv, fv;
  std::cout << "Reading reference coordinates from files...";
  if (!read_sparse(rif, rdf, ro, ri, rv)) {
    std::cout << std::endl << "***ERROR***" << std::endl << "Could not open files: " << rif << ", " << rdf << std::endl;
    return -1;
  }
  std::cout << "done." << std::endl;
  const bool same = (fif == rif && fdf == rdf);
  std::cout << "Reading fitting coordinates from files...";
  if (!same && !read_sparse(fif, fdf, fo, fi, fv)) {
    std::cout << std::endl << "***ERROR***" << std::endl << "Could not open files: " << fif << ", " << fdf << std::endl;
    return -1;
  }
  std::cout << "done." << std::endl;
  const int nr = (int)ro.size() - 1, nf = same ? nr : (int)fo.size() - 1;
  if (nr < 1) {
    std::cout << "***ERROR*** no reference vectors" << std::endl;
    return -1;
  }
  mds_ctx* ctx = nullptr;
  int rc = mds_create(p.i("device"), 0, &ctx);
  if (rc) return cli::fail(ctx, rc);
  const int kk = sort ? std::max(0, std::min(k, nr - 1)) : nr;
  std::vector<double> d((size_t)nf * kk);
  std::vector<int32_t> idx((size_t)nf * kk);
  int kused = 0;
  rc = mds_knn_data_sparse(ctx, ro.data(), ri.data(), rv.data(), nr, same ? nullptr : fo.data(),
                           same ? nullptr : fi.data(), same ? nullptr : fv.data(), same ? 0 : nf, k,
                           sort ? 0u : MDS_FULL, d.data(), idx.data(), &kused);
  if (rc) return cli::fail(ctx, rc);
  mds_destroy(ctx);
  if (!cli::write_file(p.str("distance-file"), d.data(), sizeof(double) * d.size()) ||
      !cli::write_file(p.str("index-file"), idx.data(), sizeof(int32_t) * idx.size())) {
    std::cout << "***ERROR*** could not write the output files" << std::endl;
    return -1;
  }
  std::cout << std::endl << std::endl;
  return 0;
}
