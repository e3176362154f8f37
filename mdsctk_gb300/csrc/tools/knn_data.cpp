// knn_data -- drop-in for MDSCTK's knn_data (knn_data.cpp): k nearest
// neighbours of raw double vectors, Euclidean or (-c) correlation distance,
// computed by libmdsgpu on the GPU. Same options, same input (.pts: records of
// -v doubles until end of file; a partial last record is dropped) and same
// outputs (distances.dat: double[n_fit][k]; indices.dat: int[n_fit][k]).
// With -s false the full distance rows are written and indices.dat holds
// 0..N_ref-1 per row (the reference writes an uninitialised vector there).
#include "cli.h"

static bool read_pts(const std::string& path, int dim, std::vector<double>& x, int& n) {
  std::vector<char> b;
  if (!cli::read_file(path, b)) return false;
  size_t rec = sizeof(double) * (size_t)dim;
  n = (int)(b.size() / rec);
  x.resize((size_t)n * dim);
  if (n) std::memcpy(x.data(), b.data(), rec * n);
  return true;
}

int main(int argc, char** argv) {
  const char* prog = "knn_data";
  cli::banner(prog);
  std::cout << "   Computes the k nearest neighbors of all pairs of" << std::endl
            << "   vectors in the given binary data files." << std::endl << std::endl;
  cli::Parser p(prog);
  p.add("threads", 't', cli::INT, "Input:  Number of threads to start (int; accepted, the GPU is used)", "1");
  p.add("knn", 'k', cli::INT, "Input:  K-nearest neighbors (int)");
  p.add("sort", 's', cli::BOOL, "Input:  Find K-nn,false=full distance matix (bool)", "1");
  p.add("vector-size", 'v', cli::INT, "Input:  Data vector length (int)");
  p.add("block-size", 'b', cli::INT, "Input:  Workgroup block size in # frames (int; accepted)", "128");
  p.add("correlation", 'c', cli::SWITCH, "Input:  Use correlation distance (bool)");
  p.add("reference-file", 'r', cli::STRING, "Input:  Reference data file (string:filename)", "reference.pts");
  p.add("fit-file", 'f', cli::STRING, "Input:  Fitting data file (string:filename)");
  p.add("distance-file", 'd', cli::STRING, "Output: K-nn distances file (string:filename)", "distances.dat");
  p.add("index-file", 'i', cli::STRING, "Output: K-nn indices file (string:filename)", "indices.dat");
  p.add("precision", 0, cli::STRING, "Input:  candidate screen: fp32 or bf16x3 (outputs are exact either way)",
        "bf16x3");
  p.add("device", 0, cli::INT, "Input:  CUDA device (int)", "0");
  int pr = p.parse(argc, argv);
  if (pr == 1) return 1;
  if (pr < 0) return -1;
  bool ok = true;
  const bool sort = p.b("sort");
  if (!p.is_set("knn") && sort) {
    std::cout << "ERROR: --knn not supplied." << std::endl << std::endl;
    ok = false;
  }
  if (!p.is_set("vector-size")) {
    std::cout << "ERROR: --vector-size not supplied." << std::endl << std::endl;
    ok = false;
  }
  unsigned prec = MDS_PREC_BF16X3;
  const std::string ps = p.str("precision");
  if (ps == "fp32") prec = MDS_PREC_FP32;
  else if (ps != "bf16x3") {
    std::cout << "ERROR: --precision must be fp32 or bf16x3" << std::endl;
    ok = false;
  }
  if (!ok) return -1;
  std::string ref = p.str("reference-file");
  std::string fit = p.is_set("fit-file") ? p.str("fit-file") : ref;
  int k = p.is_set("knn") ? p.i("knn") : 0, dim = p.i("vector-size");
  std::cout << "Running with the following options:" << std::endl
            << "knn =            " << k << std::endl
            << "sort =           " << sort << std::endl
            << "vector-size =    " << dim << std::endl
            << "reference-file = " << ref << std::endl
            << "fit-file =       " << fit << std::endl
            << "distance-file =  " << p.str("distance-file") << std::endl
            << "index-file =     " << p.str("index-file") << std::endl << std::endl;
  if (dim < 1) {
    std::cout << "ERROR: --vector-size must be positive." << std::endl;
    return -1;
  }
  std::vector<double> xr, xf;
  int nr = 0, nf = 0;
  if (!read_pts(ref, dim, xr, nr)) {
    std::cout << "***ERROR***" << std::endl << "Could not open file: " << ref << std::endl;
    return -1;
  }
  std::cout << "Number of reference coordinates: " << nr << std::endl;
  bool same = (fit == ref);
  if (!same && !read_pts(fit, dim, xf, nf)) {
    std::cout << "***ERROR***" << std::endl << "Could not open file: " << fit << std::endl;
    return -1;
  }
  if (same) nf = nr;
  std::cout << "Number of fitting coordinates: " << nf << std::endl;
  if (nr < 1) {
    std::cout << "***ERROR*** no reference vectors" << std::endl;
    return -1;
  }
  mds_ctx* ctx = nullptr;
  int rc = mds_create(p.i("device"), 0, &ctx);
  if (rc) return cli::fail(ctx, rc);
  unsigned flags = (p.b("correlation") ? MDS_CORRELATION : 0u) | (sort ? 0u : MDS_FULL) | prec;
  int kk = sort ? std::max(0, std::min(k, nr - 1)) : nr;
  std::vector<double> d((size_t)nf * kk);
  std::vector<int32_t> idx((size_t)nf * kk);
  int kused = 0;
  rc = mds_knn_data(ctx, xr.data(), nr, same ? nullptr : xf.data(), same ? 0 : nf, dim, k, flags, d.data(),
                    idx.data(), &kused);
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
