// knn_rms -- drop-in for MDSCTK's knn_rms (knn_rms.cpp): k nearest frames by
// minimum mass-weighted RMSD after optimal superposition, computed on the GPU
// by libmdsgpu. Same options and outputs (distances.dat: double[n_fit][k] in
// Angstrom; indices.dat: int[n_fit][k]).
//
// Inputs: -p topology (.pdb or .gro: atom count and masses by element, the
// masses GROMACS assigns to the common elements), -r/-f coordinates: GROMACS
// .xtc trajectories (decoded on the GPU by mds_xtc_decode; an atom count
// that differs from the topology's exits with status 4, knn_rms.cpp:157-178)
// or raw float32 frames [natoms][3] in nm (the layout flatten_xtc writes).
#include <algorithm>
#include <cctype>
#include <sstream>

#include "cli.h"
#include "frames.h"
#include "topology.h"

int main(int argc, char** argv) {
  const char* prog = "knn_rms";
  cli::banner(prog);
  std::cout << "   Computes the k nearest neighbors of all reference" << std::endl
            << "   structures for each structure in the fitting file." << std::endl << std::endl;
  cli::Parser p(prog);
  p.add("threads", 't', cli::INT, "Input:  Number of threads to start (int; accepted, the GPU is used)", "1");
  p.add("knn", 'k', cli::INT, "Input:  K-nearest neighbors (int)");
  p.add("sort", 's', cli::BOOL, "Input:  Find K-nn,false=full distance matix (bool)", "1");
  p.add("nofit", 'n', cli::BOOL, "Input:  DO NOT rotate+fit before RMSD calculation (bool)", "0");
  p.add("block-size", 'b', cli::INT, "Input:  Workgroup block size in # frames (int; accepted)", "128");
  p.add("topology-file", 'p', cli::STRING, "Input:  Topology file [.pdb,.gro] (string:filename)", "topology.pdb");
  p.add("reference-file", 'r', cli::STRING, "Input:  Reference coordinates (string:filename)", "reference.xtc");
  p.add("fit-file", 'f', cli::STRING, "Input:  Fitting coordinates (string:filename)");
  p.add("distance-file", 'd', cli::STRING, "Output: K-nn distances file (string:filename)", "distances.dat");
  p.add("index-file", 'i', cli::STRING, "Output: K-nn indices file (string:filename)", "indices.dat");
  p.add("precision", 0, cli::STRING, "Input:  candidate screen: fp32, bf16x3 or fp16x3 (outputs are exact either way)",
        "bf16x3");
  p.add("device", 0, cli::INT, "Input:  CUDA device (int)", "0");
  int pr = p.parse(argc, argv);
  if (pr == 1) return 1;
  if (pr < 0) return -1;
  const bool sort = p.b("sort");
  if (!p.is_set("knn") && sort) {
    std::cout << "ERROR: --knn not supplied." << std::endl << std::endl;
    return -1;
  }
  std::string ref = p.str("reference-file");
  std::string fit = p.is_set("fit-file") ? p.str("fit-file") : ref;
  const int k = p.is_set("knn") ? p.i("knn") : 0;
  std::cout << "Running with the following options:" << std::endl
            << "knn =            " << k << std::endl
            << "sort =           " << sort << std::endl
            << "nofit =          " << p.b("nofit") << std::endl
            << "topology-file =  " << p.str("topology-file") << std::endl
            << "reference-file = " << ref << std::endl
            << "fit-file =       " << fit << std::endl
            << "distance-file =  " << p.str("distance-file") << std::endl
            << "index-file =     " << p.str("index-file") << std::endl << std::endl;
  unsigned prec = MDS_PREC_BF16X3;
  std::string ps = p.str("precision");
  if (ps == "fp32") prec = MDS_PREC_FP32;
  else if (ps == "fp16x3") prec = MDS_PREC_FP16X3;
  else if (ps != "bf16x3") {
    std::cout << "ERROR: --precision must be fp32, bf16x3 or fp16x3" << std::endl;
    return -1;
  }
  std::cout << "Reading topology information from " << p.str("topology-file") << " ... ";
  Topology top;
  if (!read_topology(p.str("topology-file"), top) || top.mass.empty()) {
    std::cout << std::endl << "*** ERROR *** could not read atoms from " << p.str("topology-file") << std::endl;
    return -1;
  }
  std::cout << "done." << std::endl;
  const std::vector<float>& mass = top.mass;
  const int natoms = (int)mass.size();
  mds_ctx* ctx = nullptr;
  int rc = mds_create(p.i("device"), 0, &ctx);
  if (rc) return cli::fail(ctx, rc);
  std::vector<float> xr, xf;
  int nr = 0, nf = 0;
  for (int pass = 0; pass < 2; ++pass) {
    const std::string& fn = pass ? fit : ref;
    if (pass && fit == ref) break;
    int xa = 0;
    int rr = read_frames(ctx, fn, natoms, pass ? xf : xr, pass ? nf : nr, &xa);
    if (rr == -1) {
      std::cout << "*** ERROR *** could not open " << fn << std::endl;
      return -1;
    }
    if (rr == -3) {
      std::cout << "*** ERROR *** " << fn << " is not a readable XTC trajectory" << std::endl;
      return -1;
    }
    if (rr == -4) {
      std::cout << "*** ERROR ***" << std::endl
                << "Number of atoms in topology file (" << natoms << ") "
                << "does not match the number of atoms in the XTC file (" << fn << " : " << xa << ")."
                << std::endl;
      return 4;
    }
  }
  if (fit == ref) nf = nr;
  if (nr < 1) {
    std::cout << "*** ERROR *** no reference frames" << std::endl;
    return -1;
  }
  unsigned flags = prec | (p.b("nofit") ? MDS_NOFIT : 0u) | (sort ? 0u : MDS_FULL);
  int kk = sort ? std::max(0, std::min(k, nr - 1)) : nr;
  std::vector<double> d((size_t)nf * kk);
  std::vector<int32_t> idx((size_t)nf * kk);
  int kused = 0;
  rc = mds_knn_rms(ctx, xr.data(), nr, fit == ref ? nullptr : xf.data(), fit == ref ? 0 : nf, natoms, mass.data(), k,
                   flags, d.data(), idx.data(), &kused);
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
