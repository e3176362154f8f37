// frames.h -- coordinate input of the drop-in tools: a GROMACS .xtc
// trajectory (decoded on the GPU by mds_xtc_index / mds_xtc_decode, what
// read_first_xtc / read_next_xtc do in the reference, knn_rms.cpp:155-203)
// or raw float32 frames [natoms][3] in nm (the layout flatten_xtc writes).
#pragma once

#include "cli.h"

// Returns 0, -1 (cannot open), -3 (malformed .xtc), or -4 (the .xtc holds
// `*xtc_atoms` atoms, not natoms).
inline int read_frames(mds_ctx* ctx, const std::string& path, int natoms, std::vector<float>& x, int& n,
                       int* xtc_atoms) {
  std::vector<char> b;
  if (!cli::read_file(path, b)) return -1;
  const unsigned char* u = reinterpret_cast<const unsigned char*>(b.data());
  if (b.size() >= 4 && ((u[0] << 24) | (u[1] << 16) | (u[2] << 8) | u[3]) == 1995) {
    int nfr = 0, na = 0;
    if (mds_xtc_index(u, b.size(), nullptr, 0, &nfr, &na) != MDS_OK) return -3;
    if (na != natoms) {
      *xtc_atoms = na;
      return -4;
    }
    std::vector<int64_t> off(nfr + 1);
    if (mds_xtc_index(u, b.size(), off.data(), nfr + 1, &nfr, &na) != MDS_OK) return -3;
    x.resize((size_t)nfr * 3 * natoms);
    if (nfr && mds_xtc_decode(ctx, u, b.size(), off.data(), nfr, natoms, 0, x.data(), nullptr, nullptr,
                              nullptr) != MDS_OK) {
      std::cout << "*** ERROR *** " << mds_last_error(ctx) << std::endl;
      return -3;
    }
    n = nfr;
    return 0;
  }
  size_t fr = sizeof(float) * 3 * (size_t)natoms;
  n = (int)(b.size() / fr);
  x.resize((size_t)n * 3 * natoms);
  if (n) std::memcpy(x.data(), b.data(), fr * n);
  return 0;
}

