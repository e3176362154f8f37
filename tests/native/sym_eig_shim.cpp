// Test shim: exposes the host dense symmetric eigensolver of
// mdsctk_gb300/csrc/sym_eig.h to ctypes for the CPU tests.
#include <vector>

#include "sym_eig.h"

extern "C" int symeig_shim(int m, const double* a, double* w, double* z) {
  std::vector<double> A(a, a + (size_t)m * m), W, Z;
  if (!mds_symeig::sym_eig(A, m, W, Z)) return 1;
  for (int i = 0; i < m; ++i) w[i] = W[i];
  for (size_t i = 0; i < (size_t)m * m; ++i) z[i] = Z[i];
  return 0;
}
