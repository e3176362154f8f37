// knn_files.h -- reading distances.dat / indices.dat the way make_sysparse
// and make_gesparse do (make_sysparse.cpp:225-243): rows of maxk values are
// read from both files in lock step while either stream is still good. A
// stream that runs out keeps the bytes of its last read in the row buffer (a
// short read fills the front of the buffer; later reads leave it as it is),
// so the row count is the larger number of complete rows.
#pragma once
#include "cli.h"

namespace cli {

inline bool read_knn_pair(const std::string& dpath, const std::string& ipath, int maxk, std::vector<double>& dist,
                          std::vector<int32_t>& idx, int& nrows) {
  std::vector<char> db, ib;
  if (!read_file(dpath, db) || !read_file(ipath, ib)) return false;
  const size_t drow = sizeof(double) * (size_t)maxk, irow = sizeof(int32_t) * (size_t)maxk;
  const size_t rows_d = db.size() / drow, rows_i = ib.size() / irow;
  nrows = (int)std::max(rows_d, rows_i);
  dist.assign((size_t)nrows * maxk, 0.0);
  idx.assign((size_t)nrows * maxk, 0);
  std::vector<char> dbuf(drow, 0), ibuf(irow, 0);
  bool dfail = false, ifail = false;
  for (int r = 0; r < nrows; ++r) {
    for (int f = 0; f < 2; ++f) {
      std::vector<char>& src = f ? ib : db;
      std::vector<char>& buf = f ? ibuf : dbuf;
      bool& failed = f ? ifail : dfail;
      size_t rowb = f ? irow : drow;
      if (failed) continue;
      size_t off = (size_t)r * rowb;
      if (off + rowb <= src.size()) {
        std::memcpy(buf.data(), src.data() + off, rowb);
      } else {
        if (off < src.size()) std::memcpy(buf.data(), src.data() + off, src.size() - off);
        failed = true;
      }
    }
    std::memcpy(&dist[(size_t)r * maxk], dbuf.data(), drow);
    std::memcpy(&idx[(size_t)r * maxk], ibuf.data(), irow);
  }
  return true;
}

}  // namespace cli
