// cli.h -- command-line parsing and file helpers shared by the drop-in tools.
//
// Accepts the option syntax of the reference's Boost.program_options
// command lines: "-k 10", "--knn 10", "--knn=10", boolean values given as
// 1/0/true/false/yes/no/on/off ("-s 0"), and switches ("-c"). -h/--help
// prints the usage and exits with 1; a missing required option prints
// "ERROR: --<name> not supplied." and exits with 255 (return -1), as the
// reference's tools do.
#pragma once

#include <cerrno>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <string>
#include <vector>

#include "../../../include/mdsgpu.h"

namespace cli {

enum Kind { INT, DOUBLE, STRING, BOOL, SWITCH };

struct Opt {
  std::string lname;
  char sname;
  Kind kind;
  std::string help;
  std::string value;
  bool has_default = false;
  bool seen = false;
};

class Parser {
 public:
  explicit Parser(const char* prog) : prog_(prog) {}
  void add(const char* lname, char sname, Kind k, const char* help, const char* def = nullptr) {
    Opt o;
    o.lname = lname;
    o.sname = sname;
    o.kind = k;
    o.help = help;
    if (def) {
      o.value = def;
      o.has_default = true;
    }
    if (k == SWITCH && !def) {
      o.value = "0";
      o.has_default = true;
    }
    opts_.push_back(o);
  }
  // returns 0 ok, 1 help printed, -1 error
  int parse(int argc, char** argv) {
    add("help", 'h', SWITCH, "show this help message and exit");
    for (int i = 1; i < argc; ++i) {
      std::string a = argv[i];
      Opt* o = nullptr;
      std::string val;
      bool has_val = false;
      if (a.rfind("--", 0) == 0) {
        std::string name = a.substr(2);
        size_t eq = name.find('=');
        if (eq != std::string::npos) {
          val = name.substr(eq + 1);
          name = name.substr(0, eq);
          has_val = true;
        }
        o = find_long(name);
      } else if (a.size() >= 2 && a[0] == '-') {
        o = find_short(a[1]);
        if (o && a.size() > 2) {
          val = a.substr(2);
          has_val = true;
        }
      }
      if (!o) {
        std::cerr << "ERROR: unrecognised option '" << a << "'" << std::endl;
        return -1;
      }
      if (o->kind == SWITCH) {
        o->value = "1";
        o->seen = true;
        continue;
      }
      if (!has_val) {
        if (i + 1 >= argc) {
          std::cerr << "ERROR: the required argument for option '--" << o->lname << "' is missing" << std::endl;
          return -1;
        }
        val = argv[++i];
      }
      if (o->kind == BOOL) {
        std::string v = val;
        for (auto& ch : v) ch = (char)std::tolower(ch);
        if (v == "1" || v == "true" || v == "yes" || v == "on") val = "1";
        else if (v == "0" || v == "false" || v == "no" || v == "off") val = "0";
        else {
          std::cerr << "ERROR: invalid boolean value '" << val << "' for --" << o->lname << std::endl;
          return -1;
        }
      }
      o->value = val;
      o->seen = true;
    }
    if (is_set("help")) {
      std::cout << "usage: " << prog_ << " [options]" << std::endl << "Program options:" << std::endl;
      for (auto& o : opts_)
        std::cout << "  " << (o.sname ? std::string("-") + o.sname + " [ --" + o.lname + " ] " : "--" + o.lname + " ") << o.help
                  << (o.has_default && o.kind != SWITCH ? " (=" + o.value + ")" : std::string()) << std::endl;
      return 1;
    }
    return 0;
  }
  bool count(const char* lname) const {
    const Opt* o = find_long_c(lname);
    return o && (o->seen || (o->has_default && o->kind != SWITCH));
  }
  bool is_set(const char* lname) const {
    const Opt* o = find_long_c(lname);
    return o && o->seen;
  }
  std::string str(const char* lname) const { return find_long_c(lname)->value; }
  int i(const char* lname) const { return std::atoi(find_long_c(lname)->value.c_str()); }
  double d(const char* lname) const { return std::atof(find_long_c(lname)->value.c_str()); }
  bool b(const char* lname) const { return find_long_c(lname)->value == "1"; }

 private:
  Opt* find_long(const std::string& n) {
    for (auto& o : opts_)
      if (o.lname == n) return &o;
    return nullptr;
  }
  Opt* find_short(char c) {
    for (auto& o : opts_)
      if (o.sname == c) return &o;
    return nullptr;
  }
  const Opt* find_long_c(const char* n) const {
    for (auto& o : opts_)
      if (o.lname == n) return &o;
    return nullptr;
  }
  const char* prog_;
  std::vector<Opt> opts_;
};

inline void banner(const char* program_name) {
  std::cout << std::endl
            << "   " << program_name << " (mdsctk_gb300, GB300 implementation of MDSCTK 1.2.5)" << std::endl
            << std::endl;
}

inline bool read_file(const std::string& path, std::vector<char>& buf) {
  std::ifstream f(path.c_str(), std::ios::binary);
  if (!f.good()) return false;
  f.seekg(0, std::ios::end);
  std::streamoff n = f.tellg();
  f.seekg(0, std::ios::beg);
  buf.resize((size_t)n);
  if (n > 0) f.read(buf.data(), n);
  return true;
}

inline bool write_file(const std::string& path, const void* p, size_t n, bool append = false) {
  std::ofstream f(path.c_str(), std::ios::binary | (append ? std::ios::app : std::ios::trunc));
  if (!f.good()) return false;
  f.write(reinterpret_cast<const char*>(p), (std::streamsize)n);
  return f.good();
}

// A binary sparse matrix file (.ssm / .gsm): int n; int pcol[n+1];
// int irow[nnz]; double val[nnz] (CSC_matrix, mdsctk.cpp:44-59).
struct Csc {
  int n = 0;
  std::vector<int32_t> pcol, irow;
  std::vector<double> val;
};

inline bool read_csc(const std::string& path, Csc& m) {
  std::vector<char> b;
  if (!read_file(path, b) || b.size() < sizeof(int)) return false;
  std::memcpy(&m.n, b.data(), sizeof(int));
  if (m.n < 0) return false;
  size_t off = sizeof(int);
  if (b.size() < off + sizeof(int) * (size_t)(m.n + 1)) return false;
  m.pcol.resize(m.n + 1);
  std::memcpy(m.pcol.data(), b.data() + off, sizeof(int) * (m.n + 1));
  off += sizeof(int) * (m.n + 1);
  int64_t nnz = m.pcol[m.n];
  if (nnz < 0 || b.size() < off + (sizeof(int) + sizeof(double)) * (size_t)nnz) return false;
  m.irow.resize(nnz);
  m.val.resize(nnz);
  std::memcpy(m.irow.data(), b.data() + off, sizeof(int) * nnz);
  off += sizeof(int) * nnz;
  std::memcpy(m.val.data(), b.data() + off, sizeof(double) * nnz);
  return true;
}

inline bool write_csc(const std::string& path, int n, const int32_t* pcol, const int32_t* irow, const double* val) {
  std::ofstream f(path.c_str(), std::ios::binary | std::ios::trunc);
  if (!f.good()) return false;
  int64_t nnz = pcol[n];
  f.write(reinterpret_cast<const char*>(&n), sizeof(int));
  f.write(reinterpret_cast<const char*>(pcol), sizeof(int) * (n + 1));
  f.write(reinterpret_cast<const char*>(irow), sizeof(int) * nnz);
  f.write(reinterpret_cast<const char*>(val), sizeof(double) * nnz);
  return f.good();
}

inline int fail(mds_ctx* ctx, int rc) {
  std::cerr << "*** ERROR *** " << (ctx ? mds_last_error(ctx) : "") << " (code " << rc << ")" << std::endl;
  return 2;
}

}  // namespace cli
