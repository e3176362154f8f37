// topology.h -- the topology reader of the drop-in tools (what they take from
// GROMACS read_tps_conf in the reference, knn_rms.cpp:150,
// contact_profile.cpp:134): atom count, names, residue names and masses
// from a .pdb or .gro file. Masses are assigned by element, with the masses
// GROMACS uses for the common elements; a PDB's element column (77-78) is
// used when present, else the first letter of the atom name (protein atom
// names: CA = alpha carbon, not calcium). .tpr files are not read.
#pragma once

#include <cctype>
#include <cstdlib>
#include <fstream>
#include <string>
#include <vector>

struct Topology {
  std::vector<std::string> name;     // atom names, blanks trimmed
  std::vector<std::string> resname;  // residue names, blanks trimmed
  std::vector<float> mass;
};

inline float element_mass(const std::string& el) {
  static const std::pair<const char*, float> table[] = {
      {"H", 1.008f},     {"C", 12.011f},   {"N", 14.0067f}, {"O", 15.9994f}, {"S", 32.06f},
      {"P", 30.973762f}, {"F", 18.9984f},  {"CL", 35.45f},  {"BR", 79.904f}, {"I", 126.904f},
      {"NA", 22.98977f}, {"K", 39.0983f},  {"MG", 24.305f}, {"CA", 40.078f}, {"ZN", 65.38f},
      {"FE", 55.845f},   {"SE", 78.971f}};
  for (auto& e : table)
    if (el == e.first) return e.second;
  return 0.0f;
}

// element from a PDB/GRO atom name: leading digits skipped, the first letter
inline std::string element_from_name(const std::string& name) {
  std::string s;
  for (char c : name)
    if (std::isalpha((unsigned char)c)) s += (char)std::toupper((unsigned char)c);
  if (s.empty()) return s;
  return s.substr(0, 1);
}

inline std::string trim_blanks(const std::string& s) {
  size_t a = s.find_first_not_of(" \t\r\n"), b = s.find_last_not_of(" \t\r\n");
  return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
}

inline bool read_topology(const std::string& path, Topology& top) {
  std::ifstream f(path.c_str());
  if (!f.good()) return false;
  top = Topology();
  std::string line;
  const bool gro = path.size() > 4 && path.substr(path.size() - 4) == ".gro";
  if (gro) {
    std::getline(f, line);  // title
    std::getline(f, line);
    const int n = std::atoi(line.c_str());
    for (int i = 0; i < n && std::getline(f, line); ++i) {
      const std::string name = line.size() >= 15 ? line.substr(10, 5) : "";
      top.name.push_back(trim_blanks(name));
      top.resname.push_back(trim_blanks(line.size() >= 10 ? line.substr(5, 5) : ""));
      top.mass.push_back(element_mass(element_from_name(name)));
    }
    return true;
  }
  while (std::getline(f, line)) {
    if (line.rfind("ATOM", 0) != 0 && line.rfind("HETATM", 0) != 0) continue;
    std::string el;
    if (line.size() >= 78) {
      for (char c : line.substr(76, 2))
        if (std::isalpha((unsigned char)c)) el += (char)std::toupper((unsigned char)c);
    }
    const std::string name = line.size() >= 16 ? line.substr(12, 4) : "";
    if (el.empty()) el = element_from_name(name);
    float m = element_mass(el);
    if (m == 0.0f) m = element_mass(el.substr(0, 1));
    top.name.push_back(trim_blanks(name));
    top.resname.push_back(trim_blanks(line.size() >= 20 ? line.substr(17, 3) : ""));
    top.mass.push_back(m);
  }
  return true;
}
