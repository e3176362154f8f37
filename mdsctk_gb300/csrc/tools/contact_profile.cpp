// contact_profile -- drop-in for MDSCTK's contact_profile (contact_profile.cpp):
// the standard atomic contacts of every frame of an .xtc trajectory between
// two atom groups, as sparse binary vectors, computed by libmdsgpu on the GPU.
// Same options and outputs:
//   -e cutoff in Angstrom (9.0), -p topology (.pdb/.gro), -x trajectory
//   (.xtc, or raw float32 frames), -n index file (.ndx), -i/-d the sparse
//   vector index file (records [int n][int idx[n]], idx = i * n2 + j of the
//   pairs (group1[i], group2[j]) in contact, ascending) and data file
//   (records [double 1.0 ...]); defaults reference.svi / reference.svd.
// The two groups are chosen as GROMACS get_index does: the groups are listed
// and two group numbers are read from standard input (or given with
// --group1/--group2). Groups come from the .ndx file; without one, the
// default groups offered are System, C-alpha (atoms named CA), Backbone
// (N, CA, C) and Heavy (non-hydrogen atoms) -- GROMACS derives a longer
// default list from residue tables, so with -n the numbering matches
// GROMACS exactly and without it only these four groups exist.
// An atom count that differs between the topology and the trajectory exits
// with status 4, as the reference does (contact_profile.cpp:144-153).
#include <iomanip>
#include <sstream>

#include "cli.h"
#include "frames.h"
#include "topology.h"

struct Group {
  std::string name;
  std::vector<int> atoms;  // 0-based
};

static bool read_ndx(const std::string& path, std::vector<Group>& groups) {
  std::ifstream f(path.c_str());
  if (!f.good()) return false;
  std::string line;
  while (std::getline(f, line)) {
    const std::string t = trim_blanks(line);
    if (t.empty()) continue;
    if (t[0] == '[') {
      const size_t e = t.find(']');
      groups.push_back(Group{trim_blanks(t.substr(1, e == std::string::npos ? std::string::npos : e - 1)), {}});
      continue;
    }
    if (groups.empty()) continue;
    std::istringstream is(t);
    long a;
    while (is >> a) groups.back().atoms.push_back((int)(a - 1));
  }
  return true;
}

static void default_groups(const Topology& top, std::vector<Group>& groups) {
  Group sys{"System", {}}, ca{"C-alpha", {}}, bb{"Backbone", {}}, heavy{"Heavy", {}};
  for (int a = 0; a < (int)top.name.size(); ++a) {
    const std::string& n = top.name[a];
    sys.atoms.push_back(a);
    if (n == "CA") ca.atoms.push_back(a);
    if (n == "N" || n == "CA" || n == "C") bb.atoms.push_back(a);
    if (element_from_name(n) != "H") heavy.atoms.push_back(a);
  }
  groups = {sys, ca, bb, heavy};
}

static int choose_group(const std::vector<Group>& groups, const cli::Parser& p, const char* opt) {
  for (size_t g = 0; g < groups.size(); ++g)
    std::cout << "Group " << std::setw(5) << g << " (" << std::setw(15) << groups[g].name << ") has "
              << std::setw(6) << groups[g].atoms.size() << " elements" << std::endl;
  int sel = -1;
  if (p.is_set(opt)) {
    sel = p.i(opt);
  } else {
    std::cout << "Select a group: ";
    std::cout.flush();
    if (!(std::cin >> sel)) sel = -1;
  }
  if (sel < 0 || sel >= (int)groups.size()) return -1;
  std::cout << "Selected " << sel << ": '" << groups[sel].name << "'" << std::endl;
  return sel;
}

int main(int argc, char** argv) {
  const char* prog = "contact_profile";
  cli::banner(prog);
  std::cout << "   Computes the standard atomic contacts for structures in" << std::endl
            << "   the given xtc file. A topology PDB file and atom index file" << std::endl
            << "   should be provided for determining the atoms to compare." << std::endl
            << "   The resulting sparse contact distance profiles are" << std::endl
            << "   in sparse vector format (index-file and data-file)." << std::endl << std::endl;
  cli::Parser p(prog);
  p.add("threads", 't', cli::INT, "Input:  Number of threads to start (int; accepted, the GPU is used)", "1");
  p.add("epsilon", 'e', cli::DOUBLE, "Input:  Contact cutoff (real)", "9.0");
  p.add("topology-file", 'p', cli::STRING, "Input:  Topology file [.pdb,.gro] (string:filename)", "topology.pdb");
  p.add("xtc-file", 'x', cli::STRING, "Input:  Trajectory file (string:filename)", "traj.xtc");
  p.add("ndx-file", 'n', cli::STRING, "Input:  Index file with the atom groups (string:filename)");
  p.add("index-file", 'i', cli::STRING, "Output: Sparse vector indices file (string:filename)", "reference.svi");
  p.add("data-file", 'd', cli::STRING, "Output: Sparse vector data file (string:filename)", "reference.svd");
  p.add("group1", 0, cli::INT, "Input:  First group number (int; default: read from standard input)");
  p.add("group2", 0, cli::INT, "Input:  Second group number (int; default: read from standard input)");
  p.add("device", 0, cli::INT, "Input:  CUDA device (int)", "0");
  int pr = p.parse(argc, argv);
  if (pr == 1) return 1;
  if (pr < 0) return -1;
  std::cout << "Running with the following options:" << std::endl
            << "topology-file = " << p.str("topology-file") << std::endl
            << "xtc-file =      " << p.str("xtc-file") << std::endl
            << "ndx-file =      " << (p.is_set("ndx-file") ? p.str("ndx-file") : std::string()) << std::endl
            << "index-file =    " << p.str("index-file") << std::endl
            << "data-file =     " << p.str("data-file") << std::endl << std::endl;
  std::cout << "Reading topology information from " << p.str("topology-file") << " ... ";
  Topology top;
  if (!read_topology(p.str("topology-file"), top) || top.name.empty()) {
    std::cout << std::endl << "*** ERROR *** could not read atoms from " << p.str("topology-file") << std::endl;
    return -1;
  }
  std::cout << "done." << std::endl;
  const int natoms = (int)top.name.size();
  mds_ctx* ctx = nullptr;
  int rc = mds_create(p.i("device"), 0, &ctx);
  if (rc) return cli::fail(ctx, rc);
  std::vector<float> x;
  int nframes = 0, xtc_atoms = 0;
  const int fr = read_frames(ctx, p.str("xtc-file"), natoms, x, nframes, &xtc_atoms);
  if (fr == -4) {
    std::cout << "*** ERROR ***" << std::endl
              << "Number of atoms in topology file (" << natoms << ") does not match the number of atoms in the XTC file ("
              << p.str("xtc-file") << " : " << xtc_atoms << ")." << std::endl;
    mds_destroy(ctx);
    return 4;
  }
  if (fr != 0) {
    std::cout << "***ERROR***" << std::endl << "Could not read coordinates from " << p.str("xtc-file") << std::endl;
    mds_destroy(ctx);
    return -1;
  }
  std::vector<Group> groups;
  if (p.is_set("ndx-file")) {
    if (!read_ndx(p.str("ndx-file"), groups) || groups.empty()) {
      std::cout << "*** ERROR *** could not read groups from " << p.str("ndx-file") << std::endl;
      mds_destroy(ctx);
      return -1;
    }
  } else {
    default_groups(top, groups);
  }
  std::cout << "Please select two (non-overlapping) groups for contact profiling..." << std::endl;
  const int s1 = choose_group(groups, p, "group1");
  if (s1 < 0) {
    std::cout << "*** ERROR *** invalid group" << std::endl;
    mds_destroy(ctx);
    return -1;
  }
  std::cout << std::endl;
  const int s2 = choose_group(groups, p, "group2");
  if (s2 < 0) {
    std::cout << "*** ERROR *** invalid group" << std::endl;
    mds_destroy(ctx);
    return -1;
  }
  std::cout << std::endl;
  const std::vector<int>& g1 = groups[s1].atoms;
  const std::vector<int>& g2 = groups[s2].atoms;
  for (int a : g1)
    if (a < 0 || a >= natoms) {
      std::cout << "*** ERROR *** atom " << a + 1 << " of group " << s1 << " is not in the topology" << std::endl;
      mds_destroy(ctx);
      return -1;
    }
  for (int a : g2)
    if (a < 0 || a >= natoms) {
      std::cout << "*** ERROR *** atom " << a + 1 << " of group " << s2 << " is not in the topology" << std::endl;
      mds_destroy(ctx);
      return -1;
    }
  std::cout << "Total grid size is " << g1.size() << " x " << g2.size() << " = " << (g1.size() * g2.size())
            << std::endl;
  std::vector<int64_t> off((size_t)nframes + 1, 0);
  std::vector<int32_t> idx;
  if (nframes > 0 && !g1.empty() && !g2.empty()) {
    rc = mds_contact_profile(ctx, x.data(), nframes, natoms, g1.data(), (int)g1.size(), g2.data(), (int)g2.size(),
                             p.d("epsilon"), off.data(), nullptr, 0);
    if (rc) return cli::fail(ctx, rc);
    idx.resize((size_t)std::max<int64_t>(off[nframes], 1));
    rc = mds_contact_profile(ctx, x.data(), nframes, natoms, g1.data(), (int)g1.size(), g2.data(), (int)g2.size(),
                             p.d("epsilon"), off.data(), idx.data(), (int64_t)idx.size());
    if (rc) return cli::fail(ctx, rc);
  }
  mds_destroy(ctx);
  // records: [int total][int idx...] and [double 1.0 ...] per frame
  std::vector<char> ib, db;
  for (int f = 0; f < nframes; ++f) {
    const int32_t total = (int32_t)(off[f + 1] - off[f]);
    const char* t = reinterpret_cast<const char*>(&total);
    ib.insert(ib.end(), t, t + sizeof(total));
    const char* ii = reinterpret_cast<const char*>(idx.data() + off[f]);
    ib.insert(ib.end(), ii, ii + sizeof(int32_t) * (size_t)total);
    const double one = 1.0;
    for (int32_t e = 0; e < total; ++e) {
      const char* o = reinterpret_cast<const char*>(&one);
      db.insert(db.end(), o, o + sizeof(one));
    }
  }
  if (!cli::write_file(p.str("index-file"), ib.data(), ib.size()) ||
      !cli::write_file(p.str("data-file"), db.data(), db.size())) {
    std::cout << "***ERROR*** could not write the output files" << std::endl;
    return -1;
  }
  std::cout << std::endl << std::endl;
  return 0;
}
