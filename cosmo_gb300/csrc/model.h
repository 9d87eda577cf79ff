// Host-side model of one CI problem: the XML system description, the m-scheme
// single-particle table and the m-scheme Hamiltonian operator terms.
//
// Everything here is setup-sized (at most a few thousand s.p. pairs); the large
// objects (basis, Hamiltonian, vectors) live on the GPU.
#pragma once
#include <array>
#include <cstdint>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

namespace cg {

// Error carrying a C-ABI status code; never crosses the C ABI.
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

// ---------------------------------------------------------------- XML subset
struct XmlNode {
  std::string tag;
  std::vector<std::pair<std::string, std::string>> attrs;
  std::string text;
  std::vector<XmlNode> children;
  const std::string* attr(const std::string& k) const;
  const XmlNode* child(const std::string& t, int index = 0) const;
  int count(const std::string& t) const;
};
XmlNode parse_xml_file(const std::string& path);
// doubled spin from its text form ("5/2" -> 5, "3" -> 6)
int parse_spin2(const std::string& t);

// ---------------------------------------------------------- s.p. states
// One m-scheme single-particle state.  Quantum numbers are stored doubled
// where they can be half-integer (j2 = 2j, m2 = 2m, t2 = 2t, tz2 = 2tz), as in
// the reference's `spin` class (include/sm/spinclass.cxx).
struct SPState {
  int level;   // orbit index (XML index - 1)
  int n, l;    // radial and orbital quantum numbers
  int j2, m2;  // 2j, 2m
  int t2, tz2; // 2t (=1), 2tz: +1 neutron, -1 proton
  int parity;  // l & 1 unless given explicitly
};

struct Orbit {
  std::string name;
  int index;  // XML index (1-based)
  int n, l, j2, parity, t2;
  std::string type;  // "pn", "p" or "n"
};

// A CI problem: valence space, particle numbers, M sector and interaction files.
struct System {
  std::string name;
  std::vector<Orbit> orbits;     // sorted by XML index
  std::vector<SPState> sps;      // neutrons first, then protons
  int n_neutron_states = 0;      // sps[0, n_neutron_states) are neutrons
  int nv = 0, zv = 0;            // valence neutrons / protons
  int twom = 0;                  // 2 * Jz
  int parity = 0;                // 0 for '+', 1 for '-'
  double jj = 0.0;               // lambda of lambda * J-J+
  bool has_jj = false;
  std::vector<std::string> int_files;
  std::vector<std::array<double, 10>> int_scale;  // per file, rank-indexed scaling
  std::string mbs_name;          // ManyBodyStates name attribute (may be empty)
  int filter_twoJ = -1;          // system J / T attributes: XSHLJT keeps only these states
  int filter_twoT = -1;
  std::string xml_dir;
  // basis truncations of the system node (hwmax attribute, <hwrejection>,
  // <rejection>, xmlshell/xmbs/XsysmbsOMP.cpp:214-300), listed; the basis
  // builder refuses a truncated system instead of building the full basis
  std::string truncation;
};

System load_system(const std::string& xml_path, const std::string& system_name);

// Throws CG_ERR_UNSUPPORTED for a system with a basis truncation: every route
// that builds a basis (single problem, batch, XSHLJT) calls it before any
// device work, so no truncated system is ever solved on the full basis.
void refuse_truncated(const System& sys);

// ------------------------------------------------------------ operators
// Forward-ordered m-scheme operator terms.  Keys follow the reference's
// STensor convention: the first half of a key is annihilated, the second half
// created; one-body (i, f) with i <= f, two-body (b0 < b1 ; b2 < b3) with
// (b0, b1) <= (b2, b3) lexicographically.
using Key2 = std::array<int, 2>;
using Key4 = std::array<int, 4>;
struct Operator {
  std::map<Key2, double> one;  // ESP
  std::map<Key4, double> two;  // VSPX
};

// Spherical Oxbash interaction as read from the files.
struct SphericalInt {
  std::vector<double> spe;                    // ENT, per orbit level
  std::map<std::array<int, 6>, double> tbme;  // (c, d, a, b, J, T) as the reference keys it
};

SphericalInt read_oxbash(const System& sys);
Operator build_operator(const System& sys);

// Clebsch-Gordan coefficient <j1 m1 j2 m2 | j3 m3>, all arguments doubled.
double clebsch_gordan(int j1, int m1, int j2, int m2, int j3, int m3);

}  // namespace cg
