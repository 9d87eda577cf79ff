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

// Basis truncation of a system (XsysmbsOMP, xmlshell/xmbs/XsysmbsOMP.cpp:
// 214-300): oscillator quanta Q = sum of 2n + l over the occupied states,
// counted above the core quanta Ncore / Pcore (the quanta of the first Nv
// neutron / Zv proton s.p. states in list order, SM::CoreQuanta,
// include/sm/SingleParticleStates.cxx:155-168); a neutron configuration is
// kept when Qn - Ncore is in [0, hwmax], a proton one when Qp - Pcore is, a
// determinant when (Qn - Ncore) + (Qp - Pcore) is in [hwmin, hwmax]
// (PartitionClass.cxx:151-190, 390-413); and for each rejection the number
// of particles in its flagged s.p. states is in [nmin, nmax]
// (TestRestriction, PartitionClass.cxx:23-40).
struct Truncation {
  bool hw = false;
  int hwmin = 0, hwmax = 0;
  struct Rejection {
    int nmin = 0, nmax = 0;
    uint64_t mask = 0;          // flagged s.p. states (global index, neutrons first; spaces of <= 64 states)
    uint64_t nmask = 0, pmask = 0;  // the same per species (species-local bits)
  };
  std::vector<Rejection> rejections;
  bool active() const { return hw || !rejections.empty(); }
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
  // basis truncations of the system node (hwmax, <hwrejection>, <rejection>),
  // listed in `truncation` and given in `trunc`
  std::string truncation;
  Truncation trunc;
};

System load_system(const std::string& xml_path, const std::string& system_name);

// Oscillator quanta 2n + l of s.p. state i.
inline int sp_quanta(const SPState& s) { return 2 * s.n + s.l; }

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

// One-body raising operators keyed (annihilated, created): J+ (SPJPlus, same
// orbit and species, m -> m + 1, sqrt((j - m)(j + m + 1))) and T+ (SPTPlus,
// proton -> neutron in the same orbit and m, value 1), include/sm/
// spherical2sp.cxx:629-700; and the Hermitian square O+ O of such an operator
// as forward-ordered one- and two-body terms (SPSqrM + StripHermitianOperator,
// include/sm/cioperators.cxx:200-287): <psi| O+ O |psi> = ||O psi||^2, which
// gives <J-J+> and <T-T+> in the basis of psi itself.
std::map<Key2, double> j_plus_terms(const std::vector<SPState>& sps);
std::map<Key2, double> t_plus_terms(const System& sys);
Operator square_operator(const std::map<Key2, double>& raise);

// Clebsch-Gordan coefficient <j1 m1 j2 m2 | j3 m3>, all arguments doubled.
double clebsch_gordan(int j1, int m1, int j2, int m2, int j3, int m3);

}  // namespace cg
