// XSHLJT: spin / isospin of eigenpairs and the <state> nodes of the system XML
// (include/xsm/XSHLJT.cxx:38-142, include/xsm/xState.cxx:113-236).
#pragma once
#include <cstdint>
#include <string>
#include <utility>
#include <vector>

#include "em.h"
#include "model.h"

namespace cg {

struct Basis;

struct NewState {
  int twoJ = -1, twoT = -1, parity = 0, twoJz = 0, twoTz = 0, id = 0;
  double E = 0, dE = 0;  // E with the lambda * J-J+ penalty removed
  std::string file;
};

// "5/2" for odd, "3" for even doubled spins (SM::spin's string form)
std::string spin_text(int twice);

// The XML text with the system's <state> children merged with `add` and
// re-organised (AddState + OrganizeStates); everything else unchanged.
std::string xml_add_states(const std::string& text, const std::string& system_name,
                           const std::vector<NewState>& add);

// Read the first nstates (all when <= 0) eigenpairs of an .EE file, compute
// <J-J+> / <T-T+> on the GPU and return the state records XSHLJT would add.
std::vector<NewState> xshljt_states(const System& sys, const Basis& b, const std::string& ee_path, int nstates,
                                    const std::string& file_attr, std::vector<double>* jj_out,
                                    std::vector<double>* tt_out);

// A <state> child of a system node with its <wavefunction> (the first one):
// J, T, P, E (as written), name, Ex; Jz, Tz, .EE file and index
// (include/xsm/xState.cxx:23-46).
struct StateRecord {
  std::string name, ex, e_text;
  int twoJ = 0, twoT = 0, parity = 0, twoJz = 0, twoTz = 0, id = 0;
  double E = 0;
  std::string file;
};
std::vector<StateRecord> read_states(const std::string& xml_path, const std::string& system_name);
// vector `id` of an .EE file (as given, else beside the XML: xml_dir), its
// energy in *energy when not null
std::vector<double> read_vector(const std::string& file, const std::string& xml_dir, int id, uint64_t n,
                                double* energy);
std::string dir_of(const std::string& path);

// Child element text added to the <state> children of a system, in document
// order: front[k] right after the start tag of state k, back[k] before its end
// tag (a self-closed state gets an end tag).  Everything else is unchanged.
std::string xml_state_children(const std::string& text, const std::string& system_name,
                               const std::vector<std::vector<std::string>>& front,
                               const std::vector<std::vector<std::string>>& back);
// Attributes appended to the index-th <operator> element (in document order).
std::string xml_append_attrs(const std::string& text, const std::string& tag, int index,
                             const std::vector<std::pair<std::string, std::string>>& attrs);
// The text form of a double as the reference's addAttribute writes it (the
// default C++ stream format, 6 significant digits).
std::string num_text(double x);

// XSHLSF (xmlshell/XSHLSF.cpp:40-222): spectroscopic factors between the
// states of a parent system and a daughter system with one particle less
// (overlaps when the particle numbers are equal), table written to out_path
// (none when empty), per orbital l or, with full, per s.p. state.
void xshlsf(const std::string& parent_xml, const std::string& parent_system, const std::string& daughter_xml,
            const std::string& daughter_system, const std::string& out_path, bool full);

}  // namespace cg

namespace cg {

// XSHLEMB (xmlshell/XSHLEMB.cpp:116-372): reduced transition probabilities
// B(op) between the states of a parent system and a daughter system (the
// parent itself when daughter_xml is empty) for the <operator> node of the
// parent XML (the first one, or the one named `op_name`), written as
// <transition> (and, for diagonal elements of K < 3, <moment>) children of
// the parent's states into out_xml (the parent XML when empty).  Options:
// Weisskopf units (-w), standard units (-u), log ft (-ft), oscillator radial
// functions positive at infinity (-p).
struct XshlembOptions {
  bool weisskopf = false, units = false, logft = false, phase_infinity = false;
  std::string op_name;
};
// The <operator> child of the XML root named op_name (the first one when
// empty) as a TransitionOp; *index: its position among the <operator> nodes;
// *added: the M-operator attributes that were absent and took their defaults.
TransitionOp read_transition_operator(const XmlNode& root, const std::string& op_name, bool phase_infinity, int* index,
                                      std::vector<std::pair<std::string, std::string>>* added);
// Xlevels (xmlshell/Xlevels.cpp:60-134): the <state>s of every space of the
// files that holds some, organized together (energy order, names J P (k),
// Ex from the lowest) and listed one per line as "name T=T Ex E [Ex(data)]",
// with the mean shift and RMS against <data Ex> children when there are any;
// the organized states written to out_xml when not empty.  Returns the listing.
std::string xlevels(const std::vector<std::string>& files, const std::string& out_xml);
// XSHLAO (xmlshell/XSHLAO.cpp:22-101): orbital occupation numbers of the
// system's <state>s as <occupation name N Z/> children, into out_xml (the
// input when empty).
void xshlao(const std::string& xml, const std::string& system_name, const std::string& out_xml);
void xshlemb(const std::string& parent_xml, const std::string& parent_system, const std::string& daughter_xml,
             const std::string& daughter_system, const std::string& out_xml, const XshlembOptions& opt);

}  // namespace cg
