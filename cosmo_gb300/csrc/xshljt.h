// XSHLJT: spin / isospin of eigenpairs and the <state> nodes of the system XML
// (include/xsm/XSHLJT.cxx:38-142, include/xsm/xState.cxx:113-236).
#pragma once
#include <string>
#include <vector>

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

// XSHLSF (xmlshell/XSHLSF.cpp:40-222): spectroscopic factors between the
// states of a parent system and a daughter system with one particle less
// (overlaps when the particle numbers are equal), table written to out_path
// (none when empty), per orbital l or, with full, per s.p. state.
void xshlsf(const std::string& parent_xml, const std::string& parent_system, const std::string& daughter_xml,
            const std::string& daughter_system, const std::string& out_path, bool full);

}  // namespace cg
