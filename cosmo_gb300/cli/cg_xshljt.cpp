// Drop-in for XSHLJT (xmlshell/XSHLJT.cpp, include/xsm/XSHLJT.cxx:38-142): spin
// and isospin of the eigenpairs in an .EE file, recorded as <state> nodes of
// the system XML (in place unless -o).
//
//   cg_xshljt system.xml [-n states] [-e file.EE] [-o out.xml] [--system NAME]
//
// The .EE file defaults to <system>.HH.EE, the file cg_dexhvjt writes.
#include "cli.h"

int main(int argc, char** argv) {
  cli::Args a = cli::parse(argc, argv, {"-n", "-e", "-o", "--system"});
  if (a.pos.size() != 1) {
    std::fprintf(stderr, "usage: cg_xshljt system.xml [-n states] [-e file.EE] [-o out.xml] [--system NAME]\n");
    return 1;
  }
  const std::string want = a.gets("--system", "");
  const std::string ee = a.gets("-e", cli::system_name(a.pos[0].c_str(), want.c_str()) + ".HH.EE");
  const std::string out = a.gets("-o", "");
  int32_t added = 0;
  cli::check(cg_xshljt(a.pos[0].c_str(), want.empty() ? nullptr : want.c_str(), ee.c_str(), a.geti("-n", 10),
                       out.empty() ? nullptr : out.c_str(), &added),
             "xshljt");
  std::fprintf(stderr, "%d states recorded\n", added);
  return 0;
}
