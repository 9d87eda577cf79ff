// Drop-in for XSHLAO (xmlshell/XSHLAO.cpp:22-101): occupation numbers of every
// orbital (neutrons and protons apart) for the <state>s of a system, added to
// the states as <occupation name N Z/> nodes.
//
//   cg_xshlao system.xml [-o out.xml] [--system NAME]
#include "cli.h"

int main(int argc, char** argv) {
  cli::Args a = cli::parse(argc, argv, {"-o", "--system"});
  if (a.pos.size() != 1) {
    std::fprintf(stderr, "usage: cg_xshlao system.xml [-o out.xml] [--system NAME]\n");
    return 1;
  }
  const std::string out = a.gets("-o", ""), sys = a.gets("--system", "");
  cli::check(cg_xshlao(a.pos[0].c_str(), sys.empty() ? nullptr : sys.c_str(), out.empty() ? nullptr : out.c_str()),
             "xshlao");
  return 0;
}
