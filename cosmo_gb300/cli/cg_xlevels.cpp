// Drop-in for Xlevels (xmlshell/Xlevels.cpp:60-134): the levels of the
// <state>s in a set of XML files, organized together and listed with their
// excitation energies (and the comparison with <data Ex> children).
//
//   cg_xlevels a.xml [b.xml ...] [-o out.xml]
#include <vector>

#include "cli.h"

int main(int argc, char** argv) {
  cli::Args a = cli::parse(argc, argv, {"-o"});
  if (a.pos.empty()) {
    std::fprintf(stderr, "usage: cg_xlevels a.xml [b.xml ...] [-o out.xml]\n");
    return 1;
  }
  std::vector<const char*> f;
  for (const std::string& s : a.pos) f.push_back(s.c_str());
  const std::string out = a.gets("-o", "");
  cli::check(cg_xlevels(f.data(), int32_t(f.size()), out.empty() ? nullptr : out.c_str()), "xlevels");
  return 0;
}
