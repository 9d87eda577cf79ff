// Drop-in for Xsysmbs / XsysmbsOMP (xmlshell/xmbs/Xsysmbs.cpp:53-414): the
// M-scheme basis of a system written as a .mbs file (int32 N, uint64 n, n x N
// uint16; Many_Body_States::Write, include/sm/ManyBodyStates.cxx:199-206),
// enumerated on the GPU.
//
//   cg_xsysmbs system.xml [-o file.mbs] [--system NAME]
#include "cli.h"

int main(int argc, char** argv) {
  cli::Args a = cli::parse(argc, argv, {"-o", "--system"});
  if (a.pos.size() != 1) {
    std::fprintf(stderr, "usage: cg_xsysmbs system.xml [-o file.mbs] [--system NAME]\n");
    return 1;
  }
  const std::string want = a.gets("--system", "");
  const std::string out = a.gets("-o", cli::system_name(a.pos[0].c_str(), want.c_str()) + ".mbs");
  cg_problem* p;
  cli::check(cg_problem_load_xml(a.pos[0].c_str(), want.empty() ? nullptr : want.c_str(), &p), "load xml");
  cg_basis* b;
  cli::check(cg_basis_build(p, &b), "basis");
  uint64_t n = 0;
  int32_t N = 0;
  cli::check(cg_basis_dims(b, &n, &N), "dims");
  cli::check(cg_basis_write_mbs(b, out.c_str()), "write .mbs");
  std::fprintf(stderr, "%s: %llu states of %d particles\n", out.c_str(), (unsigned long long)n, N);
  cg_basis_destroy(b);
  cg_problem_destroy(p);
  return 0;
}
