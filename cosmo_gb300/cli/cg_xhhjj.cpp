// Drop-in for XHH+JJ (xmlshell/XHH+JJ.cpp:38-90): H + lambda J-J+ of a system
// built on the GPU and written as the row-sparse .HH file (PPMatrix::Write,
// include/sm/PPMatrix.cxx:413-465).
//
//   cg_xhhjj system.xml [-o file.HH] [--system NAME]
#include "cli.h"

int main(int argc, char** argv) {
  cli::Args a = cli::parse(argc, argv, {"-o", "--system"});
  if (a.pos.size() != 1) {
    std::fprintf(stderr, "usage: cg_xhhjj system.xml [-o file.HH] [--system NAME]\n");
    return 1;
  }
  const std::string want = a.gets("--system", "");
  const std::string out = a.gets("-o", cli::system_name(a.pos[0].c_str(), want.c_str()) + ".HH");
  cg_problem* p;
  cli::check(cg_problem_load_xml(a.pos[0].c_str(), want.empty() ? nullptr : want.c_str(), &p), "load xml");
  cg_basis* b;
  cli::check(cg_basis_build(p, &b), "basis");
  cg_hamiltonian* h;
  cli::check(cg_hamiltonian_build(p, b, CG_PREC_FP64, &h), "H");
  cli::check(cg_hamiltonian_write_hh(h, out.c_str()), "write .HH");
  cg_hamiltonian_info inf;
  cli::check(cg_hamiltonian_get_info(h, &inf), "info");
  std::fprintf(stderr, "%s: dimension %llu, %llu upper entries\n", out.c_str(), (unsigned long long)inf.n,
               (unsigned long long)inf.nnz_upper);
  cg_hamiltonian_destroy(h);
  cg_basis_destroy(b);
  cg_problem_destroy(p);
  return 0;
}
