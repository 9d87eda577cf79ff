// Drop-in for davidson_vfile (davidson/davidson_vfile.cpp:28-75): Davidson on a
// matrix stored in a .HH file, eigenpairs written to <file>.EE.
//
//   cg_davidson_vfile file.HH [-n states] [-i iterations] [-b block] [-f init.EE] [--fp32]
//
// Default: the FP64 matrix and the reference's FP64 control flow (block =
// max(block, states)); --fp32: FP32 (hi + lo) storage and the mixed solve.
#include <vector>

#include "cli.h"

int main(int argc, char** argv) {
  cli::Args a = cli::parse(argc, argv, {"-n", "-i", "-b", "-f"});
  if (a.pos.size() != 1) {
    std::fprintf(stderr, "usage: cg_davidson_vfile file.HH [-n states] [-i iterations] [-b block] [-f init.EE] [--fp32]\n");
    return 1;
  }
  const std::string hh = a.pos[0];
  const bool fp32 = a.has("--fp32");
  cg_hamiltonian* h;
  cli::check(cg_hamiltonian_read_hh(hh.c_str(), fp32 ? CG_PREC_FP32 : CG_PREC_FP64, &h), "read .HH");
  cg_hamiltonian_info inf;
  cli::check(cg_hamiltonian_get_info(h, &inf), "info");
  const uint64_t n = inf.n;
  int nst = a.geti("-n", 0);
  if (nst <= 0) nst = 10;
  if (uint64_t(nst) > n) nst = int(n);
  cg_davidson_params prm;
  cg_davidson_defaults(&prm, nst);
  prm.precision = fp32 ? CG_PREC_FP32 : CG_PREC_FP64;
  if (a.has("-i")) prm.maxiter = a.geti("-i", prm.maxiter);
  if (fp32) {
    prm.tol_resid = 1e-5;
    prm.block = nst < 8 ? nst : 8;
    prm.lim = 64;
    prm.keep = 32;
  }
  std::vector<double> init;
  int ninit = 0;
  if (a.has("-f")) {
    FILE* f = std::fopen(a.opt["-f"].c_str(), "rb");
    uint32_t cnt = 0;
    uint64_t nn = 0;
    if (f && std::fread(&cnt, 4, 1, f) == 1) {
      for (uint32_t k = 0; k < cnt; ++k) {
        double hdr[3];
        if (std::fread(hdr, 8, 3, f) != 3 || std::fread(&nn, 8, 1, f) != 1 || nn != n) break;
        init.resize(size_t(ninit + 1) * n);
        if (std::fread(init.data() + size_t(ninit) * n, 8, n, f) != n) break;
        ++ninit;
      }
    }
    if (f) std::fclose(f);
  }
  std::vector<double> E(nst), dE(nst), R(nst), V(size_t(nst) * n);
  cg_davidson_stats st;
  cli::check(cg_davidson(h, &prm, ninit ? init.data() : nullptr, ninit, E.data(), dE.data(), R.data(), V.data(),
                         &st),
             "davidson");
  for (int k = 0; k < nst; ++k) std::printf("%.10f ", E[k]);
  std::printf("\n");
  cli::check(cg_write_ee((hh + ".EE").c_str(), nst, n, E.data(), dE.data(), R.data(), V.data()), "write .EE");
  cg_hamiltonian_destroy(h);
  return 0;
}
