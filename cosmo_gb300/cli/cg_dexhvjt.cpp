// Drop-in for DEXHVJTcsb (davidson/DEXHVJTcsb.cpp:36-77): basis, H + lambda J-J+,
// Davidson for the lowest states and the spin analysis of XSHLJT, on the GPU.
//
//   cg_dexhvjt system.xml [-n states] [-i iterations] [-b block] [-f init.EE]
//              [-o out.xml] [--system NAME] [--fp64] [--virtual] [--mbs]
//
// Writes <system>.HH.EE (Davidson::Save layout) and <state> nodes into the XML
// (in place unless -o).  Default: stored FP32 (hi + lo) matrix and the mixed
// solve (resid <= 1e-5); --fp64: FP64 matrix and the reference's FP64 control
// flow (block = states, limit states + 20); --virtual: on-the-fly product
// (nothing stored); --mbs: also write <system>.mbs.  -l limit (default 1000,
// 0: never): a stored matrix of at most that dimension is diagonalized
// exactly in FP64 instead, and the .EE file then holds every state, as the
// reference's DXHV writes it (include/xsm/DEXHVcsb.cxx:80-110).
#include <vector>

#include "cli.h"

int main(int argc, char** argv) {
  cli::Args a = cli::parse(argc, argv, {"-n", "-i", "-b", "-f", "-o", "-l", "--system", "--tol"});
  if (a.pos.size() != 1) {
    std::fprintf(stderr,
                 "usage: cg_dexhvjt system.xml [-n states] [-i iterations] [-b block] [-f init.EE] [-o out.xml]"
                 " [--system NAME] [--fp64] [--virtual] [--mbs]\n");
    return 1;
  }
  const char* xml = a.pos[0].c_str();
  const std::string want = a.gets("--system", "");
  const std::string sys = cli::system_name(xml, want.c_str());
  int nst = a.geti("-n", 0);
  if (nst <= 0) nst = 10;
  const bool fp64 = a.has("--fp64"), virt = a.has("--virtual");
  cg_problem* p;
  cli::check(cg_problem_load_xml(xml, want.empty() ? nullptr : want.c_str(), &p), "load xml");
  cg_basis* b;
  cli::check(cg_basis_build(p, &b), "basis");
  uint64_t n = 0;
  cli::check(cg_basis_dims(b, &n, nullptr), "basis dims");
  std::fprintf(stderr, "dimension %llu\n", (unsigned long long)n);
  if (a.has("--mbs")) cli::check(cg_basis_write_mbs(b, (sys + ".mbs").c_str()), "write .mbs");
  if (uint64_t(nst) > n) nst = int(n);
  const int limit = a.geti("-l", 1000);
  if (!virt && limit > 0 && n <= uint64_t(limit) && n > 0) {
    // exact diagonalization: every state, FP64 matrix
    std::fprintf(stderr, "Matrix is small for davidson. Using exact diagonalization\n");
    cg_hamiltonian* h;
    cli::check(cg_hamiltonian_build(p, b, CG_PREC_FP64, &h), "H");
    std::vector<double> E(n), Z(n), V(size_t(n) * n);
    cli::check(cg_dense_eigensolve(h, E.data(), V.data()), "exact diagonalization");
    for (int k = 0; k < nst; ++k) std::printf("%.10f ", E[k]);
    std::printf("\n");
    const std::string ee = sys + ".HH.EE";
    cli::check(cg_write_ee(ee.c_str(), int32_t(n), n, E.data(), Z.data(), Z.data(), V.data()), "write .EE");
    int32_t added = 0;
    const std::string out = a.gets("-o", "");
    cli::check(cg_xshljt(xml, want.empty() ? nullptr : want.c_str(), ee.c_str(), nst,
                         out.empty() ? nullptr : out.c_str(), &added),
               "xshljt");
    std::fprintf(stderr, "%d states recorded\n", added);
    cg_hamiltonian_destroy(h);
    cg_basis_destroy(b);
    cg_problem_destroy(p);
    return 0;
  }
  const int prec = fp64 ? CG_PREC_FP64 : CG_PREC_FP32;
  cg_hamiltonian* h;
  cli::check(virt ? cg_hamiltonian_build_virtual(p, b, prec, &h) : cg_hamiltonian_build(p, b, prec, &h), "H");
  cg_davidson_params prm;
  cg_davidson_defaults(&prm, nst);
  prm.precision = prec;
  if (a.has("-i")) prm.maxiter = a.geti("-i", prm.maxiter);
  if (fp64) {
    int blk = a.geti("-b", nst);
    prm.block = blk < nst ? nst : blk;  // the reference forces block >= states
    if (prm.block > nst) prm.block = nst;
  } else {
    prm.tol_resid = a.getd("--tol", 1e-5);
    prm.block = nst < 8 ? nst : 8;
    prm.lim = 96;
    prm.keep = 32;
  }
  std::vector<double> init;
  int ninit = 0;
  if (a.has("-f")) {
    uint32_t cnt = 0;
    uint64_t nn = 0;
    FILE* f = std::fopen(a.opt["-f"].c_str(), "rb");
    if (!f) {
      std::fprintf(stderr, "cannot open %s\n", a.opt["-f"].c_str());
      return 1;
    }
    if (std::fread(&cnt, 4, 1, f) == 1) {
      for (uint32_t k = 0; k < cnt; ++k) {
        double hdr[3];
        if (std::fread(hdr, 8, 3, f) != 3 || std::fread(&nn, 8, 1, f) != 1 || nn != n) break;
        init.resize(size_t(ninit + 1) * n);
        if (std::fread(init.data() + size_t(ninit) * n, 8, n, f) != n) break;
        ++ninit;
      }
    }
    std::fclose(f);
  }
  std::vector<double> E(nst), dE(nst), R(nst), V(size_t(nst) * n);
  cg_davidson_stats st;
  cli::check(cg_davidson(h, &prm, ninit ? init.data() : nullptr, ninit, E.data(), dE.data(), R.data(), V.data(),
                         &st),
             "davidson");
  for (int k = 0; k < nst; ++k) std::printf("%.10f ", E[k]);
  std::printf("\n");
  std::fprintf(stderr, "iterations %d + %d refinement, %.3f s, converged %d\n", st.iterations,
               st.refine_iterations, st.seconds, st.converged);
  const std::string ee = sys + ".HH.EE";
  cli::check(cg_write_ee(ee.c_str(), nst, n, E.data(), dE.data(), R.data(), V.data()), "write .EE");
  int32_t added = 0;
  const std::string out = a.gets("-o", "");
  cli::check(cg_xshljt(xml, want.empty() ? nullptr : want.c_str(), ee.c_str(), nst, out.empty() ? nullptr : out.c_str(),
                       &added),
             "xshljt");
  std::fprintf(stderr, "%d states recorded\n", added);
  cg_hamiltonian_destroy(h);
  cg_basis_destroy(b);
  cg_problem_destroy(p);
  return 0;
}
