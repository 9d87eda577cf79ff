// Test-infrastructure harness (oracle side, never shipped): calls the reference
// CoSMo headers as they lie in the reference tree and dumps every intermediate
// of the CI hot path so the GB300 library can be pinned against it.
//
// It follows the logic of xsm::DXHV (include/xsm/DEXHVcsb.cxx:33-71) without
// the Eigen fallback, which is the path DEXHVJTcsb (davidson/DEXHVJTcsb.cpp:36)
// runs for n > limit.
//
// usage: ref_dump <system.xml> <out_prefix> [nstates iters block]
//   block defaults to max(10, nstates), as DEXHVJTcsb forces (davidson/DEXHVJTcsb.cpp:52,58)
//   <out_prefix>.sps.txt    s.p. table            (SM::Make, xSingleParticleStates.cxx:26)
//   <out_prefix>.esp.txt    one-body terms ESP    (xReadSPInt, xReadSPInt.cxx:24)
//   <out_prefix>.vspx.txt   two-body terms VSPX   (forward ordered, incl. lambda*J-J+)
//   <system>.mbs            basis, written by SM::Get -> MakeMBS2 into the cwd
//   <out_prefix>.rows.bin   upper-triangle H from PPMatrix2CSBBlk (PPMatrix.cxx:571)
//                           as u64 nnz, u32 row[nnz], u32 col[nnz], f64 val[nnz]
//                           sorted by (row, col)
//   <out_prefix>.spmm.bin   u64 n, u32 m, f64 x[m*n], f64 y[m*n] with y = H x from
//                           SparseMatrixCSB::TimesMatrix (csbmatrix.cxx:680)
//   <out_prefix>.EE         DavidsonDiagonalization output (kdav/davidson.cxx:168)
#include <cstdint>
typedef uint16_t spsint;
typedef unsigned long long uint_nbasis;
#include <av/argparser.cxx>
#include <av/statusclass.cxx>
#include <chrono>
#include <xsm/xManyBodyStates.cxx>
#include <xsm/xsphericalint.cxx>
#include <sm/MakeSPO.cxx>
#include <sm/spherical2sp.cxx>
#include <tav/sparse.cxx>
#include <tav/csbmatrix.cxx>
#include <xsm/xReadSPInt.cxx>
#include <sm/PPMatrix.cxx>
#include <kdav/davidson.cxx>
#include <algorithm>
#include <cstdio>
#include <string>
#include <vector>

static double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

int main(int argc, char** argv) {
  if (argc < 3) {
    std::fprintf(stderr, "usage: ref_dump <system.xml> <out_prefix> [nstates iters]\n");
    return 2;
  }
  std::string prefix = argv[2];
  int nstates = argc > 3 ? std::atoi(argv[3]) : 0;
  int iters = argc > 4 ? std::atoi(argv[4]) : 0;
  int block = argc > 5 ? std::atoi(argv[5]) : 10;
  if (block < nstates) block = nstates;

  XMLNode xMainNode = XMLNode::openFileHelper(argv[1], xsm::cosmo);
  XMLNode xSystemNode = xml::SelectNode(xMainNode, xsm::system, "name");
  SM::SingleParticleStates sps;
  Make(sps, xMainNode.getChildNode(xsm::valencespace));
  {
    FILE* f = std::fopen((prefix + ".sps.txt").c_str(), "w");
    for (size_t i = 0; i < sps.size(); ++i)
      std::fprintf(f, "%zu %d %d %d %d %d %d %d %d\n", i, sps[i].level, int(sps[i].N), int(sps[i].L),
                   int(sps[i].J), int(sps[i].Jz), int(sps[i].T), int(sps[i].Tz), int(sps[i].P));
    std::fclose(f);
  }
  SM::Many_Body_States st;
  double t0 = now_s();
  SM::Get(st, xMainNode, xSystemNode);
  double t1 = now_s();
  std::fprintf(stderr, "ref_dump: basis n=%llu N=%d (%.3f s)\n", (unsigned long long)st.n, st.N, t1 - t0);

  tav::STensor<spsint, double> ESP(2);
  tav::STensor<spsint, double> VSPX(4);
  xReadSPInt(ESP, VSPX, xSystemNode, xMainNode, sps);
  {
    FILE* f = std::fopen((prefix + ".esp.txt").c_str(), "w");
    for (auto it = ESP.begin(); it != ESP.end(); ++it)
      std::fprintf(f, "%d %d %.17g\n", int(it->first[0]), int(it->first[1]), it->second);
    std::fclose(f);
    f = std::fopen((prefix + ".vspx.txt").c_str(), "w");
    for (auto it = VSPX.begin(); it != VSPX.end(); ++it)
      std::fprintf(f, "%d %d %d %d %.17g\n", int(it->first[0]), int(it->first[1]), int(it->first[2]),
                   int(it->first[3]), it->second);
    std::fclose(f);
  }
  if (st.n == 0) return 0;

  SM::PPMatrix HH(st);
  HH.push_back(&ESP);
  HH.push_back(&VSPX);
  uint16_t br = std::sqrt(1. * st.n) + 1;
  tav::SparseMatrixCSB<double, uint32_t, uint16_t> FHH(st.n, br, br, true);
  double t2 = now_s();
  PPMatrix2CSBBlk(FHH, HH);
  double t3 = now_s();

  // Flatten the CSB blocks into a sorted (row, col, val) list.
  struct E { uint32_t r, c; double v; };
  std::vector<E> ent;
  for (int i = 0; i < FHH.numBlockRow; i++)
    for (int j = 0; j < FHH.numBlockCol; j++) {
      auto& B = FHH.Blocks[i][j];
      for (uint32_t k = 0; k < B.nnz; ++k)
        ent.push_back({uint32_t(i) * br + B.indRow[k], uint32_t(j) * br + B.indCol[k], B.elem[k]});
    }
  std::sort(ent.begin(), ent.end(), [](const E& a, const E& b) { return a.r != b.r ? a.r < b.r : a.c < b.c; });
  std::fprintf(stderr, "ref_dump: csb build %.3f s, nnz_upper=%zu, br=%d\n", t3 - t2, ent.size(), int(br));
  {
    FILE* f = std::fopen((prefix + ".rows.bin").c_str(), "wb");
    uint64_t nnz = ent.size();
    std::fwrite(&nnz, 8, 1, f);
    for (auto& e : ent) std::fwrite(&e.r, 4, 1, f);
    for (auto& e : ent) std::fwrite(&e.c, 4, 1, f);
    for (auto& e : ent) std::fwrite(&e.v, 8, 1, f);
    std::fclose(f);
  }
  {
    // y = H x for three deterministic vectors through the reference's own SpMM.
    const uint32_t m = 3;
    uint64_t n = st.n;
    std::vector<double> x(m * n), y(m * n, 0.0);
    for (uint32_t k = 0; k < m; ++k)
      for (uint64_t i = 0; i < n; ++i) x[k * n + i] = std::sin(0.37 * double(i) + 1.1 * k) + 0.25 * k;
    double t4 = now_s();
    FHH.TimesMatrix(y.data(), x.data(), m);
    double t5 = now_s();
    std::fprintf(stderr, "ref_dump: spmm m=%u %.4f s\n", m, t5 - t4);
    FILE* f = std::fopen((prefix + ".spmm.bin").c_str(), "wb");
    std::fwrite(&n, 8, 1, f);
    std::fwrite(&m, 4, 1, f);
    std::fwrite(x.data(), 8, m * n, f);
    std::fwrite(y.data(), 8, m * n, f);
    std::fclose(f);
  }
  if (nstates > 0) {
    double t6 = now_s();
    DavidsonDiagonalization((prefix + ".EE").c_str(), FHH, block, iters, nstates);
    double t7 = now_s();
    std::fprintf(stderr, "ref_dump: davidson %.3f s\n", t7 - t6);
  }
  return 0;
}
