// Test-infrastructure harness (oracle side, never shipped): the <J-J+> and
// <T-T+> computation of the reference's XSHLJT (include/xsm/XSHLJT.cxx:38-142)
// run with the reference headers as they lie in the reference tree, printing
// full-precision values instead of XSHLJT's 6-digit log lines, plus the
// eigenvectors it read, so the GPU kernel can be pinned to the same numbers.
//
// usage: ref_jt <system.xml> <file.EE> <nstates> <out_prefix>
//   <out_prefix>.jt.txt    per state: E dE dV <J-J+> <T-T+> 2J 2T
//   <out_prefix>.vecs.bin  nstates x n doubles (the vectors as read)
#include <cstdint>
typedef uint16_t spsint;
typedef unsigned long long uint_nbasis;
#include <sm/SingleParticleStates.cxx>
#include <xsm/xManyBodyStates.cxx>
#include <xsm/xState.cxx>
#include <sm/parityclass.cxx>
#include <sm/spherical2sp.cxx>
#include <sm/PPMatrix.cxx>
#include <cstdio>
#include <fstream>
#include <string>

int main(int argc, char** argv) {
  if (argc < 5) {
    std::fprintf(stderr, "usage: ref_jt <system.xml> <file.EE> <nstates> <out_prefix>\n");
    return 2;
  }
  XMLNode xMainNode = XMLNode::openFileHelper(argv[1], xsm::cosmo);
  XMLNode xSystemNode = xml::SelectNode(xMainNode, xsm::system, "name");
  SM::SingleParticleStates sps;
  Make(sps, xMainNode.getChildNode(xsm::valencespace));
  SM::QN x;
  ReadXMLQN(x, xSystemNode);
  SM::Many_Body_States st;
  SM::Get(st, xMainNode, xSystemNode);
  tav::STensor<spsint, double> JO(2);
  SM::SPJPlus(JO, sps);
  tav::STensor<spsint, double> TO(2);
  SM::SPTPlus(TO, sps);
  SM::PPMatrix JJ(st);
  JJ.push_back(&JO);
  SM::PPMatrix TT(st);
  TT.push_back(&TO);
  std::ifstream inf(argv[2], std::ios::binary);
  unsigned count = 1;
  rw::Read(count, inf);
  int want = std::atoi(argv[3]);
  if (want > 0 && unsigned(want) < count) count = unsigned(want);
  std::string prefix = argv[4];
  FILE* ft = std::fopen((prefix + ".jt.txt").c_str(), "w");
  FILE* fv = std::fopen((prefix + ".vecs.bin").c_str(), "wb");
  tav::Tensor<1, double> z;
  for (unsigned k = 0; k < count; ++k) {
    double E, dE, dV;
    rw::Read(E, inf);
    rw::Read(dE, inf);
    rw::Read(dV, inf);
    z.Read(inf);
    double je = JJ.Sqr(z);
    int J = int(SM::JJSpin(je, x.Jz));
    double te = TT.Sqr(z);
    int T = int(SM::JJSpin(te, x.Tz));
    std::fprintf(ft, "%.17g %.17g %.17g %.17g %.17g %d %d\n", E, dE, dV, je, te, J, T);
    std::fwrite(&z[0], sizeof(double), st.n, fv);
  }
  std::fclose(ft);
  std::fclose(fv);
  return 0;
}
