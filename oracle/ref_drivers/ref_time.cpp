// Test-infrastructure harness (oracle side, never shipped): times the
// reference's own CPU path for the CI hot path, compiled from the reference
// headers as they lie in the reference tree (oracle/Makefile).
//
// Same steps as xsm::DXHV (include/xsm/DEXHVcsb.cxx:33-71) without the Eigen
// fallback: basis (SM::Get), interaction (xReadSPInt), PPMatrix2CSBBlk
// (include/sm/PPMatrix.cxx:571-656) and DavidsonDiagonalization
// (include/kdav/davidson.cxx:168-225) with its default thresholds and block =
// nstates.  The matrix reaches the Davidson through the reference's own seam:
// DavidsonDiagonalization wraps its argument in MyMatrixDiagonal
// (include/kdav/MandD.cxx:8-43), a MatB::MatrixBase (include/kdav/matrixbase.h:8-25);
// the argument here is SeamTimer, which forwards size/ReadDiagonal/TimesMatrix
// to the reference CSB and records the wall-clock interval of every product,
// so each Davidson iteration's time is known (one block product per iteration).
//
// usage: ref_time <system.xml> <out_prefix> <nstates> <maxiter>
//   maxiter 0: the reference default max(40 * nstates, 200)
//   stdout: one line "ref_time {json}" with the phase times, the product log
//   and E, dE, resid of the saved states (<out_prefix>.EE).
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
#include <cstdio>
#include <fstream>
#include <memory>
#include <string>
#include <vector>

static double now_s() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

typedef tav::SparseMatrixCSB<double, uint32_t, uint16_t> RefCSB;

struct ProductLog {
  std::vector<double> start, end;
  std::vector<int> m;
};

// What MyMatrixDiagonal<SomeMatrix> needs of SomeMatrix: size(),
// ReadDiagonal(double*) and both TimesMatrix forms.  Copies share the matrix
// and the log (MyMatrixDiagonal copy-constructs its argument).
class SeamTimer {
 public:
  SeamTimer(RefCSB* m, std::shared_ptr<ProductLog> log) : m_(m), log_(std::move(log)) {}
  size_t size() { return m_->size(); }
  void ReadDiagonal(double* d) { m_->ReadDiagonal(d); }
  void TimesMatrix(double** y, double** x, int m) const {
    const double t = now_s();
    m_->TimesMatrix(y, x, m);
    record(t, m);
  }
  void TimesMatrix(double* y, double* x, int m) const {
    const double t = now_s();
    m_->TimesMatrix(y, x, m);
    record(t, m);
  }

 private:
  void record(double t, int m) const {
    log_->start.push_back(t);
    log_->end.push_back(now_s());
    log_->m.push_back(m);
  }
  RefCSB* m_;
  std::shared_ptr<ProductLog> log_;
};

int main(int argc, char** argv) {
  if (argc < 5) {
    std::fprintf(stderr, "usage: ref_time <system.xml> <out_prefix> <nstates> <maxiter>\n");
    return 2;
  }
  const std::string prefix = argv[2];
  const int nstates = std::atoi(argv[3]);
  const int maxiter = std::atoi(argv[4]);
  XMLNode xMainNode = XMLNode::openFileHelper(argv[1], xsm::cosmo);
  XMLNode xSystemNode = xml::SelectNode(xMainNode, xsm::system, "name");
  SM::SingleParticleStates sps;
  Make(sps, xMainNode.getChildNode(xsm::valencespace));
  SM::Many_Body_States st;
  const double t0 = now_s();
  SM::Get(st, xMainNode, xSystemNode);
  const double t1 = now_s();
  tav::STensor<spsint, double> ESP(2);
  tav::STensor<spsint, double> VSPX(4);
  xReadSPInt(ESP, VSPX, xSystemNode, xMainNode, sps);
  const double t2 = now_s();
  SM::PPMatrix HH(st);
  HH.push_back(&ESP);
  HH.push_back(&VSPX);
  uint16_t br = std::sqrt(1. * st.n) + 1;
  RefCSB FHH(st.n, br, br, true);
  PPMatrix2CSBBlk(FHH, HH);
  const double t3 = now_s();
  auto log = std::make_shared<ProductLog>();
  SeamTimer seam(&FHH, log);
  const std::string ee = prefix + ".EE";
  DavidsonDiagonalization(ee.c_str(), seam, nstates, maxiter, nstates);
  const double t4 = now_s();

  std::printf("ref_time {\"n\": %llu, \"threads\": %d, \"basis_s\": %.6f, \"interaction_s\": %.6f, "
              "\"csb_s\": %.6f, \"davidson_s\": %.6f, \"products\": [",
              (unsigned long long)st.n, omp_get_max_threads(), t1 - t0, t2 - t1, t3 - t2, t4 - t3);
  for (size_t i = 0; i < log->m.size(); ++i)
    std::printf("%s[%.6f, %.6f, %d]", i ? ", " : "", log->start[i] - t3, log->end[i] - t3, log->m[i]);
  std::printf("], \"states\": [");
  std::ifstream f(ee, std::ios::binary);
  uint32_t cnt = 0;
  f.read(reinterpret_cast<char*>(&cnt), 4);
  for (uint32_t i = 0; i < cnt && f; ++i) {
    double e[3];
    uint64_t n = 0;
    f.read(reinterpret_cast<char*>(e), 24);
    f.read(reinterpret_cast<char*>(&n), 8);
    f.seekg(std::streamoff(8 * n), std::ios::cur);
    std::printf("%s[%.17g, %.17g, %.17g]", i ? ", " : "", e[0], e[1], e[2]);
  }
  std::printf("]}\n");
  return 0;
}
