// Test driver: the reference's own DavidsonDiagonalization (include/kdav/
// davidson.cxx:168-225, compiled from the reference headers) driving a matrix
// through cosmo_gb300::MatrixSeam, the adapter of include/cosmo_gb300_matrix.hpp.
//
//   reference_davidson_seam oracle <rows.bin> <out.EE> <block> <saved states>
//       product from the CPU oracle's CSB (liboracle.so), which equals the
//       reference's own CSB product bit for bit: exercises the adapter's
//       layout handling under the reference solver on a machine without a GPU
//   reference_davidson_seam gpu <system.xml> <out.EE> <block> <saved states>
//       product from the GPU Hamiltonian (libcosmo_gb300.so, FP64)
// block: the Davidson block = number of eigenpairs computed (the DEXHVJTcsb
// tools pass max(10, states), davidson/DEXHVJTcsb.cpp:52,58).
// rows.bin: u64 n, u64 nnz, u64 rowptr[n + 1], u32 col[nnz], f64 val[nnz]
// (upper triangle, rows ascending).
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include <kdav/davidson.cxx>

#include "cosmo_gb300_matrix.hpp"

extern "C" {
void* oracle_csb_from_upper(uint64_t n, const uint64_t* rp, const uint32_t* cols, const double* vals);
void oracle_csb_times_matrix(const void* h, const double* x, double* y, int m, int nthreads);
void oracle_diagonal(uint64_t n, const uint64_t* rp, const uint32_t* cols, const double* vals, double* d);
}

struct OracleBackend {
  uint64_t rows = 0;
  std::vector<uint64_t> rp;
  std::vector<uint32_t> col;
  std::vector<double> val;
  void* csb = nullptr;
  uint64_t n() const { return rows; }
  void diagonal(double* d) const { oracle_diagonal(rows, rp.data(), col.data(), val.data(), d); }
  void product(const double* x, double* y, int m) const { oracle_csb_times_matrix(csb, x, y, m, 0); }
};

int main(int argc, char** argv) {
  if (argc < 6) {
    std::fprintf(stderr, "usage: reference_davidson_seam oracle|gpu <input> <out.EE> <block> <saved states>\n");
    return 2;
  }
  const std::string mode = argv[1];
  const int block = std::atoi(argv[4]), saved = std::atoi(argv[5]);
  if (mode == "gpu") {
    cosmo_gb300::GpuBackend g(argv[2], nullptr, CG_PREC_FP64);
    cosmo_gb300::MatrixSeam<cosmo_gb300::GpuBackend> M(g);
    DavidsonDiagonalization(argv[3], M, block, 0, saved);
    return 0;
  }
  auto b = std::make_shared<OracleBackend>();
  FILE* f = std::fopen(argv[2], "rb");
  if (!f) return 3;
  uint64_t nnz = 0;
  if (std::fread(&b->rows, 8, 1, f) != 1 || std::fread(&nnz, 8, 1, f) != 1) return 3;
  b->rp.resize(b->rows + 1);
  b->col.resize(nnz);
  b->val.resize(nnz);
  if (std::fread(b->rp.data(), 8, b->rows + 1, f) != b->rows + 1 || std::fread(b->col.data(), 4, nnz, f) != nnz ||
      std::fread(b->val.data(), 8, nnz, f) != nnz)
    return 3;
  std::fclose(f);
  b->csb = oracle_csb_from_upper(b->rows, b->rp.data(), b->col.data(), b->val.data());
  cosmo_gb300::MatrixSeam<OracleBackend> M{std::shared_ptr<const OracleBackend>(b)};
  DavidsonDiagonalization(argv[3], M, block, 0, saved);
  return 0;
}
