// Batched lockstep solve of many independent CI problems (see batched.cu).
#pragma once
#include <cstdint>
#include <vector>

#include "device.h"

namespace cg {

struct BatchChunk {  // rows [row0, row1) of one problem, reduced by one warp
  uint32_t prob;
  uint32_t row0, row1;
};

struct BatchSet {
  int device = 0;
  int np = 0;                     // problems
  int nq = 0, nd = 0;             // Davidson problems, exactly solved small problems
  std::vector<uint64_t> dims;     // per problem
  std::vector<int> kind;          // 0 empty, 1 dense, 2 Davidson
  std::vector<int> slot;          // index among its kind
  Hamiltonian H;                  // block-diagonal FP32 (hi + lo) matrix of the Davidson problems
  DBuf<uint32_t> rowprob;         // Davidson row -> problem slot
  DBuf<BatchChunk> chunks;
  DBuf<uint32_t> pchunk;          // per slot: first chunk (nq + 1)
  int nchunks = 0;
  std::vector<uint64_t> qrow0;    // per slot: first row (nq + 1)
  std::vector<int> qprob;         // slot -> problem
  DBuf<double> diag;
  std::vector<double> h_diag;
  DBuf<double> dense;             // nd x 64 x 64 FP64 matrices of the small problems
  std::vector<int> ddim;
  double build_seconds = 0;
  double tune_seconds = 0;        // launch-shape autotuning of H inside build_seconds
  cudaStream_t stream = nullptr;
  ~BatchSet();
};

struct BatchParams {
  int nev = 5;            // eigenpairs per problem
  int block = 8;          // vectors added per iteration (>= nev)
  int lim = 40;           // basis limit
  int keep = 16;          // Ritz vectors kept at a restart
  int maxiter = 300;      // per phase
  double tol_resid = 1e-5;
  double switch_resid = 1e-4;  // FP32 phase stops here, FP64 phase continues
  bool use_graph = true;
};

struct BatchResult {
  std::vector<double> eig, resid;  // problems x nev (NaN where a problem has fewer states)
  std::vector<int> nconv, found;   // per problem
  int iterations32 = 0, iterations64 = 0;
  uint64_t graph_launches = 0;
  int graph_kernels = 0;
  uint64_t graph_kernel_launches = 0;  // kernels replayed by graph launches
  uint64_t launches = 0;           // kernel launches incl. those replayed by graphs
  double seconds = 0, spmm_seconds = 0;
};

void batch_build(const std::vector<const System*>& sys, const std::vector<const Operator*>& ops, BatchSet& bs);
void batch_solve(BatchSet& bs, const BatchParams& prm, BatchResult& res);

}  // namespace cg
