// Block Davidson engine: configuration and results.
#pragma once
#include <cstdint>
#include <vector>

namespace cg {

struct Hamiltonian;

struct DavConfig {
  int nume = 10;       // wanted eigenpairs
  int block = 10;      // vectors added per iteration
  int lim = 30;        // basis size that triggers a collapse
  int maxiter = 400;
  double crite = 1e-15, critc = 1e-12, critr = 1e-8, ortho = 1e-9;
  int spmm_prec = 0;   // CG_PREC_*
  bool seq_ortho = true;  // reference one-vector-at-a-time Gram-Schmidt
  bool pip = false;       // block Gram-Schmidt with Pythagorean inner products (Cholesky-QR folded in)
  bool modern = false;    // residual-driven iteration with thick restart
  int keep = 0;           // Ritz vectors kept at a restart (modern; 0: 2 * nume)
  int precond = 1;        // modern: 1 diagonal preconditioner, 0 plain residuals
  bool fp32_corr = false; // refinement (modern): correction blocks multiplied in FP32, result checked in double-float
  int verbose = 0;
};

struct DavOutcome {
  std::vector<double> eig, de, resid;
  int iterations = 0, restarts = 0, ierr = 0;
  int64_t matvecs = 0;
  double seconds = 0, spmm_seconds = 0;
};

struct DavidsonRequest {
  int nume = 10;
  DavConfig phase1;          // FP64 engine, or the FP32 engine of the mixed solve
  bool refine = false;       // run the FP64 refinement phase after an FP32 phase
  DavConfig phase2;          // refinement configuration
  const double* init = nullptr;  // host, column-major, ninit vectors
  int ninit = 0;
  double* vecs_out = nullptr;    // host, column-major, nume vectors (may be null)
};

struct DavResult {
  DavOutcome phase1, phase2, final_;
  bool refined = false;
  double seconds = 0;
};

DavResult davidson_solve(const Hamiltonian& h, const DavidsonRequest& rq);

}  // namespace cg
