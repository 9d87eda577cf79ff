// Header-only C++ adapter that lets the reference's own Davidson solver
// (DavidsonDiagonalization, include/kdav/davidson.cxx:168-225) drive the GPU
// product of libcosmo_gb300.
//
// The reference wraps its matrix argument in MyMatrixDiagonal<SomeMatrix>
// (include/kdav/MandD.cxx:8-43), a MatB::MatrixBase (include/kdav/
// matrixbase.h:8-25), and needs of SomeMatrix: size(), ReadDiagonal(double*)
// and TimesMatrix(double** y, double** x, int m) / TimesMatrix(double* y,
// double* x, int m) const -- the members SparseMatrixCSB provides
// (include/tav/csbmatrix.cxx:393,623-672,719).  MatrixSeam<Backend> provides
// exactly those over a backend with
//     uint64_t n() const;
//     void diagonal(double* d) const;                       // n values
//     void product(const double* x, double* y, int m) const; // m contiguous blocks of n
// and GpuBackend is that backend over the C ABI (cg_spmm, cg_hamiltonian_diagonal).
// Copies share the backend (MyMatrixDiagonal copy-constructs its argument,
// as the reference's CSB copy shares its block pointers).  Errors throw int,
// as the reference's FatalError does (include/debug.h:81).
//
//   GpuBackend g("sys.xml", "sys", CG_PREC_FP64);
//   MatrixSeam<GpuBackend> M(g);
//   DavidsonDiagonalization("sys.HH.EE", M, 10, 0, 10);
#pragma once

#include <cstdint>
#include <cstring>
#include <memory>
#include <vector>

#include "cosmo_gb300.h"

namespace cosmo_gb300 {

template <class Backend>
class MatrixSeam {
 public:
  explicit MatrixSeam(std::shared_ptr<const Backend> b) : b_(std::move(b)), st_(std::make_shared<Staging>()) {}
  explicit MatrixSeam(const Backend& b) : MatrixSeam(std::make_shared<const Backend>(b)) {}

  size_t size() const { return size_t(b_->n()); }
  int ReadDiagonal(double* d) const {
    b_->diagonal(d);
    return 0;
  }
  // y[k], x[k]: the k-th of m column vectors of n doubles
  int TimesMatrix(double** y, double** x, int m) const {
    const uint64_t n = b_->n();
    st_->x.resize(n * uint64_t(m));
    st_->y.resize(n * uint64_t(m));
    for (int k = 0; k < m; ++k) std::memcpy(st_->x.data() + uint64_t(k) * n, x[k], n * sizeof(double));
    b_->product(st_->x.data(), st_->y.data(), m);
    for (int k = 0; k < m; ++k) std::memcpy(y[k], st_->y.data() + uint64_t(k) * n, n * sizeof(double));
    return 0;
  }
  // y, x: m contiguous column vectors of n doubles
  int TimesMatrix(double* y, double* x, int m) const {
    b_->product(x, y, m);
    return 0;
  }

 private:
  struct Staging {
    std::vector<double> x, y;
  };
  std::shared_ptr<const Backend> b_;
  std::shared_ptr<Staging> st_;  // host staging of the pointer-block form, reused between calls
};

// The GPU Hamiltonian behind the C ABI.  Owns its handle.
class GpuBackend {
 public:
  GpuBackend(const char* xml, const char* system, int32_t precision = CG_PREC_FP64) : prec_(precision) {
    cg_problem* p = nullptr;
    cg_basis* b = nullptr;
    cg_hamiltonian* h = nullptr;
    if (cg_problem_load_xml(xml, system, &p) != CG_OK) throw 1;
    const cg_status sb = cg_basis_build(p, &b);
    const cg_status sh = sb == CG_OK ? cg_hamiltonian_build(p, b, precision, &h) : sb;
    if (sb == CG_OK) cg_basis_dims(b, &n_, nullptr);
    if (b) cg_basis_destroy(b);
    cg_problem_destroy(p);
    if (sh != CG_OK) throw 1;
    h_.reset(h, cg_hamiltonian_destroy);
  }
  // an existing handle, not owned
  GpuBackend(cg_hamiltonian* h, uint64_t n, int32_t precision) : h_(h, [](cg_hamiltonian*) {}), n_(n), prec_(precision) {}

  uint64_t n() const { return n_; }
  void diagonal(double* d) const {
    if (cg_hamiltonian_diagonal(h_.get(), d) != CG_OK) throw 1;
  }
  void product(const double* x, double* y, int m) const {
    if (cg_spmm(h_.get(), x, y, m, prec_) != CG_OK) throw 1;
  }

 private:
  std::shared_ptr<cg_hamiltonian> h_;
  uint64_t n_ = 0;
  int32_t prec_ = CG_PREC_FP64;
};

}  // namespace cosmo_gb300
