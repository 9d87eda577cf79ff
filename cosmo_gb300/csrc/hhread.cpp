// .HH row-sparse matrix file -> GPU Hamiltonian (the input side of
// davidson_vfile, davidson/davidson_vfile.cpp:28-75).
//
// Layout (PPMatrix::Write, include/sm/PPMatrix.cxx:413-465; read by
// SparseMatrix::Read, include/tav/sparse.cxx:402-445): uint64 n, then per row
// uint32 nz, uint64 ind[nz], double elem[nz].  The matrix is symmetric and each
// off-diagonal pair is stored once (SparseMatrix type 1, TimesMatrix
// include/tav/sparse.cxx:274-291 applies it to both triangles), so the reader
// mirrors every off-diagonal entry into the other triangle and stores the full
// CSR (columns ascending) that the GPU products use.
#include <algorithm>
#include <cmath>
#include <fstream>

#include "device.h"

namespace cg {

void hamiltonian_read_hh(const std::string& path, int precision, Hamiltonian& h) {
  if (precision != CG_PREC_FP64 && precision != CG_PREC_FP32)
    throw Error(CG_ERR_ARG, "Hamiltonian precision must be CG_PREC_FP64 or CG_PREC_FP32");
  std::ifstream f(path, std::ios::binary);
  if (!f) throw Error(CG_ERR_IO, "cannot open " + path);
  uint64_t n = 0;
  f.read(reinterpret_cast<char*>(&n), 8);
  if (!f) throw Error(CG_ERR_IO, "short .HH file " + path);
  if (n >= (1ull << 32)) throw Error(CG_ERR_UNSUPPORTED, ".HH dimension >= 2^32");
  // pass 1: the stored rows
  std::vector<uint64_t> srp(n + 1, 0);
  std::vector<uint32_t> scol;
  std::vector<double> sval;
  std::vector<uint64_t> ind;
  for (uint64_t r = 0; r < n; ++r) {
    uint32_t nz = 0;
    f.read(reinterpret_cast<char*>(&nz), 4);
    ind.resize(nz);
    f.read(reinterpret_cast<char*>(ind.data()), std::streamsize(8) * nz);
    const size_t base = sval.size();
    sval.resize(base + nz);
    f.read(reinterpret_cast<char*>(sval.data() + base), std::streamsize(8) * nz);
    if (!f) throw Error(CG_ERR_IO, "short .HH file " + path);
    for (uint32_t k = 0; k < nz; ++k) {
      if (ind[k] >= n) throw Error(CG_ERR_PARSE, ".HH column index out of range");
      scol.push_back(uint32_t(ind[k]));
    }
    srp[r + 1] = sval.size();
  }
  // pass 2: both triangles
  std::vector<uint64_t> cnt(n + 1, 0);
  uint64_t upper = 0;
  for (uint64_t r = 0; r < n; ++r)
    for (uint64_t e = srp[r]; e < srp[r + 1]; ++e) {
      ++cnt[r + 1];
      if (scol[e] != r) ++cnt[scol[e] + 1];
    }
  for (uint64_t r = 0; r < n; ++r) cnt[r + 1] += cnt[r];
  const uint64_t nnz = cnt[n];
  std::vector<uint64_t> rp = cnt, pos(cnt.begin(), cnt.end() - 1);
  std::vector<uint32_t> col(nnz);
  std::vector<double> val(nnz), diag(n, 0.0);
  for (uint64_t r = 0; r < n; ++r)
    for (uint64_t e = srp[r]; e < srp[r + 1]; ++e) {
      const uint32_t c = scol[e];
      col[pos[r]] = c;
      val[pos[r]++] = sval[e];
      if (c != r) {
        col[pos[c]] = uint32_t(r);
        val[pos[c]++] = sval[e];
      } else {
        diag[r] += sval[e];
      }
    }
  int max_row = 0;
  std::vector<std::pair<uint32_t, double>> tmp;
  for (uint64_t r = 0; r < n; ++r) {
    const uint64_t b = rp[r], e = rp[r + 1];
    max_row = std::max<int>(max_row, int(e - b));
    bool sorted = true;
    for (uint64_t k = b + 1; k < e; ++k) sorted = sorted && col[k - 1] <= col[k];
    if (!sorted) {
      tmp.clear();
      for (uint64_t k = b; k < e; ++k) tmp.emplace_back(col[k], val[k]);
      std::stable_sort(tmp.begin(), tmp.end(),
                       [](const std::pair<uint32_t, double>& x, const std::pair<uint32_t, double>& y) {
                         return x.first < y.first;
                       });
      for (uint64_t k = b; k < e; ++k) {
        col[k] = tmp[k - b].first;
        val[k] = tmp[k - b].second;
      }
    }
    for (uint64_t k = b; k < e; ++k) upper += col[k] >= r;
  }
  CG_CUDA(cudaGetDevice(&h.device));
  if (!h.stream) CG_CUDA(cudaStreamCreateWithFlags(&h.stream, cudaStreamNonBlocking));
  cudaStream_t s = h.stream;
  h.precision = precision;
  h.n = n;
  h.nnz = nnz;
  h.nnz_upper = upper;
  h.max_row = max_row;
  h.rowptr.upload(rp, s);
  h.col.upload(col, s);
  if (precision == CG_PREC_FP64) {
    h.val64.upload(val, s);
  } else {
    std::vector<float> hi(nnz), lo(nnz);
    for (uint64_t k = 0; k < nnz; ++k) {
      hi[k] = float(val[k]);
      lo[k] = float(val[k] - double(hi[k]));
    }
    h.hi.upload(hi, s);
    h.lo.upload(lo, s);
  }
  h.diag.upload(diag, s);
  CG_CUDA(cudaStreamSynchronize(s));
}

}  // namespace cg
