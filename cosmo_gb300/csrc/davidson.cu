// Block Davidson on the GPU.
//
// The control flow restates dvdrvr2 (include/kdav/fsdavidson.cxx:615-775) as
// set up by DavidsonDiagonalization (include/kdav/davidson.cxx:168-225):
// Rayleigh-Ritz on S = B^T A B, convergence test on eigenvalue change and on
// the last Ritz coefficients (Test_Convergence, :212-281), residuals
// r = A B s - lambda B s with the diagonal preconditioner r / (lambda - A_ii)
// guarded at 1e-13 (Add_Vectors_To_Basis, :426-516), classical Gram-Schmidt
// with re-orthogonalisation while the overlap exceeds `ortho`
// (Orthogonalize_Basis, :313-390), collapse to the Ritz vectors when the basis
// reaches `lim` (Collapse_Matrix/Collapse_S, :99-121, :517-539) and unit start
// vectors on the lowest diagonal elements (setup_2d, :540-611).
//
// Layout: the basis B and the products AB are row-interleaved n x L arrays in
// HBM (row i holds component i of every basis vector), so the SpMM gathers all
// new vectors of a column with one vector load and every tall-skinny kernel
// streams whole rows.  Storage is FP64 or FP32; in the FP32 engine all
// products are FP32, summed in FP32 within a 32-row tile and in FP64 across
// tiles (GB300's FP64 rate is ~1/60 of FP32), and the projected matrix and its
// eigensolve are FP64.  The small host-side steps (projected eigenproblem, the
// convergence bookkeeping) act on at most lim x lim numbers.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <numeric>

#include "davidson.h"
#include "dense.h"
#include "device.h"

namespace cg {
namespace {

constexpr int kTile = 32;   // rows per tile
constexpr int kMaxK = 64;   // basis columns per tall-skinny call
constexpr int kMaxJ = 16;   // right-hand columns per call
constexpr int kThreads = 256;

template <class T>
__global__ void __launch_bounds__(kThreads) k_xty(uint64_t n, const T* __restrict__ X, int ldx, int xo, int K,
                                                  const T* __restrict__ Y, int ldy, int yo, int J,
                                                  double* __restrict__ part, uint64_t rows_per_cta) {
  __shared__ T xs[kTile * kMaxK];
  __shared__ T ys[kTile * kMaxJ];
  const int nout = K * J;
  double acc[4] = {0.0, 0.0, 0.0, 0.0};
  const uint64_t r0 = uint64_t(blockIdx.x) * rows_per_cta;
  const uint64_t r1 = min(n, r0 + rows_per_cta);
  for (uint64_t base = r0; base < r1; base += kTile) {
    const int rows = int(min(uint64_t(kTile), r1 - base));
    for (int idx = threadIdx.x; idx < kTile * K; idx += blockDim.x) {
      int r = idx / K, k = idx - r * K;
      xs[idx] = r < rows ? X[(base + r) * ldx + xo + k] : T(0);
    }
    for (int idx = threadIdx.x; idx < kTile * J; idx += blockDim.x) {
      int r = idx / J, j = idx - r * J;
      ys[idx] = r < rows ? Y[(base + r) * ldy + yo + j] : T(0);
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      int o = threadIdx.x + q * kThreads;
      if (o < nout) {
        int k = o / J, j = o - k * J;
        T t = T(0);
#pragma unroll 8
        for (int r = 0; r < kTile; ++r) t = fma(xs[r * K + k], ys[r * J + j], t);
        acc[q] += double(t);
      }
    }
    __syncthreads();
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    int o = threadIdx.x + q * kThreads;
    if (o < nout) part[uint64_t(blockIdx.x) * nout + o] = acc[q];
  }
}

__global__ void k_reduce_parts(const double* __restrict__ part, int nparts, int nout, double* __restrict__ out) {
  int o = blockIdx.x * blockDim.x + threadIdx.x;
  if (o >= nout) return;
  double s = 0.0;
  for (int c = 0; c < nparts; ++c) s += part[uint64_t(c) * nout + o];
  out[o] = s;
}

// Y[:, yo:yo+J] = beta * Y + alpha * X[:, xo:xo+K] G  (G is K x J, FP64).
// A CTA stages its whole row tile of X before writing, so X and Y may alias.
template <class T>
__global__ void __launch_bounds__(kThreads) k_rows_gemm(uint64_t n, const T* X, int ldx, int xo, int K,
                                                        const double* __restrict__ G, T* Y, int ldy, int yo, int J,
                                                        double alpha, double beta) {
  __shared__ T xs[kTile * kMaxK];
  __shared__ T gs[kMaxK * kMaxJ];
  for (int i = threadIdx.x; i < K * J; i += blockDim.x) gs[i] = T(alpha * G[i]);
  const T tb = T(beta);
  const uint64_t ntiles = (n + kTile - 1) / kTile;
  for (uint64_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const uint64_t base = tile * kTile;
    const int rows = int(min(uint64_t(kTile), n - base));
    __syncthreads();
    for (int idx = threadIdx.x; idx < kTile * K; idx += blockDim.x) {
      int r = idx / K, k = idx - r * K;
      xs[idx] = r < rows ? X[(base + r) * ldx + xo + k] : T(0);
    }
    __syncthreads();
    for (int idx = threadIdx.x; idx < rows * J; idx += blockDim.x) {
      int r = idx / J, j = idx - r * J;
      T t = T(0);
      for (int k = 0; k < K; ++k) t = fma(xs[r * K + k], gs[k * J + j], t);
      T* yp = Y + (base + r) * ldy + yo + j;
      *yp = (beta == 0.0) ? t : fma(tb, *yp, t);
    }
  }
}

// Residuals of C Ritz candidates: R[:, c] = AB Sc[:, c] - lam[c] B Sc[:, c],
// with per-CTA partial sums of |R[:, c]|^2.
template <class T>
__global__ void __launch_bounds__(kThreads) k_residual(uint64_t n, const T* __restrict__ B, const T* __restrict__ AB,
                                                       int ld, int K, const double* __restrict__ Sc,
                                                       const double* __restrict__ lam, int C, T* __restrict__ R,
                                                       int ldr, double* __restrict__ part, uint64_t rows_per_cta) {
  __shared__ T bs[kTile * kMaxK];
  __shared__ T abs_[kTile * kMaxK];
  __shared__ T ss[kMaxK * kMaxJ];
  __shared__ double red[kThreads];
  for (int i = threadIdx.x; i < K * C; i += blockDim.x) ss[i] = T(Sc[i]);
  const int c = threadIdx.x % C, rstep = kThreads / C, r_first = threadIdx.x / C;
  const bool active = threadIdx.x < rstep * C;
  const T lc = active ? T(lam[c]) : T(0);
  double acc = 0.0;
  const uint64_t r0 = uint64_t(blockIdx.x) * rows_per_cta;
  const uint64_t r1 = min(n, r0 + rows_per_cta);
  for (uint64_t base = r0; base < r1; base += kTile) {
    const int rows = int(min(uint64_t(kTile), r1 - base));
    __syncthreads();
    for (int idx = threadIdx.x; idx < kTile * K; idx += blockDim.x) {
      int r = idx / K, k = idx - r * K;
      bool ok = r < rows;
      bs[idx] = ok ? B[(base + r) * ld + k] : T(0);
      abs_[idx] = ok ? AB[(base + r) * ld + k] : T(0);
    }
    __syncthreads();
    if (active) {
      T tile = T(0);
      for (int r = r_first; r < rows; r += rstep) {
        T a = T(0), b = T(0);
        for (int k = 0; k < K; ++k) {
          T s = ss[k * C + c];
          a = fma(abs_[r * K + k], s, a);
          b = fma(bs[r * K + k], s, b);
        }
        T res = a - lc * b;
        R[(base + r) * ldr + c] = res;
        tile = fma(res, res, tile);
      }
      acc += double(tile);
    }
  }
  red[threadIdx.x] = active ? acc : 0.0;
  __syncthreads();
  if (threadIdx.x < C) {
    double s = 0.0;
    for (int t = threadIdx.x; t < rstep * C; t += C) s += red[t];
    part[uint64_t(blockIdx.x) * C + threadIdx.x] = s;
  }
}

// B[:, bo + a] = R[:, sel[a]] / g, g = lam[a] - diag_i, |g| <= 1e-13 -> 1e-13.
template <class T>
__global__ void k_precond_copy(uint64_t n, const T* __restrict__ R, int ldr, const int* __restrict__ sel,
                               const double* __restrict__ lam, int A, const double* __restrict__ diag, T* __restrict__ B,
                               int ld, int bo) {
  uint64_t idx = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (idx >= n * A) return;
  uint64_t i = idx / A;
  int a = int(idx - i * A);
  double g = lam[a] - diag[i];
  if (!(fabs(g) > 1e-13)) g = 1e-13;
  B[i * ld + bo + a] = T(double(R[i * ldr + sel[a]]) / g);
}

template <class T>
__global__ void k_scale_cols(uint64_t n, T* __restrict__ B, int ld, int bo, int J, const double* __restrict__ sc) {
  uint64_t idx = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (idx >= n * J) return;
  uint64_t i = idx / J;
  int j = int(idx - i * J);
  B[i * ld + bo + j] = T(double(B[i * ld + bo + j]) * sc[j]);
}

template <class T>
__global__ void k_zero_cols(uint64_t n, T* __restrict__ B, int ld, int bo, int J) {
  uint64_t idx = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (idx >= n * J) return;
  uint64_t i = idx / J;
  B[i * ld + bo + (idx - i * J)] = T(0);
}

template <class T>
__global__ void k_copy_cols(uint64_t n, const T* S, int lds, int so, T* D, int ldd, int dof,
                            int J) {
  uint64_t idx = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (idx >= n * J) return;
  uint64_t i = idx / J;
  int j = int(idx - i * J);
  D[i * ldd + dof + j] = S[i * lds + so + j];
}

template <class T>
__global__ void k_set_units(T* __restrict__ B, int ld, const uint64_t* __restrict__ rows, int m) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < m) B[rows[k] * ld + k] = T(1);
}

// host column-major doubles (vector k at k*n) <-> device row-interleaved
template <class T>
__global__ void k_cm_to_rm(uint64_t n, int m, const double* __restrict__ src, T* __restrict__ dst, int ld, int off) {
  uint64_t idx = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (idx >= n * m) return;
  uint64_t i = idx / m;
  int k = int(idx - i * m);
  dst[i * ld + off + k] = T(src[uint64_t(k) * n + i]);
}
template <class T>
__global__ void k_rm_to_cm(uint64_t n, int m, const T* __restrict__ src, int ld, int off, double* __restrict__ dst) {
  uint64_t idx = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (idx >= n * m) return;
  uint64_t i = idx / m;
  int k = int(idx - i * m);
  dst[uint64_t(k) * n + i] = double(src[i * ld + off + k]);
}

inline unsigned blocks_for(uint64_t work, int t = 256) { return unsigned((work + t - 1) / t); }

}  // namespace

// ------------------------------------------------------------ engine
template <class T>
struct Engine {
  const Hamiltonian& H;
  DavConfig cfg;
  cudaStream_t s;
  uint64_t n;
  int L;           // leading dimension of B / AB (>= lim, padded)
  int nparts;      // CTAs of the reduction kernels
  uint64_t rows_per_cta;
  DBuf<T> B, AB, R;
  int ldr;
  DBuf<double> part, small, small2, dlam;
  DBuf<int> dsel;
  DBuf<uint64_t> drows;
  double spmm_s = 0;
  cudaEvent_t ev0, ev1;
  // reference state
  int kpass = 0, nume, lim, mblock;
  std::vector<double> S;      // lim x lim, FP64
  std::vector<double> eigs, old, zvec;  // zvec: kpass x kpass, columns eigenvectors
  std::vector<int> icv;

  Engine(const Hamiltonian& h, const DavConfig& c, cudaStream_t st) : H(h), cfg(c), s(st) {
    n = h.n;
    nume = c.nume;
    lim = c.lim;
    mblock = c.block;
    int align = sizeof(T) == 4 ? 4 : 2;
    L = (lim + align - 1) / align * align;
    if (lim > kMaxK) throw Error(CG_ERR_ARG, "lim above 64 is not supported");
    if (mblock > kMaxJ || nume > kMaxJ) throw Error(CG_ERR_ARG, "block and nstates must be <= 16");
    int nsm = 0;
    CG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, h.device));
    nparts = std::max(1, std::min<int>(nsm * 2, int((n + kTile - 1) / kTile)));
    rows_per_cta = (n + nparts - 1) / nparts;
    rows_per_cta = (rows_per_cta + kTile - 1) / kTile * kTile;
    nparts = int((n + rows_per_cta - 1) / rows_per_cta);
    B.alloc(n * L);
    AB.alloc(n * L);
    ldr = (std::max(nume, 1) + align - 1) / align * align;
    R.alloc(n * ldr);
    part.alloc(size_t(nparts) * kMaxK * kMaxJ);
    small.alloc(kMaxK * kMaxK);
    small2.alloc(kMaxK * kMaxK);
    dlam.alloc(kMaxK);
    dsel.alloc(kMaxK);
    drows.alloc(kMaxK);
    CG_CUDA(cudaMemsetAsync(B.p, 0, B.bytes(), s));
    CG_CUDA(cudaMemsetAsync(AB.p, 0, AB.bytes(), s));
    CG_CUDA(cudaEventCreate(&ev0));
    CG_CUDA(cudaEventCreate(&ev1));
    S.assign(size_t(lim) * lim, 0.0);
    eigs.assign(lim, 0.0);
    old.assign(lim, 0.0);
    icv.assign(nume, 0);
  }
  ~Engine() {
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
  }

  // G (K x J, row-major, host) = X[:, xo:xo+K]^T Y[:, yo:yo+J]
  void xty(const T* X, int xo, int K, const T* Y, int yo, int J, std::vector<double>& G) {
    k_xty<T><<<nparts, kThreads, 0, s>>>(n, X, L, xo, K, Y, L, yo, J, part.p, rows_per_cta);
    CG_CUDA(cudaGetLastError());
    k_reduce_parts<<<blocks_for(K * J), 256, 0, s>>>(part.p, nparts, K * J, small.p);
    G.resize(size_t(K) * J);
    CG_CUDA(cudaMemcpyAsync(G.data(), small.p, sizeof(double) * K * J, cudaMemcpyDeviceToHost, s));
    CG_CUDA(cudaStreamSynchronize(s));
  }
  // Y[:, yo:yo+J] = beta Y + alpha X[:, xo:xo+K] G (G host K x J)
  void gemm(T* Xp, int xo, int K, const std::vector<double>& G, T* Yp, int yo, int J, double alpha, double beta) {
    CG_CUDA(cudaMemcpyAsync(small2.p, G.data(), sizeof(double) * K * J, cudaMemcpyHostToDevice, s));
    unsigned grid = unsigned(std::min<uint64_t>((n + kTile - 1) / kTile, uint64_t(nparts) * 4));
    k_rows_gemm<T><<<grid, kThreads, 0, s>>>(n, Xp, L, xo, K, small2.p, Yp, L, yo, J, alpha, beta);
    CG_CUDA(cudaGetLastError());
    CG_CUDA(cudaStreamSynchronize(s));  // G's staging buffer is reused by the next call
  }
  void spmm(int c0, int m) {
    CG_CUDA(cudaEventRecord(ev0, s));
    spmm_launch(H, cfg.spmm_prec, B.p + c0, L, AB.p + c0, L, m, s);
    CG_CUDA(cudaEventRecord(ev1, s));
    CG_CUDA(cudaEventSynchronize(ev1));
    float ms = 0;
    CG_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
    spmm_s += ms * 1e-3;
  }
  // new columns of S from AB[:, c0:c0+m] (Add_Vectors_To_AB_S, fsdavidson.cxx:161-211)
  void add_ab_s(int c0, int m, int64_t& nmv) {
    spmm(c0, m);
    nmv += m;
    std::vector<double> G;
    xty(B.p, 0, c0 + m, AB.p, c0, m, G);  // G[j][c] = b_j . ab_{c0+c}
    for (int c = 0; c < m; ++c) {
      int i = c0 + c;
      for (int j = 0; j <= i; ++j) {
        double v = G[size_t(j) * m + c];  // S[i][j] = b_j . ab_i for j <= i
        S[size_t(i) * lim + j] = v;
        S[size_t(j) * lim + i] = v;
      }
    }
  }
  void diagonalize() {
    std::vector<double> a(size_t(kpass) * kpass);
    for (int i = 0; i < kpass; ++i)
      for (int j = 0; j < kpass; ++j) a[size_t(i) * kpass + j] = S[size_t(i) * lim + j];
    std::vector<double> w;
    sym_eig(kpass, a, w, zvec);
    for (int i = 0; i < nume; ++i) eigs[i] = w[i];
  }
  double svec(int state, int row) const { return zvec[size_t(row) * kpass + state]; }
  // B[:, 0:nume] = B[:, 0:kp] Z[:, 0:nume], same for AB
  void collapse(int kp) {
    std::vector<double> G(size_t(kp) * nume);
    for (int k = 0; k < kp; ++k)
      for (int j = 0; j < nume; ++j) G[size_t(k) * nume + j] = svec(j, k);
    gemm(B.p, 0, kp, G, B.p, 0, nume, 1.0, 0.0);
    gemm(AB.p, 0, kp, G, AB.p, 0, nume, 1.0, 0.0);
  }
  void collapse_s() {
    std::fill(S.begin(), S.end(), 0.0);
    for (int i = 0; i < nume; ++i) S[size_t(i) * lim + i] = eigs[i];
    zvec.assign(size_t(nume) * nume, 0.0);
    for (int i = 0; i < nume; ++i) zvec[size_t(i) * nume + i] = 1.0;
  }
  // residuals of candidate states `st` (0-based); returns norms
  std::vector<double> residuals(const std::vector<int>& st) {
    int C = int(st.size());
    std::vector<double> Sc(size_t(kpass) * C), lam(C);
    for (int c = 0; c < C; ++c) {
      lam[c] = eigs[st[c]];
      for (int k = 0; k < kpass; ++k) Sc[size_t(k) * C + c] = svec(st[c], k);
    }
    CG_CUDA(cudaMemcpyAsync(small2.p, Sc.data(), sizeof(double) * Sc.size(), cudaMemcpyHostToDevice, s));
    CG_CUDA(cudaMemcpyAsync(dlam.p, lam.data(), sizeof(double) * C, cudaMemcpyHostToDevice, s));
    k_residual<T><<<nparts, kThreads, 0, s>>>(n, B.p, AB.p, L, kpass, small2.p, dlam.p, C, R.p, ldr, part.p,
                                              rows_per_cta);
    CG_CUDA(cudaGetLastError());
    k_reduce_parts<<<1, 256, 0, s>>>(part.p, nparts, C, small.p);
    std::vector<double> nr(C);
    CG_CUDA(cudaMemcpyAsync(nr.data(), small.p, sizeof(double) * C, cudaMemcpyDeviceToHost, s));
    CG_CUDA(cudaStreamSynchronize(s));
    for (auto& x : nr) x = std::sqrt(std::max(x, 0.0));
    return nr;
  }
  void precond_copy(const std::vector<int>& sel_r, const std::vector<double>& lam, int bo) {
    int A = int(sel_r.size());
    if (!A) return;
    CG_CUDA(cudaMemcpyAsync(dsel.p, sel_r.data(), sizeof(int) * A, cudaMemcpyHostToDevice, s));
    CG_CUDA(cudaMemcpyAsync(dlam.p, lam.data(), sizeof(double) * A, cudaMemcpyHostToDevice, s));
    k_precond_copy<T><<<blocks_for(n * A), 256, 0, s>>>(n, R.p, ldr, dsel.p, dlam.p, A, H.diag.p, B.p, L, bo);
    CG_CUDA(cudaGetLastError());
  }
  void scale_col(int c, double f) {
    CG_CUDA(cudaMemcpyAsync(small2.p, &f, sizeof(double), cudaMemcpyHostToDevice, s));
    k_scale_cols<T><<<blocks_for(n), 256, 0, s>>>(n, B.p, L, c, 1, small2.p);
    CG_CUDA(cudaGetLastError());
    CG_CUDA(cudaStreamSynchronize(s));
  }
  void copy_col(int from, int to) {
    k_copy_cols<T><<<blocks_for(n), 256, 0, s>>>(n, B.p, L, from, B.p, L, to, 1);
    CG_CUDA(cudaGetLastError());
  }

  // Orthogonalize_Basis (fsdavidson.cxx:313-390), one vector at a time.
  // Returns false (restart) when the overlap grows between passes.
  bool orthogonalize_seq(int basis_dim, int& nncv) {
    int iv = 1, icur = basis_dim;
    while (iv <= nncv) {
      double dprev = 1.0e7;
      bool again;
      do {
        again = false;
        int k = basis_dim + iv - 1;
        std::vector<double> G;
        xty(B.p, 0, k, B.p, icur, 1, G);
        double dcur = 0.0;
        for (double g : G) dcur = std::max(dcur, std::fabs(g));
        gemm(B.p, 0, k, G, B.p, icur, 1, -1.0, 1.0);
        if (dcur >= cfg.ortho) {
          if (dcur > dprev) {
            nncv = iv - 1;
            return false;
          }
          dprev = dcur;
          again = true;
        }
      } while (again);
      std::vector<double> nn;
      xty(B.p, icur, 1, B.p, icur, 1, nn);
      double nrm = std::sqrt(std::max(nn[0], 0.0));
      if (nrm < 1e-14) {
        // drop: replace by the last new vector (the reference indexes the
        // replacement absolutely; the last new vector is what is meant)
        if (basis_dim + nncv - 1 != icur) copy_col(basis_dim + nncv - 1, icur);
        --nncv;
      } else {
        scale_col(icur, 1.0 / nrm);
        ++icur;
        ++iv;
      }
    }
    return true;
  }

  // Block classical Gram-Schmidt against the basis (two passes), then
  // Cholesky-QR twice inside the new block.  Columns are first scaled to unit
  // norm; a column whose norm falls below `drop` after the projection carries
  // nothing the basis does not already span and is removed.
  void compact(int basis_dim, int& m, const std::vector<int>& keep) {
    for (int a = 0; a < int(keep.size()); ++a)
      if (keep[a] != a) copy_col(basis_dim + keep[a], basis_dim + a);
    m = int(keep.size());
  }
  void gram(int basis_dim, int m, std::vector<double>& M) { xty(B.p, basis_dim, m, B.p, basis_dim, m, M); }
  void scale_block(int basis_dim, int m, const std::vector<double>& f) {
    CG_CUDA(cudaMemcpyAsync(small2.p, f.data(), sizeof(double) * m, cudaMemcpyHostToDevice, s));
    k_scale_cols<T><<<blocks_for(n * m), 256, 0, s>>>(n, B.p, L, basis_dim, m, small2.p);
    CG_CUDA(cudaGetLastError());
    CG_CUDA(cudaStreamSynchronize(s));
  }
  bool orthogonalize_block(int basis_dim, int& nncv) {
    const double drop = sizeof(T) == 4 ? 1e-8 : 1e-20;  // squared norm after projection
    int m = nncv;
    if (m == 0) return true;
    std::vector<double> M;
    gram(basis_dim, m, M);
    {
      std::vector<int> keep;
      std::vector<double> f;
      for (int j = 0; j < m; ++j) {
        double d = M[size_t(j) * m + j];
        if (d > 0.0 && std::isfinite(d)) { keep.push_back(j); f.push_back(1.0 / std::sqrt(d)); }
      }
      compact(basis_dim, m, keep);
      if (m) scale_block(basis_dim, m, f);
    }
    for (int pass = 0; pass < 2 && m > 0 && basis_dim > 0; ++pass) {
      std::vector<double> G;
      xty(B.p, 0, basis_dim, B.p, basis_dim, m, G);
      gemm(B.p, 0, basis_dim, G, B.p, basis_dim, m, -1.0, 1.0);
    }
    int good = 0;
    for (int attempt = 0; attempt < 2 * kMaxJ && m > 0 && good < 2; ++attempt) {
      gram(basis_dim, m, M);
      std::vector<int> keep;
      for (int j = 0; j < m; ++j)
        if (M[size_t(j) * m + j] > drop) keep.push_back(j);
      if (int(keep.size()) < m) {
        compact(basis_dim, m, keep);
        good = 0;
        continue;
      }
      std::vector<double> Lc(M);
      int bad = cholesky(m, Lc);
      if (bad >= 0) {
        std::vector<int> k2;
        for (int j = 0; j < m; ++j)
          if (j != bad) k2.push_back(j);
        compact(basis_dim, m, k2);
        good = 0;
        continue;
      }
      // B_new <- B_new L^{-T}
      std::vector<double> Ginv(size_t(m) * m, 0.0);
      for (int j = 0; j < m; ++j) {
        std::vector<double> x(m, 0.0);
        for (int i = m - 1; i >= 0; --i) {
          double r = (i == j) ? 1.0 : 0.0;
          for (int k = i + 1; k < m; ++k) r -= Lc[size_t(k) * m + i] * x[k];
          x[i] = r / Lc[size_t(i) * m + i];
        }
        for (int i = 0; i < m; ++i) Ginv[size_t(i) * m + j] = x[i];
      }
      gemm(B.p, basis_dim, m, Ginv, B.p, basis_dim, m, 1.0, 0.0);
      ++good;
    }
    nncv = m;
    return true;
  }

  void set_unit_start(int first, int count, const std::vector<uint64_t>& rows) {
    if (count <= 0) return;
    CG_CUDA(cudaMemcpyAsync(drows.p, rows.data() + first, sizeof(uint64_t) * count, cudaMemcpyHostToDevice, s));
    k_set_units<T><<<1, 64, 0, s>>>(B.p + first, L, drows.p, count);
    CG_CUDA(cudaGetLastError());
  }

  // Run the iteration.  niv: number of valid starting columns already in B.
  DavOutcome run(int niv, const std::vector<double>& hdiag) {
    auto t0 = std::chrono::steady_clock::now();
    DavOutcome out;
    int64_t nmv = 0;
    if (niv > lim || niv < nume) {
      // setup_2d: unit vectors at the nume lowest diagonal elements (first index on ties)
      std::vector<uint64_t> idx(n);
      std::iota(idx.begin(), idx.end(), 0);
      int want = nume;
      std::partial_sort(idx.begin(), idx.begin() + std::min<uint64_t>(want, n), idx.end(),
                        [&](uint64_t a, uint64_t b) { return hdiag[a] < hdiag[b] || (hdiag[a] == hdiag[b] && a < b); });
      if (niv > lim) niv = 0;
      set_unit_start(niv, nume - niv, idx);
      if (niv) {
        int a = nume - niv;
        if (cfg.seq_ortho) orthogonalize_seq(niv, a); else orthogonalize_block(niv, a);
      }
      niv = nume;
    }
    else {
      // provided start vectors: make them orthonormal in this engine's precision
      int a = niv;
      orthogonalize_block(0, a);
      if (a < nume) {
        std::vector<uint64_t> idx(n);
        std::iota(idx.begin(), idx.end(), 0);
        std::partial_sort(idx.begin(), idx.begin() + std::min<uint64_t>(nume, n), idx.end(),
                          [&](uint64_t x, uint64_t y) { return hdiag[x] < hdiag[y] || (hdiag[x] == hdiag[y] && x < y); });
        k_zero_cols<T><<<blocks_for(n * (nume - a)), 256, 0, s>>>(n, B.p, L, a, nume - a);
        set_unit_start(a, nume - a, idx);
        int b2 = nume - a;
        orthogonalize_block(a, b2);
        a += b2;
      }
      niv = a;
    }
    kpass = niv;
    add_ab_s(0, kpass, nmv);
    int nncv = kpass;
    std::vector<int> incv;
    bool restart = false, first = true, done = false, hit_cap = true;
    int nloops = 0, ierr = 0;
    std::fill(eigs.begin(), eigs.end(), 0.0);
    do {
      for (int i = 0; i < nume; ++i) old[i] = eigs[i];
      diagonalize();
      // Test_Convergence
      {
        int nnce = 0;
        for (int i = 0; i < nume; ++i)
          if (std::fabs(old[i] - eigs[i]) >= cfg.crite) ++nnce;
        if (nnce == 0) {
          done = true;
        } else {
          std::vector<int> ind;
          std::vector<double> rowlast;
          for (int i = 0; i < nume; ++i) {
            if (icv[i]) continue;
            double tmax = std::fabs(svec(i, kpass - 1));
            for (int l = 1; l <= nncv - 1; ++l) tmax = std::max(tmax, std::fabs(svec(i, kpass - l - 1)));
            if (tmax < cfg.critc) icv[i] = 1;
            else { ind.push_back(i); rowlast.push_back(tmax); }
          }
          nncv = int(ind.size());
          done = nncv == 0;
          // order by decreasing coefficient (first maximum wins ties)
          for (int i = 0; i < nncv; ++i) {
            int mx = i;
            for (int j = i + 1; j < nncv; ++j)
              if (rowlast[j] > rowlast[mx]) mx = j;
            std::swap(rowlast[i], rowlast[mx]);
            std::swap(ind[i], ind[mx]);
          }
          incv = ind;
        }
      }
      if (done || uint64_t(kpass) >= n) { hit_cap = false; break; }
      if (kpass == lim) {
        collapse(lim);
        collapse_s();
        kpass = nume;
        ++out.restarts;
      }
      // Add_Vectors_To_Basis
      {
        int limadd = std::min(lim, mblock + kpass);
        std::vector<double> rn = residuals(incv);
        std::vector<int> sel_r;
        std::vector<double> lam;
        std::vector<int> added;
        int icvc = 0;
        bool early_done = false;
        for (int i = 0; i < nncv; ++i) {
          int st = incv[i];
          if (rn[i] < cfg.critr) {
            ++icvc;
            icv[st] = 1;
            if (icvc < nncv) continue;
            early_done = true;
            break;
          }
          sel_r.push_back(i);
          lam.push_back(eigs[st]);
          added.push_back(st);
          if (int(added.size()) + kpass == limadd) break;
        }
        if (cfg.verbose) {
          double mx = 0;
          for (double r : rn) mx = std::max(mx, r);
          std::fprintf(stderr, "dav[%s] it %d kpass %d cand %d max_resid %.3e E0 %.8f\n",
                       sizeof(T) == 4 ? "fp32" : "fp64", nloops, kpass, nncv, mx, eigs[0]);
        }
        if (early_done) { done = true; }
        else {
          nncv = int(added.size());
          precond_copy(sel_r, lam, kpass);
          restart = !(cfg.seq_ortho ? orthogonalize_seq(kpass, nncv) : orthogonalize_block(kpass, nncv));
          incv = added;
        }
      }
      if (!restart) {
        first = true;
      } else if (first) {
        first = false;
        collapse(kpass);
        collapse_s();
        for (int i = 0; i < nume; ++i) eigs[i] = 1e30;
        kpass = nume;
        restart = false;
        ++out.restarts;
        continue;
      } else {
        ierr += 1024;
        hit_cap = false;
        break;
      }
      if (done) { hit_cap = false; break; }
      if (nncv == 0) { hit_cap = false; break; }
      add_ab_s(kpass, nncv, nmv);
      kpass += nncv;
      ++nloops;
    } while (nloops < cfg.maxiter);
    if (hit_cap) {
      ierr += 2048;
      kpass -= nncv;
      // the last S columns were never diagonalised: redo on the reduced basis
      diagonalize();
    }
    // final results (fsdavidson.cxx:751-771)
    out.de.resize(nume);
    for (int i = 0; i < nume; ++i) out.de[i] = std::fabs(old[i] - eigs[i]);
    if (kpass != nume) collapse(kpass);
    kpass = nume;
    zvec.assign(size_t(nume) * nume, 0.0);
    for (int i = 0; i < nume; ++i) zvec[size_t(i) * nume + i] = 1.0;
    std::vector<int> all(nume);
    std::iota(all.begin(), all.end(), 0);
    out.resid = residuals(all);
    out.eig.assign(eigs.begin(), eigs.begin() + nume);
    out.iterations = nloops;
    out.matvecs = nmv;
    out.ierr = ierr;
    out.spmm_seconds = spmm_s;
    out.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return out;
  }
};

template <class T>
static void load_start(Engine<T>& e, const double* init_dev_cm, int ninit) {
  if (!ninit) return;
  k_cm_to_rm<T><<<blocks_for(e.n * ninit), 256, 0, e.s>>>(e.n, ninit, init_dev_cm, e.B.p, e.L, 0);
  CG_CUDA(cudaGetLastError());
}

template <class T>
static void store_vectors(Engine<T>& e, int m, double* dst_dev_cm) {
  k_rm_to_cm<T><<<blocks_for(e.n * m), 256, 0, e.s>>>(e.n, m, e.B.p, e.L, 0, dst_dev_cm);
  CG_CUDA(cudaGetLastError());
}

DavResult davidson_solve(const Hamiltonian& h, const DavidsonRequest& rq) {
  cudaStream_t s = h.stream;
  DavResult res;
  const uint64_t n = h.n;
  const int nume = rq.nume;
  if (nume < 1 || uint64_t(nume) > n) throw Error(CG_ERR_ARG, "nstates out of range");
  std::vector<double> hdiag(n);
  CG_CUDA(cudaMemcpyAsync(hdiag.data(), h.diag.p, n * 8, cudaMemcpyDeviceToHost, s));
  CG_CUDA(cudaStreamSynchronize(s));
  DBuf<double> vecs(n * nume);  // column-major result on device
  DBuf<double> init;
  int ninit = rq.ninit;
  if (ninit) {
    init.alloc(n * ninit);
    init.upload(rq.init, n * ninit, s);
  }
  auto t0 = std::chrono::steady_clock::now();
  if (rq.phase1.spmm_prec == CG_PREC_FP64) {
    Engine<double> e(h, rq.phase1, s);
    load_start(e, init.p, std::min(ninit, e.lim));
    DavOutcome o = e.run(std::min(ninit, e.lim + 1), hdiag);
    store_vectors(e, nume, vecs.p);
    res.phase1 = o;
    res.final_ = o;
  } else {
    DavOutcome o1;
    {
      Engine<float> e(h, rq.phase1, s);
      load_start(e, init.p, std::min(ninit, e.lim));
      o1 = e.run(std::min(ninit, e.lim + 1), hdiag);
      store_vectors(e, nume, vecs.p);
    }
    res.phase1 = o1;
    res.final_ = o1;
    if (rq.refine) {
      Engine<double> e(h, rq.phase2, s);
      load_start(e, vecs.p, nume);
      DavOutcome o2 = e.run(nume, hdiag);
      store_vectors(e, nume, vecs.p);
      res.phase2 = o2;
      res.final_ = o2;
      res.refined = true;
    }
  }
  CG_CUDA(cudaStreamSynchronize(s));
  res.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  if (rq.vecs_out) CG_CUDA(cudaMemcpy(rq.vecs_out, vecs.p, n * nume * 8, cudaMemcpyDeviceToHost));
  return res;
}

}  // namespace cg
