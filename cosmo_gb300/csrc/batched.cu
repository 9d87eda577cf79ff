// Batched solve of many independent CI problems (uneven dimensions) in lockstep.
//
// The reference solves one system per DEXHVJTcsb run (davidson/DEXHVJTcsb.cpp:
// 36-77, DavidsonDiagonalization include/kdav/davidson.cxx:168-281).  Here a
// whole set of problems is solved at once on one GPU:
//   * every problem's basis and stored H (FP32 hi + lo) is built on the GPU and
//     the matrices are concatenated into one block-diagonal CSR, so a single
//     SpMM launch multiplies the blocks of all problems;
//   * problems of dimension <= kDense are diagonalised exactly: their dense H
//     (hi + lo summed in FP64) goes through the batched Jacobi eigensolver;
//   * the others run one block Davidson in lockstep (same block size, basis
//     limit and thick-restart length for all, each with its own vectors,
//     projected matrix and Ritz pairs): tall-skinny products are segmented by
//     problem (warp chunks never cross a problem boundary, per-problem partial
//     sums reduced in a fixed order), the projected eigenproblems are solved on
//     the device by a parallel cyclic Jacobi (one CTA per problem), and every
//     iteration shape (basis size) is captured once into a CUDA graph and
//     replayed, so an iteration is one graph launch for all problems;
//   * FP32 vectors and products with FP64 projections until the residuals reach
//     the switch threshold, then the same engine in FP64 with the FP64-accurate
//     (hi + lo) product to the final tolerance.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <numeric>
#include <type_traits>

#include "batched.h"
#include "dfloat.h"
#include "dense.h"

namespace cg {

namespace {

constexpr int kDense = 64;     // problems up to this dimension are solved exactly
constexpr int kJac = 64;       // largest matrix of the batched Jacobi
constexpr int kChunk = 64;     // rows summed in the working precision before an FP64 add
constexpr int kTile = 16 * kChunk;  // rows of one problem per CTA of the segmented products
constexpr int kMaxB = 8;       // block size limit
constexpr int kMaxLim = 40;    // basis limit

// ------------------------------------------------------------ assembly
__global__ void k_concat_rows(uint64_t n, const uint64_t* __restrict__ rp, uint64_t base, uint64_t row0,
                              uint64_t* __restrict__ out) {
  uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i < n) out[row0 + i] = base + rp[i];
}
__global__ void k_concat_cols(uint64_t nnz, const uint32_t* __restrict__ c, uint32_t off, uint32_t* __restrict__ out) {
  uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i < nnz) out[i] = c[i] + off;
}
// dense FP64 matrix (n x n, row-major, ld kJac) of rows [r0, r0 + n) of a CSR whose columns start at r0
__global__ void k_dense_fill(int n, uint64_t r0, const uint64_t* __restrict__ rp, const uint32_t* __restrict__ col,
                             const float* __restrict__ hi, const float* __restrict__ lo, double* __restrict__ A) {
  const int i = blockIdx.x;
  for (int j = threadIdx.x; j < kJac; j += blockDim.x) A[i * kJac + j] = 0.0;
  __syncthreads();
  for (uint64_t e = rp[r0 + i] + threadIdx.x; e < rp[r0 + i + 1]; e += blockDim.x)
    A[i * kJac + int(col[e] - r0)] = double(hi[e]) + double(lo[e]);
}

// ------------------------------------------------ batched Jacobi eigensolver
// One CTA per matrix: A (k x k, symmetric, FP64 in, ld kJac) -> eigenvalues
// ascending w[0..k) and eigenvectors Z (column j of the k x k block, ld kJac),
// computed in R: FP64 (off-diagonal norm down to 1e-12 of the Frobenius norm)
// or FP32 (1e-6).  FP32 vectors alone, off by ~eps32 |S| / gap, kept the
// FP32 Davidson phase from reaching its 1e-4 residuals (300 instead of 133
// iterations), so that phase runs the FP32 Jacobi and then the FP64 one from
// its vectors (re-orthonormalized: ortho), which leaves the FP64 pipe only
// one or two sweeps.  Cyclic Jacobi with the round-robin ordering: each round
// applies k/2 disjoint rotations at once, skipping those whose |a_pq| is
// below 1e-17 (FP32: 1e-7) of sqrt|a_pp a_qq|; at most 40 sweeps.
template <class R>
constexpr size_t jac_smem() {
  return (size_t(3) * kJac * (kJac + 1) + 256 + kJac) * sizeof(R) + (2 * kJac + 8) * sizeof(int);
}

// Warm start (kprev > 0): the leading kprev x kprev block of A is the
// previous step's projected matrix, whose eigenvectors Zout still holds; the
// sweeps start from A' = P^T A P, P = diag(Z_prev, I), whose leading block is
// already diagonal, with Z = P, so only the coupling to the newest rows is
// left to rotate away.  kprev = k takes Zout as approximate eigenvectors of
// the whole matrix (from the FP32 solve of the same A).
template <class R>
__global__ void __launch_bounds__(256) k_bjacobi(const double* __restrict__ Ain, const int* __restrict__ kdim,
                                                 int kconst, double* __restrict__ w, double* Zout,
                                                 const int* __restrict__ fz, int kprev, int ortho) {
  constexpr R kConv = sizeof(R) == 4 ? R(1e-12) : R(1e-24);   // (off / total)^2 at convergence
  constexpr R kTiny = sizeof(R) == 4 ? R(1e-30) : R(1e-300);
  constexpr R kSkip = sizeof(R) == 4 ? R(1e-7) : R(1e-17);
  if (fz && fz[blockIdx.x]) return;
  extern __shared__ __align__(16) unsigned char jsm_raw[];
  R* jsm = reinterpret_cast<R*>(jsm_raw);
  R(*A)[kJac + 1] = reinterpret_cast<R(*)[kJac + 1]>(jsm);
  R(*Z)[kJac + 1] = reinterpret_cast<R(*)[kJac + 1]>(jsm + kJac * (kJac + 1));
  R(*Tm)[kJac + 1] = reinterpret_cast<R(*)[kJac + 1]>(jsm + 2 * kJac * (kJac + 1));
  R* red = jsm + 3 * kJac * (kJac + 1);
  R* rc = red + 256;
  R* rs = rc + kJac / 2;
  int* rp = reinterpret_cast<int*>(rs + kJac / 2);
  int* rq = rp + kJac / 2;
  int* order = rq + kJac / 2;
  int& done = order[kJac];
  const int b = blockIdx.x, tid = threadIdx.x;
  const int k = kdim ? kdim[b] : kconst;
  const double* Ab = Ain + size_t(b) * kJac * kJac;
  const int kp = (kprev > 0 && kprev <= k) ? kprev : 0;
  const double* Zp = Zout + size_t(b) * kJac * kJac;
  for (int i = tid; i < kJac * kJac; i += blockDim.x) {
    const int r = i / kJac, c = i % kJac;
    Z[r][c] = (r < kp && c < kp) ? R(Zp[r * kJac + c]) : (r == c && r >= kp ? R(1) : R(0));
  }
  __syncthreads();
  if (ortho && kp > 0) {
    // vectors from a lower-precision solve: one Newton-Schulz step,
    // P <- P (3 I - P^T P) / 2, squares their deviation from orthonormality
    // (A's storage holds the new P until A is loaded)
    for (int i = tid; i < kp * kp; i += blockDim.x) {
      const int r = i / kp, c = i % kp;
      R v = 0;
      for (int t = 0; t < kp; ++t) v += Z[t][r] * Z[t][c];
      Tm[r][c] = (r == c ? R(1.5) : R(0)) - R(0.5) * v;
    }
    __syncthreads();
    for (int i = tid; i < kp * kp; i += blockDim.x) {
      const int r = i / kp, c = i % kp;
      R v = 0;
      for (int t = 0; t < kp; ++t) v += Z[r][t] * Tm[t][c];
      A[r][c] = v;
    }
    __syncthreads();
    for (int i = tid; i < kp * kp; i += blockDim.x) {
      const int r = i / kp, c = i % kp;
      Z[r][c] = A[r][c];
    }
    __syncthreads();
  }
  for (int i = tid; i < kJac * kJac; i += blockDim.x) {
    const int r = i / kJac, c = i % kJac;
    A[r][c] = (r < k && c < k) ? R(Ab[r * kJac + c]) : R(0);
  }
  __syncthreads();
  if (kp > 0) {
    // Tm = A P (only the first kp columns change), then A = P^T Tm (first kp rows)
    for (int i = tid; i < k * k; i += blockDim.x) {
      const int r = i / k, c = i % k;
      R v = 0;
      if (c < kp)
        for (int t = 0; t < kp; ++t) v += A[r][t] * Z[t][c];
      else
        v = A[r][c];
      Tm[r][c] = v;
    }
    __syncthreads();
    for (int i = tid; i < k * k; i += blockDim.x) {
      const int r = i / k, c = i % k;
      R v = 0;
      if (r < kp)
        for (int t = 0; t < kp; ++t) v += Z[t][r] * Tm[t][c];
      else
        v = Tm[r][c];
      A[r][c] = v;
    }
    __syncthreads();
    // exact symmetry (the two products round differently)
    for (int i = tid; i < k * k; i += blockDim.x) {
      const int r = i / k, c = i % k;
      if (r < c) {
        const R v = R(0.5) * (A[r][c] + A[c][r]);
        A[r][c] = v;
        A[c][r] = v;
      }
    }
    __syncthreads();
  }
  const int kk = k + (k & 1);  // even player count; player k (if odd) is idle
  for (int sweep = 0; sweep < 40 && k > 1; ++sweep) {
    // convergence: off-diagonal vs total
    R off = 0, tot = 0;
    for (int i = tid; i < k * k; i += blockDim.x) {
      const int r = i / k, c = i % k;
      const R v = A[r][c] * A[r][c];
      tot += v;
      if (r != c) off += v;
    }
    // warp sums, then the 8 warps' in a fixed order
    for (int o = 16; o; o >>= 1) {
      off += __shfl_xor_sync(0xffffffffu, off, o);
      tot += __shfl_xor_sync(0xffffffffu, tot, o);
    }
    if ((tid & 31) == 0) {
      red[tid >> 5] = off;
      red[8 + (tid >> 5)] = tot;
    }
    __syncthreads();
    if (tid == 0) {
      R offs = 0, tots = 0;
      for (int w8 = 0; w8 < int(blockDim.x >> 5); ++w8) {
        offs += red[w8];
        tots += red[8 + w8];
      }
      done = offs <= kConv * tots || offs == R(0);
    }
    __syncthreads();
    if (done) break;
    for (int round = 0; round < kk - 1; ++round) {
      // pairs of this round: player 0 fixed, the others rotate
      if (tid < kk / 2) {
        auto player = [&](int pos) { return pos == 0 ? 0 : 1 + (pos - 1 + round) % (kk - 1); };
        int p = player(tid), q = player(kk - 1 - tid);
        if (p > q) { int t = p; p = q; q = t; }
        R c = 1, s = 0;
        if (q < k) {
          const R apq = A[p][q];
          if (fabs(apq) > kTiny && fabs(apq) > kSkip * sqrt(fabs(A[p][p] * A[q][q]))) {
            const R tau = (A[q][q] - A[p][p]) / (R(2) * apq);
            const R t = (tau >= 0 ? R(1) : R(-1)) / (fabs(tau) + sqrt(R(1) + tau * tau));
            c = R(1) / sqrt(R(1) + t * t);
            s = t * c;
          }
        }
        rp[tid] = p;
        rq[tid] = q;  // >= k: the idle player of an odd k
        rc[tid] = c;  // (1, 0) when this pair is not rotated
        rs[tid] = s;
      }
      __syncthreads();
      // A <- J^T A J and Z <- Z J in one pass: the pairs of a round are
      // disjoint and cover every index, so each 2 x 2 block (pair a rows,
      // pair b columns) is rotated from both sides by one thread; the rows of
      // Z's column pairs go to the threads after the blocks
      const int np2 = kk / 2;
      for (int i = tid; i < np2 * np2 + k * np2; i += blockDim.x) {
        if (i < np2 * np2) {
          const int a = i / np2, bb = i - a * np2;
          const int pa = rp[a], qa = rq[a], pb = rp[bb], qb = rq[bb];
          const bool va = qa < k, vb = qb < k;
          const R ca = rc[a], sa = rs[a], cb = rc[bb], sb = rs[bb];
          if ((sa == R(0)) && (sb == R(0))) continue;
          const R x00 = A[pa][pb], x01 = vb ? A[pa][qb] : R(0);
          const R x10 = va ? A[qa][pb] : R(0), x11 = (va && vb) ? A[qa][qb] : R(0);
          // rows p, q of the block: J_a^T
          const R y00 = ca * x00 - sa * x10, y01 = ca * x01 - sa * x11;
          const R y10 = sa * x00 + ca * x10, y11 = sa * x01 + ca * x11;
          // columns p, q: J_b
          A[pa][pb] = cb * y00 - sb * y01;
          if (vb) A[pa][qb] = sb * y00 + cb * y01;
          if (va) A[qa][pb] = cb * y10 - sb * y11;
          if (va && vb) A[qa][qb] = sb * y10 + cb * y11;
        } else {
          const int t = i - np2 * np2, bb = t / k, r = t - bb * k;
          const int pb = rp[bb], qb = rq[bb];
          const R cb = rc[bb], sb = rs[bb];
          if (qb >= k || sb == R(0)) continue;
          const R zp = Z[r][pb], zq = Z[r][qb];
          Z[r][pb] = cb * zp - sb * zq;
          Z[r][qb] = sb * zp + cb * zq;
        }
      }
      __syncthreads();
    }
  }
  // ascending order (ties by index)
  for (int i = tid; i < k; i += blockDim.x) {
    int rank = 0;
    const R di = A[i][i];
    for (int j = 0; j < k; ++j) {
      const R dj = A[j][j];
      rank += (dj < di) || (dj == di && j < i);
    }
    order[rank] = i;
  }
  __syncthreads();
  double* wb = w + size_t(b) * kJac;
  double* Zb = Zout + size_t(b) * kJac * kJac;
  for (int i = tid; i < kJac; i += blockDim.x) wb[i] = i < k ? double(A[order[i]][order[i]]) : 0.0;
  for (int i = tid; i < kJac * kJac; i += blockDim.x) {
    const int r = i / kJac, c = i % kJac;
    Zb[r * kJac + c] = (r < k && c < k) ? double(Z[r][order[c]]) : 0.0;
  }
}

// ------------------------------------------------ segmented tall-skinny ops
// Per-tile partials of G = X[:, xo:xo+K]^T Y[:, yo:yo+J]: one CTA per tile (rows
// of one problem), warp w takes every 8th chunk of the tile; the chunk's J
// columns of Y are staged in shared memory, lane l owns columns l and l + 32 of
// X with four rows of loads in flight.  FP32 engine: FP32 products summed over
// a 64-row chunk, chunks in FP64.  FP64 engine: double-float products (FP64
// operands split once into FP32 pairs) summed over a 32-row chunk, chunks in
// FP64.  The 8 warps are added in a fixed order.
template <class T>
__global__ void __launch_bounds__(256) k_bxty(const BatchChunk* __restrict__ tiles, const T* __restrict__ X, int ldx,
                                              int xo, int K, const T* __restrict__ Y, int ldy, int yo, int J,
                                              double* __restrict__ part, const int* __restrict__ fz) {
  constexpr bool DF = sizeof(T) == 8;
  constexpr int CH = DF ? 32 : kChunk;
  __shared__ double red[8][kMaxLim * kMaxB];
  __shared__ __align__(16) float yh[8][CH * kMaxB];
  __shared__ __align__(16) float yl[8][DF ? CH * kMaxB : 1];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const BatchChunk tl = tiles[blockIdx.x];
  if (fz[tl.prob]) return;
  const bool a0 = lane < K, a1 = lane + 32 < K;
  double d0[kMaxB], d1[kMaxB];
#pragma unroll
  for (int j = 0; j < kMaxB; ++j) { d0[j] = 0.0; d1[j] = 0.0; }
  for (uint32_t c0 = tl.row0 + uint32_t(w) * CH; c0 < tl.row1; c0 += 8u * CH) {
    const int rows = int(min(tl.row1 - c0, uint32_t(CH)));
    __syncwarp();
    for (int i = lane; i < CH * kMaxB; i += 32) {
      const int rr = i / kMaxB, j = i - rr * kMaxB;
      const T v = (rr < rows && j < J) ? Y[size_t(c0 + rr) * ldy + yo + j] : T(0);
      if constexpr (DF) df_split(double(v), yh[w][i], yl[w][i]);
      else yh[w][i] = float(v);
    }
    __syncwarp();
    float sh0[kMaxB], sh1[kMaxB], sl0[kMaxB], sl1[kMaxB];
#pragma unroll
    for (int j = 0; j < kMaxB; ++j) { sh0[j] = sh1[j] = sl0[j] = sl1[j] = 0.f; }
    for (int rr = 0; rr < rows; rr += 4) {
      T xa[4], xb[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const bool ok = rr + u < rows;
        const T* xr = X + size_t(c0 + rr + u) * ldx + xo;
        xa[u] = (ok && a0) ? xr[lane] : T(0);
        xb[u] = (ok && a1) ? xr[lane + 32] : T(0);
      }
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const float* yr = yh[w] + (rr + u) * kMaxB;
        if constexpr (DF) {
          const float* ylr = yl[w] + (rr + u) * kMaxB;
          float ah, al, bh, bl;
          df_split(double(xa[u]), ah, al);
          df_split(double(xb[u]), bh, bl);
#pragma unroll
          for (int j = 0; j < kMaxB; ++j)
            if (j < J) {
              df_mac(sh0[j], sl0[j], ah, al, yr[j], ylr[j]);
              if (a1) df_mac(sh1[j], sl1[j], bh, bl, yr[j], ylr[j]);
            }
        } else {
#pragma unroll
          for (int j = 0; j < kMaxB; ++j) {
            sh0[j] = fmaf(float(xa[u]), yr[j], sh0[j]);
            sh1[j] = fmaf(float(xb[u]), yr[j], sh1[j]);
          }
        }
      }
    }
#pragma unroll
    for (int j = 0; j < kMaxB; ++j) {
      d0[j] += double(sh0[j]) + double(sl0[j]);
      d1[j] += double(sh1[j]) + double(sl1[j]);
    }
  }
#pragma unroll
  for (int j = 0; j < kMaxB; ++j)
    if (j < J) {
      if (a0) red[w][lane * J + j] = d0[j];
      if (a1) red[w][(lane + 32) * J + j] = d1[j];
    }
  __syncthreads();
  for (int o = threadIdx.x; o < K * J; o += blockDim.x) {
    double sum = 0.0;
    for (int i = 0; i < 8; ++i) sum += red[i][o];
    part[size_t(blockIdx.x) * (kMaxLim * kMaxB) + o] = sum;
  }
}

// G[q][K x J] = sum of the partials of problem q's chunks, in chunk order
__global__ void k_breduce(const uint32_t* __restrict__ pchunk, const double* __restrict__ part, int K, int J,
                          double* __restrict__ G, const int* __restrict__ fz) {
  const int q = blockIdx.x;
  if (fz[q]) return;
  for (int o = threadIdx.x; o < K * J; o += blockDim.x) {
    double s = 0.0;
    for (uint32_t c = pchunk[q]; c < pchunk[q + 1]; ++c) s += part[size_t(c) * (kMaxLim * kMaxB) + o];
    G[size_t(q) * (kMaxLim * kMaxB) + o] = s;
  }
}

// S[q][i][c0 + j] = S[q][c0 + j][i] = G[q][i * J + j] for i < K (K = c0 + J)
__global__ void k_bset_proj(int K, int J, int c0, const double* __restrict__ G, double* __restrict__ S,
                            const int* __restrict__ fz) {
  const int q = blockIdx.x;
  if (fz[q]) return;
  double* Sq = S + size_t(q) * kJac * kJac;
  const double* Gq = G + size_t(q) * (kMaxLim * kMaxB);
  for (int o = threadIdx.x; o < K * J; o += blockDim.x) {
    const int i = o / J, j = o % J;
    const double v = Gq[o];
    if (i >= c0 && i - c0 > j) continue;  // lower part of the new block comes from its mirror
    Sq[i * kJac + c0 + j] = v;
    Sq[(c0 + j) * kJac + i] = v;
  }
}

// Y[r][yo + j] = beta * Y[r][yo + j] + alpha * sum_i X[r][xo + i] M[q][i][j]  (M ld mld, per problem),
// computed in T.  One CTA per tile (rows of one problem, M staged in shared
// memory), one thread per row: the row is read completely before it is
// written (in-place safe).
template <class T>
__global__ void __launch_bounds__(256) k_bgemm(const BatchChunk* __restrict__ tiles, const T* X, int ldx, int xo,
                                               int K, const double* __restrict__ M, size_t mstride, int mld, T* Y,
                                               int ldy, int yo, int J, double alpha, double beta,
                                               const int* __restrict__ fz) {
  constexpr bool DF = sizeof(T) == 8;  // FP64 engine: double-float arithmetic
  __shared__ float Mh[kMaxLim * kMaxLim];
  __shared__ float Ml[DF ? kMaxLim * kMaxLim : 1];
  const BatchChunk tl = tiles[blockIdx.x];
  if (fz[tl.prob]) return;
  const double* Mq = M + size_t(tl.prob) * mstride;
  for (int i = threadIdx.x; i < K * J; i += blockDim.x) {
    const double v = alpha * Mq[(i / J) * mld + (i % J)];
    if constexpr (DF) df_split(v, Mh[i], Ml[i]);
    else Mh[i] = float(v);
  }
  __syncthreads();
  for (uint32_t r = tl.row0 + threadIdx.x; r < tl.row1; r += blockDim.x) {
    float ah[kMaxLim], al[kMaxLim];
#pragma unroll
    for (int j = 0; j < kMaxLim; ++j) { ah[j] = 0.f; al[j] = 0.f; }
    const T* xr = X + size_t(r) * ldx + xo;
    for (int i = 0; i < K; ++i) {
      if constexpr (DF) {
        float xh, xl;
        df_split(double(xr[i]), xh, xl);
#pragma unroll
        for (int j = 0; j < kMaxLim; ++j)
          if (j < J) df_mac(ah[j], al[j], xh, xl, Mh[i * J + j], Ml[i * J + j]);
      } else {
        const float xv = float(xr[i]);
#pragma unroll
        for (int j = 0; j < kMaxLim; ++j)
          if (j < J) ah[j] = fmaf(xv, Mh[i * J + j], ah[j]);
      }
    }
    T* yr = Y + size_t(r) * ldy + yo;
#pragma unroll
    for (int j = 0; j < kMaxLim; ++j)
      if (j < J) {
        const T v = DF ? T(double(ah[j]) + double(al[j])) : T(ah[j]);
        yr[j] = beta == 0.0 ? v : T(beta) * yr[j] + v;
      }
  }
}

// R[r][j] = sum_i (AV[r][i] - theta[q][j] V[r][i]) Z[q][i][j], j < b  (computed in T;
// one CTA per tile with Z[:, 0:b] and theta staged in shared memory)
template <class T>
__global__ void __launch_bounds__(256) k_bresid(const BatchChunk* __restrict__ tiles, const T* __restrict__ V,
                                                const T* __restrict__ AV, int ld, int K, const double* __restrict__ w,
                                                const double* __restrict__ Z, T* __restrict__ R, int ldr, int b,
                                                const int* __restrict__ fz) {
  constexpr bool DF = sizeof(T) == 8;  // FP64 engine: double-float arithmetic
  __shared__ float Zh[kMaxLim * kMaxB];
  __shared__ float Zl[DF ? kMaxLim * kMaxB : 1];
  __shared__ double th[kMaxB];
  const BatchChunk tl = tiles[blockIdx.x];
  if (fz[tl.prob]) return;
  const double* Zq = Z + size_t(tl.prob) * kJac * kJac;
  for (int i = threadIdx.x; i < K * b; i += blockDim.x) {
    const double v = Zq[(i / b) * kJac + (i % b)];
    if constexpr (DF) df_split(v, Zh[i], Zl[i]);
    else Zh[i] = float(v);
  }
  if (threadIdx.x < b) th[threadIdx.x] = w[size_t(tl.prob) * kJac + threadIdx.x];
  __syncthreads();
  for (uint32_t r = tl.row0 + threadIdx.x; r < tl.row1; r += blockDim.x) {
    // AV z_j and V z_j separately, then R = AV z - theta V z
    float ah[kMaxB], al[kMaxB], bh[kMaxB], bl[kMaxB];
#pragma unroll
    for (int j = 0; j < kMaxB; ++j) { ah[j] = al[j] = bh[j] = bl[j] = 0.f; }
    for (int i = 0; i < K; ++i) {
      const T v = V[size_t(r) * ld + i], av = AV[size_t(r) * ld + i];
      if constexpr (DF) {
        float vh, vl, ach, acl;
        df_split(double(v), vh, vl);
        df_split(double(av), ach, acl);
#pragma unroll
        for (int j = 0; j < kMaxB; ++j)
          if (j < b) {
            df_mac(ah[j], al[j], ach, acl, Zh[i * b + j], Zl[i * b + j]);
            df_mac(bh[j], bl[j], vh, vl, Zh[i * b + j], Zl[i * b + j]);
          }
      } else {
#pragma unroll
        for (int j = 0; j < kMaxB; ++j)
          if (j < b) {
            ah[j] = fmaf(float(av), Zh[i * b + j], ah[j]);
            bh[j] = fmaf(float(v), Zh[i * b + j], bh[j]);
          }
      }
    }
#pragma unroll
    for (int j = 0; j < kMaxB; ++j)
      if (j < b) {
        if constexpr (DF)
          R[size_t(r) * ldr + j] = T((double(ah[j]) + double(al[j])) - th[j] * (double(bh[j]) + double(bl[j])));
        else
          R[size_t(r) * ldr + j] = T(ah[j] - float(th[j]) * bh[j]);
      }
  }
}

// V[r][c0 + j] = R[r][j] / (theta[q][j] - diag[r]) with the reference's 1e-13 floor
template <class T>
__global__ void k_bprecond(uint32_t nrows, const uint32_t* __restrict__ rowprob, const T* __restrict__ R, int ldr,
                           const double* __restrict__ w, const double* __restrict__ diag, T* __restrict__ V, int ld,
                           int c0, int b, const int* __restrict__ fz) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrows || fz[rowprob[r]]) return;
  const double* wq = w + size_t(rowprob[r]) * kJac;
  for (int j = 0; j < b; ++j) {
    double den = wq[j] - diag[r];
    if (fabs(den) < 1e-13) den = den < 0 ? -1e-13 : 1e-13;
    V[size_t(r) * ld + c0 + j] = T(double(R[size_t(r) * ldr + j]) / den);
  }
}

// per problem: residual norms of the b Ritz pairs from diag(G) (G = R^T R); a
// problem whose first nev residuals are all <= tol is frozen (every later kernel
// of the engine skips it, so its basis, Ritz values and vectors stay those of
// this iteration; kfreeze records the basis size).  nconv = frozen problems.
__global__ void k_bconv(int Q, int nev, int b, const double* __restrict__ G, double tol, double* __restrict__ rnorm,
                        int* __restrict__ fz, int* __restrict__ kfreeze, int k, int* __restrict__ nconv) {
  __shared__ int cnt;
  if (threadIdx.x == 0) cnt = 0;
  __syncthreads();
  for (int q = threadIdx.x; q < Q; q += blockDim.x) {
    if (!fz[q]) {
      bool ok = true;
      for (int j = 0; j < b; ++j) {
        const double r = sqrt(fmax(G[size_t(q) * (kMaxLim * kMaxB) + j * b + j], 0.0));
        rnorm[q * kMaxB + j] = r;
        if (j < nev) ok = ok && r <= tol;
      }
      if (ok) {
        fz[q] = 1;
        kfreeze[q] = k;
      }
    }
    if (fz[q]) atomicAdd(&cnt, 1);
  }
  __syncthreads();
  if (threadIdx.x == 0) *nconv = cnt;
}

// replace marked columns by a fixed pseudo-random vector (hash of row and column)
template <class T>
__global__ void k_bfill(uint32_t nrows, const uint32_t* __restrict__ rowprob, const int* __restrict__ bad, T* V,
                        int ld, int c0, int b, uint32_t salt, const int* __restrict__ fz) {
  const uint32_t r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nrows || fz[rowprob[r]]) return;
  const int m = bad[rowprob[r]];
  if (!m) return;
  for (int j = 0; j < b; ++j)
    if (m >> j & 1) {
      uint32_t h = r * 0x9E3779B1u ^ (uint32_t(j + 1) * 0x85EBCA77u) ^ salt;
      h ^= h >> 15; h *= 0x2C1B3C6Du; h ^= h >> 12; h *= 0x297A2D39u; h ^= h >> 15;
      V[size_t(r) * ld + c0 + j] = T(double(h) * (1.0 / 4294967296.0) - 0.5);
    }
}

// S[q] = diag(w[q][0..keep)), rest zero
// after a thick restart: S = diag(kept Ritz values); the eigenvectors of that
// block are the identity (the warm start of the next Jacobi reads them from Z)
__global__ void k_bset_diag(int keep, const double* __restrict__ w, double* __restrict__ S, double* __restrict__ Z,
                            const int* __restrict__ fz) {
  const int q = blockIdx.x;
  if (fz[q]) return;
  double* Sq = S + size_t(q) * kJac * kJac;
  double* Zq = Z + size_t(q) * kJac * kJac;
  for (int i = threadIdx.x; i < kJac * kJac; i += blockDim.x) {
    const int r = i / kJac, c = i % kJac;
    Sq[i] = (r == c && r < keep) ? w[size_t(q) * kJac + r] : 0.0;
    Zq[i] = (r == c && r < keep) ? 1.0 : 0.0;
  }
}

// Block Gram-Schmidt with Pythagorean inner products for each problem: W =
// [V_basis | T]^T T ((c0 + b) x b, ld b) gives the projections Gp (first c0
// rows) and the block Gram Mt; S = Mt - Gp^T Gp is the Gram of the projected
// block.  Columns with |T_perp|^2 / |T|^2 >= min_ratio are orthonormalised by
// the Cholesky factor of S restricted to them (scaled to unit columns);
// weaker columns are only projected (the next pass normalises them), and a
// column with nothing left is marked in bad[] for replacement.  Writes the
// update coefficients C ((c0 + b) x b, ld kMaxB): T <- [V_basis | T] C.
__global__ void __launch_bounds__(64) k_bpip(int Q, int c0, int b, const double* __restrict__ G,
                                              double* __restrict__ M, int* __restrict__ bad,
                                              const int* __restrict__ fz, double min_ratio) {
  // one CTA of 64 threads per problem: the b x b Gram correction and the
  // (c0 + b) x b coefficients in parallel, the b x b factorisation on thread 0
  const int q = blockIdx.x, tid = threadIdx.x;
  if (q >= Q) return;
  if (fz[q]) {
    if (tid == 0) bad[q] = 0;
    return;
  }
  __shared__ double w[kMaxLim * kMaxB], S[kMaxB][kMaxB], R[kMaxB][kMaxB], d[kMaxB];
  __shared__ int bmask;
  const int K = c0 + b;
  for (int i = tid; i < K * b; i += blockDim.x) w[i] = G[size_t(q) * (kMaxLim * kMaxB) + i];
  __syncthreads();
  if (tid < b) {
    const double mjj = w[(c0 + tid) * b + tid];
    d[tid] = mjj > 0.0 ? 1.0 / sqrt(mjj) : 0.0;
  }
  __syncthreads();
  for (int t = tid; t < b * b; t += blockDim.x) {
    const int i = t / b, j = t % b;
    double v = w[(c0 + i) * b + j];
    for (int k = 0; k < c0; ++k) v -= w[k * b + i] * w[k * b + j];
    S[i][j] = v * d[i] * d[j];
  }
  __syncthreads();
  if (tid == 0) {
    int weak = 0, badmask = 0;
    for (int j = 0; j < b; ++j) {
      if (!(d[j] > 0.0)) badmask |= 1 << j;
      else if (!(S[j][j] >= min_ratio)) {
        weak |= 1 << j;
        if (!(S[j][j] > 1e-24)) badmask |= 1 << j;  // nothing outside the basis
      }
    }
    const int skip = weak | badmask;
    // Cholesky of S on the healthy columns (skipped rows/columns: identity)
    double L[kMaxB][kMaxB];
    for (int i = 0; i < b; ++i)
      for (int j = 0; j <= i; ++j) {
        if ((skip >> i & 1) || (skip >> j & 1)) {
          L[i][j] = i == j ? 1.0 : 0.0;
          continue;
        }
        double sum = S[i][j];
        for (int t = 0; t < j; ++t) sum -= L[i][t] * L[j][t];
        if (i == j) {
          if (!(sum > 1e-24)) {  // numerically dependent on the columns before: project only
            weak |= 1 << i;
            L[i][i] = 1.0;
            for (int t = 0; t < i; ++t) L[i][t] = 0.0;
          } else {
            L[i][i] = sqrt(sum);
          }
        } else {
          L[i][j] = (weak >> i & 1) ? 0.0 : sum / L[j][j];
        }
      }
    const int proj = weak | badmask;  // columns that are only projected
    // R = D L^{-T} on the healthy columns, e_j on the others (upper triangular)
    for (int j = 0; j < b; ++j) {
      for (int i = 0; i < b; ++i) R[i][j] = 0.0;
      if (proj >> j & 1) {
        R[j][j] = 1.0;
        continue;
      }
      double x[kMaxB];
      for (int i = b - 1; i >= 0; --i) {
        if (proj >> i & 1) {
          x[i] = 0.0;
          continue;
        }
        double r = i == j ? 1.0 : 0.0;
        for (int k = i + 1; k < b; ++k) r -= L[k][i] * x[k];
        x[i] = r / L[i][i];
      }
      for (int i = 0; i < b; ++i) R[i][j] = d[i] * x[i];
    }
    bmask = badmask;
  }
  __syncthreads();
  double* c = M + size_t(q) * (kMaxLim * kMaxB);
  for (int t = tid; t < K * b; t += blockDim.x) {
    const int k = t / b, j = t % b;
    double v;
    if (k < c0) {
      v = 0.0;
      for (int i = 0; i < b; ++i) v -= w[k * b + i] * R[i][j];
    } else {
      v = R[k - c0][j];
    }
    c[k * kMaxB + j] = v;
  }
  if (tid == 0) bad[q] = bmask;
}

template <class T>
__global__ void k_bpack(uint32_t nrows, const T* __restrict__ V, int ld, int c0, int b, T* __restrict__ W, int ldw) {
  uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i >= uint64_t(nrows) * ldw) return;
  const uint64_t r = i / ldw;
  const int j = int(i - r * ldw);
  W[i] = j < b ? V[r * ld + c0 + j] : T(0);
}

__global__ void k_bunits(int Q, const uint32_t* __restrict__ rows, int b, float* V32, double* V64, int ld) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= Q * b) return;
  const int j = i % b;
  if (V32) V32[size_t(rows[i]) * ld + j] = 1.f;
  if (V64) V64[size_t(rows[i]) * ld + j] = 1.0;
}

// X[r][0:b] = Ritz vectors of the problem of tile: V[:, 0:K] Z[:, 0:b] with K the
// freeze-time basis size for frozen problems; otherwise the last iteration's
// (V[:, 0:b] when that iteration restarted, V[:, 0:last_k] Z otherwise)
template <class T, class D>
__global__ void __launch_bounds__(256) k_britz(const BatchChunk* __restrict__ tiles, const T* __restrict__ V, int ld,
                                               const double* __restrict__ Z, const int* __restrict__ fz,
                                               const int* __restrict__ kfreeze, int last_k, int last_restarted,
                                               D* __restrict__ X, int ldx, int b) {
  __shared__ double Zs[kMaxLim * kMaxB];
  const BatchChunk tl = tiles[blockIdx.x];
  const bool frozen = fz[tl.prob] != 0;
  const bool copy = !frozen && last_restarted;
  const int K = frozen ? kfreeze[tl.prob] : last_k;
  const double* Zq = Z + size_t(tl.prob) * kJac * kJac;
  for (int i = threadIdx.x; i < K * b; i += blockDim.x) Zs[i] = Zq[(i / b) * kJac + (i % b)];
  __syncthreads();
  for (uint32_t r = tl.row0 + threadIdx.x; r < tl.row1; r += blockDim.x) {
    const T* vr = V + size_t(r) * ld;
    for (int j = 0; j < b; ++j) {
      double a = 0.0;
      if (copy) {
        a = double(vr[j]);
      } else {
        for (int i = 0; i < K; ++i) a += double(vr[i]) * Zs[i * b + j];
      }
      X[size_t(r) * ldx + j] = D(a);
    }
  }
}

inline unsigned nblk(uint64_t n, int t = 256) { return unsigned((n + t - 1) / t); }

// ---------------------------------------------------------------- engine
template <class T>
struct BEngine {
  BatchSet& bs;
  cudaStream_t s;
  int Q, nev, b, lim, keep;
  uint32_t N;
  DBuf<T> V, AV, R, W;        // N x lim, N x lim, N x 8, N x 8 (SpMM staging, FP32 engine)
  DBuf<double> S, Z, w, G, M, part, rnorm;
  DBuf<float> dfstage;        // N x 16 (FP64 engine: double-float staging)
  DBuf<int> fz, kfreeze, nconv, bad;
  int* h_nconv = nullptr;     // pinned
  std::vector<cudaGraphExec_t> graphs;  // per basis size
  std::vector<int> graph_kernels;
  int kernels_per_graph = 0;
  uint64_t graph_launches = 0, graph_kernel_launches = 0;
  double iter_s = 0;
  int last_k = 0;

  BEngine(BatchSet& b_, int nev0, int b0, int lim0, int keep0)
      : bs(b_), s(b_.stream), Q(b_.nq), nev(nev0), b(b0), lim(lim0), keep(keep0), N(uint32_t(b_.H.n)) {
    V.alloc(size_t(N) * lim);
    AV.alloc(size_t(N) * lim);
    R.alloc(size_t(N) * 8);
    W.alloc(size_t(N) * 8);
    if (sizeof(T) == 8) dfstage.alloc(size_t(N) * 16);
    S.alloc(size_t(Q) * kJac * kJac);
    Z.alloc(size_t(Q) * kJac * kJac);
    w.alloc(size_t(Q) * kJac);
    G.alloc(size_t(Q) * kMaxLim * kMaxB);
    M.alloc(size_t(Q) * kMaxLim * kMaxB);
    part.alloc(size_t(bs.nchunks) * kMaxLim * kMaxB);
    rnorm.alloc(size_t(Q) * kMaxB);
    fz.alloc(Q);
    kfreeze.alloc(Q);
    nconv.alloc(1);
    bad.alloc(Q);
    CG_CUDA(cudaMallocHost(&h_nconv, sizeof(int)));
    CG_CUDA(cudaMemsetAsync(V.p, 0, V.bytes(), s));
    CG_CUDA(cudaMemsetAsync(AV.p, 0, AV.bytes(), s));
    CG_CUDA(cudaMemsetAsync(S.p, 0, S.bytes(), s));
    CG_CUDA(cudaMemsetAsync(fz.p, 0, fz.bytes(), s));
    CG_CUDA(cudaMemsetAsync(kfreeze.p, 0, kfreeze.bytes(), s));
    CG_CUDA(cudaMemsetAsync(bad.p, 0, bad.bytes(), s));
    graphs.assign(lim + 1, nullptr);
    graph_kernels.assign(lim + 1, 0);
  }
  ~BEngine() {
    for (auto g : graphs)
      if (g) cudaGraphExecDestroy(g);
    if (h_nconv) cudaFreeHost(h_nconv);
  }

  // G[q] = X[:, xo:xo+K]^T Y[:, yo:yo+J] per (unfrozen) problem
  void xty(const T* X, int ldx, int xo, int K, const T* Y, int ldy, int yo, int J) {
    k_bxty<T><<<unsigned(bs.nchunks), 256, 0, s>>>(bs.chunks.p, X, ldx, xo, K, Y, ldy, yo, J, part.p, fz.p);
    k_breduce<<<Q, 128, 0, s>>>(bs.pchunk.p, part.p, K, J, G.p, fz.p);
  }
  void gemm(const T* X, int ldx, int xo, int K, const double* Mm, size_t mstride, int mld, T* Y, int ldy, int yo,
            int J, double alpha, double beta) {
    k_bgemm<T><<<unsigned(bs.nchunks), 256, 0, s>>>(bs.chunks.p, X, ldx, xo, K, Mm, mstride, mld, Y, ldy, yo, J,
                                                     alpha, beta, fz.p);
  }
  void spmm(int c0) {
    if constexpr (sizeof(T) == 4) {
      k_bpack<float><<<nblk(uint64_t(N) * 8), 256, 0, s>>>(N, V.p, lim, c0, b, W.p, 8);
      spmm_f32_padded(bs.H, W.p, 8, AV.p + c0, lim, b, s);
    } else {
      spmm_refine_df(bs.H, V.p + c0, lim, AV.p + c0, lim, b, dfstage.p, s);
    }
  }
  // orthonormalise V[:, c0:c0+b] against V[:, 0:c0] and within the block:
  // two passes of block Gram-Schmidt with Pythagorean inner products (one
  // X^T Y and one X C over basis + block per pass, k_bpip)
  void orthonormalise(int c0) {
    const size_t ms = kMaxLim * kMaxB;
    for (int pass = 0; pass < 2; ++pass) {
      // first pass: columns mostly inside the basis are only projected; the
      // second normalises every column that has anything left
      const double min_ratio = pass ? 0.0 : (sizeof(T) == 4 ? 1e-3 : 1e-8);
      xty(V.p, lim, 0, c0 + b, V.p, lim, c0, b);  // [V_basis | T]^T T
      k_bpip<<<Q, 64, 0, s>>>(Q, c0, b, G.p, M.p, bad.p, fz.p, min_ratio);
      gemm(V.p, lim, 0, c0 + b, M.p, ms, kMaxB, V.p, lim, c0, b, 1.0, 0.0);
      k_bfill<T><<<nblk(N), 256, 0, s>>>(N, bs.rowprob.p, bad.p, V.p, lim, c0, b, 0x1234567u + pass, fz.p);
    }
  }
  // one iteration with current basis size k (the newest b columns not yet multiplied)
  void enqueue_step(int k, double tol) {
    spmm(k - b);
    xty(V.p, lim, 0, k, AV.p, lim, k - b, b);
    k_bset_proj<<<Q, 128, 0, s>>>(k, b, k - b, G.p, S.p, fz.p);
    // warm start from the previous step's eigenvectors (size k - b; after a
    // restart the kept block is diagonal and Z's leading block the identity).
    // FP32 phase: FP32 sweeps first, then FP64 sweeps from their
    // (re-orthonormalized) vectors, which leave only ~1e-7 couplings, so the
    // FP64 pipe does one or two sweeps instead of a full solve
    if (sizeof(T) == 4) {
      k_bjacobi<float><<<Q, 256, jac_smem<float>(), s>>>(S.p, nullptr, k, w.p, Z.p, fz.p, k - b, 0);
      k_bjacobi<double><<<Q, 256, jac_smem<double>(), s>>>(S.p, nullptr, k, w.p, Z.p, fz.p, k, 1);
    } else {
      k_bjacobi<double><<<Q, 256, jac_smem<double>(), s>>>(S.p, nullptr, k, w.p, Z.p, fz.p, k - b, 0);
    }
    k_bresid<T><<<unsigned(bs.nchunks), 256, 0, s>>>(bs.chunks.p, V.p, AV.p, lim, k, w.p, Z.p, R.p, 8, b, fz.p);
    xty(R.p, 8, 0, b, R.p, 8, 0, b);
    k_bconv<<<1, 256, 0, s>>>(Q, nev, b, G.p, tol, rnorm.p, fz.p, kfreeze.p, k, nconv.p);
    CG_CUDA(cudaMemcpyAsync(h_nconv, nconv.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    int c0 = k;
    if (k + b > lim) {  // thick restart to the `keep` lowest Ritz vectors
      const size_t zs = size_t(kJac) * kJac;
      gemm(V.p, lim, 0, k, Z.p, zs, kJac, V.p, lim, 0, keep, 1.0, 0.0);
      gemm(AV.p, lim, 0, k, Z.p, zs, kJac, AV.p, lim, 0, keep, 1.0, 0.0);
      k_bset_diag<<<Q, 256, 0, s>>>(keep, w.p, S.p, Z.p, fz.p);
      c0 = keep;
    }
    k_bprecond<T><<<nblk(N, 128), 128, 0, s>>>(N, bs.rowprob.p, R.p, 8, w.p, bs.diag.p, V.p, lim, c0, b, fz.p);
    orthonormalise(c0);
  }
  int next_k(int k) const { return (k + b > lim ? keep : k) + b; }

  // run until every problem's first nev residuals are <= tol or maxiter; returns iterations
  int run(double tol, int maxiter, bool use_graph) {
    int k = b;
    int it = 0;
    for (; it < maxiter; ++it) {
      last_k = k;
      auto t0 = std::chrono::steady_clock::now();
      if (use_graph) {
        if (!graphs[k]) {
          cudaGraph_t g;
          CG_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
          enqueue_step(k, tol);
          CG_CUDA(cudaStreamEndCapture(s, &g));
          size_t nn = 0;
          CG_CUDA(cudaGraphGetNodes(g, nullptr, &nn));
          std::vector<cudaGraphNode_t> nodes(nn);
          CG_CUDA(cudaGraphGetNodes(g, nodes.data(), &nn));
          int nk = 0;
          for (auto nd : nodes) {
            cudaGraphNodeType ty;
            CG_CUDA(cudaGraphNodeGetType(nd, &ty));
            nk += ty == cudaGraphNodeTypeKernel;
          }
          graph_kernels[k] = nk;
          kernels_per_graph = std::max(kernels_per_graph, nk);
          CG_CUDA(cudaGraphInstantiate(&graphs[k], g, 0));
          CG_CUDA(cudaGraphDestroy(g));
        }
        CG_CUDA(cudaGraphLaunch(graphs[k], s));
        ++graph_launches;
        graph_kernel_launches += uint64_t(graph_kernels[k]);
      } else {
        enqueue_step(k, tol);
      }
      CG_CUDA(cudaStreamSynchronize(s));
      iter_s += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
      if (*h_nconv == Q) {
        ++it;
        break;
      }
      k = next_k(k);
    }
    return it;
  }
  // Ritz vectors (b per problem) into X (N x b, ld ldx)
  template <class D>
  void ritz_vectors(D* X, int ldx) {
    k_britz<T, D><<<unsigned(bs.nchunks), 256, 0, s>>>(bs.chunks.p, V.p, lim, Z.p, fz.p, kfreeze.p, last_k,
                                                        last_k + b > lim ? 1 : 0, X, ldx, b);
    CG_CUDA(cudaGetLastError());
    count_launch();
  }
};

}  // namespace

BatchSet::~BatchSet() {
  if (stream) cudaStreamDestroy(stream);
}

void batch_build(const std::vector<const System*>& sys, const std::vector<const Operator*>& ops, BatchSet& bs) {
  CG_CUDA(cudaGetDevice(&bs.device));
  if (!bs.stream) CG_CUDA(cudaStreamCreateWithFlags(&bs.stream, cudaStreamNonBlocking));
  cudaStream_t s = bs.stream;
  const int P = int(sys.size());
  bs.np = P;
  bs.dims.assign(P, 0);
  bs.kind.assign(P, 0);
  bs.slot.assign(P, -1);
  std::vector<std::unique_ptr<Hamiltonian>> hs(P);
  auto t0 = std::chrono::steady_clock::now();
  uint64_t ntot = 0, nnz = 0;
  int nq = 0, nd = 0;
  for (int p = 0; p < P; ++p) {
    Basis b;
    basis_build(*sys[p], b);
    bs.dims[p] = b.n;
    if (b.n == 0) continue;
    hs[p] = std::make_unique<Hamiltonian>();
    hamiltonian_build(*sys[p], *ops[p], b, CG_PREC_FP32, *hs[p], false);  // rows go into the block-diagonal CSR
    if (b.n <= uint64_t(kDense)) {
      bs.kind[p] = 1;
      bs.slot[p] = nd++;
    } else {
      bs.kind[p] = 2;
      bs.slot[p] = nq++;
      ntot += b.n;
      nnz += hs[p]->nnz;
    }
  }
  if (ntot >= (1ull << 32)) throw Error(CG_ERR_UNSUPPORTED, "batched rows beyond 2^32");
  bs.nq = nq;
  bs.nd = nd;
  // block-diagonal FP32 (hi + lo) matrix of the Davidson problems
  Hamiltonian& H = bs.H;
  H.device = bs.device;
  H.precision = CG_PREC_FP32;
  H.n = ntot;
  H.nnz = nnz;
  H.rowptr.alloc(ntot + 1);
  H.col.alloc(std::max<uint64_t>(nnz, 1));
  H.hi.alloc(std::max<uint64_t>(nnz, 1));
  H.lo.alloc(std::max<uint64_t>(nnz, 1));
  H.diag.alloc(std::max<uint64_t>(ntot, 1));
  std::vector<uint32_t> rowprob(ntot), pchunk(nq + 1, 0);
  std::vector<BatchChunk> chunks;
  bs.qrow0.assign(nq + 1, 0);
  bs.qprob.assign(nq, 0);
  uint64_t row = 0, e = 0;
  for (int p = 0; p < P; ++p) {
    if (bs.kind[p] != 2) continue;
    const Hamiltonian& h = *hs[p];
    const int q = bs.slot[p];
    bs.qprob[q] = p;
    bs.qrow0[q] = row;
    k_concat_rows<<<nblk(h.n), 256, 0, s>>>(h.n, h.rowptr.p, e, row, H.rowptr.p);
    k_concat_cols<<<nblk(h.nnz), 256, 0, s>>>(h.nnz, h.col.p, uint32_t(row), H.col.p + e);
    CG_CUDA(cudaMemcpyAsync(H.hi.p + e, h.hi.p, h.nnz * 4, cudaMemcpyDeviceToDevice, s));
    CG_CUDA(cudaMemcpyAsync(H.lo.p + e, h.lo.p, h.nnz * 4, cudaMemcpyDeviceToDevice, s));
    CG_CUDA(cudaMemcpyAsync(H.diag.p + row, h.diag.p, h.n * 8, cudaMemcpyDeviceToDevice, s));
    count_launch(2);
    pchunk[q] = uint32_t(chunks.size());
    for (uint64_t r0 = 0; r0 < h.n; r0 += kTile)
      chunks.push_back(BatchChunk{uint32_t(q), uint32_t(row + r0), uint32_t(row + std::min<uint64_t>(h.n, r0 + kTile))});
    for (uint64_t i = 0; i < h.n; ++i) rowprob[row + i] = uint32_t(q);
    row += h.n;
    e += h.nnz;
  }
  pchunk[nq] = uint32_t(chunks.size());
  bs.qrow0[nq] = row;
  CG_CUDA(cudaMemcpyAsync(H.rowptr.p + ntot, &e, 8, cudaMemcpyHostToDevice, s));
  bs.nchunks = int(chunks.size());
  bs.chunks.upload(chunks, s);
  bs.pchunk.upload(pchunk, s);
  bs.rowprob.upload(rowprob, s);
  bs.diag.alloc(std::max<uint64_t>(ntot, 1));
  CG_CUDA(cudaMemcpyAsync(bs.diag.p, H.diag.p, ntot * 8, cudaMemcpyDeviceToDevice, s));
  // host diagonal for the starting vectors
  bs.h_diag.resize(ntot);
  CG_CUDA(cudaMemcpyAsync(bs.h_diag.data(), H.diag.p, ntot * 8, cudaMemcpyDeviceToHost, s));
  // dense matrices of the small problems
  bs.dense.alloc(std::max<size_t>(size_t(nd) * kJac * kJac, 1));
  bs.ddim.assign(nd, 0);
  for (int p = 0; p < P; ++p) {
    if (bs.kind[p] != 1) continue;
    const Hamiltonian& h = *hs[p];
    const int d = bs.slot[p];
    bs.ddim[d] = int(h.n);
    k_dense_fill<<<unsigned(h.n), 64, 0, s>>>(int(h.n), 0, h.rowptr.p, h.col.p, h.hi.p, h.lo.p,
                                               bs.dense.p + size_t(d) * kJac * kJac);
    count_launch();
  }
  CG_CUDA(cudaGetLastError());
  CG_CUDA(cudaStreamSynchronize(s));  // the per-problem matrices (hs) are released after their copies
  // launch shape of the block-diagonal product (warps per CTA x resident CTAs
  // per SM), timed on this matrix with the solve's 8-vector rows; the iteration
  // graphs capture the chosen shape
  if (H.n > 0) {
    const auto ta = std::chrono::steady_clock::now();
    struct StreamLoan {  // H destroys its own stream; the batch's is only lent
      Hamiltonian& h;
      ~StreamLoan() { h.stream = nullptr; }
    } loan{H};
    H.stream = s;
    spmm_autotune(H, kMaxB, 2);
    bs.tune_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - ta).count();
  }
  bs.build_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

void batch_solve(BatchSet& bs, const BatchParams& prm, BatchResult& res) {
  // (also loads both Jacobi kernels before any iteration is captured into a graph)
  CG_CUDA(cudaFuncSetAttribute(k_bjacobi<double>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               int(jac_smem<double>())));
  CG_CUDA(cudaFuncSetAttribute(k_bjacobi<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               int(jac_smem<float>())));
  if (prm.nev < 1 || prm.nev > kMaxB) throw Error(CG_ERR_ARG, "batched solve: nstates must be in 1..8");
  if (prm.block < prm.nev || prm.block > kMaxB) throw Error(CG_ERR_ARG, "batched solve: block must be in nstates..8");
  if (prm.lim > kMaxLim || prm.keep < prm.block || prm.keep + prm.block > prm.lim)
    throw Error(CG_ERR_ARG, "batched solve: need block <= keep, keep + block <= lim <= 40");
  cudaStream_t s = bs.stream;
  const int P = bs.np, nev = prm.nev;
  res.eig.assign(size_t(P) * nev, std::nan(""));
  res.resid.assign(size_t(P) * nev, std::nan(""));
  res.nconv.assign(P, 0);
  res.found.assign(P, 0);
  auto t0 = std::chrono::steady_clock::now();
  const uint64_t l0 = launch_counter();
  // exact solves of the small problems (one launch)
  std::vector<double> dw, dz;
  if (bs.nd > 0) {
    DBuf<double> w(size_t(bs.nd) * kJac), Z(size_t(bs.nd) * kJac * kJac);
    DBuf<int> kd;
    kd.upload(bs.ddim, s);
    k_bjacobi<double><<<bs.nd, 256, jac_smem<double>(), s>>>(bs.dense.p, kd.p, 0, w.p, Z.p, nullptr, 0, 0);
    CG_CUDA(cudaGetLastError());
    count_launch();
    dw.resize(size_t(bs.nd) * kJac);
    CG_CUDA(cudaMemcpyAsync(dw.data(), w.p, dw.size() * 8, cudaMemcpyDeviceToHost, s));
    CG_CUDA(cudaStreamSynchronize(s));
  }
  for (int p = 0; p < P; ++p) {
    if (bs.kind[p] != 1) continue;
    const int d = bs.slot[p], k = bs.ddim[d], m = std::min(k, nev);
    for (int j = 0; j < m; ++j) {
      res.eig[size_t(p) * nev + j] = dw[size_t(d) * kJac + j];
      res.resid[size_t(p) * nev + j] = 0.0;
    }
    res.nconv[p] = m;
    res.found[p] = m;
  }
  // lockstep Davidson of the others
  if (bs.nq > 0) {
    const int Q = bs.nq;
    const int blk = prm.block;
    BEngine<float> e32(bs, nev, blk, prm.lim, prm.keep);
    // starting vectors: unit vectors at the nev lowest diagonal entries of each problem
    std::vector<uint32_t> urows(size_t(Q) * blk);
    for (int q = 0; q < Q; ++q) {
      const uint64_t r0 = bs.qrow0[q], r1 = bs.qrow0[q + 1];
      std::vector<uint32_t> idx(r1 - r0);
      std::iota(idx.begin(), idx.end(), 0u);
      std::partial_sort(idx.begin(), idx.begin() + blk, idx.end(), [&](uint32_t a, uint32_t c) {
        return bs.h_diag[r0 + a] < bs.h_diag[r0 + c] || (bs.h_diag[r0 + a] == bs.h_diag[r0 + c] && a < c);
      });
      for (int j = 0; j < blk; ++j) urows[size_t(q) * blk + j] = uint32_t(r0 + idx[j]);
    }
    DBuf<uint32_t> du;
    du.upload(urows, s);
    k_bunits<<<nblk(size_t(Q) * blk), 256, 0, s>>>(Q, du.p, blk, e32.V.p, nullptr, prm.lim);
    count_launch();
    const double sw = std::max(prm.switch_resid, prm.tol_resid);
    res.iterations32 = e32.run(sw, prm.maxiter, prm.use_graph);
    res.graph_launches += e32.graph_launches;
    res.graph_kernels = std::max(res.graph_kernels, e32.kernels_per_graph);
    res.graph_kernel_launches += e32.graph_kernel_launches;
    // FP64 phase from the FP32 Ritz vectors
    BEngine<double> e64(bs, nev, blk, prm.lim, prm.keep);
    e32.ritz_vectors(e64.V.p, prm.lim);  // FP32 Ritz vectors, widened, start the FP64 phase
    e64.orthonormalise(0);
    res.iterations64 = e64.run(prm.tol_resid, prm.maxiter, prm.use_graph);
    res.graph_launches += e64.graph_launches;
    res.graph_kernels = std::max(res.graph_kernels, e64.kernels_per_graph);
    res.graph_kernel_launches += e64.graph_kernel_launches;
    std::vector<double> w(size_t(Q) * kJac), rn(size_t(Q) * kMaxB);
    std::vector<int> cv(Q);
    CG_CUDA(cudaMemcpyAsync(w.data(), e64.w.p, w.size() * 8, cudaMemcpyDeviceToHost, s));
    CG_CUDA(cudaMemcpyAsync(rn.data(), e64.rnorm.p, rn.size() * 8, cudaMemcpyDeviceToHost, s));
    CG_CUDA(cudaStreamSynchronize(s));
    for (int q = 0; q < Q; ++q) {
      const int p = bs.qprob[q];
      int c = 0;
      for (int j = 0; j < nev; ++j) {
        res.eig[size_t(p) * nev + j] = w[size_t(q) * kJac + j];
        res.resid[size_t(p) * nev + j] = rn[size_t(q) * kMaxB + j];
        c += rn[size_t(q) * kMaxB + j] <= prm.tol_resid;
      }
      res.nconv[p] = c;
      res.found[p] = nev;
    }
    res.spmm_seconds = e32.iter_s + e64.iter_s;
  }
  res.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  res.launches = launch_counter() - l0 + res.graph_kernel_launches;
  count_launch(res.graph_kernel_launches);
}

}  // namespace cg
