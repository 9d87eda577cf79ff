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
#include "dfloat.h"
#include "virtual.h"
#include "dense.h"
#include "device.h"

namespace cg {
namespace {

constexpr int kTile = 32;   // rows per tile
constexpr int kMaxK = 64;   // basis columns per tall-skinny kernel call
constexpr int kMaxLim = 128;  // basis limit (calls over more than kMaxK columns are split or use the 128-row forms)
constexpr int kMaxKeep = 64;  // Ritz vectors kept at a thick restart
constexpr int kMaxJ = 32;   // right-hand columns per call
constexpr int kMaxC = 16;   // residual candidates per call
constexpr int kThreads = 256;

template <class T>
__global__ void __launch_bounds__(kThreads) k_xty(uint64_t n, const T* __restrict__ X, int ldx, int xo, int K,
                                                  const T* __restrict__ Y, int ldy, int yo, int J,
                                                  double* __restrict__ part, uint64_t rows_per_cta) {
  __shared__ T xs[kTile * kMaxK];
  __shared__ T ys[kTile * kMaxJ];
  const int nout = K * J;
  double acc[8] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
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
    for (int q = 0; q < 8; ++q) {
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
  for (int q = 0; q < 8; ++q) {
    int o = threadIdx.x + q * kThreads;
    if (o < nout) part[uint64_t(blockIdx.x) * nout + o] = acc[q];
  }
}

// out[o] = sum_c part[c * nout + o]: one CTA per output, strided per-thread
// sums and a fixed-order tree, so the result is deterministic.
__global__ void k_reduce_parts(const double* __restrict__ part, int nparts, int nout, double* __restrict__ out) {
  __shared__ double red[128];
  const int o = blockIdx.x;
  double s = 0.0;
  for (int c = threadIdx.x; c < nparts; c += 128) s += part[uint64_t(c) * nout + o];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int w = 64; w; w >>= 1) {
    if (threadIdx.x < w) red[threadIdx.x] += red[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[o] = red[0];
}

// ---- streaming tall-skinny kernels -------------------------------------
// G (K x J) partials = X[:, xo:xo+K]^T Y[:, yo:yo+J] over this CTA's rows.
// KP = K rounded up to a power of two (<= 64) threads share one row, thread
// k of the group owns column k of X and all J outputs of that column; FP32
// products are summed over 64-row chunks and the chunks in FP64.
template <class T, int JMAX>
__global__ void __launch_bounds__(256) k_xty_s(uint64_t n, const T* __restrict__ X, int ldx, int xo, int K,
                                               const T* __restrict__ Y, int ldy, int yo, int J, int KP,
                                               double* __restrict__ part, uint64_t rows_per_cta) {
  __shared__ double red[256 * 2];
  const int k = threadIdx.x % KP, rg = threadIdx.x / KP, ngroups = 256 / KP;
  const bool active = k < K;
  double acc[JMAX];
  T ch[JMAX];
#pragma unroll
  for (int j = 0; j < JMAX; ++j) { acc[j] = 0.0; ch[j] = T(0); }
  const uint64_t r0 = uint64_t(blockIdx.x) * rows_per_cta;
  const uint64_t r1 = min(n, r0 + rows_per_cta);
  int cnt = 0;
  for (uint64_t r = r0 + rg; r < r1; r += ngroups) {
    const T xv = active ? X[r * ldx + xo + k] : T(0);
    const T* yr = Y + r * ldy + yo;
#pragma unroll
    for (int j = 0; j < JMAX; ++j)
      if (j < J) ch[j] = fma(xv, __ldg(yr + j), ch[j]);
    if (++cnt == 64) {
#pragma unroll
      for (int j = 0; j < JMAX; ++j) { acc[j] += double(ch[j]); ch[j] = T(0); }
      cnt = 0;
    }
  }
#pragma unroll
  for (int j = 0; j < JMAX; ++j) acc[j] += double(ch[j]);
  // reduce the row groups: for each j, sum acc over rg (same k); J is uniform
#pragma unroll
  for (int j = 0; j < JMAX; ++j) {
    if (j < J) {
      red[threadIdx.x] = acc[j];
      __syncthreads();
      if (rg == 0 && active) {
        double sum = 0.0;
        for (int g = 0; g < ngroups; ++g) sum += red[g * KP + k];
        part[uint64_t(blockIdx.x) * (K * J) + k * J + j] = sum;
      }
      __syncthreads();
    }
  }
}

// Warp-per-row-chunk X^T Y: lane l owns columns l and l + 32 of X (K <= 64);
// four rows are loaded before they are used so each warp keeps several rows of
// loads in flight.  FP32 (or FP64) products, 64-row chunks summed in FP64;
// per-warp partials go to part[warp][k * J + j].
template <class T, int JMAX>
__global__ void __launch_bounds__(256) k_xty_w(uint64_t n, const T* __restrict__ X, int ldx, int xo, int K,
                                               const T* __restrict__ Y, int ldy, int yo, int J,
                                               double* __restrict__ part, uint64_t rows_per_warp) {
  const int lane = threadIdx.x & 31;
  const uint64_t gw = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  // Y rows as float4 when every row start is 16-byte aligned; the columns past
  // J in the last float4 are zero-weighted below (yv beyond J only meets c0/c1
  // of columns j >= J, which are never written out)
  const bool vec_y = (reinterpret_cast<uintptr_t>(Y + yo) % 16 == 0) && (ldy % 4 == 0) && (J % 4 == 0);
  const uint64_t r0 = gw * rows_per_warp;
  const uint64_t r1 = min(n, r0 + rows_per_warp);
  const bool a0 = lane < K, a1 = lane + 32 < K;
  T c0[JMAX], c1[JMAX];
  double d0[JMAX], d1[JMAX];
#pragma unroll
  for (int j = 0; j < JMAX; ++j) { c0[j] = c1[j] = T(0); d0[j] = d1[j] = 0.0; }
  int cnt = 0;
  for (uint64_t r = r0; r < r1; r += 4) {
    T x0[4], x1[4], yv[4][JMAX];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const bool ok = r + u < r1;
      const T* xr = X + (r + u) * ldx + xo;
      x0[u] = (ok && a0) ? xr[lane] : T(0);
      x1[u] = (ok && a1) ? xr[lane + 32] : T(0);
      const T* yr = Y + (r + u) * ldy + yo;
      if constexpr (sizeof(T) == 4 && JMAX % 4 == 0) {
        if (vec_y) {  // J values of the row as 16-byte loads (broadcast across the warp)
#pragma unroll
          for (int j4 = 0; j4 < JMAX / 4; ++j4) {
            const float4 v = (ok && 4 * j4 < J) ? __ldg(reinterpret_cast<const float4*>(yr) + j4)
                                                : make_float4(0.f, 0.f, 0.f, 0.f);
            yv[u][4 * j4] = v.x;
            yv[u][4 * j4 + 1] = v.y;
            yv[u][4 * j4 + 2] = v.z;
            yv[u][4 * j4 + 3] = v.w;
          }
          continue;
        }
      }
#pragma unroll
      for (int j = 0; j < JMAX; ++j) yv[u][j] = (ok && j < J) ? __ldg(yr + j) : T(0);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int j = 0; j < JMAX; ++j) {
        c0[j] = fma(x0[u], yv[u][j], c0[j]);
        c1[j] = fma(x1[u], yv[u][j], c1[j]);
      }
    cnt += 4;
    if (cnt >= 64) {
#pragma unroll
      for (int j = 0; j < JMAX; ++j) { d0[j] += double(c0[j]); d1[j] += double(c1[j]); c0[j] = c1[j] = T(0); }
      cnt = 0;
    }
  }
  double* out = part + gw * uint64_t(K * J);
#pragma unroll
  for (int j = 0; j < JMAX; ++j) {
    if (j < J) {
      if (a0) out[lane * J + j] = d0[j] + double(c0[j]);
      if (a1) out[(lane + 32) * J + j] = d1[j] + double(c1[j]);
    }
  }
}

// ---- double-float arithmetic for the FP64 engine (dfloat.h) ----------------

// X^T Y of the FP64 engine in double-float: as k_xty_t, with the staged Y chunk
// held as FP32 pairs and 32-row chunks summed in double-float, then in FP64.
template <int JMAX>
__global__ void __launch_bounds__(256) k_xty_df(uint64_t n, const double* __restrict__ X, int ldx, int xo, int K,
                                                const double* __restrict__ Y, int ldy, int yo, int J,
                                                double* __restrict__ part, uint64_t rows_per_warp) {
  constexpr int CH = 32;
  __shared__ __align__(16) float yh[8][CH * JMAX], yl[8][CH * JMAX];
  __shared__ double dsh[8][2 * JMAX][32];
  const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
  const uint64_t gw = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const uint64_t r0 = gw * rows_per_warp;
  const uint64_t r1 = min(n, r0 + rows_per_warp);
  const bool a0 = lane < K, a1 = lane + 32 < K;
#pragma unroll
  for (int j = 0; j < 2 * JMAX; ++j) dsh[wl][j][lane] = 0.0;
  for (uint64_t c0 = r0; c0 < r1; c0 += CH) {
    const int rows = int(min(uint64_t(CH), r1 - c0));
    __syncwarp();
    for (int i = lane; i < CH * JMAX; i += 32) {
      const int rr = i / JMAX, j = i - rr * JMAX;
      const double v = (rr < rows && j < J) ? Y[(c0 + rr) * ldy + yo + j] : 0.0;
      df_split(v, yh[wl][i], yl[wl][i]);
    }
    __syncwarp();
    float c0h[JMAX], c0l[JMAX], c1h[JMAX], c1l[JMAX];
#pragma unroll
    for (int j = 0; j < JMAX; ++j) { c0h[j] = c0l[j] = c1h[j] = c1l[j] = 0.f; }
    for (int rr = 0; rr < rows; ++rr) {
      const double* xr = X + (c0 + rr) * ldx + xo;
      float xah = 0.f, xal = 0.f, xbh = 0.f, xbl = 0.f;
      if (a0) df_split(xr[lane], xah, xal);
      if (a1) df_split(xr[lane + 32], xbh, xbl);
      const float* yhr = yh[wl] + rr * JMAX;
      const float* ylr = yl[wl] + rr * JMAX;
#pragma unroll
      for (int j = 0; j < JMAX; ++j) {
        df_mac(c0h[j], c0l[j], xah, xal, yhr[j], ylr[j]);
        if (a1) df_mac(c1h[j], c1l[j], xbh, xbl, yhr[j], ylr[j]);
      }
    }
#pragma unroll
    for (int j = 0; j < JMAX; ++j) {
      dsh[wl][j][lane] += double(c0h[j]) + double(c0l[j]);
      dsh[wl][JMAX + j][lane] += double(c1h[j]) + double(c1l[j]);
    }
  }
  double* out = part + gw * uint64_t(K * J);
#pragma unroll
  for (int j = 0; j < JMAX; ++j) {
    if (j < J) {
      if (a0) out[lane * J + j] = dsh[wl][j][lane];
      if (a1) out[(lane + 32) * J + j] = dsh[wl][JMAX + j][lane];
    }
  }
}

// R = AB s_c - lam_c B s_c of the FP64 engine in double-float, one thread per
// row; s and lam as FP32 pairs in shared memory; R and the norms in FP64.
template <int CMAX, int KM>
__global__ void __launch_bounds__(256) k_resid_df(uint64_t n, const double* __restrict__ B,
                                                  const double* __restrict__ AB, int ld, int K,
                                                  const double* __restrict__ Sc, const double* __restrict__ lam, int C,
                                                  double* __restrict__ R, int ldr, double* __restrict__ part) {
  __shared__ float sh_[KM * CMAX], sl_[KM * CMAX];
  __shared__ double ls[CMAX];
  __shared__ double red[8][CMAX];
  for (int i = threadIdx.x; i < KM * CMAX; i += blockDim.x) {
    const int k = i / CMAX, c = i % CMAX;
    df_split((k < K && c < C) ? Sc[k * C + c] : 0.0, sh_[i], sl_[i]);
  }
  for (int i = threadIdx.x; i < CMAX; i += blockDim.x) ls[i] = i < C ? lam[i] : 0.0;
  __syncthreads();
  double nrm[CMAX];
#pragma unroll
  for (int c = 0; c < CMAX; ++c) nrm[c] = 0.0;
  for (uint64_t r = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; r < n; r += uint64_t(gridDim.x) * blockDim.x) {
    float ah[CMAX], al[CMAX], bh[CMAX], bl[CMAX];
#pragma unroll
    for (int c = 0; c < CMAX; ++c) { ah[c] = al[c] = bh[c] = bl[c] = 0.f; }
    const double* br = B + r * ld;
    const double* abr = AB + r * ld;
    for (int k = 0; k < K; ++k) {
      float xbh, xbl, xah, xal;
      df_split(br[k], xbh, xbl);
      df_split(abr[k], xah, xal);
#pragma unroll
      for (int c = 0; c < CMAX; ++c) {
        const float s0 = sh_[k * CMAX + c], s1 = sl_[k * CMAX + c];
        df_mac(ah[c], al[c], xah, xal, s0, s1);
        df_mac(bh[c], bl[c], xbh, xbl, s0, s1);
      }
    }
#pragma unroll
    for (int c = 0; c < CMAX; ++c)
      if (c < C) {
        const double res = (double(ah[c]) + double(al[c])) - ls[c] * (double(bh[c]) + double(bl[c]));
        R[r * ldr + c] = res;
        nrm[c] += res * res;
      }
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int c = 0; c < CMAX; ++c) {
    double v = nrm[c];
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(~0u, v, o);
    if (lane == 0) red[w][c] = v;
  }
  __syncthreads();
  if (threadIdx.x < C) {
    double v = 0.0;
    for (int i = 0; i < int(blockDim.x >> 5); ++i) v += red[i][threadIdx.x];
    part[uint64_t(blockIdx.x) * C + threadIdx.x] = v;
  }
}

// Y = beta Y + alpha X G of the FP64 engine in double-float: one thread per
// row, alpha G as FP32 pairs in shared memory, outputs combined in FP64.  A row
// is read completely before it is written (X and Y may alias).
template <int JMAX, int KM>
__global__ void __launch_bounds__(256) k_gemm_df(uint64_t n, const double* X, int ldx, int xo, int K,
                                                 const double* __restrict__ G, double* Y, int ldy, int yo, int J,
                                                 double alpha, double beta) {
  __shared__ float gh[KM * JMAX], gl[KM * JMAX];
  for (int i = threadIdx.x; i < KM * JMAX; i += blockDim.x) {
    const int k = i / JMAX, j = i % JMAX;
    df_split((k < K && j < J) ? alpha * G[k * J + j] : 0.0, gh[i], gl[i]);
  }
  __syncthreads();
  for (uint64_t r = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; r < n; r += uint64_t(gridDim.x) * blockDim.x) {
    float ah[JMAX], al[JMAX];
#pragma unroll
    for (int j = 0; j < JMAX; ++j) { ah[j] = 0.f; al[j] = 0.f; }
    const double* xr = X + r * ldx + xo;
    for (int k = 0; k < K; ++k) {
      float xh, xl;
      df_split(xr[k], xh, xl);
#pragma unroll
      for (int j = 0; j < JMAX; ++j) df_mac(ah[j], al[j], xh, xl, gh[k * JMAX + j], gl[k * JMAX + j]);
    }
    double* yr = Y + r * ldy + yo;
#pragma unroll
    for (int j = 0; j < JMAX; ++j)
      if (j < J) {
        const double v = double(ah[j]) + double(al[j]);
        yr[j] = beta == 0.0 ? v : fma(beta, yr[j], v);
      }
  }
}

// X^T Y with the Y sub-block of each 64-row chunk staged in shared memory:
// the warp first copies the chunk's J columns of Y (coalesced: lane groups of
// J read consecutive rows), then lane l owns columns l and l + 32 of X and
// reads the J values of a row as shared-memory broadcasts.  FP32 products are
// summed over the chunk and the chunks in FP64; per-warp partials go to
// part[warp][k * J + j].  Any column offset yo (no alignment needed).
template <class T, int JMAX>
__global__ void __launch_bounds__(256, 4) k_xty_t(uint64_t n, const T* __restrict__ X, int ldx, int xo, int K,
                                               const T* __restrict__ Y, int ldy, int yo, int J,
                                               double* __restrict__ part, uint64_t rows_per_warp) {
  constexpr int CH = JMAX * sizeof(T) > 32 ? 32 : 64;  // staged rows per chunk (<= 32 KB per CTA)
  __shared__ __align__(16) T ys[8][CH * JMAX];
  // FP64 chunk sums of lane l, column j at dsh[warp][j][l] (x0) and [JMAX + j][l] (x1)
  __shared__ double dsh[8][2 * JMAX][32];
  const int lane = threadIdx.x & 31, wl = threadIdx.x >> 5;
  const uint64_t gw = (uint64_t(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
  const uint64_t r0 = gw * rows_per_warp;
  const uint64_t r1 = min(n, r0 + rows_per_warp);
  const bool a0 = lane < K, a1 = lane + 32 < K;
  T* yw = ys[wl];
#pragma unroll
  for (int j = 0; j < 2 * JMAX; ++j) dsh[wl][j][lane] = 0.0;
  for (uint64_t c0 = r0; c0 < r1; c0 += CH) {
    const int rows = int(min(uint64_t(CH), r1 - c0));
    __syncwarp();
    for (int i = lane; i < CH * JMAX; i += 32) {
      const int rr = i / JMAX, j = i - rr * JMAX;
      yw[i] = (rr < rows && j < J) ? Y[(c0 + rr) * ldy + yo + j] : T(0);
    }
    __syncwarp();
    T c0v[JMAX], c1v[JMAX];
#pragma unroll
    for (int j = 0; j < JMAX; ++j) { c0v[j] = T(0); c1v[j] = T(0); }
    constexpr int U = sizeof(T) == 4 ? 8 : 4;  // rows of X loads in flight per lane
    for (int rr = 0; rr < rows; rr += U) {
      const T* xr0 = X + (c0 + rr) * ldx + xo;
      T xa[U], xb[U];
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const bool ok = rr + u < rows;
        xa[u] = (a0 && ok) ? xr0[u * ldx + lane] : T(0);
        xb[u] = (a1 && ok) ? xr0[u * ldx + lane + 32] : T(0);
      }
#pragma unroll
      for (int u = 0; u < U; ++u) {
        const T* ya = yw + (rr + u) * JMAX;
#pragma unroll
        for (int j = 0; j < JMAX; ++j) {
          const T v = ya[j];
          c0v[j] = fma(xa[u], v, c0v[j]);
          c1v[j] = fma(xb[u], v, c1v[j]);
        }
      }
    }
#pragma unroll
    for (int j = 0; j < JMAX; ++j) {
      dsh[wl][j][lane] += double(c0v[j]);
      dsh[wl][JMAX + j][lane] += double(c1v[j]);
    }
  }
  double* out = part + gw * uint64_t(K * J);
#pragma unroll
  for (int j = 0; j < JMAX; ++j) {
    if (j < J) {
      if (a0) out[lane * J + j] = dsh[wl][j][lane];
      if (a1) out[(lane + 32) * J + j] = dsh[wl][JMAX + j][lane];
    }
  }
}

// 32-byte load of 8 consecutive floats (32-byte aligned address): one L1
// request per thread for a whole 8-float segment of a row (thread-per-row
// kernels read rows 256 bytes apart, so every request touches one sector per
// lane; halving the requests halves the L1 work).  Coherent (not .nc): the
// gemm may write the rows it reads.
__device__ __forceinline__ void ld8c(const float* p, float (&v)[8]) {
  asm volatile("ld.global.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7])
               : "l"(p)
               : "memory");
}

// 32-byte store of 8 consecutive floats (32-byte aligned address): one L1
// request per thread instead of eight partial-sector stores.
__device__ __forceinline__ void st8(float* p, const float (&v)[8]) {
  asm volatile("st.global.v8.f32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};"
               :
               : "l"(p), "f"(v[0]), "f"(v[1]), "f"(v[2]), "f"(v[3]), "f"(v[4]), "f"(v[5]), "f"(v[6]), "f"(v[7])
               : "memory");
}

// R[:, c] = AB s_c - lam_c B s_c for C candidates, one thread per row with the
// row read 8 values (32 bytes) at a time when aligned, s in shared memory, R
// rows written 8 columns at a time; per-CTA partial |R[:, c]|^2 (FP32 over a
// thread's rows, FP64 across threads, fixed order).
template <class T, int CMAX, int KM>
__global__ void __launch_bounds__(256) k_resid_v(uint64_t n, const T* __restrict__ B, const T* __restrict__ AB,
                                                 int ld, int K, const double* __restrict__ Sc,
                                                 const double* __restrict__ lam, int C, T* __restrict__ R, int ldr,
                                                 double* __restrict__ part, bool vec, bool vec_r) {
  __shared__ __align__(16) T ss[KM * CMAX];
  __shared__ T ls[CMAX];
  __shared__ double red[8][CMAX];
  for (int i = threadIdx.x; i < KM * CMAX; i += blockDim.x) {
    const int k = i / CMAX, c = i % CMAX;
    ss[i] = (k < K && c < C) ? T(Sc[k * C + c]) : T(0);
  }
  for (int i = threadIdx.x; i < CMAX; i += blockDim.x) ls[i] = i < C ? T(lam[i]) : T(0);
  __syncthreads();
  T nrm[CMAX];
#pragma unroll
  for (int c = 0; c < CMAX; ++c) nrm[c] = T(0);
  // columns written by 32-byte stores: whole groups of 8, the ones past C
  // hold exact zeros (zero weights in ss and ls), so no sector is written in part
  const int cvec = (sizeof(T) == 4 && vec_r) ? (C + 7) / 8 * 8 : 0;
  for (uint64_t r = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; r < n; r += uint64_t(gridDim.x) * blockDim.x) {
    // res_c = sum_k (AB_k - lam_c B_k) s_kc: one accumulator per candidate
    T res[CMAX];
#pragma unroll
    for (int c = 0; c < CMAX; ++c) res[c] = T(0);
    const T* br = B + r * ld;
    const T* abr = AB + r * ld;
    int k = 0;
    if constexpr (sizeof(T) == 4) {
      if (vec) {  // rows 32-byte aligned
        for (; k + 8 <= K; k += 8) {
          float bb[8], aa[8];
          ld8c(br + k, bb);
          ld8c(abr + k, aa);
#pragma unroll
          for (int u = 0; u < 8; ++u)
#pragma unroll
            for (int c = 0; c < CMAX; ++c)
              res[c] = fma(fma(-ls[c], bb[u], aa[u]), ss[(k + u) * CMAX + c], res[c]);
        }
      }
    }
    for (; k < K; ++k) {
      const T bv = br[k], av = abr[k];
#pragma unroll
      for (int c = 0; c < CMAX; ++c) res[c] = fma(fma(-ls[c], bv, av), ss[k * CMAX + c], res[c]);
    }
#pragma unroll
    for (int c = 0; c < CMAX; ++c)
      if (c < C) nrm[c] = fma(res[c], res[c], nrm[c]);
    T* rr = R + r * ldr;
    if constexpr (sizeof(T) == 4) {
      // R rows 32-byte aligned: whole 8-column groups as one store each
#pragma unroll
      for (int g = 0; g < CMAX / 8; ++g)
        if (8 * g + 8 <= cvec) {
          float v[8];
#pragma unroll
          for (int u = 0; u < 8; ++u) v[u] = res[8 * g + u];
          st8(rr + 8 * g, v);
        }
    }
#pragma unroll
    for (int c = 0; c < CMAX; ++c)
      if (c >= cvec && c < C) rr[c] = res[c];
  }
  // CTA partials: warp shuffles then the 8 warps in order
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int c = 0; c < CMAX; ++c) {
    double v = double(nrm[c]);
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(~0u, v, o);
    if (lane == 0) red[w][c] = v;
  }
  __syncthreads();
  if (threadIdx.x < C) {
    double v = 0.0;
    for (int i = 0; i < int(blockDim.x >> 5); ++i) v += red[i][threadIdx.x];
    part[uint64_t(blockIdx.x) * C + threadIdx.x] = v;
  }
}

// Y[:, yo:yo+J] = beta Y + alpha X[:, xo:xo+K] G, one thread per row, all J
// outputs of the row in registers, G (alpha folded in) in shared memory read
// as broadcast; FP32 X rows read 8 values (32 bytes) at a time when aligned.  A row is
// read completely before it is written, so X and Y may alias.
template <class T, int JMAX, int KM>
__global__ void __launch_bounds__(256) k_gemm_r(uint64_t n, const T* X, int ldx, int xo, int K,
                                                const double* __restrict__ G, T* Y, int ldy, int yo, int J,
                                                double alpha, double beta, bool vec_x, bool vec_y) {
  __shared__ __align__(16) T gs[KM * JMAX];
  for (int i = threadIdx.x; i < KM * JMAX; i += blockDim.x) {
    const int k = i / JMAX, j = i % JMAX;
    gs[i] = (k < K && j < J) ? T(alpha * G[k * J + j]) : T(0);
  }
  __syncthreads();
  const T tb = T(beta);
  for (uint64_t r = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; r < n; r += uint64_t(gridDim.x) * blockDim.x) {
    T acc[JMAX];
#pragma unroll
    for (int j = 0; j < JMAX; ++j) acc[j] = T(0);
    const T* xr = X + r * ldx + xo;
    int k = 0;
    if constexpr (sizeof(T) == 4) {
      if (vec_x) {  // row segment 32-byte aligned
        for (; k + 8 <= K; k += 8) {
          float xv[8];
          ld8c(xr + k, xv);
#pragma unroll
          for (int u = 0; u < 8; ++u)
#pragma unroll
            for (int j = 0; j < JMAX; ++j) acc[j] = fma(xv[u], gs[(k + u) * JMAX + j], acc[j]);
        }
      }
    }
    for (; k < K; ++k) {
      const T xv = xr[k];
#pragma unroll
      for (int j = 0; j < JMAX; ++j) acc[j] = fma(xv, gs[k * JMAX + j], acc[j]);
    }
    T* yr = Y + r * ldy + yo;
    if constexpr (sizeof(T) == 4 && JMAX % 8 == 0) {
      if (vec_y) {  // Y segment 32-byte aligned, J a multiple of 8: 32-byte stores
#pragma unroll
        for (int g = 0; g < JMAX / 8; ++g)
          if (8 * g < J) {
            float v[8];
            if (beta != 0.0) {
              float o[8];
              ld8c(yr + 8 * g, o);
#pragma unroll
              for (int u = 0; u < 8; ++u) v[u] = fma(tb, o[u], acc[8 * g + u]);
            } else {
#pragma unroll
              for (int u = 0; u < 8; ++u) v[u] = acc[8 * g + u];
            }
            st8(yr + 8 * g, v);
          }
        continue;
      }
    }
#pragma unroll
    for (int j = 0; j < JMAX; ++j)
      if (j < J) yr[j] = (beta == 0.0) ? acc[j] : fma(tb, yr[j], acc[j]);
  }
}

// Thread per row: R[:, c] = AB s_c - lam_c B s_c for C candidates, plus
// per-CTA partial |R[:, c]|^2 (FP32 over 16-row chunks, FP64 across).
template <class T, int CMAX>
__global__ void __launch_bounds__(256) k_resid_s(uint64_t n, const T* __restrict__ B, const T* __restrict__ AB,
                                                 int ld, int K, const double* __restrict__ Sc,
                                                 const double* __restrict__ lam, int C, T* __restrict__ R, int ldr,
                                                 double* __restrict__ part) {
  __shared__ T ss[64 * CMAX];
  __shared__ T ls[CMAX];
  __shared__ double red[256];
  for (int i = threadIdx.x; i < K * C; i += blockDim.x) ss[(i / C) * CMAX + (i % C)] = T(Sc[i]);
  for (int i = threadIdx.x; i < CMAX; i += blockDim.x) ls[i] = i < C ? T(lam[i]) : T(0);
  __syncthreads();
  double nacc[CMAX];
  T nch[CMAX];
#pragma unroll
  for (int c = 0; c < CMAX; ++c) { nacc[c] = 0.0; nch[c] = T(0); }
  int cnt = 0;
  for (uint64_t r = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; r < n; r += uint64_t(gridDim.x) * blockDim.x) {
    T a[CMAX], b[CMAX];
#pragma unroll
    for (int c = 0; c < CMAX; ++c) { a[c] = T(0); b[c] = T(0); }
    const T* br = B + r * ld;
    const T* abr = AB + r * ld;
    for (int k = 0; k < K; ++k) {
      const T bv = br[k], av = abr[k];
#pragma unroll
      for (int c = 0; c < CMAX; ++c) {
        a[c] = fma(av, ss[k * CMAX + c], a[c]);
        b[c] = fma(bv, ss[k * CMAX + c], b[c]);
      }
    }
#pragma unroll
    for (int c = 0; c < CMAX; ++c)
      if (c < C) {
        const T res = a[c] - ls[c] * b[c];
        R[r * ldr + c] = res;
        nch[c] = fma(res, res, nch[c]);
      }
    if (++cnt == 16) {
#pragma unroll
      for (int c = 0; c < CMAX; ++c) { nacc[c] += double(nch[c]); nch[c] = T(0); }
      cnt = 0;
    }
  }
#pragma unroll
  for (int c = 0; c < CMAX; ++c) {
    if (c < C) {
      red[threadIdx.x] = nacc[c] + double(nch[c]);
      __syncthreads();
      for (int o = 128; o; o >>= 1) {
        if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
        __syncthreads();
      }
      if (threadIdx.x == 0) part[uint64_t(blockIdx.x) * C + c] = red[0];
      __syncthreads();
    }
  }
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
  __shared__ T ss[kMaxK * kMaxC];
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
  // the difference in FP64 (theta and diag agree to many digits near
  // convergence), the division in the vectors' precision
  T g = T(lam[a] - diag[i]);
  if (!(fabs(g) > T(1e-13))) g = T(1e-13);
  B[i * ld + bo + a] = R[i * ldr + sel[a]] / g;
}

template <class T>
__global__ void k_scale_cols(uint64_t n, T* __restrict__ B, int ld, int bo, int J, const double* __restrict__ sc) {
  uint64_t idx = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (idx >= n * J) return;
  uint64_t i = idx / J;
  int j = int(idx - i * J);
  B[i * ld + bo + j] = B[i * ld + bo + j] * T(sc[j]);
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

// W (n x pad, packed 32/64-byte rows) = B[:, c0:c0+m] padded with zero columns
__global__ void k_stage_block(uint64_t n, const float* __restrict__ B, int ld, int c0, int m, float* __restrict__ W,
                              int pad) {
  uint64_t idx = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (idx >= n * pad) return;
  uint64_t i = idx / pad;
  int j = int(idx - i * pad);
  W[idx] = j < m ? B[i * ld + c0 + j] : 0.f;
}

// W (n x 8 FP32, zero-padded) = columns c0 .. c0+m of the FP64 block B, rounded
__global__ void k_narrow8(uint64_t n, const double* __restrict__ B, int ld, int c0, int m, float* __restrict__ W) {
  uint64_t idx = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (idx >= n * 8) return;
  uint64_t i = idx >> 3;
  int j = int(idx & 7);
  W[idx] = j < m ? float(B[i * ld + c0 + j]) : 0.f;
}

// Y[:, c0 .. c0+m] (FP64) = W (n x 8 FP32), first m columns
__global__ void k_widen8(uint64_t n, const float* __restrict__ W, int m, double* __restrict__ Y, int ld, int c0) {
  uint64_t idx = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (idx >= n * 8) return;
  uint64_t i = idx >> 3;
  int j = int(idx & 7);
  if (j < m) Y[i * ld + c0 + j] = double(W[idx]);
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
  int nsm_ = 1;
  uint64_t xwarps_ = 8, xrows_ = 1;  // warps of the X^T Y kernel and rows per warp
  uint64_t rows_per_cta;
  DBuf<T> B, AB, R;
  int ldr;
  DBuf<double> part, small, small2, dlam;
  DBuf<int> dsel;
  DBuf<uint64_t> drows;
  double spmm_s = 0;
  // host wall time per phase (verbose >= 2 prints them)
  double t_eig = 0, t_resid = 0, t_ortho = 0, t_collapse = 0, t_abs = 0;
  int pip_calls_ = 0, pip_fallbacks_ = 0;
  int gemm_occ_[8] = {0, 0, 0, 0, 0, 0, 0, 0};  // resident CTAs per SM of k_gemm_r<T, 4|8|16|32, 64|kMaxLim>
  static double now() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
  }
  cudaEvent_t ev0, ev1;
  // reference state
  int kpass = 0, nume, lim, mblock;
  std::vector<double> S;      // lim x lim, FP64
  std::vector<double> eigs, old, zvec;  // zvec: kpass x kpass, columns eigenvectors
  std::vector<double> wall_;            // all eigenvalues of the last projected problem
  std::vector<int> icv;

  Engine(const Hamiltonian& h, const DavConfig& c, cudaStream_t st) : H(h), cfg(c), s(st) {
    n = h.n;
    nume = c.nume;
    lim = c.lim;
    mblock = c.block;
    int align = sizeof(T) == 4 ? 4 : 2;
    L = (lim + align - 1) / align * align;
    if (lim > kMaxLim) throw Error(CG_ERR_ARG, "lim above 128 is not supported");
    if (mblock > kMaxC || nume > kMaxC) throw Error(CG_ERR_ARG, "block and nstates must be <= 16");
    int nsm = 0;
    CG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, h.device));
    nsm_ = nsm;
    nparts = std::max(1, std::min<int>(nsm * 4, int((n + kTile - 1) / kTile)));
    rows_per_cta = (n + nparts - 1) / nparts;
    rows_per_cta = (rows_per_cta + kTile - 1) / kTile * kTile;
    nparts = int((n + rows_per_cta - 1) / rows_per_cta);
    B.alloc(n * L);
    AB.alloc(n * L);
    // FP32 residual rows padded to 32 bytes (stored 8 columns at a time)
    const int ralign = sizeof(T) == 4 ? 8 : 2;
    ldr = (std::max(nume, 1) + ralign - 1) / ralign * ralign;
    R.alloc(n * ldr);
    xwarps_ = uint64_t(nsm) * 32;  // 4 CTAs of 8 warps per SM
    xrows_ = (n + xwarps_ - 1) / xwarps_;
    xrows_ = (xrows_ + 3) / 4 * 4;
    xwarps_ = std::max<uint64_t>(8, (n + xrows_ - 1) / xrows_);
    xwarps_ = (xwarps_ + 7) / 8 * 8;
    part.alloc(std::max<size_t>(std::max<size_t>(size_t(nparts) * kMaxK * kMaxJ, size_t(nsm * 8) * kMaxC),
                                size_t(xwarps_) * 64 * 16));
    small.alloc(kMaxLim * kMaxLim);
    small2.alloc(kMaxLim * kMaxLim);
    dlam.alloc(kMaxLim);
    dsel.alloc(kMaxLim);
    drows.alloc(kMaxLim);
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

  // G (K x J, row-major, host) = X[:, xo:xo+K]^T Y[:, yo:yo+J]; more than
  // kMaxK columns of X go through the kernels kMaxK at a time (rows of G)
  void xty(const T* X, int xo, int K, const T* Y, int yo, int J, std::vector<double>& G) {
    if (K > kMaxK && J > 0) {
      if (K > kMaxLim) throw Error(CG_ERR_INTERNAL, "xty shape out of range");
      G.assign(size_t(K) * J, 0.0);
      std::vector<double> Gc;
      for (int k0 = 0; k0 < K; k0 += kMaxK) {
        const int kc = std::min(kMaxK, K - k0);
        xty(X, xo + k0, kc, Y, yo, J, Gc);
        std::copy(Gc.begin(), Gc.end(), G.begin() + size_t(k0) * J);
      }
      return;
    }
    if (K == 0 || J == 0) { G.assign(size_t(K) * J, 0.0); return; }
    if (J > 16 || K > kMaxK) throw Error(CG_ERR_INTERNAL, "xty shape out of range");
    const unsigned blocks = unsigned(xwarps_ / 8);
    // the refinement phase of the mixed solve multiplies in double-float; the
    // plain FP64 solve (and any product of fewer than 3 columns) stays FP64
    const bool df = sizeof(T) == 8 && cfg.spmm_prec == CG_PREC_REFINE && J >= 3;
    if constexpr (sizeof(T) == 8) {
      if (df && J <= 4) k_xty_df<4><<<blocks, 256, 0, s>>>(n, X, L, xo, K, Y, L, yo, J, part.p, xrows_);
      else if (df && J <= 8) k_xty_df<8><<<blocks, 256, 0, s>>>(n, X, L, xo, K, Y, L, yo, J, part.p, xrows_);
      else if (J <= 4) k_xty_t<T, 4><<<blocks, 256, 0, s>>>(n, X, L, xo, K, Y, L, yo, J, part.p, xrows_);
      else if (J <= 8) k_xty_t<T, 8><<<blocks, 256, 0, s>>>(n, X, L, xo, K, Y, L, yo, J, part.p, xrows_);
      else k_xty_w<T, 16><<<blocks, 256, 0, s>>>(n, X, L, xo, K, Y, L, yo, J, part.p, xrows_);
    } else if (J <= 4) k_xty_t<T, 4><<<blocks, 256, 0, s>>>(n, X, L, xo, K, Y, L, yo, J, part.p, xrows_);
    else if (J <= 8) k_xty_t<T, 8><<<blocks, 256, 0, s>>>(n, X, L, xo, K, Y, L, yo, J, part.p, xrows_);
    else k_xty_w<T, 16><<<blocks, 256, 0, s>>>(n, X, L, xo, K, Y, L, yo, J, part.p, xrows_);
    CG_CUDA(cudaGetLastError());
    count_launch();
    k_reduce_parts<<<K * J, 128, 0, s>>>(part.p, int(xwarps_), K * J, small.p);
    CG_CUDA(cudaGetLastError());
    count_launch();
    G.resize(size_t(K) * J);
    CG_CUDA(cudaMemcpyAsync(G.data(), small.p, sizeof(double) * K * J, cudaMemcpyDeviceToHost, s));
    CG_CUDA(cudaStreamSynchronize(s));
  }
  // Y[:, yo:yo+J] = beta Y + alpha X[:, xo:xo+K] G (G host K x J).  More
  // than kMaxJ outputs (beta 0 only: the thick restart keeping more than 32
  // Ritz vectors, X and Y the same block) go kMaxJ columns at a time into a
  // scratch block, then into Y, so no output overwrites an input still read.
  DBuf<T> wide_;
  void gemm(T* Xp, int xo, int K, const std::vector<double>& G, T* Yp, int yo, int J, double alpha, double beta) {
    if (J > kMaxJ) {
      if (beta != 0.0 || J > kMaxKeep) throw Error(CG_ERR_INTERNAL, "gemm shape out of range");
      if (wide_.n < n * uint64_t(J)) wide_.alloc(n * uint64_t(J));
      std::vector<double> Gc;
      for (int j0 = 0; j0 < J; j0 += kMaxJ) {
        const int jc = std::min(kMaxJ, J - j0);
        Gc.assign(size_t(K) * jc, 0.0);
        for (int k = 0; k < K; ++k)
          for (int j = 0; j < jc; ++j) Gc[size_t(k) * jc + j] = G[size_t(k) * J + j0 + j];
        gemm_ld(Xp, xo, K, Gc, wide_.p, J, j0, jc, alpha, 0.0);
      }
      k_copy_cols<T><<<blocks_for(n * uint64_t(J)), 256, 0, s>>>(n, wide_.p, J, 0, Yp, L, yo, J);
      CG_CUDA(cudaGetLastError());
      count_launch();
      CG_CUDA(cudaStreamSynchronize(s));
      return;
    }
    gemm_ld(Xp, xo, K, G, Yp, L, yo, J, alpha, beta);
  }
  void gemm_ld(T* Xp, int xo, int K, const std::vector<double>& G, T* Yp, int ldy, int yo, int J, double alpha,
               double beta) {
    // every kernel below holds G (K x J) in shared memory sized 64 (or, for
    // K > 64, kMaxLim) x kMaxJ and gives a row at most 32 lanes
    if (K < 0 || K > kMaxLim || J < 0 || J > kMaxJ) throw Error(CG_ERR_INTERNAL, "gemm shape out of range");
    const bool wide = K > kMaxK;
    if (K == 0 || J == 0) return;
    CG_CUDA(cudaMemcpyAsync(small2.p, G.data(), sizeof(double) * K * J, cudaMemcpyHostToDevice, s));
    const bool vx = reinterpret_cast<uintptr_t>(Xp + xo) % 32 == 0 && L % 8 == 0;
    const bool vy = reinterpret_cast<uintptr_t>(Yp + yo) % 32 == 0 && ldy % 8 == 0 && J % 8 == 0;
    unsigned grid = unsigned(std::min<uint64_t>((n + 255) / 256, uint64_t(nsm_) * 8));
    if constexpr (sizeof(T) == 8) {
      if (J <= 32 && J >= 3 && cfg.spmm_prec == CG_PREC_REFINE) {
        const double* Xd = reinterpret_cast<const double*>(Xp);
        double* Yd = reinterpret_cast<double*>(Yp);
#define CG_GEMM_DF(JM, KM) k_gemm_df<JM, KM><<<grid, 256, 0, s>>>(n, Xd, L, xo, K, small2.p, Yd, ldy, yo, J, alpha, beta)
        if (J <= 8) { if (wide) CG_GEMM_DF(8, kMaxLim); else CG_GEMM_DF(8, kMaxK); }
        else if (J <= 16) { if (wide) CG_GEMM_DF(16, kMaxLim); else CG_GEMM_DF(16, kMaxK); }
        else { if (wide) CG_GEMM_DF(32, kMaxLim); else CG_GEMM_DF(32, kMaxK); }
#undef CG_GEMM_DF
        CG_CUDA(cudaGetLastError());
        count_launch();
        CG_CUDA(cudaStreamSynchronize(s));
        return;
      }
    }
    // one wave of resident CTAs (the grid-stride loop gives each thread whole
    // rows, so the grid changes no result)
    const int jc = (J <= 4 ? 0 : J <= 8 ? 1 : J <= 16 ? 2 : 3) + (wide ? 4 : 0);
    if (!gemm_occ_[jc]) {
      int per_sm = 0;
      switch (jc) {
        case 0: CG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gemm_r<T, 4, kMaxK>, 256, 0)); break;
        case 1: CG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gemm_r<T, 8, kMaxK>, 256, 0)); break;
        case 2: CG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gemm_r<T, 16, kMaxK>, 256, 0)); break;
        case 3: CG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gemm_r<T, 32, kMaxK>, 256, 0)); break;
        case 4: CG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gemm_r<T, 4, kMaxLim>, 256, 0)); break;
        case 5: CG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gemm_r<T, 8, kMaxLim>, 256, 0)); break;
        case 6: CG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gemm_r<T, 16, kMaxLim>, 256, 0)); break;
        default: CG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_gemm_r<T, 32, kMaxLim>, 256, 0)); break;
      }
      gemm_occ_[jc] = std::max(per_sm, 1);
    }
    grid = unsigned(std::max<uint64_t>(1, std::min<uint64_t>((n + 255) / 256, uint64_t(nsm_) * gemm_occ_[jc])));
#define CG_GEMM_R(JM, KM) k_gemm_r<T, JM, KM><<<grid, 256, 0, s>>>(n, Xp, L, xo, K, small2.p, Yp, ldy, yo, J, alpha, beta, vx, vy)
    if (J <= 4) { if (wide) CG_GEMM_R(4, kMaxLim); else CG_GEMM_R(4, kMaxK); }
    else if (J <= 8) { if (wide) CG_GEMM_R(8, kMaxLim); else CG_GEMM_R(8, kMaxK); }
    else if (J <= 16) { if (wide) CG_GEMM_R(16, kMaxLim); else CG_GEMM_R(16, kMaxK); }
    else { if (wide) CG_GEMM_R(32, kMaxLim); else CG_GEMM_R(32, kMaxK); }
#undef CG_GEMM_R
    CG_CUDA(cudaGetLastError());
    count_launch();
    CG_CUDA(cudaStreamSynchronize(s));  // G's staging buffer is reused by the next call
  }
  DBuf<float> stage;  // FP32 engine: aligned SpMM input block (n x 16)
  // Refinement phase: once the starting vectors' products are in AB (double-
  // float), the correction blocks are multiplied in FP32 (FP32 matrix values,
  // vectors rounded to FP32).  A correction enters a converged Ritz vector
  // with a coefficient of the order of the residual (<= the switch residual,
  // 3e-5 in the mixed solve), so the FP32 product's ~1e-7 relative error
  // reaches the Ritz vector's product as ~1e-7 |H| * 3e-5, far below the
  // residual threshold; the final Ritz vectors are multiplied again in
  // double-float and their residuals checked before the phase ends (and the
  // phase goes on in double-float if the residuals stall first).
  bool fp32_corr_ = false;
  double corr_best_ = 1e300;  // smallest largest-residual seen on FP32 correction products
  int corr_stall_ = 0;        // iterations since it last dropped by 10 %
  DBuf<float> y32_;
  void spmm_narrow(int c0, int m) {
    if (!stage.p) stage.alloc(n * 16);
    if (!y32_.p) y32_.alloc(n * 8);
    const double* Bd = reinterpret_cast<const double*>(B.p);
    double* ABd = reinterpret_cast<double*>(AB.p);
    for (int c = 0; c < m; c += 8) {
      const int mc = std::min(8, m - c);
      k_narrow8<<<blocks_for(n * 8), 256, 0, s>>>(n, Bd, L, c0 + c, mc, stage.p);
      CG_CUDA(cudaGetLastError());
      count_launch();
      if (H.virt) virtual_product_f32(H, stage.p, y32_.p, 8, mc, s);
      else spmm_f32_padded(H, stage.p, 8, y32_.p, 8, mc, s);
      k_widen8<<<blocks_for(n * 8), 256, 0, s>>>(n, y32_.p, mc, ABd, L, c0 + c);
      CG_CUDA(cudaGetLastError());
      count_launch();
    }
  }
  void spmm(int c0, int m) {
    CG_CUDA(cudaEventRecord(ev0, s));
    if (fp32_corr_) {
      spmm_narrow(c0, m);
    } else if (H.virt) {
      // on-the-fly product: pack 8 (FP32) or 4 (FP64) columns at a time
      if (!stage.p) stage.alloc(n * 16);
      if constexpr (sizeof(T) == 4) {
        for (int c = 0; c < m; c += kVirtualVB32) {
          const int mc = std::min(kVirtualVB32, m - c);
          virtual_pack_f32(n, reinterpret_cast<const float*>(B.p), L, c0 + c, mc, stage.p, s);
          virtual_product_f32(H, stage.p, reinterpret_cast<float*>(AB.p) + c0 + c, L, mc, s);
        }
      } else if (cfg.spmm_prec == CG_PREC_REFINE) {
        // refinement: double-float product, 4 vectors a pass as (hi, lo) pairs
        for (int c = 0; c < m; c += 4) {
          const int mc = std::min(4, m - c);
          virtual_pack_df(n, reinterpret_cast<const double*>(B.p), L, c0 + c, mc, stage.p, s);
          virtual_product_df(H, stage.p, reinterpret_cast<double*>(AB.p) + c0 + c, L, mc, s);
        }
      } else {
        double* w = reinterpret_cast<double*>(stage.p);
        for (int c = 0; c < m; c += kVirtualVB64) {
          const int mc = std::min(kVirtualVB64, m - c);
          virtual_pack_f64(n, reinterpret_cast<const double*>(B.p), L, c0 + c, mc, w, s);
          virtual_product_f64(H, w, reinterpret_cast<double*>(AB.p) + c0 + c, L, mc, s);
        }
      }
    } else if constexpr (sizeof(T) == 4) {
      if (cfg.spmm_prec == CG_PREC_FP32) {
        if (!stage.p) stage.alloc(n * 16);
        int pad = m <= 8 ? 8 : 16;
        k_stage_block<<<blocks_for(n * pad), 256, 0, s>>>(n, reinterpret_cast<const float*>(B.p), L, c0, m,
                                                            stage.p, pad);
        CG_CUDA(cudaGetLastError());
    count_launch();
        spmm_f32_padded(H, stage.p, pad, reinterpret_cast<float*>(AB.p) + c0, L, m, s);
      } else {
        spmm_launch(H, cfg.spmm_prec, B.p + c0, L, AB.p + c0, L, m, s);
      }
    } else if (cfg.spmm_prec == CG_PREC_REFINE) {
      if (!stage.p) stage.alloc(n * 16);
      spmm_refine_df(H, reinterpret_cast<const double*>(B.p) + c0, L, reinterpret_cast<double*>(AB.p) + c0, L, m,
                     stage.p, s);
    } else {
      spmm_launch(H, cfg.spmm_prec, B.p + c0, L, AB.p + c0, L, m, s);
    }
    CG_CUDA(cudaEventRecord(ev1, s));
    CG_CUDA(cudaEventSynchronize(ev1));
    float ms = 0;
    CG_CUDA(cudaEventElapsedTime(&ms, ev0, ev1));
    spmm_s += ms * 1e-3;
  }
  // new columns of S from AB[:, c0:c0+m] (Add_Vectors_To_AB_S, fsdavidson.cxx:161-211)
  void add_ab_s(int c0, int m, int64_t& nmv) {
    double t0 = now();
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
    t_abs += now() - t0;
  }
  void diagonalize() {
    double t0 = now();
    struct Acc { double& t; double t0; ~Acc() { t += now() - t0; } } acc_{t_eig, t0};
    std::vector<double> a(size_t(kpass) * kpass);
    for (int i = 0; i < kpass; ++i)
      for (int j = 0; j < kpass; ++j) a[size_t(i) * kpass + j] = S[size_t(i) * lim + j];
    sym_eig(kpass, a, wall_, zvec);
    for (int i = 0; i < nume; ++i) eigs[i] = wall_[i];
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
    struct Acc { double& t; double t0; ~Acc() { t += now() - t0; } } acc_{t_resid, now()};
    int C = int(st.size());
    std::vector<double> Sc(size_t(kpass) * C), lam(C);
    for (int c = 0; c < C; ++c) {
      lam[c] = eigs[st[c]];
      for (int k = 0; k < kpass; ++k) Sc[size_t(k) * C + c] = svec(st[c], k);
    }
    CG_CUDA(cudaMemcpyAsync(small2.p, Sc.data(), sizeof(double) * Sc.size(), cudaMemcpyHostToDevice, s));
    CG_CUDA(cudaMemcpyAsync(dlam.p, lam.data(), sizeof(double) * C, cudaMemcpyHostToDevice, s));
    const unsigned rgrid = unsigned(std::min<uint64_t>((n + 255) / 256, uint64_t(nsm_) * 8));
    const bool vec = L % 8 == 0 && reinterpret_cast<uintptr_t>(B.p) % 32 == 0 &&
                     reinterpret_cast<uintptr_t>(AB.p) % 32 == 0;
    const bool vec_r = ldr % 8 == 0 && (C + 7) / 8 * 8 <= ldr && reinterpret_cast<uintptr_t>(R.p) % 32 == 0;
    bool done = false;
    if constexpr (sizeof(T) == 8) {
      if (cfg.spmm_prec == CG_PREC_REFINE) {
#define CG_RESID_DF(CM, KM) k_resid_df<CM, KM><<<rgrid, 256, 0, s>>>(n, B.p, AB.p, L, kpass, small2.p, dlam.p, C, R.p, ldr, part.p)
        if (C <= 8) { if (kpass > kMaxK) CG_RESID_DF(8, kMaxLim); else CG_RESID_DF(8, kMaxK); }
        else { if (kpass > kMaxK) CG_RESID_DF(16, kMaxLim); else CG_RESID_DF(16, kMaxK); }
#undef CG_RESID_DF
        done = true;
      }
    }
    if (!done) {
#define CG_RESID_V(CM, KM) k_resid_v<T, CM, KM><<<rgrid, 256, 0, s>>>(n, B.p, AB.p, L, kpass, small2.p, dlam.p, C, R.p, ldr, part.p, vec, vec_r)
      if (C <= 8) { if (kpass > kMaxK) CG_RESID_V(8, kMaxLim); else CG_RESID_V(8, kMaxK); }
      else { if (kpass > kMaxK) CG_RESID_V(16, kMaxLim); else CG_RESID_V(16, kMaxK); }
#undef CG_RESID_V
    }
    CG_CUDA(cudaGetLastError());
    count_launch();
    k_reduce_parts<<<C, 128, 0, s>>>(part.p, int(rgrid), C, small.p);
    CG_CUDA(cudaGetLastError());
    count_launch();
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
    count_launch();
  }
  void scale_col(int c, double f) {
    CG_CUDA(cudaMemcpyAsync(small2.p, &f, sizeof(double), cudaMemcpyHostToDevice, s));
    k_scale_cols<T><<<blocks_for(n), 256, 0, s>>>(n, B.p, L, c, 1, small2.p);
    CG_CUDA(cudaGetLastError());
    count_launch();
    CG_CUDA(cudaStreamSynchronize(s));
  }
  void copy_col(int from, int to) {
    k_copy_cols<T><<<blocks_for(n), 256, 0, s>>>(n, B.p, L, from, B.p, L, to, 1);
    CG_CUDA(cudaGetLastError());
    count_launch();
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
    count_launch();
    CG_CUDA(cudaStreamSynchronize(s));
  }
  // Block Gram-Schmidt with Pythagorean inner products, twice (BCGS-PIP2):
  // one X^T Y over [basis | block] gives the projections G = X^T Y and the
  // block's Gram M = Y^T Y at once; the projected block's Gram is M - G^T G
  // (X orthonormal), whose Cholesky factor L gives the whole update in one
  // product, Y <- [X Y] [-G L^-T ; L^-T].  Two passes of (X^T Y, X G) per
  // call instead of Gram + scale + 2 x (X^T Y, X G) + 2 x (Gram, Y R^-1).
  // Returns false (Y possibly updated by a first pass, still spanning the same
  // space modulo the basis) when the block is nearly inside the basis or a
  // factorisation fails: the classical form then takes over.
  bool orthogonalize_pip(int basis_dim, int m) {
    const int K = basis_dim + m;
    if (K > kMaxLim || m > 16) return false;
    const double min_ratio = sizeof(T) == 4 ? 1e-3 : 1e-8;  // |Y_perp|^2 / |Y|^2 below: cancellation
    for (int pass = 0; pass < 2; ++pass) {
      std::vector<double> W;
      xty(B.p, 0, K, B.p, basis_dim, m, W);  // K x m
      std::vector<double> S(size_t(m) * m), d(m);
      for (int j = 0; j < m; ++j) {
        const double mjj = W[size_t(basis_dim + j) * m + j];
        if (!(mjj > 0.0) || !std::isfinite(mjj)) return false;
        d[j] = 1.0 / std::sqrt(mjj);
      }
      for (int i = 0; i < m; ++i)
        for (int j = 0; j < m; ++j) {
          double v = W[size_t(basis_dim + i) * m + j];
          for (int k = 0; k < basis_dim; ++k) v -= W[size_t(k) * m + i] * W[size_t(k) * m + j];
          S[size_t(i) * m + j] = v * d[i] * d[j];  // scaled to unit input columns
        }
      for (int j = 0; j < m; ++j)
        if (!(S[size_t(j) * m + j] > min_ratio)) return false;
      if (cholesky(m, S) >= 0) return false;
      // R^-1 = D L^-T (upper triangular in the scaled frame, rescaled)
      std::vector<double> Ri(size_t(m) * m, 0.0);
      for (int j = 0; j < m; ++j) {
        std::vector<double> x(m, 0.0);
        for (int i = m - 1; i >= 0; --i) {
          double r = (i == j) ? 1.0 : 0.0;
          for (int k = i + 1; k < m; ++k) r -= S[size_t(k) * m + i] * x[k];
          x[i] = r / S[size_t(i) * m + i];
        }
        for (int i = 0; i < m; ++i) Ri[size_t(i) * m + j] = d[i] * x[i];
      }
      std::vector<double> C(size_t(K) * m, 0.0);
      for (int k = 0; k < basis_dim; ++k)
        for (int j = 0; j < m; ++j) {
          double v = 0.0;
          for (int i = 0; i < m; ++i) v -= W[size_t(k) * m + i] * Ri[size_t(i) * m + j];
          C[size_t(k) * m + j] = v;
        }
      for (int i = 0; i < m; ++i)
        for (int j = 0; j < m; ++j) C[size_t(basis_dim + i) * m + j] = Ri[size_t(i) * m + j];
      gemm(B.p, 0, K, C, B.p, basis_dim, m, 1.0, 0.0);  // in place: each row read before written
    }
    ++pip_calls_;
    return true;
  }
  bool orthogonalize_block(int basis_dim, int& nncv) {
    struct Acc { double& t; double t0; ~Acc() { t += now() - t0; } } acc_{t_ortho, now()};
    const double drop = sizeof(T) == 4 ? 1e-8 : 1e-20;  // squared norm after projection
    int m = nncv;
    if (m == 0) return true;
    if (cfg.pip && orthogonalize_pip(basis_dim, m)) return true;
    if (cfg.pip) ++pip_fallbacks_;
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
    count_launch();
  }

  // B[:, 0:nume], AB[:, 0:nume] = the Ritz vectors of the current projection
  // and their products; S = diag(Ritz values), kpass = nume
  void to_ritz() {
    std::vector<double> G(size_t(kpass) * nume);
    for (int k = 0; k < kpass; ++k)
      for (int j = 0; j < nume; ++j) G[size_t(k) * nume + j] = svec(j, k);
    gemm(B.p, 0, kpass, G, B.p, 0, nume, 1.0, 0.0);
    gemm(AB.p, 0, kpass, G, AB.p, 0, nume, 1.0, 0.0);
    std::fill(S.begin(), S.end(), 0.0);
    for (int i = 0; i < nume; ++i) S[size_t(i) * lim + i] = eigs[i];
    kpass = nume;
    zvec.assign(size_t(nume) * nume, 0.0);
    for (int i = 0; i < nume; ++i) zvec[size_t(i) * nume + i] = 1.0;
  }

  // Residual-driven block Davidson with thick restart (the mixed-precision
  // solve): every iteration re-checks the residual of every wanted pair, adds
  // the preconditioned residuals of the unconverged ones (largest first), and
  // when the basis is full keeps `keep` Ritz vectors instead of `nume`.
  DavOutcome run_modern(int niv, const std::vector<double>& hdiag) {
    auto t0 = std::chrono::steady_clock::now();
    DavOutcome out;
    int64_t nmv = 0;
    if (niv >= nume && niv <= lim) {
      int a = niv;
      orthogonalize_block(0, a);
      niv = a;
    } else {
      niv = 0;
    }
    if (niv < nume) {
      std::vector<uint64_t> idx(n);
      std::iota(idx.begin(), idx.end(), 0);
      std::partial_sort(idx.begin(), idx.begin() + std::min<uint64_t>(nume, n), idx.end(),
                        [&](uint64_t x, uint64_t y) { return hdiag[x] < hdiag[y] || (hdiag[x] == hdiag[y] && x < y); });
      k_zero_cols<T><<<blocks_for(n * (nume - niv)), 256, 0, s>>>(n, B.p, L, niv, nume - niv);
      set_unit_start(niv, nume - niv, idx);
      int b2 = nume - niv;
      orthogonalize_block(niv, b2);
      niv += b2;
    }
    kpass = niv;
    add_ab_s(0, kpass, nmv);
    fp32_corr_ = sizeof(T) == 8 && cfg.spmm_prec == CG_PREC_REFINE && cfg.fp32_corr;
    corr_best_ = 1e300;
    corr_stall_ = 0;
    const int keep = std::max(nume, std::min(cfg.keep > 0 ? cfg.keep : 2 * nume, lim - mblock));
    int nloops = 0;
    bool done = false;
    std::vector<double> rn;
    std::fill(eigs.begin(), eigs.end(), 0.0);
    for (;;) {
      for (int i = 0; i < nume; ++i) old[i] = eigs[i];
      diagonalize();
      if (kpass + mblock > lim) {
        double tc0 = now();
        int kp = std::min(keep, kpass);
        std::vector<double> G(size_t(kpass) * kp);
        for (int k = 0; k < kpass; ++k)
          for (int j = 0; j < kp; ++j) G[size_t(k) * kp + j] = svec(j, k);
        gemm(B.p, 0, kpass, G, B.p, 0, kp, 1.0, 0.0);
        gemm(AB.p, 0, kpass, G, AB.p, 0, kp, 1.0, 0.0);
        std::fill(S.begin(), S.end(), 0.0);
        for (int i = 0; i < kp; ++i) S[size_t(i) * lim + i] = wall_[i];
        zvec.assign(size_t(kp) * kp, 0.0);
        for (int i = 0; i < kp; ++i) zvec[size_t(i) * kp + i] = 1.0;
        kpass = kp;
        ++out.restarts;
        t_collapse += now() - tc0;
      }
      std::vector<int> all(nume);
      std::iota(all.begin(), all.end(), 0);
      rn = residuals(all);
      std::vector<int> unc;
      for (int i = 0; i < nume; ++i)
        if (!(rn[i] < cfg.critr)) unc.push_back(i);
      if (cfg.verbose & 1) {
        double mx = 0;
        for (double r : rn) mx = std::max(mx, r);
        std::fprintf(stderr, "dav[%s] it %d kpass %d unconverged %zu max_resid %.3e E0 %.8f E%d %.8f\n",
                     sizeof(T) == 4 ? "fp32" : "fp64", nloops, kpass, unc.size(), mx, eigs[0], nume - 1,
                     eigs[nume - 1]);
      }
      // FP32 correction products carry a noise floor of ~1e-7 |H| times the
      // corrections' weight in the Ritz vectors; if the largest residual has
      // not dropped by 10 % for 4 iterations the threshold may lie below that
      // floor, and the phase goes on in double-float as after a failed check
      if (fp32_corr_) {
        double mx = 0;
        for (double r : rn) mx = std::max(mx, r);
        if (mx < 0.9 * corr_best_) {
          corr_best_ = mx;
          corr_stall_ = 0;
        } else {
          ++corr_stall_;
        }
      }
      const bool stalled = fp32_corr_ && corr_stall_ >= 4;
      if (fp32_corr_ && (unc.empty() || stalled)) {
        // every residual is below the threshold on the FP32 correction
        // products (or they stall): multiply the Ritz vectors again in
        // double-float and take the residuals from those products
        fp32_corr_ = false;
        to_ritz();
        add_ab_s(0, nume, nmv);
        diagonalize();
        to_ritz();
        rn = residuals(all);
        unc.clear();
        for (int i = 0; i < nume; ++i)
          if (!(rn[i] < cfg.critr)) unc.push_back(i);
        if (cfg.verbose & 1) {
          double mx = 0;
          for (double r : rn) mx = std::max(mx, r);
          std::fprintf(stderr, "dav[fp64] double-float %s: unconverged %zu max_resid %.3e\n",
                       stalled ? "products after a stall" : "check", unc.size(), mx);
        }
      }
      if (unc.empty()) { done = true; break; }
      if (nloops >= cfg.maxiter) break;
      std::stable_sort(unc.begin(), unc.end(), [&](int a, int b) { return rn[a] > rn[b]; });
      int add = std::min<int>(int(unc.size()), std::min(mblock, lim - kpass));
      std::vector<int> sel_r(unc.begin(), unc.begin() + add);
      std::vector<double> lam(add);
      for (int a = 0; a < add; ++a) lam[a] = eigs[sel_r[a]];
      if (cfg.precond) precond_copy(sel_r, lam, kpass);
      else copy_residuals(sel_r, kpass);
      int nncv = add;
      orthogonalize_block(kpass, nncv);
      if (nncv == 0) { ierr_stall = true; break; }
      add_ab_s(kpass, nncv, nmv);
      kpass += nncv;
      ++nloops;
    }
    if (fp32_corr_) {
      // stopped (iteration cap, no new direction) while on FP32 correction
      // products: the returned residuals come from double-float products too
      fp32_corr_ = false;
      to_ritz();
      add_ab_s(0, nume, nmv);
      diagonalize();
      to_ritz();
    }
    out.de.resize(nume);
    for (int i = 0; i < nume; ++i) out.de[i] = std::fabs(old[i] - eigs[i]);
    // final Ritz vectors in B[:, 0:nume]
    if (kpass != nume) {
      std::vector<double> G(size_t(kpass) * nume);
      for (int k = 0; k < kpass; ++k)
        for (int j = 0; j < nume; ++j) G[size_t(k) * nume + j] = svec(j, k);
      gemm(B.p, 0, kpass, G, B.p, 0, nume, 1.0, 0.0);
      gemm(AB.p, 0, kpass, G, AB.p, 0, nume, 1.0, 0.0);
      kpass = nume;
      zvec.assign(size_t(nume) * nume, 0.0);
      for (int i = 0; i < nume; ++i) zvec[size_t(i) * nume + i] = 1.0;
    }
    std::vector<int> all(nume);
    std::iota(all.begin(), all.end(), 0);
    out.resid = residuals(all);
    out.eig.assign(eigs.begin(), eigs.begin() + nume);
    out.iterations = nloops;
    out.matvecs = nmv;
    out.ierr = done ? 0 : (ierr_stall ? 1024 : 2048);
    out.spmm_seconds = spmm_s;
    out.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (cfg.verbose >= 2)
      std::fprintf(stderr,
                   "dav[%s] phases: total %.3f s, spmm %.3f, ab+S %.3f, eig %.3f, resid %.3f, ortho %.3f, "
                   "collapse %.3f (iterations %d, PIP orthogonalisations %d, fallbacks %d)\n",
                   sizeof(T) == 4 ? "fp32" : "fp64", out.seconds, spmm_s, t_abs, t_eig, t_resid, t_ortho,
                   t_collapse, nloops, pip_calls_, pip_fallbacks_);
    return out;
  }
  bool ierr_stall = false;

  // B[:, bo + a] = R[:, sel[a]] (no preconditioner)
  void copy_residuals(const std::vector<int>& sel_r, int bo) {
    for (int a = 0; a < int(sel_r.size()); ++a) {
      k_copy_cols<T><<<blocks_for(n), 256, 0, s>>>(n, R.p, ldr, sel_r[a], B.p, L, bo + a, 1);
      CG_CUDA(cudaGetLastError());
    count_launch();
    }
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
    count_launch();
}

template <class T>
static void store_vectors(Engine<T>& e, int m, double* dst_dev_cm) {
  k_rm_to_cm<T><<<blocks_for(e.n * m), 256, 0, e.s>>>(e.n, m, e.B.p, e.L, 0, dst_dev_cm);
  CG_CUDA(cudaGetLastError());
    count_launch();
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
    DavOutcome o = rq.phase1.modern ? e.run_modern(std::min(ninit, e.lim + 1), hdiag)
                                    : e.run(std::min(ninit, e.lim + 1), hdiag);
    store_vectors(e, nume, vecs.p);
    res.phase1 = o;
    res.final_ = o;
  } else {
    DavOutcome o1;
    {
      Engine<float> e(h, rq.phase1, s);
      load_start(e, init.p, std::min(ninit, e.lim));
      o1 = rq.phase1.modern ? e.run_modern(std::min(ninit, e.lim + 1), hdiag)
                            : e.run(std::min(ninit, e.lim + 1), hdiag);
      store_vectors(e, nume, vecs.p);
    }
    res.phase1 = o1;
    res.final_ = o1;
    if (rq.refine) {
      Engine<double> e(h, rq.phase2, s);
      load_start(e, vecs.p, nume);
      DavOutcome o2 = rq.phase2.modern ? e.run_modern(nume, hdiag) : e.run(nume, hdiag);
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
