// Stored-Hamiltonian SpMM, Y = H X for a block of m vectors.
//
// Replaces SparseMatrixCSB::TimesMatrix (include/tav/csbmatrix.cxx:623-663):
// the reference stores the upper triangle in square CSB blocks and pulls
// y_j = sum_{i<j} B_ij^T x_i + sum_{i>=j} B_ji x_i per block row, reading every
// stored element twice and every vector separately.  Here both triangles are
// stored row-wise (one HBM stream, each element read once for all m vectors),
// the vectors are row-interleaved so one gather brings all m components of a
// column (one 32-byte sector for m = 8 FP32), one warp reduces one row with
// shuffles, and each CTA walks a contiguous row range so that the rows of one
// neutron block, which share their column structure, reuse gathered vectors
// from L1.
//
// Modes:
//   CG_PREC_FP64   FP64 values, FP64 vectors, FP64 accumulation.
//   CG_PREC_FP32   FP32 values and vectors, FP32 accumulation in each lane and
//                  across the warp (GB300 runs FP64 at ~1/60 of the FP32 rate;
//                  the FP64 accumulation lives in the Davidson projections).
//   CG_PREC_REFINE FP32 hi + FP32 lo values (h = hi + lo to ~2^-48), FP64
//                  vectors and accumulation.
#include <algorithm>
#include <mutex>
#include <string>
#include <type_traits>

#include "device.h"
#include "tiled.h"
#include "virtual.h"

namespace cg {
namespace {

constexpr int kWarpsPerCta = 8;

// NV components starting at p, loaded VW elements at a time (p must be
// aligned to VW elements; the dispatcher picks VW from the actual alignment).
template <int NV, int VW>
__device__ __forceinline__ void load_vec(const float* __restrict__ p, float (&v)[NV]) {
  if constexpr (VW == 4) {
#pragma unroll
    for (int k = 0; k < NV / 4; ++k) {
      float4 t = __ldg(reinterpret_cast<const float4*>(p) + k);
      v[4 * k] = t.x; v[4 * k + 1] = t.y; v[4 * k + 2] = t.z; v[4 * k + 3] = t.w;
    }
  } else if constexpr (VW == 2) {
#pragma unroll
    for (int k = 0; k < NV / 2; ++k) {
      float2 t = __ldg(reinterpret_cast<const float2*>(p) + k);
      v[2 * k] = t.x; v[2 * k + 1] = t.y;
    }
  } else {
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] = __ldg(p + k);
  }
}

template <int NV, int VW>
__device__ __forceinline__ void load_vec(const double* __restrict__ p, double (&v)[NV]) {
  if constexpr (VW == 2) {
#pragma unroll
    for (int k = 0; k < NV / 2; ++k) {
      double2 t = __ldg(reinterpret_cast<const double2*>(p) + k);
      v[2 * k] = t.x; v[2 * k + 1] = t.y;
    }
  } else {
#pragma unroll
    for (int k = 0; k < NV; ++k) v[k] = __ldg(p + k);
  }
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_sumf(float v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Each CTA owns rows [r0, r1); its warps take rows r0 + w, r0 + w + 8, ...
template <int NV, int MODE, int VW>
__global__ void __launch_bounds__(kWarpsPerCta * 32) k_spmm(uint64_t n, const uint64_t* __restrict__ rowptr,
                                                            const uint32_t* __restrict__ col,
                                                            const void* __restrict__ vals,
                                                            const float* __restrict__ lo, const void* __restrict__ xv,
                                                            int ldx, void* __restrict__ yv, int ldy,
                                                            uint64_t rows_per_cta) {
  using XT = typename std::conditional<MODE == CG_PREC_FP32, float, double>::type;
  const XT* x = static_cast<const XT*>(xv);
  XT* y = static_cast<XT*>(yv);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint64_t r0 = uint64_t(blockIdx.x) * rows_per_cta;
  const uint64_t r1 = min(n, r0 + rows_per_cta);
  for (uint64_t row = r0 + warp; row < r1; row += kWarpsPerCta) {
    const uint64_t b = __ldg(rowptr + row), e = __ldg(rowptr + row + 1);
    double tot[NV];
    if constexpr (MODE == CG_PREC_FP32) {
      const float* hv = static_cast<const float*>(vals);
      float acc[NV];
#pragma unroll
      for (int k = 0; k < NV; ++k) acc[k] = 0.f;
      for (uint64_t p = b + lane; p < e; p += 32) {
        const uint32_t c = __ldcs(col + p);
        const float h = __ldcs(hv + p);
        float xx[NV];
        load_vec<NV, VW>(x + uint64_t(c) * ldx, xx);
#pragma unroll
        for (int k = 0; k < NV; ++k) acc[k] = fmaf(h, xx[k], acc[k]);
      }
      // cross-lane sum in FP32: on GB300 an FP64 warp reduction per row costs
      // more FP64-pipe time than the whole row's memory traffic
#pragma unroll
      for (int k = 0; k < NV; ++k) tot[k] = double(warp_sumf(acc[k]));
    } else {
      double acc[NV];
#pragma unroll
      for (int k = 0; k < NV; ++k) acc[k] = 0.0;
      for (uint64_t p = b + lane; p < e; p += 32) {
        const uint32_t c = __ldcs(col + p);
        double h;
        if constexpr (MODE == CG_PREC_FP64) h = __ldcs(static_cast<const double*>(vals) + p);
        else h = double(__ldcs(static_cast<const float*>(vals) + p)) + double(__ldcs(lo + p));
        double xx[NV];
        load_vec<NV, VW>(x + uint64_t(c) * ldx, xx);
#pragma unroll
        for (int k = 0; k < NV; ++k) acc[k] = fma(h, xx[k], acc[k]);
      }
#pragma unroll
      for (int k = 0; k < NV; ++k) tot[k] = warp_sum(acc[k]);
    }
    // lane k writes component k (all lanes hold every total after the xor-reduction)
    double mine = 0.0;
#pragma unroll
    for (int k = 0; k < NV; ++k)
      if (lane == k) mine = tot[k];
    if (lane < NV) y[row * uint64_t(ldy) + lane] = XT(mine);
  }
}

// 256-bit gather of 8 consecutive FP32 components (one 32-byte sector).
__device__ __forceinline__ void ld8(const float* __restrict__ p, float (&v)[8]) {
  asm volatile("ld.global.nc.v8.f32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7])
               : "l"(p));
}

// FP32 product for NV = 8 or 16 vectors whose rows are 32-byte aligned.
// Per stored entry one lane issues NV/8 sector-wide gathers (the L1 data pipe
// is charged per sector touched by an instruction, so one wide load per 8
// vectors is the cheapest gather).  The row sum uses a reduce-scatter across
// the warp: at each halving step a lane keeps one half of its partial sums
// and receives the partner's other half, so NV = 8 costs 9 shuffles per row
// instead of 5 * NV.  Only the first m_out components are stored.
template <int NV, int WARPS>
__global__ void __launch_bounds__(WARPS * 32) k_spmm_f32w(uint64_t n, const uint64_t* __restrict__ rowptr,
                                                                 const uint32_t* __restrict__ col,
                                                                 const float* __restrict__ vals,
                                                                 const float* __restrict__ x, int ldx,
                                                                 float* __restrict__ y, int ldy, int m_out,
                                                                 uint64_t rows_per_cta) {
  static_assert(NV == 8 || NV == 16, "NV must be 8 or 16");
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint64_t r0 = uint64_t(blockIdx.x) * rows_per_cta;
  const uint64_t r1 = min(n, r0 + rows_per_cta);
  for (uint64_t row = r0 + warp; row < r1; row += WARPS) {
    const uint64_t b = __ldg(rowptr + row), e = __ldg(rowptr + row + 1);
    float acc[NV];
#pragma unroll
    for (int k = 0; k < NV; ++k) acc[k] = 0.f;
    // four entries per lane per step, all loads issued before any use, so each
    // lane keeps four gathers in flight (the loop is latency bound otherwise)
    uint64_t p = b + lane;
    for (; p + 96 < e; p += 128) {
      uint32_t c[4];
      float h[4];
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        c[u] = __ldcs(col + p + 32 * u);
        h[u] = __ldcs(vals + p + 32 * u);
      }
      float xx[4][NV];
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int g = 0; g < NV / 8; ++g) {
          float t[8];
          ld8(x + uint64_t(c[u]) * ldx + 8 * g, t);
#pragma unroll
          for (int j = 0; j < 8; ++j) xx[u][8 * g + j] = t[j];
        }
#pragma unroll
      for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int k = 0; k < NV; ++k) acc[k] = fmaf(h[u], xx[u][k], acc[k]);
    }
    for (; p < e; p += 32) {
      const uint32_t c = __ldcs(col + p);
      const float h = __ldcs(vals + p);
      const float* xp = x + uint64_t(c) * ldx;
#pragma unroll
      for (int g = 0; g < NV / 8; ++g) {
        float xx[8];
        ld8(xp + 8 * g, xx);
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[8 * g + j] = fmaf(h, xx[j], acc[8 * g + j]);
      }
    }
    // reduce-scatter: offsets 16, 8, 4 (and 2 for NV = 16) halve the values per lane
#pragma unroll
    for (int o = 16, c = NV; c > 1; o >>= 1, c >>= 1) {
      const bool up = lane & o;
#pragma unroll
      for (int k = 0; k < c / 2; ++k) {
        float send = up ? acc[k] : acc[c / 2 + k];
        float keep = up ? acc[c / 2 + k] : acc[k];
        acc[k] = keep + __shfl_xor_sync(0xffffffffu, send, o);
      }
    }
    // the lane group sharing a vector index finishes with plain xor steps
    constexpr int kShift = NV == 8 ? 2 : 1;  // lanes per vector index = 32 / NV
#pragma unroll
    for (int o = (1 << kShift) >> 1; o; o >>= 1) acc[0] += __shfl_xor_sync(0xffffffffu, acc[0], o);
    const int vi = lane >> kShift;
    if ((lane & ((1 << kShift) - 1)) == 0 && vi < m_out) y[row * uint64_t(ldy) + vi] = acc[0];
  }
}

template <int MODE, int NV, int VW>
void run_kernel(const Hamiltonian& h, const void* vals, const void* x, int ldx, void* y, int ldy, cudaStream_t s) {
  int nsm = 0;
  CG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, h.device));
  int per_sm = 0;
  CG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_spmm<NV, MODE, VW>, kWarpsPerCta * 32, 0));
  uint64_t ctas = uint64_t(nsm) * std::max(per_sm, 1) * 4;
  uint64_t rpc = (h.n + ctas - 1) / ctas;
  rpc = (rpc + kWarpsPerCta - 1) / kWarpsPerCta * kWarpsPerCta;
  if (rpc == 0) rpc = kWarpsPerCta;
  unsigned grid = unsigned((h.n + rpc - 1) / rpc);
  if (grid == 0) return;
  k_spmm<NV, MODE, VW><<<grid, kWarpsPerCta * 32, 0, s>>>(h.n, h.rowptr.p, h.col.p, vals, h.lo.p, x, ldx, y, ldy,
                                                           rpc);
  CG_CUDA(cudaGetLastError());
    count_launch();
}

// Widest vector load the operands allow: VW elements divide NV, the base
// address and the row pitch.
// ---- double-float refinement product ------------------------------------
// Error-free transformations (Knuth two-sum, FMA two-product) on FP32 pairs
// (hi, lo): ~48-bit accurate sums and products on the FP32 pipe, which GB300
// runs ~60x faster than FP64.
struct df32 {
  float hi, lo;
};
__device__ __forceinline__ df32 two_sum(float a, float b) {
  float s = a + b;
  float bb = s - a;
  float e = (a - (s - bb)) + (b - bb);
  return {s, e};
}
__device__ __forceinline__ df32 quick_two_sum(float a, float b) {
  float s = a + b;
  return {s, b - (s - a)};
}
// acc += (ah + al) * (bh + bl)
__device__ __forceinline__ void df_fma(df32& acc, float ah, float al, float bh, float bl) {
  float p = ah * bh;
  float pe = fmaf(ah, bh, -p);
  pe = fmaf(ah, bl, fmaf(al, bh, pe));
  df32 s = two_sum(acc.hi, p);
  s.lo += acc.lo + pe;
  acc = quick_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ df32 df_add(df32 a, df32 b) {
  df32 s = two_sum(a.hi, b.hi);
  s.lo += a.lo + b.lo;
  return quick_two_sum(s.hi, s.lo);
}

// Y = H X for 8 vectors in double-float.  X is staged as rows of 16 floats:
// 8 hi parts then 8 lo parts (two sector-wide gathers per stored entry); the
// matrix values are the stored (hi, lo) pair; Y is written as FP64.
template <int WARPS>
__global__ void __launch_bounds__(WARPS * 32) k_spmm_df8(uint64_t n, const uint64_t* __restrict__ rowptr,
                                                         const uint32_t* __restrict__ col,
                                                         const float* __restrict__ vhi,
                                                         const float* __restrict__ vlo,
                                                         const float* __restrict__ x, double* __restrict__ y,
                                                         int ldy, int m_out, uint64_t rows_per_cta) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint64_t r0 = uint64_t(blockIdx.x) * rows_per_cta;
  const uint64_t r1 = min(n, r0 + rows_per_cta);
  for (uint64_t row = r0 + warp; row < r1; row += WARPS) {
    const uint64_t b = __ldg(rowptr + row), e = __ldg(rowptr + row + 1);
    df32 acc[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) acc[k] = {0.f, 0.f};
    uint64_t p = b + lane;
    for (; p + 32 < e; p += 64) {
      uint32_t c[2];
      float hh[2], hl[2], xh[2][8], xl[2][8];
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        c[u] = __ldcs(col + p + 32 * u);
        hh[u] = __ldcs(vhi + p + 32 * u);
        hl[u] = __ldcs(vlo + p + 32 * u);
      }
#pragma unroll
      for (int u = 0; u < 2; ++u) {
        ld8(x + uint64_t(c[u]) * 16, xh[u]);
        ld8(x + uint64_t(c[u]) * 16 + 8, xl[u]);
      }
#pragma unroll
      for (int u = 0; u < 2; ++u)
#pragma unroll
        for (int k = 0; k < 8; ++k) df_fma(acc[k], hh[u], hl[u], xh[u][k], xl[u][k]);
    }
    for (; p < e; p += 32) {
      const uint32_t c = __ldcs(col + p);
      const float hh = __ldcs(vhi + p), hl = __ldcs(vlo + p);
      float xh[8], xl[8];
      ld8(x + uint64_t(c) * 16, xh);
      ld8(x + uint64_t(c) * 16 + 8, xl);
#pragma unroll
      for (int k = 0; k < 8; ++k) df_fma(acc[k], hh, hl, xh[k], xl[k]);
    }
    // reduce-scatter across the warp (offsets 16, 8, 4), then offsets 2, 1
#pragma unroll
    for (int o = 16, cnt = 8; cnt > 1; o >>= 1, cnt >>= 1) {
      const bool up = lane & o;
#pragma unroll
      for (int k = 0; k < cnt / 2; ++k) {
        df32 send = up ? acc[k] : acc[cnt / 2 + k];
        df32 keep = up ? acc[cnt / 2 + k] : acc[k];
        df32 got{__shfl_xor_sync(0xffffffffu, send.hi, o), __shfl_xor_sync(0xffffffffu, send.lo, o)};
        acc[k] = df_add(keep, got);
      }
    }
#pragma unroll
    for (int o = 2; o; o >>= 1) {
      df32 got{__shfl_xor_sync(0xffffffffu, acc[0].hi, o), __shfl_xor_sync(0xffffffffu, acc[0].lo, o)};
      acc[0] = df_add(acc[0], got);
    }
    const int vi = lane >> 2;
    if ((lane & 3) == 0 && vi < m_out) y[row * uint64_t(ldy) + vi] = double(acc[0].hi) + double(acc[0].lo);
  }
}

// x (FP64, row-interleaved, m <= 8 columns) -> staging rows of 8 hi + 8 lo floats
__global__ void k_stage_df(uint64_t n, const double* __restrict__ x, int ldx, int m, float* __restrict__ w) {
  uint64_t idx = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (idx >= n * 8) return;
  uint64_t i = idx >> 3;
  int j = int(idx & 7);
  double v = j < m ? x[i * ldx + j] : 0.0;
  float h = float(v);
  w[i * 16 + j] = h;
  w[i * 16 + 8 + j] = float(v - double(h));
}

// Launch shape of the FP32 product: WARPS warps per CTA, CTAS CTAs per SM,
// each CTA walking one contiguous row range (so the warps sharing an SM work on
// neighbouring rows, whose columns overlap, and reuse gathered vectors in L1).
template <int NV, int WARPS>
void launch_wide(const Hamiltonian& h, const float* x, int ldx, float* y, int ldy, int m_out, int ctas_per_sm,
                 cudaStream_t s) {
  int nsm = 0;
  CG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, h.device));
  int per_sm = 0;
  CG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_spmm_f32w<NV, WARPS>, WARPS * 32, 0));
  int use = std::max(1, std::min(per_sm, ctas_per_sm));
  uint64_t ctas = uint64_t(nsm) * use;
  uint64_t rpc = (h.n + ctas - 1) / ctas;
  rpc = (rpc + WARPS - 1) / WARPS * WARPS;
  if (rpc == 0) rpc = WARPS;
  unsigned grid = unsigned((h.n + rpc - 1) / rpc);
  if (grid == 0) return;
  k_spmm_f32w<NV, WARPS><<<grid, WARPS * 32, 0, s>>>(h.n, h.rowptr.p, h.col.p, h.hi.p, x, ldx, y, ldy, m_out, rpc);
  CG_CUDA(cudaGetLastError());
    count_launch();
}

template <int NV>
void run_wide(const Hamiltonian& h, const float* x, int ldx, float* y, int ldy, int m_out, cudaStream_t s) {
  const SpmmTuning& t = h.tuning;
  switch (t.warps) {
    case 4: return launch_wide<NV, 4>(h, x, ldx, y, ldy, m_out, t.ctas_per_sm, s);
    case 8: return launch_wide<NV, 8>(h, x, ldx, y, ldy, m_out, t.ctas_per_sm, s);
    case 16: return launch_wide<NV, 16>(h, x, ldx, y, ldy, m_out, t.ctas_per_sm, s);
    case 32: return launch_wide<NV, 32>(h, x, ldx, y, ldy, m_out, t.ctas_per_sm, s);
    default: throw Error(CG_ERR_ARG, "SpMM tuning: warps per CTA must be 4, 8, 16 or 32");
  }
}

template <int MODE, int NV>
void run_nv(const Hamiltonian& h, const void* vals, const void* x, int ldx, void* y, int ldy, cudaStream_t s) {
  constexpr size_t esz = MODE == CG_PREC_FP32 ? 4 : 8;
  if constexpr (MODE == CG_PREC_FP32 && (NV == 8 || NV == 16)) {
    if (reinterpret_cast<uintptr_t>(x) % 32 == 0 && ldx % 8 == 0)
      return run_wide<NV>(h, static_cast<const float*>(x), ldx, static_cast<float*>(y), ldy, NV, s);
  }
  auto ok = [&](size_t vw) {
    return NV % vw == 0 && reinterpret_cast<uintptr_t>(x) % (vw * esz) == 0 && (size_t(ldx) % vw) == 0;
  };
  if constexpr (MODE == CG_PREC_FP32 && NV % 4 == 0) {
    if (ok(4)) return run_kernel<MODE, NV, 4>(h, vals, x, ldx, y, ldy, s);
  }
  if constexpr (NV % 2 == 0) {
    if (ok(2)) return run_kernel<MODE, NV, 2>(h, vals, x, ldx, y, ldy, s);
  }
  if (reinterpret_cast<uintptr_t>(x) % esz) throw Error(CG_ERR_ARG, "x is not aligned to its element size");
  run_kernel<MODE, NV, 1>(h, vals, x, ldx, y, ldy, s);
}

template <int MODE>
void dispatch_nv(int m, const Hamiltonian& h, const void* vals, const void* x, int ldx, void* y, int ldy,
                 cudaStream_t s) {
  switch (m) {
#define CG_NV(N) \
  case N: run_nv<MODE, N>(h, vals, x, ldx, y, ldy, s); break;
    CG_NV(1) CG_NV(2) CG_NV(3) CG_NV(4) CG_NV(5) CG_NV(6) CG_NV(7) CG_NV(8)
    CG_NV(9) CG_NV(10) CG_NV(11) CG_NV(12) CG_NV(13) CG_NV(14) CG_NV(15) CG_NV(16)
#undef CG_NV
    default: throw Error(CG_ERR_ARG, "SpMM supports 1..16 vectors per call");
  }
}

template <class T>
__global__ void k_cm_to_rm(uint64_t n, int m, const double* __restrict__ src, T* __restrict__ dst, int ld) {
  uint64_t idx = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (idx >= n * m) return;
  uint64_t i = idx / m;
  int k = int(idx - i * m);
  dst[i * ld + k] = T(src[uint64_t(k) * n + i]);
}
template <class T>
__global__ void k_rm_to_cm(uint64_t n, int m, const T* __restrict__ src, int ld, double* __restrict__ dst) {
  uint64_t idx = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (idx >= n * m) return;
  uint64_t i = idx / m;
  int k = int(idx - i * m);
  dst[uint64_t(k) * n + i] = double(src[i * ld + k]);
}

template <class T>
void spmm_host_t(const Hamiltonian& h, int precision, const double* x, double* y, int m) {
  const uint64_t n = h.n;
  cudaStream_t s = h.stream;
  DBuf<double> cm(n * m);
  cm.upload(x, n * m, s);
  for (int c0 = 0; c0 < m; c0 += 16) {
    int mc = std::min(16, m - c0);
    int ld = (mc + 3) / 4 * 4;
    DBuf<T> xi(n * ld), yi(n * ld);
    unsigned g = unsigned((n * mc + 255) / 256);
    if (g) k_cm_to_rm<T><<<g, 256, 0, s>>>(n, mc, cm.p + uint64_t(c0) * n, xi.p, ld);
    CG_CUDA(cudaGetLastError());
    count_launch();
    if constexpr (std::is_same<T, double>::value) {
      if (precision == CG_PREC_REFINE) {
        DBuf<float> stage(n * 16);
        spmm_refine_df(h, xi.p, ld, yi.p, ld, mc, stage.p, s);
      } else {
        spmm_launch(h, precision, xi.p, ld, yi.p, ld, mc, s);
      }
    } else {
      spmm_launch(h, precision, xi.p, ld, yi.p, ld, mc, s);
    }
    if (g) k_rm_to_cm<T><<<g, 256, 0, s>>>(n, mc, yi.p, ld, cm.p + uint64_t(c0) * n);
    CG_CUDA(cudaGetLastError());
    count_launch();
    CG_CUDA(cudaStreamSynchronize(s));
  }
  CG_CUDA(cudaMemcpyAsync(y, cm.p, n * m * 8, cudaMemcpyDeviceToHost, s));
  CG_CUDA(cudaStreamSynchronize(s));
}

}  // namespace

void spmm_host(const Hamiltonian& h, int precision, const double* x, double* y, int m) {
  if (m < 1) throw Error(CG_ERR_ARG, "m must be >= 1");
  if (precision == CG_PREC_FP32) spmm_host_t<float>(h, precision, x, y, m);
  else spmm_host_t<double>(h, precision, x, y, m);
}

// Autotuner: time every candidate launch shape of the row-wise FP32 product on
// this matrix and, for up to 8 vectors, the block-tiled product (CUDA events
// on the handle's stream, median of `reps`); keep the fastest in h.tuning /
// h.use_tiled.  Returns the per-candidate times (the tiled candidate carries
// ctas_per_sm = 0).  Shapes with fewer than 16 resident warps per SM are not
// tried (the gathers of the row-wise product need more in flight; they were
// 2-6x slower than the best on every matrix measured), and a candidate whose
// warm-up launch takes more than twice the best median so far is not
// repeated.
std::vector<SpmmCandidate> spmm_autotune(Hamiltonian& h, int m, int reps) {
  if (h.virt) throw Error(CG_ERR_UNSUPPORTED, "launch-shape tuning applies to stored matrices");
  if (h.precision != CG_PREC_FP32) throw Error(CG_ERR_ARG, "autotuning applies to FP32 matrices");
  const int ld = m <= 8 ? 8 : 16;
  cudaStream_t s = h.stream;
  DBuf<float> x(h.n * ld), y(h.n * ld);
  CG_CUDA(cudaMemsetAsync(x.p, 0, x.bytes(), s));
  cudaEvent_t e0, e1;
  CG_CUDA(cudaEventCreate(&e0));
  CG_CUDA(cudaEventCreate(&e1));
  float best = 1e30f;
  auto time_once = [&]() {
    CG_CUDA(cudaEventRecord(e0, s));
    spmm_f32_padded(h, x.p, ld, y.p, ld, m, s);  // warm
    CG_CUDA(cudaEventRecord(e1, s));
    CG_CUDA(cudaEventSynchronize(e1));
    float warm = 0;
    CG_CUDA(cudaEventElapsedTime(&warm, e0, e1));
    if (warm > 2.0f * best) return warm;
    std::vector<float> ts;
    for (int r = 0; r < reps; ++r) {
      CG_CUDA(cudaEventRecord(e0, s));
      spmm_f32_padded(h, x.p, ld, y.p, ld, m, s);
      CG_CUDA(cudaEventRecord(e1, s));
      CG_CUDA(cudaEventSynchronize(e1));
      float ms = 0;
      CG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      ts.push_back(ms);
    }
    std::sort(ts.begin(), ts.end());
    return ts[ts.size() / 2];
  };
  std::vector<SpmmCandidate> out;
  const SpmmTuning keep = h.tuning;
  SpmmTuning bt = keep;
  bool tiled_best = false;
  h.use_tiled = false;
  for (int w : {4, 8, 16, 32})
    for (int c : {1, 2, 4, 8}) {
      if (w * c > 64 || w * c < 16) continue;  // 16..64 resident warps per SM
      h.tuning.warps = w;
      h.tuning.ctas_per_sm = c;
      const float med = time_once();
      out.push_back({w, c, med});
      if (med < best) { best = med; bt = h.tuning; }
    }
  if (h.tiled && m <= 8) {
    // tiled launch shapes: slices per consumer warp x ring slots
    TiledOp& t = *h.tiled;
    int brps = t.rps, bst = t.stages;
    float tbest = 1e30f;
    h.use_tiled = true;
    for (int rps : {1, 2, 3})
      for (int st : {2, 3, 4, 6}) {
        if ((t.smax + rps - 1) / rps > 31) continue;  // at most 31 consumer warps
        if (tiled_smem(t, st) > 227 * 1024) continue;
        t.rps = rps;
        t.warps = (t.smax + rps - 1) / rps;
        t.stages = st;
        const float med = time_once();
        if (med < tbest) { tbest = med; brps = rps; bst = st; }
      }
    t.rps = brps;
    t.warps = (t.smax + brps - 1) / brps;
    t.stages = bst;
    const int bw = t.warps;
    out.push_back({bw, 0, tbest});
    if (tbest < best) { best = tbest; tiled_best = true; }
  }
  h.tuning = bt;
  h.tuning.tuned = true;
  h.use_tiled = tiled_best;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return out;
}

// ---- gather-rate probe ---------------------------------------------------
// Random 32-byte gathers (one sector per lane, four in flight per lane) from a
// table of `rows` 32-byte rows; `share` consecutive lanes read consecutive rows
// (share = 4 puts four lanes in one 128-byte line).  Measures the ceiling of
// the SpMM's dominant traffic on this device.
__global__ void k_gather_probe(const uint32_t* __restrict__ idx, uint64_t nidx, const float* __restrict__ x,
                               float* __restrict__ out) {
  float acc = 0.f;
  const uint64_t t = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x, stride = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t i = t; i < nidx; i += stride * 4) {
    uint32_t c[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) c[u] = (i + u * stride < nidx) ? __ldg(idx + i + u * stride) : 0u;
    float v[4][8];
#pragma unroll
    for (int u = 0; u < 4; ++u) ld8(x + 8ull * c[u], v[u]);
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
      for (int j = 0; j < 8; ++j) acc += v[u][j];
  }
  if (acc == 1234.5f) out[0] = acc;  // keeps the loads live
}

__global__ void k_probe_index(uint32_t* __restrict__ idx, uint64_t n, uint64_t rows, int share, uint64_t seed) {
  uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  uint64_t g = i / share;
  uint64_t z = (g + seed) * 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  z ^= z >> 31;
  uint64_t base = z % (rows / share);
  idx[i] = uint32_t(base * share + i % share);
}

double gather_probe(int device, uint64_t rows, int share) {
  if (share < 1 || rows < uint64_t(share)) throw Error(CG_ERR_ARG, "bad probe shape");
  CG_CUDA(cudaSetDevice(device));
  cudaStream_t s;
  CG_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  const uint64_t n = 1ull << 26;
  DBuf<uint32_t> idx(n);
  DBuf<float> x(rows * 8), out(1);
  CG_CUDA(cudaMemsetAsync(x.p, 0, x.bytes(), s));
  k_probe_index<<<unsigned((n + 255) / 256), 256, 0, s>>>(idx.p, n, rows, share, 12345);
  CG_CUDA(cudaGetLastError());
  int nsm = 0;
  CG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, device));
  cudaEvent_t e0, e1;
  CG_CUDA(cudaEventCreate(&e0));
  CG_CUDA(cudaEventCreate(&e1));
  k_gather_probe<<<nsm * 8, 256, 0, s>>>(idx.p, n, x.p, out.p);
  CG_CUDA(cudaEventRecord(e0, s));
  const int reps = 3;
  for (int r = 0; r < reps; ++r) k_gather_probe<<<nsm * 8, 256, 0, s>>>(idx.p, n, x.p, out.p);
  CG_CUDA(cudaEventRecord(e1, s));
  CG_CUDA(cudaEventSynchronize(e1));
  CG_CUDA(cudaGetLastError());
  float ms = 0;
  CG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(s);
  return double(n) * reps / (ms * 1e-3);
}

void spmm_refine_df(const Hamiltonian& h, const double* x, int ldx, double* y, int ldy, int m, float* stage,
                    cudaStream_t s) {
  if (h.virt) return virtual_launch(h, CG_PREC_REFINE, x, ldx, y, ldy, m, s);
  if (h.precision != CG_PREC_FP32) throw Error(CG_ERR_ARG, "refinement product needs an FP32 (hi+lo) matrix");
  for (int c0 = 0; c0 < m; c0 += 8) {
    const int mc = std::min(8, m - c0);
    k_stage_df<<<unsigned((h.n * 8 + 255) / 256), 256, 0, s>>>(h.n, x + c0, ldx, mc, stage);
    CG_CUDA(cudaGetLastError());
    count_launch();
    int nsm = 0;
    CG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, h.device));
    constexpr int W = 8;
    int per_sm = 0;
    CG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_spmm_df8<W>, W * 32, 0));
    uint64_t ctas = uint64_t(nsm) * std::max(per_sm, 1);
    uint64_t rpc = (h.n + ctas - 1) / ctas;
    rpc = (rpc + W - 1) / W * W;
    if (rpc == 0) rpc = W;
    unsigned grid = unsigned((h.n + rpc - 1) / rpc);
    if (grid)
      k_spmm_df8<W><<<grid, W * 32, 0, s>>>(h.n, h.rowptr.p, h.col.p, h.hi.p, h.lo.p, stage, y + c0, ldy, mc, rpc);
    CG_CUDA(cudaGetLastError());
    count_launch();
  }
}

// ---- allocation-free refinement product ------------------------------------
// The double-float product stages each block of 8 columns of x as 16 floats per
// row (8 high parts, then 8 low parts).  spmm_refine_static keeps that staging
// area in the fixed device array below instead of a per-call allocation, for
// callers that cannot allocate device memory: a host eigensolver that drives
// the product while the stored matrix and its vector basis hold the device's
// memory, or a caller that must not stall other streams (cudaMalloc/cudaFree
// can synchronize the whole device).  The array is one per device and shared
// by every call; k_stage_df writes every element it later reads, so nothing in
// it has to start at zero.
constexpr uint64_t kStaticStageBytes = uint64_t(8) << 20;  // 8 MiB
constexpr uint64_t kStaticStageRows = kStaticStageBytes / (16 * sizeof(float));  // 131,072 rows
constexpr int kStaticMaxDevices = 64;
static __device__ __align__(256) float g_static_stage[kStaticStageBytes / sizeof(float)];

namespace {
// Address of g_static_stage on `device`, looked up once per device (the first
// call on a device does this set-up; make it before any stream capture
// begins).  The caller has made `device` current.
float* static_stage(int device) {
  static std::mutex mu;
  static float* addr[kStaticMaxDevices] = {};
  if (device < 0 || device >= kStaticMaxDevices) throw Error(CG_ERR_ARG, "device ordinal beyond 63");
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_static_stage);
    if (e != cudaSuccess || !p)
      throw Error(CG_ERR_CUDA, std::string("cudaGetSymbolAddress(static staging area): ") + cudaGetErrorString(e));
    addr[device] = static_cast<float*>(p);
  }
  return addr[device];
}
}  // namespace

uint64_t spmm_refine_static_max_rows() { return kStaticStageRows; }

void spmm_refine_static(const Hamiltonian& h, const double* x, int ldx, double* y, int ldy, int m,
                        cudaStream_t s) {
  if (h.virt) throw Error(CG_ERR_ARG, "the allocation-free product needs a stored FP32 (hi+lo) matrix");
  if (h.precision != CG_PREC_FP32) throw Error(CG_ERR_ARG, "refinement product needs an FP32 (hi+lo) matrix");
  if (m < 1 || m > 16) throw Error(CG_ERR_ARG, "the allocation-free product takes 1..16 vectors per call");
  if (ldx < m || ldy < m) throw Error(CG_ERR_ARG, "leading dimension smaller than the vector count");
  if (reinterpret_cast<uintptr_t>(x) % 8 || reinterpret_cast<uintptr_t>(y) % 8)
    throw Error(CG_ERR_ARG, "x and y must be 8-byte aligned FP64 buffers");
  if (h.n > kStaticStageRows)
    throw Error(CG_ERR_ARG, "allocation-free product: " + std::to_string(h.n) +
                                " rows exceed its static staging area of " + std::to_string(kStaticStageRows) +
                                " rows (8 MiB); use cg_spmm_device or cg_spmm");
  spmm_refine_df(h, x, ldx, y, ldy, m, static_stage(h.device), s);
}

void spmm_f32_padded(const Hamiltonian& h, const float* x, int ldx, float* y, int ldy, int m, cudaStream_t s) {
  if (h.virt) return virtual_launch(h, CG_PREC_FP32, x, ldx, y, ldy, m, s);
  if (h.precision != CG_PREC_FP32) throw Error(CG_ERR_ARG, "FP32 product needs an FP32 matrix");
  if (m < 1 || m > 16) throw Error(CG_ERR_ARG, "padded FP32 SpMM takes 1..16 vectors");
  if (reinterpret_cast<uintptr_t>(x) % 32 || ldx % 8) throw Error(CG_ERR_ARG, "padded FP32 SpMM needs 32-byte rows");
  if (m <= 8 && ldx == 8 && h.tiled && h.use_tiled) return tiled_product(h, x, y, ldy, m, s);
  if (m <= 8) {
    if (ldx < 8) throw Error(CG_ERR_ARG, "ldx < 8");
    run_wide<8>(h, x, ldx, y, ldy, m, s);
  } else {
    if (ldx < 16) throw Error(CG_ERR_ARG, "ldx < 16");
    run_wide<16>(h, x, ldx, y, ldy, m, s);
  }
}

void spmm_launch(const Hamiltonian& h, int precision, const void* x, int ldx, void* y, int ldy, int m,
                 cudaStream_t s) {
  if (m < 1 || m > 16) throw Error(CG_ERR_ARG, "SpMM supports 1..16 vectors per call");
  if (h.virt) return virtual_launch(h, precision, x, ldx, y, ldy, m, s);
  if (ldx < m || ldy < m) throw Error(CG_ERR_ARG, "leading dimension smaller than the vector count");
  switch (precision) {
    case CG_PREC_FP64:
      if (h.precision != CG_PREC_FP64) throw Error(CG_ERR_ARG, "FP64 product needs an FP64 matrix");
      dispatch_nv<CG_PREC_FP64>(m, h, h.val64.p, x, ldx, y, ldy, s);
      break;
    case CG_PREC_FP32:
      if (h.precision != CG_PREC_FP32) throw Error(CG_ERR_ARG, "FP32 product needs an FP32 matrix");
      if (m <= 8 && ldx == 8 && h.tiled && h.use_tiled && reinterpret_cast<uintptr_t>(x) % 16 == 0)
        return tiled_product(h, static_cast<const float*>(x), static_cast<float*>(y), ldy, m, s);
      dispatch_nv<CG_PREC_FP32>(m, h, h.hi.p, x, ldx, y, ldy, s);
      break;
    case CG_PREC_REFINE:
      if (h.precision != CG_PREC_FP32) throw Error(CG_ERR_ARG, "refinement product needs an FP32 (hi+lo) matrix");
      dispatch_nv<CG_PREC_REFINE>(m, h, h.hi.p, x, ldx, y, ldy, s);
      break;
    default:
      throw Error(CG_ERR_ARG, "unknown precision");
  }
}

}  // namespace cg
