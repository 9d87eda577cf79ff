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
//   CG_PREC_FP32   FP32 values and vectors; each lane accumulates its products
//                  in FP32, the cross-lane (across row blocks) sum is FP64, the
//                  result is rounded once to FP32.
//   CG_PREC_REFINE FP32 hi + FP32 lo values (h = hi + lo to ~2^-48), FP64
//                  vectors and accumulation.
#include <algorithm>
#include <type_traits>

#include "device.h"

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
#pragma unroll
      for (int k = 0; k < NV; ++k) tot[k] = warp_sum(double(acc[k]));
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
}

// Widest vector load the operands allow: VW elements divide NV, the base
// address and the row pitch.
template <int MODE, int NV>
void run_nv(const Hamiltonian& h, const void* vals, const void* x, int ldx, void* y, int ldy, cudaStream_t s) {
  constexpr size_t esz = MODE == CG_PREC_FP32 ? 4 : 8;
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
    spmm_launch(h, precision, xi.p, ld, yi.p, ld, mc, s);
    if (g) k_rm_to_cm<T><<<g, 256, 0, s>>>(n, mc, yi.p, ld, cm.p + uint64_t(c0) * n);
    CG_CUDA(cudaGetLastError());
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

void spmm_launch(const Hamiltonian& h, int precision, const void* x, int ldx, void* y, int ldy, int m,
                 cudaStream_t s) {
  if (m < 1 || m > 16) throw Error(CG_ERR_ARG, "SpMM supports 1..16 vectors per call");
  if (ldx < m || ldy < m) throw Error(CG_ERR_ARG, "leading dimension smaller than the vector count");
  switch (precision) {
    case CG_PREC_FP64:
      if (h.precision != CG_PREC_FP64) throw Error(CG_ERR_ARG, "FP64 product needs an FP64 matrix");
      dispatch_nv<CG_PREC_FP64>(m, h, h.val64.p, x, ldx, y, ldy, s);
      break;
    case CG_PREC_FP32:
      if (h.precision != CG_PREC_FP32) throw Error(CG_ERR_ARG, "FP32 product needs an FP32 matrix");
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
