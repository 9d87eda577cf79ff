// Block-tiled 8-vector FP32 product (layout described in tiled.h).
//
// Product kernel: one CTA per row block b (longest first), warp w owning the
// 32-row slices w, w + NW, ... of b and the 8 accumulators of each of its
// rows in registers for the whole CTA.  The CTA walks the tiles of b in
// ascending column block; thread 0 keeps `stages` tiles in flight, each x[c]
// brought into a shared-memory ring slot by one cp.async.bulk whose completion
// is counted on that slot's `full` mbarrier, and a slot is refilled once every
// warp has arrived on its `empty` mbarrier.  Warps therefore run up to
// stages - 1 tiles apart and never meet at a CTA-wide barrier inside the loop.
// Each stored entry costs one 2-byte column, one FP32 value (both streamed,
// coalesced) and one 32-byte row read from shared memory.
//
// The reference's blocked format is PPMatrix2CSBBlk (include/sm/PPMatrix.cxx:
// 571-656, square blocks of floor(sqrt(n)) + 1 rows, 16-bit in-block indices)
// multiplied by SparseMatrixCSB::TimesMatrix (include/tav/csbmatrix.cxx:
// 623-663); here the blocks follow the basis' neutron blocks so that a tile is
// one (neutron configuration, neutron configuration) pair and both triangles
// are stored.
#include <algorithm>

#include "bulk.h"
#include "tiled.h"

namespace cg {

namespace {

constexpr int kTiledHead = kTiledHeadBytes;

__global__ void k_colblk(int nb, const uint64_t* __restrict__ bstart, uint32_t* __restrict__ colblk) {
  for (int b = blockIdx.x; b < nb; b += gridDim.x)
    for (uint64_t r = bstart[b] + threadIdx.x; r < bstart[b + 1]; r += blockDim.x) colblk[r] = uint32_t(b);
}

// first position in [lo, hi) whose column is >= c (columns ascending)
__device__ __forceinline__ uint64_t lower_col(const uint32_t* __restrict__ col, uint64_t lo, uint64_t hi, uint64_t c) {
  while (lo < hi) {
    const uint64_t mid = (lo + hi) >> 1;
    if (col[mid] < c) lo = mid + 1; else hi = mid;
  }
  return lo;
}

// mark the (row block, column block) pairs that hold entries
__global__ void k_tmark(uint64_t n, const uint64_t* __restrict__ rowptr, const uint32_t* __restrict__ col,
                        const uint32_t* __restrict__ colblk, int words, uint32_t* __restrict__ bitmap) {
  const int lane = threadIdx.x & 31;
  const uint64_t w0 = (blockIdx.x * uint64_t(blockDim.x) + threadIdx.x) >> 5;
  const uint64_t nw = (uint64_t(gridDim.x) * blockDim.x) >> 5;
  for (uint64_t r = w0; r < n; r += nw) {
    const uint64_t rb = rowptr[r], re = rowptr[r + 1];
    const uint32_t b = colblk[r];
    for (uint64_t e = rb + lane; e < re; e += 32) {
      const uint32_t cb = colblk[col[e]];
      const uint32_t prev = e == rb ? ~0u : colblk[col[e - 1]];
      if (cb != prev) atomicOr(&bitmap[size_t(b) * words + (cb >> 5)], 1u << (cb & 31));
    }
  }
}

struct TileIndex {
  const uint64_t* bstart;
  const uint32_t* colblk;
  const uint32_t* bitmap;
  const uint32_t* wrank;  // per (block, word): tiles of the block before this word (global tile index)
  const uint32_t* tptr;
  const uint32_t* runbase;
  int words;
  __device__ __forceinline__ uint32_t run(uint32_t b, uint32_t cb, uint64_t r) const {
    const size_t w = size_t(b) * words + (cb >> 5);
    const uint32_t tile = wrank[w] + __popc(bitmap[w] & ((1u << (cb & 31)) - 1u));
    const uint32_t slices = uint32_t((bstart[b + 1] - bstart[b] + 31) >> 5);
    return runbase[b] + (tile - tptr[b]) * slices + uint32_t((r - bstart[b]) >> 5);
  }
};

// width (entries of the longest row) of every (tile, slice) run
__global__ void k_twidth(uint64_t n, const uint64_t* __restrict__ rowptr, const uint32_t* __restrict__ col,
                         TileIndex ti, uint32_t* __restrict__ width) {
  const int lane = threadIdx.x & 31;
  const uint64_t w0 = (blockIdx.x * uint64_t(blockDim.x) + threadIdx.x) >> 5;
  const uint64_t nw = (uint64_t(gridDim.x) * blockDim.x) >> 5;
  for (uint64_t r = w0; r < n; r += nw) {
    const uint64_t rb = rowptr[r], re = rowptr[r + 1];
    const uint32_t b = ti.colblk[r];
    for (uint64_t e = rb + lane; e < re; e += 32) {
      const uint32_t cb = ti.colblk[col[e]];
      const uint32_t prev = e == rb ? ~0u : ti.colblk[col[e - 1]];
      if (cb != prev) {
        const uint64_t end = lower_col(col, e, re, ti.bstart[cb + 1]);
        atomicMax(&width[ti.run(b, cb, r)], uint32_t(end - e));
      }
    }
  }
}

__global__ void k_tfill(uint64_t n, const uint64_t* __restrict__ rowptr, const uint32_t* __restrict__ col,
                        const float* __restrict__ hi, TileIndex ti, const uint32_t* __restrict__ roff,
                        uint16_t* __restrict__ tcol, float* __restrict__ tval) {
  const int lane = threadIdx.x & 31;
  const uint64_t w0 = (blockIdx.x * uint64_t(blockDim.x) + threadIdx.x) >> 5;
  const uint64_t nw = (uint64_t(gridDim.x) * blockDim.x) >> 5;
  for (uint64_t r = w0; r < n; r += nw) {
    const uint64_t rb = rowptr[r], re = rowptr[r + 1];
    const uint32_t b = ti.colblk[r];
    const uint32_t l = uint32_t(r - ti.bstart[b]) & 31;
    for (uint64_t e = rb + lane; e < re; e += 32) {
      const uint32_t c = col[e];
      const uint32_t cb = ti.colblk[c];
      const uint64_t cs = ti.bstart[cb];
      const uint64_t first = lower_col(col, rb, e + 1, cs);
      const uint64_t dst = (uint64_t(roff[ti.run(b, cb, r)]) + (e - first)) * 32 + l;
      tcol[dst] = uint16_t(c - cs);
      tval[dst] = hi[e];
    }
  }
}

struct TArgs {
  const uint64_t* bstart;
  const uint32_t* order;
  const uint32_t* tptr;
  const uint32_t* tcb;
  const uint32_t* runbase;
  const uint32_t* roff;
  const uint16_t* col;
  const float* val;
  int lmax, stages;
};

// Row read of 8 floats as two 16-byte halves, odd lanes second half first (the
// first load of a warp then covers all eight 16-byte bank groups); the halves
// stay swapped in the lane's registers and accumulators.
__device__ __forceinline__ void row8(const float* p, int sw, float (&v)[8]) {
  const float4 a = reinterpret_cast<const float4*>(p)[sw], b = reinterpret_cast<const float4*>(p)[sw ^ 1];
  v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
}

template <int NW, int RPS>
__global__ void __launch_bounds__(NW * 32) k_tiled(TArgs a, const float* __restrict__ x, float* __restrict__ y,
                                                   int ldy, int m, int* __restrict__ err) {
  constexpr int U = 4;  // entry steps whose loads are in flight together
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int S = a.stages;
  uint64_t* full = reinterpret_cast<uint64_t*>(smem_raw);
  uint64_t* empty = full + S;
  volatile int* abort_flag = reinterpret_cast<volatile int*>(empty + S);
  float* ring = reinterpret_cast<float*>(smem_raw + kTiledHead);
  const size_t slot_floats = size_t(a.lmax) * 8;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, sw = lane & 1;
  const uint32_t b = a.order[blockIdx.x];
  const uint64_t start = a.bstart[b];
  const int L = int(a.bstart[b + 1] - start);
  const int slices = (L + 31) >> 5;
  const uint32_t t0 = a.tptr[b];
  const int T = int(a.tptr[b + 1] - t0);
  const uint32_t rb = a.runbase[b];

  if (tid == 0) {
    for (int i = 0; i < S; ++i) {
      bulk::mbar_init(&full[i], 1);
      bulk::mbar_init(&empty[i], NW);
    }
    *abort_flag = 0;
    bulk::fence_mbar_init();
  }
  __syncthreads();
  auto issue = [&](int t) {
    const uint32_t cb = a.tcb[t0 + t];
    const uint64_t cs = a.bstart[cb];
    const uint32_t bytes = uint32_t(a.bstart[cb + 1] - cs) * 32u;
    bulk::bulk_load(ring + size_t(t % S) * slot_floats, x + cs * 8, bytes, &full[t % S]);
  };
  int issued = 0;
  if (tid == 0)
    for (; issued < S && issued < T; ++issued) issue(issued);

  float acc[RPS][8];
#pragma unroll
  for (int k = 0; k < RPS; ++k)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[k][j] = 0.f;

  // run offsets of this warp's slices, one tile ahead
  uint32_t nx0[RPS], nx1[RPS];
#pragma unroll
  for (int k = 0; k < RPS; ++k) {
    const int s = warp + k * NW;
    nx0[k] = nx1[k] = 0;
    if (s < slices && T > 0) {
      nx0[k] = a.roff[rb + s];
      nx1[k] = a.roff[rb + s + 1];
    }
  }
  for (int t = 0; t < T; ++t) {
    // refill the slot of the previous tile once every warp has released it
    if (tid == 0 && t >= 1 && issued < T) {
      const int p = t - 1;
      if (bulk::mbar_wait(&empty[p % S], (p / S) & 1)) {
        issue(issued);
        ++issued;
      } else {
        *abort_flag = 1;
        atomicOr(err, 1);
      }
    }
    if (__any_sync(0xffffffffu, *abort_flag != 0)) break;
    uint32_t o0[RPS], o1[RPS];
#pragma unroll
    for (int k = 0; k < RPS; ++k) {
      o0[k] = nx0[k];
      o1[k] = nx1[k];
      const int s = warp + k * NW;
      if (s < slices && t + 1 < T) {
        const uint32_t q = rb + uint32_t(t + 1) * slices + s;
        nx0[k] = a.roff[q];
        nx1[k] = a.roff[q + 1];
      }
    }
    const bool ok = bulk::mbar_wait(&full[t % S], (t / S) & 1);
    if (!__all_sync(0xffffffffu, ok)) {
      if (lane == 0) {
        *abort_flag = 1;
        atomicOr(err, 1);
      }
      break;
    }
    const float* buf = ring + size_t(t % S) * slot_floats;
#pragma unroll
    for (int k = 0; k < RPS; ++k) {
      for (uint32_t j = o0[k]; j < o1[k]; j += U) {
        uint32_t c[U];
        float v[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          c[u] = 0;
          v[u] = 0.f;
          if (j + u < o1[k]) {
            const uint64_t e = uint64_t(j + u) * 32 + lane;
            c[u] = __ldcs(a.col + e);
            v[u] = __ldcs(a.val + e);
          }
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
          if (j + u < o1[k]) {
            float xr[8];
            row8(buf + size_t(c[u]) * 8, sw, xr);
#pragma unroll
            for (int q = 0; q < 8; ++q) acc[k][q] = fmaf(v[u], xr[q], acc[k][q]);
          }
      }
    }
    __syncwarp();
    if (lane == 0) bulk::mbar_arrive(&empty[t % S]);
  }
  __syncthreads();
  if (*abort_flag) {
    // let the copies still in flight land before the CTA's shared memory goes
    if (tid == 0)
      for (int i = issued > S ? issued - S : 0; i < issued; ++i) bulk::mbar_wait(&full[i % S], (i / S) & 1);
    return;
  }
#pragma unroll
  for (int k = 0; k < RPS; ++k) {
    const int r = (warp + k * NW) * 32 + lane;
    if (r < L) {
      float* yr = y + (start + r) * size_t(ldy);
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        const int jj = sw ? (j ^ 4) : j;
        if (jj < m) yr[jj] = acc[k][j];
      }
    }
  }
}

template <int NW, int RPS>
void launch_tiled(const TiledOp& t, const TArgs& a, const float* x, float* y, int ldy, int m, int* err,
                  cudaStream_t s) {
  const size_t smem = kTiledHead + size_t(t.stages) * t.lmax * 32;
  CG_CUDA(cudaFuncSetAttribute(k_tiled<NW, RPS>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
  k_tiled<NW, RPS><<<unsigned(t.nb), NW * 32, smem, s>>>(a, x, y, ldy, m, err);
  CG_CUDA(cudaGetLastError());
  count_launch();
}

template <int NW>
void launch_nw(const TiledOp& t, const TArgs& a, const float* x, float* y, int ldy, int m, int* err, cudaStream_t s) {
  const int rps = (t.smax + NW - 1) / NW;
  switch (rps) {
    case 1: launch_tiled<NW, 1>(t, a, x, y, ldy, m, err, s); break;
    case 2: launch_tiled<NW, 2>(t, a, x, y, ldy, m, err, s); break;
    case 3: launch_tiled<NW, 3>(t, a, x, y, ldy, m, err, s); break;
    case 4: launch_tiled<NW, 4>(t, a, x, y, ldy, m, err, s); break;
    default: throw Error(CG_ERR_INTERNAL, "tiled product: too many slices per warp");
  }
}

}  // namespace

std::vector<uint64_t> tiled_uniform_blocks(uint64_t n) {
  std::vector<uint64_t> b;
  for (uint64_t r = 0; r < n; r += 512) b.push_back(r);
  b.push_back(n);
  return b;
}

void tiled_build(Hamiltonian& h, const std::vector<uint64_t>& bs) {
  h.tiled.reset();
  if (h.precision != CG_PREC_FP32 || h.n == 0 || bs.size() < 2 || bs.back() != h.n) return;
  const int nb = int(bs.size() - 1);
  int lmax = 0;
  for (int b = 0; b < nb; ++b) {
    if (bs[b + 1] < bs[b]) throw Error(CG_ERR_INTERNAL, "block starts not ascending");
    lmax = std::max<int>(lmax, int(std::min<uint64_t>(bs[b + 1] - bs[b], 1u << 30)));
  }
  if (lmax > kTiledMaxBlock) return;
  cudaStream_t s = h.stream;
  auto tp = std::make_shared<TiledOp>();
  TiledOp& t = *tp;
  t.nb = nb;
  t.lmax = std::max(lmax, 1);
  t.smax = (t.lmax + 31) / 32;
  t.nnz = h.nnz;
  t.bstart.upload(bs, s);
  std::vector<uint32_t> order(nb);
  for (int b = 0; b < nb; ++b) order[b] = uint32_t(b);
  std::stable_sort(order.begin(), order.end(),
                   [&](uint32_t p, uint32_t q) { return bs[p + 1] - bs[p] > bs[q + 1] - bs[q]; });
  t.order.upload(order, s);

  DBuf<uint32_t> colblk(h.n);
  k_colblk<<<unsigned(std::min(nb, 152 * 16)), 256, 0, s>>>(nb, t.bstart.p, colblk.p);
  CG_CUDA(cudaGetLastError());
  count_launch();
  const int words = (nb + 31) / 32;
  DBuf<uint32_t> bitmap(size_t(nb) * words);
  CG_CUDA(cudaMemsetAsync(bitmap.p, 0, bitmap.bytes(), s));
  const unsigned grid = unsigned(std::min<uint64_t>((h.n * 32 + 255) / 256, 152ull * 64));
  k_tmark<<<grid, 256, 0, s>>>(h.n, h.rowptr.p, h.col.p, colblk.p, words, bitmap.p);
  CG_CUDA(cudaGetLastError());
  count_launch();
  std::vector<uint32_t> hb(size_t(nb) * words);
  CG_CUDA(cudaMemcpyAsync(hb.data(), bitmap.p, hb.size() * 4, cudaMemcpyDeviceToHost, s));
  CG_CUDA(cudaStreamSynchronize(s));

  // tiles in ascending column block per row block; per-word tile ranks; runs
  std::vector<uint32_t> tptr(nb + 1), wrank(hb.size()), runbase(nb), tcb;
  uint64_t ntiles = 0, nruns = 0;
  for (int b = 0; b < nb; ++b) {
    tptr[b] = uint32_t(ntiles);
    runbase[b] = uint32_t(nruns);
    const uint64_t before = ntiles;
    for (int w = 0; w < words; ++w) {
      wrank[size_t(b) * words + w] = uint32_t(ntiles);
      for (uint32_t bits = hb[size_t(b) * words + w]; bits; bits &= bits - 1) {
        tcb.push_back(uint32_t(w * 32 + __builtin_ctz(bits)));
        ++ntiles;
      }
    }
    nruns += (ntiles - before) * ((bs[b + 1] - bs[b] + 31) / 32);
    if (ntiles >= (1ull << 32) || nruns >= (1ull << 32) - 1) return;  // beyond the 32-bit run index
  }
  tptr[nb] = uint32_t(ntiles);
  t.ntiles = ntiles;
  t.nruns = nruns;
  t.tptr.upload(tptr, s);
  t.tcb.upload(tcb, s);
  t.runbase.upload(runbase, s);
  DBuf<uint32_t> dwrank;
  dwrank.upload(wrank, s);
  TileIndex ti{t.bstart.p, colblk.p, bitmap.p, dwrank.p, t.tptr.p, t.runbase.p, words};

  DBuf<uint32_t> width(std::max<uint64_t>(nruns, 1));
  CG_CUDA(cudaMemsetAsync(width.p, 0, width.bytes(), s));
  k_twidth<<<grid, 256, 0, s>>>(h.n, h.rowptr.p, h.col.p, ti, width.p);
  CG_CUDA(cudaGetLastError());
  count_launch();
  std::vector<uint32_t> hw(nruns);
  if (nruns) CG_CUDA(cudaMemcpyAsync(hw.data(), width.p, nruns * 4, cudaMemcpyDeviceToHost, s));
  CG_CUDA(cudaStreamSynchronize(s));
  std::vector<uint32_t> roff(nruns + 1);
  uint64_t run = 0;
  for (uint64_t i = 0; i < nruns; ++i) {
    roff[i] = uint32_t(run);
    run += hw[i];
    if (run >= (1ull << 32)) return;  // beyond the 32-bit entry-group offsets
  }
  roff[nruns] = uint32_t(run);
  t.entries = run * 32;
  t.roff.upload(roff, s);
  t.col.alloc(std::max<uint64_t>(t.entries, 1));
  t.val.alloc(std::max<uint64_t>(t.entries, 1));
  CG_CUDA(cudaMemsetAsync(t.col.p, 0, t.col.bytes(), s));
  CG_CUDA(cudaMemsetAsync(t.val.p, 0, t.val.bytes(), s));
  k_tfill<<<grid, 256, 0, s>>>(h.n, h.rowptr.p, h.col.p, h.hi.p, ti, t.roff.p, t.col.p, t.val.p);
  CG_CUDA(cudaGetLastError());
  count_launch();
  CG_CUDA(cudaStreamSynchronize(s));

  // default launch shape (spmm_autotune refines it): 8 warps while 3 slices
  // per warp cover the longest block, else 16; as many ring slots (2..4) as
  // keep three CTAs per SM
  t.warps = t.smax <= 24 ? 8 : 16;
  const size_t slot = size_t(t.lmax) * 32;
  t.stages = int(std::max<size_t>(2, std::min<size_t>(4, (72 * 1024 - kTiledHead) / slot)));
  t.err.alloc(1);
  h.tiled = tp;
}

void tiled_product(const Hamiltonian& h, const float* x, float* y, int ldy, int m, cudaStream_t s) {
  const TiledOp& t = *h.tiled;
  if (m < 1 || m > 8) throw Error(CG_ERR_ARG, "tiled product takes 1..8 vectors");
  if (reinterpret_cast<uintptr_t>(x) % 16) throw Error(CG_ERR_ARG, "tiled product needs a 16-byte aligned x");
  if (t.stages < 2 || 2 * t.stages * 8 + 4 > kTiledHead || kTiledHead + size_t(t.stages) * t.lmax * 32 > 227 * 1024)
    throw Error(CG_ERR_ARG, "tiled product: ring slots out of range");
  TArgs a{t.bstart.p, t.order.p, t.tptr.p, t.tcb.p, t.runbase.p, t.roff.p, t.col.p, t.val.p, t.lmax, t.stages};
  CG_CUDA(cudaMemsetAsync(t.err.p, 0, sizeof(int), s));
  if (t.warps == 8) launch_nw<8>(t, a, x, y, ldy, m, t.err.p, s);
  else launch_nw<16>(t, a, x, y, ldy, m, t.err.p, s);
  int herr = 0;
  CG_CUDA(cudaMemcpyAsync(&herr, t.err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  CG_CUDA(cudaStreamSynchronize(s));
  if (herr) throw Error(CG_ERR_TIMEOUT, "tiled product: a staged copy or a slot release did not complete");
}

}  // namespace cg
