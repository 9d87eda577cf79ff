// Block-tiled 8-vector FP32 product (layout described in tiled.h).
//
// Product kernel: one CTA per row block b (longest first) with NW consumer
// warps (the longest block's slices / RPS) and one producer warp.  Consumer warp w owns the 32-row slices
// w, w + NW, ... of b and keeps the 8 accumulators of each of its rows in
// registers for the whole CTA.  The CTA walks the tiles of b in ascending
// column block, in staged units (tile, range of 32-entry groups): lane 0 of
// the producer warp fills a ring of `stages` shared-memory slots, each unit
// brought in by three cp.async.bulk copies (x of the column block, the
// unit's 16-bit columns, its FP32 values) counted on the slot's `full`
// mbarrier, and refills a slot once every consumer warp has arrived on its
// `empty` mbarrier.  Consumers therefore never touch global memory in the
// inner loop and never meet at a CTA-wide barrier inside it: per stored entry
// one 2-byte and one 4-byte shared load (coalesced) and one 32-byte row read
// of the staged x.
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

// Bank-group balancing of the staged-x row reads.  A row read is two 16-byte
// loads, lane l taking half (l & 1) first; the half of x row c read first sits
// in bank group 2 (c mod 4) + (l & 1), the second one in its partner group.
// When in every quarter warp (8 lanes) of a step the four even lanes read four
// different column classes (c mod 4) and so do the four odd lanes, both loads
// touch 8 distinct groups per quarter: no extra wavefront.  The entries of a
// row may be taken in any order (only its summation order changes) and a row
// shorter than its run may place its padding at any step, so the classes are
// matched greedily step by step: one thread per (run, quarter); lanes with the
// least slack choose first, each taking its first entry whose class is still
// free among the lanes of its parity, else padding when it has slack, else its
// next entry.
__global__ void k_tbalance(uint64_t nruns, const uint32_t* __restrict__ roff, uint16_t* __restrict__ col,
                           float* __restrict__ val) {
  const uint64_t t0 = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  const uint64_t nt = uint64_t(gridDim.x) * blockDim.x;
  for (uint64_t t = t0; t < nruns * 4; t += nt) {
    const uint64_t r = t >> 2;
    const int lq = int(t & 3) * 8;  // first lane of this quarter
    const uint64_t g0 = roff[r];
    const uint32_t w = roff[r + 1] - roff[r];
    if (w < 2) continue;
    uint32_t rem[8];
    for (int i = 0; i < 8; ++i) {
      rem[i] = 0;
      for (uint32_t q = 0; q < w; ++q) rem[i] += val[(g0 + q) * 32 + lq + i] != 0.f;
    }
    for (uint32_t j = 0; j < w; ++j) {
      uint32_t used = 0;  // bit (4 parity + class): taken in this step
      uint32_t done = 0;
      for (int pick = 0; pick < 8; ++pick) {
        int i = -1;
        uint32_t bslack = 0;
        for (int c = 0; c < 8; ++c) {
          if ((done >> c) & 1u) continue;
          const uint32_t slack = (w - j) - rem[c];
          if (i < 0 || slack < bslack) { i = c; bslack = slack; }
        }
        done |= 1u << i;
        if (rem[i] == 0) continue;  // only padding left in this row
        const uint32_t par = uint32_t(i & 1) * 4;
        const uint64_t ej = (g0 + j) * 32 + lq + i;
        uint32_t take = w;
        for (uint32_t q = j; q < w && take == w; ++q) {
          const uint64_t e = (g0 + q) * 32 + lq + i;
          if (val[e] != 0.f && !((used >> (par + (col[e] & 3u))) & 1u)) take = q;
        }
        if (take == w && bslack > 0)  // pad now: bring a padding entry to step j
          for (uint32_t q = j; q < w && take == w; ++q)
            if (val[(g0 + q) * 32 + lq + i] == 0.f) take = q;
        if (take == w)
          for (uint32_t q = j; q < w && take == w; ++q)
            if (val[(g0 + q) * 32 + lq + i] != 0.f) take = q;
        if (take != j) {
          const uint64_t eb = (g0 + take) * 32 + lq + i;
          const uint16_t tc = col[ej]; col[ej] = col[eb]; col[eb] = tc;
          const float tv = val[ej]; val[ej] = val[eb]; val[eb] = tv;
        }
        if (val[ej] != 0.f) {
          used |= 1u << (par + (col[ej] & 3u));
          --rem[i];
        }
      }
    }
  }
}

// Padding entries (value 0) still issue the row read: each points at the
// column of a real lane of the same parity and step (the same addresses in
// both loads: no extra access), in its own quarter warp when one has a real
// entry, else anywhere in the warp.  One warp per run.
__global__ void k_tpadaddr(uint64_t nruns, const uint32_t* __restrict__ roff, uint16_t* __restrict__ col,
                           const float* __restrict__ val) {
  const int lane = threadIdx.x & 31;
  const uint32_t pmask = (lane & 1) ? 0xaaaaaaaau : 0x55555555u;
  const uint64_t w0 = (blockIdx.x * uint64_t(blockDim.x) + threadIdx.x) >> 5;
  const uint64_t nw = (uint64_t(gridDim.x) * blockDim.x) >> 5;
  for (uint64_t r = w0; r < nruns; r += nw) {
    const uint64_t g0 = roff[r];
    const uint32_t w = roff[r + 1] - roff[r];
    for (uint32_t j = 0; j < w; ++j) {
      const uint64_t ej = (g0 + j) * 32 + lane;
      const bool real = val[ej] != 0.f;
      const uint32_t mine = col[ej];
      const uint32_t same = __ballot_sync(0xffffffffu, real) & pmask;
      const uint32_t inq = same & (0xffu << (lane & 24));
      const int src = inq ? __ffs(inq) - 1 : (same ? __ffs(same) - 1 : lane);
      const uint32_t other = __shfl_sync(0xffffffffu, mine, src);
      if (!real) col[ej] = uint16_t(other);
    }
  }
}

// Scaled-identity tiles: every row of the block holds exactly one entry, at
// its own position in the column block, and all values are bitwise equal (a
// two-neutron move with the protons as spectators).  One warp per tile.
__global__ void k_tident(uint64_t ntiles, const uint32_t* __restrict__ tblock, const uint64_t* __restrict__ bstart,
                         const uint32_t* __restrict__ tptr, const uint32_t* __restrict__ runbase,
                         const uint32_t* __restrict__ roff, const uint16_t* __restrict__ col,
                         const float* __restrict__ val, uint32_t* __restrict__ ident) {
  const int lane = threadIdx.x & 31;
  const uint64_t w0 = (blockIdx.x * uint64_t(blockDim.x) + threadIdx.x) >> 5;
  const uint64_t nw = (uint64_t(gridDim.x) * blockDim.x) >> 5;
  for (uint64_t t = w0; t < ntiles; t += nw) {
    const uint32_t b = tblock[t];
    const uint32_t L = uint32_t(bstart[b + 1] - bstart[b]), sl = (L + 31) / 32;
    const uint32_t q0 = runbase[b] + (uint32_t(t) - tptr[b]) * sl;
    const float v0 = val[uint64_t(roff[q0]) * 32];
    bool ok = v0 != 0.f;
    for (uint32_t s = 0; s < sl && ok; ++s) {
      const uint32_t g = roff[q0 + s];
      bool good = roff[q0 + s + 1] - g == 1;
      const uint32_t r = s * 32 + lane;
      if (good && r < L) {
        const uint64_t e = uint64_t(g) * 32 + lane;
        good = col[e] == r && __float_as_uint(val[e]) == __float_as_uint(v0);
      }
      ok = __all_sync(0xffffffffu, good);
    }
    if (lane == 0) ident[t] = ok ? __float_as_uint(v0) : 0u;
  }
}

// One staged unit: x of one column block and the entry groups [g0, g1) of one
// tile, plus the tile's run offsets (roff of its slices 0..slices, a 16-byte
// aligned copy in TiledOp::rcopy).  32 bytes.
struct __align__(16) TItem {
  uint32_t xrow, xrows;  // first row and row count of the column block
  uint32_t g0, g1;       // entry groups of this unit
  uint32_t rc, rcbytes;  // run-offset copy: first u32 in rcopy, bytes (multiple of 16)
  uint32_t pad0, pad1;
};

struct TArgs {
  const uint64_t* bstart;
  const uint32_t* order;
  const uint32_t* iptr;
  const TItem* items;
  const uint32_t* rcopy;
  const uint16_t* col;
  const float* val;
  const uint32_t* dptr;  // nb + 1: first scaled-identity tile of each block
  const uint2* iden;     // per scaled-identity tile: first x row, value bits
  int lmax, gmax, stages;
};

__device__ __forceinline__ void row8g(const float* p, int sw, float (&v)[8]) {
  const float4 a = __ldg(reinterpret_cast<const float4*>(p) + sw), b = __ldg(reinterpret_cast<const float4*>(p) + (sw ^ 1));
  v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
}

// Row read of 8 floats as two 16-byte halves, odd lanes second half first (the
// first load of a warp then covers all eight 16-byte bank groups); the halves
// stay swapped in the lane's registers and accumulators.
__device__ __forceinline__ void row8(const float* p, int sw, float (&v)[8]) {
  const float4 a = reinterpret_cast<const float4*>(p)[sw], b = reinterpret_cast<const float4*>(p)[sw ^ 1];
  v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
}

template <int RPS>
__global__ void __launch_bounds__(1024) k_tiled(TArgs a, const float* __restrict__ x, float* __restrict__ y,
                                                int ldy, int m, int* __restrict__ err) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int NW = int(blockDim.x >> 5) - 1;  // consumer warps; the last warp produces
  const int S = a.stages;
  uint64_t* full = reinterpret_cast<uint64_t*>(smem_raw);
  uint64_t* empty = full + S;
  volatile int* abort_flag = reinterpret_cast<volatile int*>(empty + S);
  unsigned char* ring = smem_raw + kTiledHead;
  // slot: header (g0, g1, pad; run offsets of the tile's slices, up to
  // kTiledSlotHead - 16 bytes) | x block (lmax rows x 32 B) | columns (gmax
  // groups x 64 B) | values (gmax groups x 128 B)
  const uint32_t xbytes = uint32_t(a.lmax) * 32u, cbytes = uint32_t(a.gmax) * 64u;
  const uint32_t slot = kTiledSlotHead + xbytes + 3u * cbytes;

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5, sw = lane & 1;
  const uint32_t b = a.order[blockIdx.x];
  const uint64_t start = a.bstart[b];
  const int L = int(a.bstart[b + 1] - start);
  const int slices = (L + 31) >> 5;
  const uint32_t i0 = a.iptr[b];
  const int I = int(a.iptr[b + 1] - i0);

  if (tid == 0) {
    for (int i = 0; i < S; ++i) {
      bulk::mbar_init(&full[i], 1);
      bulk::mbar_init(&empty[i], NW);
    }
    *abort_flag = 0;
    bulk::fence_mbar_init();
  }
  __syncthreads();

  if (warp == NW) {
    // producer warp: the lanes fetch the descriptors of 32 units at a time;
    // lane 0 refills slot i % S once every consumer warp has released the unit
    // S before, writes the unit's bounds and starts its four copies
    int issued = 0;
    bool stop = false;
    // entries are read once; x blocks are staged again by the CTAs of other row blocks
    const uint64_t once = bulk::policy_evict_first(), again = bulk::policy_evict_last();
    for (int base = 0; base < I && !stop; base += 32) {
      TItem d{};
      if (base + lane < I) d = a.items[i0 + base + lane];
      const int nb = min(32, I - base);
      for (int k = 0; k < nb; ++k) {
        const uint32_t xrow = __shfl_sync(0xffffffffu, d.xrow, k), xrows = __shfl_sync(0xffffffffu, d.xrows, k);
        const uint32_t g0 = __shfl_sync(0xffffffffu, d.g0, k), g1 = __shfl_sync(0xffffffffu, d.g1, k);
        const uint32_t rc = __shfl_sync(0xffffffffu, d.rc, k), rcb = __shfl_sync(0xffffffffu, d.rcbytes, k);
        int bad = 0;
        if (lane == 0) {
          const int i = base + k;
          if (i >= S && !bulk::mbar_wait(&empty[i % S], ((i / S) - 1) & 1)) {
            *abort_flag = 1;
            atomicOr(err, 1);
            bad = 1;
          } else if (*abort_flag) {
            bad = 1;
          } else {
            unsigned char* st = ring + size_t(i % S) * slot;
            uint32_t* hd = reinterpret_cast<uint32_t*>(st);
            hd[0] = g0;
            hd[1] = g1;
            uint64_t* bar = &full[i % S];
            const uint32_t ng = g1 - g0, xb = xrows * 32u;
            bulk::expect_tx(bar, rcb + xb + ng * 192u);
            bulk::copy(st + 16, a.rcopy + rc, rcb, bar);
            bulk::copy_hint(st + kTiledSlotHead, x + uint64_t(xrow) * 8, xb, bar, again);
            bulk::copy_hint(st + kTiledSlotHead + xbytes, a.col + uint64_t(g0) * 32, ng * 64u, bar, once);
            bulk::copy_hint(st + kTiledSlotHead + xbytes + cbytes, a.val + uint64_t(g0) * 32, ng * 128u, bar, once);
            issued = i + 1;
          }
        }
        if (__shfl_sync(0xffffffffu, bad, 0)) {
          stop = true;
          break;
        }
      }
    }
    if (lane == 0 && *abort_flag)  // let the copies still in flight land before the CTA's shared memory goes
      for (int i = issued > S ? issued - S : 0; i < issued; ++i) bulk::mbar_wait(&full[i % S], (i / S) & 1);
    __syncthreads();
    return;
  }

  float acc[RPS][8];
#pragma unroll
  for (int k = 0; k < RPS; ++k)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[k][j] = 0.f;

  // scaled-identity tiles straight from global memory (consecutive rows,
  // coalesced) while the first units stream in
  {
    const uint32_t d0 = a.dptr[b], d1 = a.dptr[b + 1];
    uint32_t d = d0;
    for (; d + 2 <= d1; d += 2) {
      const uint2 e0 = a.iden[d], e1 = a.iden[d + 1];
#pragma unroll
      for (int k = 0; k < RPS; ++k) {
        const int r = (warp + k * NW) * 32 + lane;
        if (r < L) {
          float x0[8], x1[8];
          row8g(x + (uint64_t(e0.x) + r) * 8, sw, x0);
          row8g(x + (uint64_t(e1.x) + r) * 8, sw, x1);
          const float v0 = __uint_as_float(e0.y), v1 = __uint_as_float(e1.y);
#pragma unroll
          for (int u = 0; u < 8; ++u) acc[k][u] = fmaf(v1, x1[u], fmaf(v0, x0[u], acc[k][u]));
        }
      }
    }
    if (d < d1) {
      const uint2 e0 = a.iden[d];
#pragma unroll
      for (int k = 0; k < RPS; ++k) {
        const int r = (warp + k * NW) * 32 + lane;
        if (r < L) {
          float x0[8];
          row8g(x + (uint64_t(e0.x) + r) * 8, sw, x0);
          const float v0 = __uint_as_float(e0.y);
#pragma unroll
          for (int u = 0; u < 8; ++u) acc[k][u] = fmaf(v0, x0[u], acc[k][u]);
        }
      }
    }
  }

  for (int i = 0; i < I; ++i) {
    const bool ok = bulk::mbar_wait(&full[i % S], (i / S) & 1);
    if (!__all_sync(0xffffffffu, ok && *abort_flag == 0)) {
      if (lane == 0) {
        *abort_flag = 1;
        atomicOr(err, 1);
      }
      break;
    }
    const unsigned char* st = ring + size_t(i % S) * slot;
    const uint32_t* hd = reinterpret_cast<const uint32_t*>(st);
    const uint32_t g0 = hd[0], g1 = hd[1];
    const uint32_t* ro = hd + 4;  // run offsets of the tile's slices
    const float* xs = reinterpret_cast<const float*>(st + kTiledSlotHead);
    const uint16_t* sc = reinterpret_cast<const uint16_t*>(st + kTiledSlotHead + xbytes) + lane;
    const float* sv = reinterpret_cast<const float*>(st + kTiledSlotHead + xbytes + cbytes) + lane;
#pragma unroll
    for (int k = 0; k < RPS; ++k) {
      const int s = warp + k * NW;
      if (s < slices) {
        const uint32_t lo = max(ro[s], g0), hi = min(ro[s + 1], g1);
        uint32_t j = lo;
        // two steps per pass, all shared loads issued before the FMAs; padding
        // (value 0, column 0) reads row 0 of the staged block and adds 0
        for (; j + 2 <= hi; j += 2) {
          const uint32_t q = (j - g0) * 32;
          const float v0 = sv[q], v1 = sv[q + 32];
          const uint32_t c0 = sc[q], c1 = sc[q + 32];
          float x0[8], x1[8];
          row8(xs + c0 * 8, sw, x0);
          row8(xs + c1 * 8, sw, x1);
#pragma unroll
          for (int u = 0; u < 8; ++u) acc[k][u] = fmaf(v1, x1[u], fmaf(v0, x0[u], acc[k][u]));
        }
        if (j < hi) {
          const uint32_t q = (j - g0) * 32;
          const float v0 = sv[q];
          float x0[8];
          row8(xs + uint32_t(sc[q]) * 8, sw, x0);
#pragma unroll
          for (int u = 0; u < 8; ++u) acc[k][u] = fmaf(v0, x0[u], acc[k][u]);
        }
      }
    }
    __syncwarp();
    if (lane == 0) bulk::mbar_arrive(&empty[i % S]);
  }
  __syncthreads();
  if (*abort_flag) return;
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

}  // namespace

size_t tiled_smem(const TiledOp& t, int stages) {
  return kTiledHeadBytes + size_t(stages) * (kTiledSlotHead + size_t(t.lmax) * 32 + size_t(t.gmax) * 192);
}

namespace {

template <int RPS>
void launch_tiled(const TiledOp& t, const TArgs& a, const float* x, float* y, int ldy, int m, int* err,
                  cudaStream_t s) {
  const size_t smem = tiled_smem(t, t.stages);
  const int nw = (t.smax + RPS - 1) / RPS;
  CG_CUDA(cudaFuncSetAttribute(k_tiled<RPS>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
  k_tiled<RPS><<<unsigned(t.nb), (nw + 1) * 32, smem, s>>>(a, x, y, ldy, m, err);
  CG_CUDA(cudaGetLastError());
  count_launch();
}

}  // namespace

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
  if (nruns) {
    k_tbalance<<<unsigned(std::min<uint64_t>((nruns * 4 + 255) / 256, 152ull * 64)), 256, 0, s>>>(
        nruns, t.roff.p, t.col.p, t.val.p);
    CG_CUDA(cudaGetLastError());
    count_launch();
    k_tpadaddr<<<unsigned(std::min<uint64_t>((nruns * 32 + 255) / 256, 152ull * 64)), 256, 0, s>>>(
        nruns, t.roff.p, t.col.p, t.val.p);
    CG_CUDA(cudaGetLastError());
    count_launch();
  }
  // scaled-identity tiles
  std::vector<uint32_t> tblock(ntiles);
  for (int b = 0; b < nb; ++b)
    for (uint32_t tt = tptr[b]; tt < tptr[b + 1]; ++tt) tblock[tt] = uint32_t(b);
  DBuf<uint32_t> dtblock, dident(std::max<uint64_t>(ntiles, 1));
  dtblock.upload(tblock, s);
  if (ntiles) {
    k_tident<<<unsigned(std::min<uint64_t>((ntiles * 32 + 255) / 256, 152ull * 64)), 256, 0, s>>>(
        ntiles, dtblock.p, t.bstart.p, t.tptr.p, t.runbase.p, t.roff.p, t.col.p, t.val.p, dident.p);
    CG_CUDA(cudaGetLastError());
    count_launch();
  }
  std::vector<uint32_t> ident(ntiles);
  if (ntiles) CG_CUDA(cudaMemcpyAsync(ident.data(), dident.p, ntiles * 4, cudaMemcpyDeviceToHost, s));
  CG_CUDA(cudaStreamSynchronize(s));
  // staged units: each tile's entry groups in chunks of at most gmax groups,
  // with a 16-byte aligned copy of the tile's run offsets
  t.gmax = std::max(8, t.lmax / 6);  // entry area ~ the x area of a slot
  std::vector<uint32_t> iptr(nb + 1), rcopy, dptr(nb + 1);
  std::vector<TItem> items;
  std::vector<uint2> iden;
  for (int b = 0; b < nb; ++b) {
    iptr[b] = uint32_t(items.size());
    dptr[b] = uint32_t(iden.size());
    const uint32_t sl = uint32_t((bs[b + 1] - bs[b] + 31) / 32);
    const uint32_t cpb = (sl + 1 + 3) / 4 * 16;  // bytes of one copy
    for (uint32_t tt = tptr[b]; tt < tptr[b + 1]; ++tt) {
      const uint32_t q = runbase[b] + (tt - tptr[b]) * sl;
      const uint32_t G0 = roff[q], G1 = roff[q + sl];
      if (ident[tt]) {  // read straight from x, nothing staged
        iden.push_back(make_uint2(uint32_t(bs[tcb[tt]]), ident[tt]));
        t.ident_tiles += 1;
        t.ident_nnz += bs[b + 1] - bs[b];
        continue;
      }
      const uint32_t rc = uint32_t(rcopy.size());
      for (uint32_t v = 0; v < cpb / 4; ++v) rcopy.push_back(v <= sl ? roff[q + v] : 0u);
      const uint32_t cb = tcb[tt];
      for (uint32_t g = G0; g < G1; g += uint32_t(t.gmax))
        items.push_back({uint32_t(bs[cb]), uint32_t(bs[cb + 1] - bs[cb]), g, std::min(G1, g + uint32_t(t.gmax)), rc,
                         cpb, 0, 0});
    }
    if (rcopy.size() >= (1ull << 32)) return;
  }
  iptr[nb] = uint32_t(items.size());
  dptr[nb] = uint32_t(iden.size());
  t.dptr.upload(dptr, s);
  t.iden.alloc(std::max<size_t>(iden.size(), 1) * sizeof(uint2));
  if (!iden.empty())
    CG_CUDA(cudaMemcpyAsync(t.iden.p, iden.data(), iden.size() * sizeof(uint2), cudaMemcpyHostToDevice, s));
  t.nitems = items.size();
  t.iptr.upload(iptr, s);
  t.rcopy.upload(rcopy, s);
  t.items.alloc(items.size() * sizeof(TItem));
  if (!items.empty())
    CG_CUDA(cudaMemcpyAsync(t.items.p, items.data(), items.size() * sizeof(TItem), cudaMemcpyHostToDevice, s));
  CG_CUDA(cudaStreamSynchronize(s));

  // default launch shape (spmm_autotune refines it): two slices per consumer
  // warp (one for blocks of at most 8 slices), two ring slots (on fp 4+4 this
  // keeps three CTAs per SM, the fastest of 1..3 slices x 2..4 slots)
  t.rps = t.smax <= 8 ? 1 : (t.smax <= 62 ? 2 : 3);
  t.warps = (t.smax + t.rps - 1) / t.rps;
  t.stages = 2;
  t.err.alloc(1);
  h.tiled = tp;
}

void tiled_product(const Hamiltonian& h, const float* x, float* y, int ldy, int m, cudaStream_t s) {
  const TiledOp& t = *h.tiled;
  if (m < 1 || m > 8) throw Error(CG_ERR_ARG, "tiled product takes 1..8 vectors");
  if (reinterpret_cast<uintptr_t>(x) % 16) throw Error(CG_ERR_ARG, "tiled product needs a 16-byte aligned x");
  if (t.stages < 2 || 2 * t.stages * 8 + 4 > kTiledHead || tiled_smem(t, t.stages) > 227 * 1024)
    throw Error(CG_ERR_ARG, "tiled product: ring slots out of range");
  TArgs a{t.bstart.p, t.order.p, t.iptr.p, reinterpret_cast<const TItem*>(t.items.p), t.rcopy.p, t.col.p, t.val.p,
          t.dptr.p, reinterpret_cast<const uint2*>(t.iden.p), t.lmax, t.gmax, t.stages};
  CG_CUDA(cudaMemsetAsync(t.err.p, 0, sizeof(int), s));
  if (t.warps != (t.smax + t.rps - 1) / t.rps || t.warps > 31) throw Error(CG_ERR_ARG, "tiled product: bad launch shape");
  switch (t.rps) {
    case 1: launch_tiled<1>(t, a, x, y, ldy, m, t.err.p, s); break;
    case 2: launch_tiled<2>(t, a, x, y, ldy, m, t.err.p, s); break;
    case 3: launch_tiled<3>(t, a, x, y, ldy, m, t.err.p, s); break;
    case 4: launch_tiled<4>(t, a, x, y, ldy, m, t.err.p, s); break;
    default: throw Error(CG_ERR_ARG, "tiled product: slices per warp must be 1..4");
  }
  int herr = 0;
  CG_CUDA(cudaMemcpyAsync(&herr, t.err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  CG_CUDA(cudaStreamSynchronize(s));
  if (herr) throw Error(CG_ERR_TIMEOUT, "tiled product: a staged copy or a slot release did not complete");
}

}  // namespace cg
