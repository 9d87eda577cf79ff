// On-the-fly H + lambda * J-J+ product (the element kinds and their tables are
// described in virtual.h).
//
// Host: transition tables of every neutron block and proton configuration,
// built from the same forward-ordered operator terms and the same fermion
// phase rule as the stored builder (SM::ActFermiOperator,
// include/sm/cioperators.cxx:36-62; SM::Annihilation / SM::Creation,
// include/sm/operators.cxx:121-187).
//
// Device: one CTA per neutron block beta (rows start(beta) .. + L), each thread
// owning up to RPT rows and VB vectors of each row in registers.  The own
// block's terms (diagonal, PP2, P1) read x through L1 (the block is reused by
// every row of the CTA); NN2 reads x[nu', pi] for consecutive pi, coalesced
// across the CTA; for every neutron one-body transition beta -> beta' the
// whole block x[beta'] (contiguous, L' rows) is brought into shared memory by
// one bulk TMA copy (cp.async.bulk, completion on an mbarrier, two buffers so
// the next block streams in while this one is used) together with the
// W[a][c][.][.] slice, and each row walks its proton transitions of the
// balancing 2m change, gathering from shared memory.
#include <algorithm>
#include <chrono>
#include <functional>
#include <map>
#include <numeric>
#include <unordered_map>

#include "bulk.h"
#include "dfloat.h"
#include "tiled.h"
#include "virtual.h"

namespace cg {

namespace {

constexpr double kDropV = 1e-14;
constexpr int kVirtualSmemHead = 128;  // three mbarriers; keeps the staging buffers 128-byte aligned

inline int popc(uint64_t x) { return __builtin_popcountll(x); }
inline uint64_t below_h(int b) { return b >= 64 ? ~0ull : (1ull << b) - 1ull; }
// global occupation words (neutron s.p. states from bit 0, protons above) of
// up to 128 s.p. states, host only
using G = unsigned __int128;
inline int popg(G x) { return __builtin_popcountll(uint64_t(x)) + __builtin_popcountll(uint64_t(x >> 64)); }
inline G below_g(int b) { return b >= 128 ? ~G(0) : ((G(1) << b) - 1); }
inline G gbit(int b) { return G(1) << b; }
inline int ctzg(G x) {
  const uint64_t lo = uint64_t(x);
  return lo ? __builtin_ctzll(lo) : 64 + __builtin_ctzll(uint64_t(x >> 64));
}

struct HostOp {
  int ns = 0, np_pairs = 0;
  std::vector<double> e1;      // ns x ns
  std::vector<double> v2;      // npairs x npairs
  std::vector<int32_t> pidx;   // ns x ns
  double V(int a, int b, int c, int d) const {  // a < b, c < d
    return v2[size_t(pidx[a * ns + b]) * np_pairs + pidx[c * ns + d]];
  }
  // forward two-body term (b0 < b1 annihilated, b2 < b3 created) on S0
  double term2(G S0, int b0, int b1, int b2, int b3) const {
    double v = V(b0, b1, b2, b3);
    int p = popg(S0 & below_g(b0)) + popg(S0 & below_g(b1)) - 1;
    G I = S0 & ~(gbit(b0) | gbit(b1));
    p += popg(I & below_g(b2)) + popg(I & below_g(b3));
    return (p & 1) ? -v : v;
  }
  double term1(G S0, int x, int y) const {
    double v = e1[x * ns + y];
    int p = popg(S0 & below_g(x)) + popg((S0 & ~gbit(x)) & below_g(y));
    return (p & 1) ? -v : v;
  }
};

HostOp host_operator(const System& sys, const Operator& op) {
  HostOp h;
  const int ns = int(sys.sps.size());
  h.ns = ns;
  h.pidx.assign(ns * ns, -1);
  int np = 0;
  for (int a = 0; a < ns; ++a)
    for (int b = a + 1; b < ns; ++b) h.pidx[a * ns + b] = np++;
  h.np_pairs = np;
  h.e1.assign(ns * ns, 0.0);
  for (auto& kv : op.one) h.e1[kv.first[0] * ns + kv.first[1]] = kv.second;
  h.v2.assign(size_t(std::max(np, 1)) * std::max(np, 1), 0.0);
  for (auto& kv : op.two) {
    const Key4& k = kv.first;
    if (k[0] >= k[1] || k[2] >= k[3]) continue;  // cannot act on a determinant
    h.v2[size_t(h.pidx[k[0] * ns + k[1]]) * np + h.pidx[k[2] * ns + k[3]]] = kv.second;
  }
  return h;
}

// one-body move x -> y inside a species mask: phase parity of the other
// occupied orbitals strictly between (the same from either end)
inline int move_sign(uint64_t mask, int from, int to) {
  uint64_t o = mask & ~(1ull << from);
  return (popc(o & below_h(from)) + popc(o & below_h(to))) & 1;
}

// ------------------------------------------------------------------ device
struct VArgs {
  int nn, np, ndm, dm0, lmax;
  const uint64_t* bstart;
  const uint32_t *blen, *bclass, *order;
  const void *bmask, *cmask;  // species masks: uint32_t, or uint64_t for a wide basis
  const uint32_t* cstart;
  const uint32_t* nt_off;
  const NTrans* nt;
  const uint32_t* nn_off;
  const VPair* nn2;
  const uint32_t* cslice;  // first 32-row slice of each proton class
  const uint32_t* sl_off;  // per (slice, slot): first proton-transition entry (32 lanes x count)
  const uint32_t* sl_e;    // rank | (b * np + d) << 16 | sign << 27
  const uint32_t* pp_off;  // per slice: first PP2 entry (32 lanes x count)
  const uint32_t* pp_rank;
  const double* diag;
  // truncated basis: class rank of each list member, and per list a map
  // class rank -> list rank (0xffff: outside the basis), rmax entries at most
  const uint32_t* gcr;
  const uint16_t* lmap;
  const uint32_t *lmap_off, *lmap_len;
  int rmax;
};

template <class T>
struct VTab {
  const T *W, *Un, *Up;
  const T* sl_c;  // P1 value without neutron spectators, parallel to sl_e
  const T* pp_h;  // PP2 values, parallel to pp_rank
};

__device__ __forceinline__ int lowbit(uint32_t w) { return __ffs(w) - 1; }
__device__ __forceinline__ int lowbit(unsigned long long w) { return __ffsll((long long)w) - 1; }

using bulk::bulk_load;
using bulk::fence_mbar_init;
using bulk::mbar_init;
using bulk::mbar_wait;

// One row of VB vectors (32 bytes) read as two 16-byte halves.  Odd lanes
// read the second half first and keep the halves swapped in registers (and in
// their accumulators; the store undoes it): a warp's first load then spreads
// over all eight 16-byte bank groups instead of the four even ones, which cuts
// the shared-memory wavefronts of 32 random rows from ~11 to ~6.7 per load.
template <class T, int VB>
struct Row;
template <>
struct Row<float, 8> {
  float v[8];
  __device__ __forceinline__ void load_g(const float* p, int sw) {
    float4 a = __ldg(reinterpret_cast<const float4*>(p) + sw), b = __ldg(reinterpret_cast<const float4*>(p) + (sw ^ 1));
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
  }
  __device__ __forceinline__ void load_s(const float* p, int sw) {
    float4 a = reinterpret_cast<const float4*>(p)[sw], b = reinterpret_cast<const float4*>(p)[sw ^ 1];
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
  }
};
template <>
struct Row<double, 4> {
  double v[4];
  __device__ __forceinline__ void load_g(const double* p, int sw) {
    double2 a = __ldg(reinterpret_cast<const double2*>(p) + sw), b = __ldg(reinterpret_cast<const double2*>(p) + (sw ^ 1));
    v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
  }
  __device__ __forceinline__ void load_s(const double* p, int sw) {
    double2 a = reinterpret_cast<const double2*>(p)[sw], b = reinterpret_cast<const double2*>(p)[sw ^ 1];
    v[0] = a.x; v[1] = a.y; v[2] = b.x; v[3] = b.y;
  }
};

// Element values: T for the FP32 / FP64 products, an FP32 (hi, lo) pair for
// the double-float one (FP64-accurate to ~2^-44 on the FP32 pipe).
struct DF2 {
  float h, l;
};
template <class T, bool DF>
struct VT {
  using type = T;
};
template <class T>
struct VT<T, true> {
  using type = DF2;
};
__device__ __forceinline__ float vneg(float v) { return -v; }
__device__ __forceinline__ double vneg(double v) { return -v; }
__device__ __forceinline__ DF2 vneg(DF2 v) { return {-v.h, -v.l}; }
__device__ __forceinline__ float vadd(float a, float b) { return a + b; }
__device__ __forceinline__ double vadd(double a, double b) { return a + b; }
__device__ __forceinline__ DF2 vadd(DF2 a, DF2 b) {
  DF2 r;
  df_add(r.h, r.l, a.h, a.l, b.h, b.l);
  return r;
}
template <class V>
__device__ __forceinline__ V vfrom(double d);
template <>
__device__ __forceinline__ float vfrom<float>(double d) { return float(d); }
template <>
__device__ __forceinline__ double vfrom<double>(double d) { return d; }
template <>
__device__ __forceinline__ DF2 vfrom<DF2>(double d) {
  DF2 r;
  df_split(d, r.h, r.l);
  return r;
}
// table value i: the T table, or its (hi, lo) pair
template <class V, class T>
__device__ __forceinline__ V vtab(const T* hi, const T* lo, size_t i) {
  if constexpr (sizeof(V) == 2 * sizeof(float) && sizeof(T) == sizeof(float)) return V{hi[i], lo[i]};
  else return V(hi[i]);
}
// acc += v * row: VB values of T, or VB / 2 double-float pairs (hi at even,
// lo at odd positions of the row and of the accumulators)
template <class T, int VB>
__device__ __forceinline__ void vmac(T (&acc)[VB], T v, const T (&x)[VB]) {
#pragma unroll
  for (int j = 0; j < VB; ++j) acc[j] += v * x[j];
}
template <class T, int VB>
__device__ __forceinline__ void vmac(T (&acc)[VB], DF2 v, const T (&x)[VB]) {
#pragma unroll
  for (int u = 0; u < VB / 2; ++u) df_mac(acc[2 * u], acc[2 * u + 1], x[2 * u], x[2 * u + 1], v.h, v.l);
}

// DF = false: Y = H X in T (FP32 8 vectors or FP64 4 vectors per pass).
// DF = true (T = float): X as 4 vectors of (hi, lo) FP32 pairs in the 8-float
// rows, table values as (hi, lo) pairs (tl holds the low parts), products and
// sums in double-float, Y written as FP64: the refinement product on the FP32
// pipe instead of the FP64 one.
// TR = true: a truncated basis, whose block rows are a list (the allowed
// proton configurations of the block's class).  The proton-transition tables
// then hold class ranks of the target configuration; the class-to-list map
// of every staged block comes into shared memory with its x rows, and a
// target outside the basis is skipped.  NN2 reads the target's map from global
// memory.  M: the species-mask type (uint64_t for a wide basis, which always
// takes the TR form).  ST = false (blocks whose staging does not fit in
// shared memory): the own block, the target blocks and their class-to-list
// maps are read from global memory (L2) instead of being staged.
template <class T, int VB, int RPT, bool DF, bool TR, class M, bool ST>
__global__ void __launch_bounds__(RPT <= 2 ? 1024 : 512) k_virtual(VArgs a, VTab<T> tb, VTab<T> tl,
                                                                   const T* __restrict__ x, void* __restrict__ yv,
                                                                   int ldy, int m, int* __restrict__ err) {
  using V = typename VT<T, DF>::type;
  // shared memory: [3 mbarriers | pad to 128 B] own buf0 buf1 (lmax x VB each of T)
  //                wsl0 wsl1 (np*np + 4, last = 0) un0 un1 (32) Pp (np*np + 1, last = 0), of V
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int npp = a.np * a.np, nw = npp + 4;
  uint64_t* mbar = reinterpret_cast<uint64_t*>(smem_raw);
  const size_t stg = ST ? size_t(a.lmax) * VB : 0;
  T* own = reinterpret_cast<T*>(smem_raw + kVirtualSmemHead);
  T* buf0 = own + stg;
  T* buf1 = buf0 + stg;
  V* wsl0 = reinterpret_cast<V*>(buf1 + stg);
  V* wsl1 = wsl0 + nw;
  V* un0 = wsl1 + nw;
  V* un1 = un0 + a.np;
  V* Pp = un1 + a.np;
  // TR: class-to-list maps of the own block and the two staged blocks, from the
  // first 16-byte boundary after Pp
  uint16_t* rown = reinterpret_cast<uint16_t*>((reinterpret_cast<uintptr_t>(Pp + npp + 1) + 15) & ~uintptr_t(15));
  uint16_t* rbuf0 = rown + a.rmax;
  uint16_t* rbuf1 = rbuf0 + a.rmax;

  // half-swapped row reads (Row) for up to 2 rows per thread: fp 4+4 (2 rows)
  // 4.46 -> 4.04 ms; with 4 rows per thread (fp 5+5) they measured slower
  // (75.9 -> 83.2 ms), so those launches read halves in order
  const int tid = threadIdx.x, NT = blockDim.x, lane = tid & 31, sw = RPT <= 2 ? (lane & 1) : 0;
  const uint32_t beta = a.order[blockIdx.x];
  const uint64_t start = a.bstart[beta];
  const int L = int(a.blen[beta]);
  const uint32_t cls = a.bclass[beta];
  const uint32_t cs = a.cstart[cls], slice0 = a.cslice[cls];
  const M nmask = static_cast<const M*>(a.bmask)[beta];
  const M* cmask = static_cast<const M*>(a.cmask);
  const uint32_t t0 = a.nt_off[beta], t1 = a.nt_off[beta + 1];

  if (tid == 0) {
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    mbar_init(&mbar[2], 1);
    fence_mbar_init();
  }
  // P1 neutron-spectator sums of this block: Pp[b*np+d] = sum_{q in nu} Up[b][d][q]
  for (int i = tid; i <= npp; i += NT) {
    V s = vfrom<V>(0.0);
    if (i < npp)
      for (M w = nmask; w; w &= w - 1) s = vadd(s, vtab<V>(tb.Up, tl.Up, size_t(i) * a.nn + lowbit(w)));
    Pp[i] = s;
  }
  if (tid == 0) {
    wsl0[npp] = vfrom<V>(0.0);
    wsl1[npp] = vfrom<V>(0.0);
  }
  __syncthreads();
  // one elected thread: the x rows of block blk (and, TR, its class-to-list map) onto one barrier
  auto stage = [&](T* dst, uint16_t* rdst, uint32_t blk, uint64_t* bar) {
    const uint32_t xb = a.blen[blk] * uint32_t(VB * sizeof(T));
    if constexpr (TR) {
      const uint32_t lc = a.bclass[blk], rb = a.lmap_len[lc] * 2u;
      bulk::expect_tx(bar, xb + rb);
      bulk::copy(dst, x + a.bstart[blk] * VB, xb, bar);
      bulk::copy(rdst, a.lmap + a.lmap_off[lc], rb, bar);
    } else {
      bulk_load(dst, x + a.bstart[blk] * VB, xb, bar);
    }
  };
  if (ST && tid == 0) {
    stage(own, rown, beta, &mbar[2]);
    if (t0 < t1) stage(buf0, rbuf0, a.nt[t0].target, &mbar[0]);
  }
  // where the own block's rows and map are read from
  const T* ownx = ST ? own : x + start * VB;
  auto ldrow = [&](Row<T, VB>& xr, const T* p) {
    if constexpr (ST) xr.load_s(p, sw);
    else xr.load_g(p, sw);
  };
  const uint16_t* rownp = ST ? rown : (TR ? a.lmap + a.lmap_off[cls] : nullptr);
  // TR: class rank of each own row's proton configuration
  uint32_t gr[RPT];
#pragma unroll
  for (int k = 0; k < RPT; ++k) {
    const int r = tid + k * NT;
    gr[k] = (TR && r < L) ? a.gcr[cs + r] : 0u;
  }

  T acc[RPT][VB];
#pragma unroll
  for (int k = 0; k < RPT; ++k)
#pragma unroll
    for (int j = 0; j < VB; ++j) acc[k][j] = 0;

  // NN2 first (global x, consecutive rows of the target block), while the own block streams in
  for (uint32_t e = a.nn_off[beta], e1 = a.nn_off[beta + 1]; e < e1; ++e) {
    const VPair q = a.nn2[e];
    const uint64_t ts = a.bstart[q.target];
    const V h = vfrom<V>(q.h);
#pragma unroll
    for (int k = 0; k < RPT; ++k) {
      const int r = tid + k * NT;
      if (r < L) {
        Row<T, VB> xr;
        if constexpr (TR) {  // the same proton configuration in the target's list (q.pad: its map)
          const uint32_t rr = __ldg(a.lmap + q.pad + gr[k]);
          if (rr != 0xffffu) {
            xr.load_g(x + (ts + rr) * VB, sw);
            vmac(acc[k], h, xr.v);
          }
        } else {
          xr.load_g(x + (ts + r) * VB, sw);
          vmac(acc[k], h, xr.v);
        }
      }
    }
  }
  if constexpr (ST) {
    const bool ok = mbar_wait(&mbar[2], 0);
    if (__syncthreads_or(!ok)) {
      if (tid == 0) {
        atomicOr(err, 1);
        mbar_wait(&mbar[2], 0);
        if (t0 < t1) mbar_wait(&mbar[0], 0);
      }
      __syncthreads();
      return;
    }
  }
  // diagonal, PP2 and P1 from the own block.  Rows come in 32-row slices
  // (warp-uniform), whose transition lists are stored lane-interleaved.
#pragma unroll
  for (int k = 0; k < RPT; ++k) {
    const int rb = (tid & ~31) + k * NT;  // first row of this warp's slice
    if (rb < L) {
      const int r = rb + lane;
      const uint32_t sl = slice0 + uint32_t(rb >> 5);
      Row<T, VB> xr;
      if (r < L) {
        ldrow(xr, ownx + size_t(r) * VB);
        vmac(acc[k], vfrom<V>(a.diag[start + r]), xr.v);
      }
      for (uint32_t e = a.pp_off[sl] + lane, e1 = a.pp_off[sl + 1]; e < e1; e += 32) {
        const V h = vtab<V>(tb.pp_h, tl.pp_h, e);
        ldrow(xr, ownx + size_t(a.pp_rank[e]) * VB);
        vmac(acc[k], h, xr.v);
      }
      const size_t o = size_t(sl) * a.ndm + a.dm0;
      for (uint32_t e = a.sl_off[o] + lane, e1 = a.sl_off[o + 1]; e < e1; e += 32) {
        const uint32_t q = a.sl_e[e];
        V v = Pp[(q >> 16) & 0x7ff];
        v = vadd(vtab<V>(tb.sl_c, tl.sl_c, e), ((q >> 27) & 1) ? vneg(v) : v);
        if constexpr (TR) {
          const uint32_t rr = rownp[q & 0xffff];
          if (rr != 0xffffu) {
            ldrow(xr, ownx + size_t(rr) * VB);
            vmac(acc[k], v, xr.v);
          }
        } else {
          ldrow(xr, ownx + size_t(q & 0xffff) * VB);
          vmac(acc[k], v, xr.v);
        }
      }
    }
  }
  // neutron one-body transitions: N1 (same 2m) and NP
  uint32_t u = 0;
  for (uint32_t t = t0; t < t1; ++t, ++u) {
    const int jb = u & 1;
    const NTrans tr = a.nt[t];
    V* wsl = jb ? wsl1 : wsl0;
    V* un = jb ? un1 : un0;
    const size_t wrow = (size_t(tr.a) * a.nn + tr.c) * npp;
    for (int i = tid; i < npp; i += NT) {
      const V w = vtab<V>(tb.W, tl.W, wrow + i);
      wsl[i] = tr.sign ? vneg(w) : w;
    }
    const bool same_m = tr.dmi == a.dm0;
    if (same_m && tid < a.np) {
      const V w = vtab<V>(tb.Un, tl.Un, (size_t(tr.a) * a.nn + tr.c) * a.np + tid);
      un[tid] = tr.sign ? vneg(w) : w;
    }
    __syncthreads();
    if constexpr (ST) {
      if (tid == 0 && t + 1 < t1) stage(jb ? buf0 : buf1, jb ? rbuf0 : rbuf1, a.nt[t + 1].target, &mbar[jb ^ 1]);
      const bool ok = mbar_wait(&mbar[jb], (u >> 1) & 1);
      if (__syncthreads_or(!ok)) {
        // give the copies in flight a second bounded wait, report, leave
        if (tid == 0) {
          atomicOr(err, 1);
          mbar_wait(&mbar[jb], (u >> 1) & 1);
          if (t + 1 < t1) mbar_wait(&mbar[jb ^ 1], ((u + 1) >> 1) & 1);
        }
        __syncthreads();
        return;
      }
    }
    const T* bf = ST ? (jb ? buf1 : buf0) : x + a.bstart[tr.target] * VB;
    const uint16_t* rbf = ST ? (jb ? rbuf1 : rbuf0) : (TR ? a.lmap + a.lmap_off[a.bclass[tr.target]] : nullptr);
    const int dmp = a.ndm - 2 - (tr.dmi & ~1) + (tr.dmi & 1);  // opposite 2m change, same parity change
    const V cn = vfrom<V>(tr.cn);
#pragma unroll
    for (int k = 0; k < RPT; ++k) {
      const int rb = (tid & ~31) + k * NT;
      if (rb < L) {
        const int r = rb + lane;
        const uint32_t sl = slice0 + uint32_t(rb >> 5);
        const size_t o = size_t(sl) * a.ndm + dmp;
        for (uint32_t e = a.sl_off[o] + lane, e1 = a.sl_off[o + 1]; e < e1; e += 32) {
          const uint32_t q = a.sl_e[e];
          V w = wsl[(q >> 16) & 0x7ff];
          w = ((q >> 27) & 1) ? vneg(w) : w;
          Row<T, VB> xr;
          if constexpr (TR) {
            const uint32_t rr = rbf[q & 0xffff];
            if (rr != 0xffffu) {
              ldrow(xr, bf + size_t(rr) * VB);
              vmac(acc[k], w, xr.v);
            }
          } else {
            ldrow(xr, bf + size_t(q & 0xffff) * VB);
            vmac(acc[k], w, xr.v);
          }
        }
        // N1: the same proton configuration in the target block (TR: its rank in the target's list)
        if (same_m && r < L) {
          const uint32_t rn = TR ? uint32_t(rbf[gr[k]]) : uint32_t(r);
          if (rn != 0xffffu) {
            V v = cn;
            for (M w = cmask[cs + r]; w; w &= w - 1) v = vadd(v, un[lowbit(w)]);
            Row<T, VB> xr;
            ldrow(xr, bf + size_t(rn) * VB);
            vmac(acc[k], v, xr.v);
          }
        }
      }
    }
  }
#pragma unroll
  for (int k = 0; k < RPT; ++k) {
    const int r = tid + k * NT;
    if (r < L) {
      if constexpr (DF) {
        // register pair u holds vector u, or u ^ (VB / 4) with the halves swapped
        double* yr = static_cast<double*>(yv) + (start + r) * size_t(ldy);
#pragma unroll
        for (int u = 0; u < VB / 2; ++u) {
          const int jj = sw ? (u ^ (VB / 4)) : u;
          if (jj < m) yr[jj] = double(acc[k][2 * u]) + double(acc[k][2 * u + 1]);
        }
      } else {
        T* yr = static_cast<T*>(yv) + (start + r) * size_t(ldy);
#pragma unroll
        for (int j = 0; j < VB; ++j) {
          const int jj = sw ? (j ^ (VB / 2)) : j;
          if (jj < m) yr[jj] = acc[k][j];
        }
      }
    }
  }
}

// diagonal of every row: En(block) + Ep(proton configuration) + pn part
template <class M>
__global__ void k_virtual_diag(uint64_t n, int nblocks, const uint64_t* __restrict__ bstart,
                               const uint32_t* __restrict__ bclass, const M* __restrict__ bmask,
                               const uint32_t* __restrict__ cstart, const M* __restrict__ cmask,
                               const double* __restrict__ En, const double* __restrict__ Ep,
                               const double* __restrict__ Vd, int np, double* __restrict__ diag) {
  uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  int lo = 0, hi = nblocks - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (bstart[mid] <= i) lo = mid; else hi = mid - 1;
  }
  const uint32_t g = cstart[bclass[lo]] + uint32_t(i - bstart[lo]);
  double d = En[lo] + Ep[g];
  const M pm = cmask[g];
  for (M w = bmask[lo]; w; w &= w - 1) {
    const int an = lowbit(w);
    for (M z = pm; z; z &= z - 1) d += Vd[an * np + lowbit(z)];
  }
  diag[i] = d;
}

template <class T, int VB, int RPT, bool DF, bool TR, class M, bool ST>
void launch_rpt(const Hamiltonian& h, const VArgs& a, const VTab<T>& tb, const VTab<T>& tl, const T* x, void* y,
                int ldy, int m, int threads, size_t smem, int* err, cudaStream_t s) {
  auto kern = k_virtual<T, VB, RPT, DF, TR, M, ST>;
  CG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
  kern<<<unsigned(a.lmax ? h.virt->nblocks : 0), threads, smem, s>>>(a, tb, tl, x, y, ldy, m, err);
  CG_CUDA(cudaGetLastError());
  count_launch();
}

VArgs make_args(const VirtualOp& v, const Hamiltonian& h) {
  VArgs a;
  a.nn = v.nn; a.np = v.np; a.ndm = v.ndm; a.dm0 = v.dm0; a.lmax = v.lmax;
  a.bstart = v.bstart.p; a.blen = v.blen.p; a.bclass = v.bclass.p; a.order = v.order.p;
  a.bmask = v.wide ? static_cast<const void*>(v.bmask64.p) : static_cast<const void*>(v.bmask.p);
  a.cmask = v.wide ? static_cast<const void*>(v.cmask64.p) : static_cast<const void*>(v.cmask.p);
  a.cstart = v.cstart.p;
  a.nt_off = v.nt_off.p; a.nt = v.nt.p; a.nn_off = v.nn_off.p; a.nn2 = v.nn2.p;
  a.cslice = v.cslice.p; a.sl_off = v.sl_off.p; a.sl_e = v.sl_e.p; a.pp_off = v.pp_off.p; a.pp_rank = v.pp_rank.p;
  a.diag = h.diag.p;
  a.gcr = v.gcr.p;
  a.lmap = v.lmap.p;
  a.lmap_off = v.lmap_off.p;
  a.lmap_len = v.lmap_len.p;
  a.rmax = v.rmax;
  return a;
}

// DF: x holds VB / 2 vectors as (hi, lo) pairs, y is FP64 (VB / 2 columns)
template <class T, int VB, bool DF = false>
void virtual_product(const Hamiltonian& h, const T* x, void* y, int ldy, int m, const VTab<T>& tb,
                     const VTab<T>& tl, cudaStream_t s) {
  if (!h.virt) throw Error(CG_ERR_INTERNAL, "not an on-the-fly Hamiltonian");
  const VirtualOp& v = *h.virt;
  if (m < 1 || m > (DF ? VB / 2 : VB)) throw Error(CG_ERR_ARG, "on-the-fly product: too many vectors for one pass");
  if (ldy < m) throw Error(CG_ERR_ARG, "leading dimension smaller than the vector count");
  if (reinterpret_cast<uintptr_t>(x) % 16) throw Error(CG_ERR_ARG, "on-the-fly product needs 16-byte aligned x");
  if (v.nblocks == 0) return;
  VArgs a = make_args(v, h);
  const int npp = v.np * v.np;
  const size_t vsz = DF ? 2 * sizeof(float) : sizeof(T);  // bytes of one element value
  // staged: own block, two target blocks (and, with lists, their maps) in
  // shared memory; blocks too long for that read x and the maps through L2
  const size_t tabs = (3 * size_t(npp + 4) + 2 * size_t(v.np)) * vsz;
  const size_t smem_staged = kVirtualSmemHead + size_t(3) * v.lmax * VB * sizeof(T) + tabs +
                             (v.truncated ? 16 + size_t(3) * v.rmax * sizeof(uint16_t) : 0);
  const bool staged = smem_staged <= 227 * 1024;
  const size_t smem = staged ? smem_staged : kVirtualSmemHead + tabs + 16;
  if (smem > 227 * 1024) throw Error(CG_ERR_UNSUPPORTED, "interaction slices too large for shared memory");
  // rows per thread: threads <= 512, or <= 1024 when the staging buffers
  // leave room for one CTA per SM only (long blocks, e.g. fp 5+5): there two
  // rows per thread and twice the warps hide the shared-memory latency better
  // than four rows per thread
  const int thread_cap = (staged && smem > 113 * 1024) ? 1024 : 512;
  int rpt = 1;
  while ((v.lmax + rpt - 1) / rpt > thread_cap) rpt <<= 1;
  int threads = (v.lmax + rpt - 1) / rpt;
  threads = std::max(64, (threads + 31) / 32 * 32);
  if (rpt > 8) throw Error(CG_ERR_UNSUPPORTED, "neutron block longer than 4096 rows");
  DBuf<int>& err = v.err;
  CG_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), s));
#define CG_VIRTUAL_RPT(TRV, MV, STV)                                                                         \
  switch (rpt) {                                                                                             \
    case 1: launch_rpt<T, VB, 1, DF, TRV, MV, STV>(h, a, tb, tl, x, y, ldy, m, threads, smem, err.p, s); break; \
    case 2: launch_rpt<T, VB, 2, DF, TRV, MV, STV>(h, a, tb, tl, x, y, ldy, m, threads, smem, err.p, s); break; \
    case 4: launch_rpt<T, VB, 4, DF, TRV, MV, STV>(h, a, tb, tl, x, y, ldy, m, threads, smem, err.p, s); break; \
    default: launch_rpt<T, VB, 8, DF, TRV, MV, STV>(h, a, tb, tl, x, y, ldy, m, threads, smem, err.p, s); break; \
  }
#define CG_VIRTUAL_ST(TRV, MV)    \
  if (staged) {                   \
    CG_VIRTUAL_RPT(TRV, MV, true)  \
  } else {                        \
    CG_VIRTUAL_RPT(TRV, MV, false) \
  }
  if (v.wide) {
    CG_VIRTUAL_ST(true, unsigned long long)
  } else if (v.truncated) {
    CG_VIRTUAL_ST(true, uint32_t)
  } else {
    CG_VIRTUAL_ST(false, uint32_t)
  }
#undef CG_VIRTUAL_ST
#undef CG_VIRTUAL_RPT
  int herr = 0;
  CG_CUDA(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  CG_CUDA(cudaStreamSynchronize(s));
  if (herr) throw Error(CG_ERR_TIMEOUT, "on-the-fly product: a staged copy did not complete");
}

// W (n x VB packed) = columns c0 .. c0+m of x (row-interleaved, ld), zero-padded
template <class T, int VB>
__global__ void k_pack(uint64_t n, const T* __restrict__ x, int ld, int c0, int m, T* __restrict__ w) {
  uint64_t idx = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (idx >= n * VB) return;
  uint64_t i = idx / VB;
  int j = int(idx - i * VB);
  w[idx] = j < m ? x[i * ld + c0 + j] : T(0);
}

template <class T, int VB>
void pack(uint64_t n, const T* x, int ld, int c0, int m, T* w, cudaStream_t s) {
  if (!n) return;
  k_pack<T, VB><<<unsigned((n * VB + 255) / 256), 256, 0, s>>>(n, x, ld, c0, m, w);
  CG_CUDA(cudaGetLastError());
  count_launch();
}

}  // namespace

void virtual_pack_f32(uint64_t n, const float* x, int ld, int c0, int m, float* w, cudaStream_t s) {
  pack<float, kVirtualVB32>(n, x, ld, c0, m, w, s);
}
void virtual_pack_f64(uint64_t n, const double* x, int ld, int c0, int m, double* w, cudaStream_t s) {
  pack<double, kVirtualVB64>(n, x, ld, c0, m, w, s);
}

void virtual_launch(const Hamiltonian& h, int precision, const void* x, int ldx, void* y, int ldy, int m,
                    cudaStream_t s) {
  if (m < 1) throw Error(CG_ERR_ARG, "m must be >= 1");
  if (ldx < m || ldy < m) throw Error(CG_ERR_ARG, "leading dimension smaller than the vector count");
  const uint64_t n = h.n;
  if (precision == CG_PREC_FP32) {
    DBuf<float> w(std::max<uint64_t>(n * kVirtualVB32, 1));
    for (int c0 = 0; c0 < m; c0 += kVirtualVB32) {
      const int mc = std::min(kVirtualVB32, m - c0);
      virtual_pack_f32(n, static_cast<const float*>(x), ldx, c0, mc, w.p, s);
      virtual_product_f32(h, w.p, static_cast<float*>(y) + c0, ldy, mc, s);
    }
  } else if (precision == CG_PREC_REFINE) {
    DBuf<float> w(std::max<uint64_t>(n * 8, 1));
    for (int c0 = 0; c0 < m; c0 += 4) {
      const int mc = std::min(4, m - c0);
      virtual_pack_df(n, static_cast<const double*>(x), ldx, c0, mc, w.p, s);
      virtual_product_df(h, w.p, static_cast<double*>(y) + c0, ldy, mc, s);
    }
  } else if (precision == CG_PREC_FP64) {
    DBuf<double> w(std::max<uint64_t>(n * kVirtualVB64, 1));
    for (int c0 = 0; c0 < m; c0 += kVirtualVB64) {
      const int mc = std::min(kVirtualVB64, m - c0);
      virtual_pack_f64(n, static_cast<const double*>(x), ldx, c0, mc, w.p, s);
      virtual_product_f64(h, w.p, static_cast<double*>(y) + c0, ldy, mc, s);
    }
  } else {
    throw Error(CG_ERR_ARG, "unknown precision");
  }
}

void virtual_product_f32(const Hamiltonian& h, const float* x, float* y, int ldy, int m, cudaStream_t s) {
  VTab<float> tb{h.virt->Wf.p, h.virt->Unf.p, h.virt->Upf.p, h.virt->sl_cf.p, h.virt->pp_hf.p};
  virtual_product<float, kVirtualVB32>(h, x, y, ldy, m, tb, tb, s);
}

void virtual_product_f64(const Hamiltonian& h, const double* x, double* y, int ldy, int m, cudaStream_t s) {
  VTab<double> tb{h.virt->W.p, h.virt->Un.p, h.virt->Up.p, h.virt->sl_c.p, h.virt->pp_h.p};
  virtual_product<double, kVirtualVB64>(h, x, y, ldy, m, tb, tb, s);
}

// x: 4 vectors as (hi, lo) FP32 pairs per row (virtual_pack_df), y FP64
void virtual_product_df(const Hamiltonian& h, const float* x, double* y, int ldy, int m, cudaStream_t s) {
  VTab<float> tb{h.virt->Wf.p, h.virt->Unf.p, h.virt->Upf.p, h.virt->sl_cf.p, h.virt->pp_hf.p};
  VTab<float> tl{h.virt->Wl.p, h.virt->Unl.p, h.virt->Upl.p, h.virt->sl_cl.p, h.virt->pp_hl.p};
  virtual_product<float, kVirtualVB32, true>(h, x, y, ldy, m, tb, tl, s);
}

namespace {
// 8 floats per row = 4 vectors as (hi, lo) pairs, columns c0 .. c0+m of x
__global__ void k_pack_df(uint64_t n, const double* __restrict__ x, int ld, int c0, int m, float* __restrict__ w) {
  const uint64_t idx = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (idx >= n * 4) return;
  const uint64_t i = idx >> 2;
  const int j = int(idx & 3);
  float h, l;
  df_split(j < m ? x[i * ld + c0 + j] : 0.0, h, l);
  w[i * 8 + 2 * j] = h;
  w[i * 8 + 2 * j + 1] = l;
}
}  // namespace

void virtual_pack_df(uint64_t n, const double* x, int ld, int c0, int m, float* w, cudaStream_t s) {
  if (!n) return;
  k_pack_df<<<unsigned((n * 4 + 255) / 256), 256, 0, s>>>(n, x, ld, c0, m, w);
  CG_CUDA(cudaGetLastError());
  count_launch();
}

uint64_t Hamiltonian::device_bytes() const {
  return rowptr.bytes() + col.bytes() + val64.bytes() + hi.bytes() + lo.bytes() + diag.bytes() +
         (virt ? virt->bytes() : 0) + (tiled ? tiled->bytes() : 0);
}

// ------------------------------------------------------------------- build
void virtual_build(const System& sys, const Operator& op, const Basis& b, int precision, Hamiltonian& h) {
  if (precision != CG_PREC_FP64 && precision != CG_PREC_FP32)
    throw Error(CG_ERR_ARG, "Hamiltonian precision must be CG_PREC_FP64 or CG_PREC_FP32");
  auto t_begin = std::chrono::steady_clock::now();
  CG_CUDA(cudaGetDevice(&h.device));
  if (h.device != b.device) throw Error(CG_ERR_ARG, "basis lives on another device");
  if (!h.stream) CG_CUDA(cudaStreamCreateWithFlags(&h.stream, cudaStreamNonBlocking));
  cudaStream_t s = h.stream;
  h.precision = precision;
  h.n = b.n;
  auto vp = std::make_shared<VirtualOp>();
  VirtualOp& v = *vp;
  const int nn = b.nn, np = b.np, ns = b.ns;
  const bool wide = b.wide;  // 64-bit species masks (wide.cu); the list machinery below
  if (nn > 64 || np > 45)
    throw Error(CG_ERR_UNSUPPORTED, "the on-the-fly product takes at most 64 neutron and 45 proton m-states");
  v.nn = nn;
  v.np = np;
  HostOp H = host_operator(sys, op);
  int m2max = 0;
  for (int i = 0; i < ns; ++i) m2max = std::max(m2max, std::abs(b.sp_m2[i]));
  for (int i = 0; i < ns; ++i)
    if ((b.sp_m2[i] - b.sp_m2[0]) & 1) throw Error(CG_ERR_UNSUPPORTED, "mixed integer / half-integer m");
  // transition slot = (change of 2m, change of parity): (dm2 / 2 + m2max) * 2 + dpar.  A neutron
  // transition in slot s pairs with proton transitions in slot nslot - 2 - (s & ~1) + (s & 1) (opposite
  // 2m change, same parity change), so both species land in classes of the same block.
  v.m2max = m2max;
  v.ndm = 2 * (2 * m2max + 1);
  v.dm0 = 2 * m2max;
  const auto& par = b.sp_par;
  auto dmi_of = [&](int from, int to) { return (((b.sp_m2[to] - b.sp_m2[from]) / 2 + m2max) << 1) | (par[to] ^ par[from]); };

  const int nblocks = int(b.h_bstart.size());
  const int nclasses = int(b.h_cstart.size()) - 1;
  v.nblocks = nblocks;
  // species masks of block neutrons and list protons
  auto nmask_of = [&](int beta) -> uint64_t { return wide ? b.h_wbmask[beta] : uint64_t(b.h_bmask[beta]); };
  auto pmask_of = [&](size_t g) -> uint64_t { return wide ? b.h_wcmask[g] : uint64_t(b.h_cmasks[g]); };
  const size_t nmembers = wide ? b.h_wcmask.size() : b.h_cmasks.size();
  v.nconf_p = nmembers;
  std::vector<uint32_t> blen(nblocks), order(nblocks);
  for (int i = 0; i < nblocks; ++i) {
    uint32_t c = b.h_bclass[i];
    blen[i] = b.h_cstart[c + 1] - b.h_cstart[c];
    v.lmax = std::max<int>(v.lmax, int(blen[i]));
  }
  // block of a neutron configuration (-1: not a block of the basis)
  std::vector<int32_t> block_tab(wide ? 1 : std::max<uint64_t>(b.neut.nconf, 1), -1);
  std::unordered_map<uint64_t, int32_t> block_map;
  for (int i = 0; i < nblocks; ++i) {
    if (wide) block_map[b.h_wbmask[i]] = i;
    else block_tab[colex_host(b.h_bmask[i], b.h_binom)] = i;
  }
  auto block_of = [&](uint64_t nu) -> int32_t {
    if (!wide) return block_tab[colex_host(nu, b.h_binom)];
    auto it = block_map.find(nu);
    return it == block_map.end() ? -1 : it->second;
  };
  // rank of a proton configuration in its (2m, parity) class, -1 when the
  // basis has no such configuration (a wide basis holds only the enumerated ones)
  std::unordered_map<uint64_t, uint32_t> univ;
  if (wide)
    for (size_t i = 0; i < b.h_wpuniv.size(); ++i) univ[b.h_wpuniv[i]] = uint32_t(i);
  auto class_rank = [&](uint64_t pi) -> int64_t {
    if (!wide) return b.h_pcrank[colex_host(pi, b.h_binom)];
    auto it = univ.find(pi);
    return it == univ.end() ? -1 : int64_t(b.h_wpuniv_rank[it->second]);
  };
  // truncated basis: the "classes" of the basis are its lists.  Each list
  // member keeps its rank in the untruncated class (b.h_pcrank), and each list
  // a map class rank -> list rank (0xffff: not in the list), padded to 8
  // entries so that every map is a 16-byte bulk copy
  const bool trunc = b.truncated || wide;
  std::vector<uint32_t> gcr, lmap_off, lmap_len, g_list;
  std::vector<uint16_t> lmap;
  if (trunc) {
    // class size of a proton configuration
    std::function<uint32_t(uint64_t)> class_size;
    std::map<std::pair<int, int>, uint32_t> csize;  // untruncated class sizes by (2m, parity)
    std::vector<uint32_t> key_of;
    std::vector<std::pair<int, int>> keys;
    if (wide) {
      class_size = [&](uint64_t pi) -> uint32_t { return b.h_wpuniv_csize[univ.at(pi)]; };
    } else {
      key_of.assign(std::max<uint64_t>(b.prot.nconf, 1), 0);
      for (uint64_t i = 0; i < b.prot.nconf; ++i) {
        const std::pair<int, int> k{b.prot.lex_m2[i], b.prot.lex_par[i]};
        if (csize[k]++ == 0) keys.push_back(k);
      }
      std::map<std::pair<int, int>, uint32_t> key_id;
      for (size_t i = 0; i < keys.size(); ++i) key_id[keys[i]] = uint32_t(i);
      for (uint64_t i = 0; i < b.prot.nconf; ++i)
        key_of[colex_host(b.prot.lex_mask[i], b.h_binom)] = key_id[{b.prot.lex_m2[i], b.prot.lex_par[i]}];
      class_size = [&](uint64_t pi) -> uint32_t { return csize[keys[key_of[colex_host(pi, b.h_binom)]]]; };
    }
    gcr.assign(std::max<size_t>(nmembers, 1), 0);
    g_list.assign(std::max<size_t>(nmembers, 1), 0);
    for (int L = 0; L < nclasses; ++L) {
      const uint32_t g0 = b.h_cstart[L], g1 = b.h_cstart[L + 1];
      uint32_t cs = 0;
      if (g1 > g0) cs = class_size(pmask_of(g0));
      if (cs > 0xffff) throw Error(CG_ERR_UNSUPPORTED, "proton class longer than 65535 configurations");
      const uint32_t len = std::max<uint32_t>(8, (cs + 7) / 8 * 8);
      lmap_off.push_back(uint32_t(lmap.size()));
      lmap_len.push_back(len);
      v.rmax = std::max<int>(v.rmax, int(len));
      lmap.resize(lmap.size() + len, 0xffff);
      for (uint32_t g = g0; g < g1; ++g) {
        const int64_t rr = class_rank(pmask_of(g));
        const uint32_t r = uint32_t(rr);
        if (rr < 0 || r >= cs) throw Error(CG_ERR_INTERNAL, "list member outside its class");
        gcr[g] = r;
        g_list[g] = uint32_t(L);
        lmap[lmap_off[L] + r] = uint16_t(g - g0);
      }
    }
    if (lmap.size() >= (1ull << 32)) throw Error(CG_ERR_UNSUPPORTED, "class-to-list maps beyond 2^32 entries");
  }
  v.truncated = trunc;
  v.wide = wide;
  const uint64_t nall = nn == 64 ? ~0ull : ((1ull << nn) - 1);
  const uint64_t pall_local = np == 64 ? ~0ull : ((1ull << np) - 1);
  const auto& m2 = b.sp_m2;

  // neutron transitions and NN2 per block
  std::vector<uint32_t> nt_off(nblocks + 1, 0), nn_off(nblocks + 1, 0);
  std::vector<NTrans> nt;
  std::vector<VPair> nn2;
  std::vector<double> En(nblocks, 0.0);
  for (int beta = 0; beta < nblocks; ++beta) {
    const uint64_t nu = nmask_of(beta);
    const uint64_t holes = ~nu & nall;
    double e = 0;
    for (uint64_t t = nu; t; t &= t - 1) {
      int a = __builtin_ctzll(t);
      e += H.e1[a * ns + a];
    }
    for (uint64_t t = nu; t; t &= t - 1) {
      int a = __builtin_ctzll(t);
      for (uint64_t w = t & (t - 1); w; w &= w - 1) {
        int c = __builtin_ctzll(w);
        e += H.V(a, c, a, c);
      }
    }
    En[beta] = e;
    for (uint64_t t = nu; t; t &= t - 1) {
      const int a = __builtin_ctzll(t);
      for (uint64_t w = holes; w; w &= w - 1) {
        const int c = __builtin_ctzll(w);
        const uint64_t nu2 = nu ^ (1ull << a) ^ (1ull << c);
        const int tb = block_of(nu2);
        if (tb < 0) continue;
        NTrans tr{};
        tr.target = uint32_t(tb);
        tr.a = uint8_t(a);
        tr.c = uint8_t(c);
        tr.sign = int8_t(move_sign(nu, a, c));
        tr.dmi = uint8_t(dmi_of(a, c));
        tr.cn = 0.0;
        if (tr.dmi == v.dm0) {
          const int x = std::min(a, c), yy = std::max(a, c);
          const uint64_t S0 = a < c ? nu : nu2;
          double val = H.term1(S0, x, yy);
          for (uint64_t q = nu & ~(1ull << a); q; q &= q - 1) {
            const int sc = __builtin_ctzll(q);
            val += H.term2(S0, std::min(x, sc), std::max(x, sc), std::min(yy, sc), std::max(yy, sc));
          }
          tr.cn = val;
        }
        nt.push_back(tr);
      }
    }
    nt_off[beta + 1] = uint32_t(nt.size());
    for (uint64_t t = nu; t; t &= t - 1) {
      const int a = __builtin_ctzll(t);
      for (uint64_t u = t & (t - 1); u; u &= u - 1) {
        const int bb = __builtin_ctzll(u);
        for (uint64_t w = holes; w; w &= w - 1) {
          const int c = __builtin_ctzll(w);
          for (uint64_t z = holes & ~below_h(c + 1); z; z &= z - 1) {
            const int d = __builtin_ctzll(z);
            if (m2[a] + m2[bb] != m2[c] + m2[d] || (par[a] ^ par[bb] ^ par[c] ^ par[d])) continue;
            const uint64_t K = nu ^ (1ull << a) ^ (1ull << bb) ^ (1ull << c) ^ (1ull << d);
            const int tb = block_of(K);
            if (tb < 0) {
              if (trunc) continue;  // the target block is outside the truncated basis
              throw Error(CG_ERR_INTERNAL, "two-neutron move leaves the basis");
            }
            const bool fwd = (a < c) || (a == c && bb < d);
            const double val = fwd ? H.term2(nu, a, bb, c, d) : H.term2(K, c, d, a, bb);
            // truncated basis: pad = the target list's class-to-list map
            if (std::fabs(val) >= kDropV)
              nn2.push_back(VPair{uint32_t(tb), trunc ? lmap_off[b.h_bclass[tb]] : 0u, val});
          }
        }
      }
    }
    nn_off[beta + 1] = uint32_t(nn2.size());
  }

  // proton transitions (grouped by 2m change) and PP2 per proton configuration
  const uint64_t npc = nmembers;
  std::vector<uint32_t> pt_off(npc * v.ndm + 1, 0), pp_off(npc + 1, 0);
  std::vector<uint2> pt;
  std::vector<double> pt_c, Ep(npc, 0.0);
  std::vector<VPair> pp2;
  std::vector<std::vector<std::pair<uint2, double>>> bydm(v.ndm);
  for (uint64_t g = 0; g < npc; ++g) {
    const uint64_t pi = pmask_of(g);
    const uint64_t holes = ~pi & pall_local;
    const G P = G(pi) << nn;  // global bits
    double e = 0;
    for (uint64_t t = pi; t; t &= t - 1) {
      int q = nn + __builtin_ctzll(t);
      e += H.e1[q * ns + q];
    }
    for (uint64_t t = pi; t; t &= t - 1) {
      int q = nn + __builtin_ctzll(t);
      for (uint64_t w = t & (t - 1); w; w &= w - 1) {
        int r = nn + __builtin_ctzll(w);
        e += H.V(q, r, q, r);
      }
    }
    Ep[g] = e;
    for (auto& l : bydm) l.clear();
    for (uint64_t t = pi; t; t &= t - 1) {
      const int bl = __builtin_ctzll(t);
      for (uint64_t w = holes; w; w &= w - 1) {
        const int dl = __builtin_ctzll(w);
        const uint64_t pi2 = pi ^ (1ull << bl) ^ (1ull << dl);
        const int64_t crank = class_rank(pi2);
        if (crank < 0) continue;  // a configuration no list of the basis holds
        const uint32_t rank = uint32_t(crank);
        const int bg = nn + bl, dg = nn + dl;
        const int sign = move_sign(pi, bl, dl);
        uint2 q;
        q.x = rank;
        q.y = uint32_t(bl) | (uint32_t(dl) << 8) | (uint32_t(sign) << 16);
        double cp = 0.0;
        if (dmi_of(bg, dg) == v.dm0) {
          const int x = std::min(bg, dg), yy = std::max(bg, dg);
          const G S0 = bl < dl ? P : (G(pi2) << nn);
          cp = H.term1(S0, x, yy);
          for (G z = P & ~gbit(bg); z; z &= z - 1) {
            const int sc = ctzg(z);
            cp += H.term2(S0, std::min(x, sc), std::max(x, sc), std::min(yy, sc), std::max(yy, sc));
          }
        }
        bydm[dmi_of(bg, dg)].push_back({q, cp});
      }
    }
    for (int k = 0; k < v.ndm; ++k) {
      pt_off[g * v.ndm + k] = uint32_t(pt.size());
      for (auto& qc : bydm[k]) {
        pt.push_back(qc.first);
        pt_c.push_back(qc.second);
      }
    }
    for (uint64_t t = pi; t; t &= t - 1) {
      const int a = nn + __builtin_ctzll(t);
      for (uint64_t u = t & (t - 1); u; u &= u - 1) {
        const int bb = nn + __builtin_ctzll(u);
        for (uint64_t w = holes; w; w &= w - 1) {
          const int c = nn + __builtin_ctzll(w);
          for (uint64_t z = holes & ~below_h(c - nn + 1); z; z &= z - 1) {
            const int d = nn + __builtin_ctzll(z);
            if (m2[a] + m2[bb] != m2[c] + m2[d] || (par[a] ^ par[bb] ^ par[c] ^ par[d])) continue;
            const G K = P ^ gbit(a) ^ gbit(bb) ^ gbit(c) ^ gbit(d);
            const bool fwd = (a < c) || (a == c && bb < d);
            const double val = fwd ? H.term2(P, a, bb, c, d) : H.term2(K, c, d, a, bb);
            // rank in the own block's list (the class; truncated: skip targets outside the list)
            const int64_t crank = class_rank(uint64_t(K >> nn));
            if (crank < 0) continue;
            uint32_t rank = uint32_t(crank);
            if (trunc) {
              rank = lmap[lmap_off[g_list[g]] + rank];
              if (rank == 0xffff) continue;
            }
            if (std::fabs(val) >= kDropV) pp2.push_back(VPair{rank, 0u, val});
          }
        }
      }
    }
    pp_off[g + 1] = uint32_t(pp2.size());
  }
  pt_off[npc * v.ndm] = uint32_t(pt.size());
  if (pt.size() >= (1ull << 32) || nt.size() >= (1ull << 32) || pp2.size() >= (1ull << 32) ||
      nn2.size() >= (1ull << 32))
    throw Error(CG_ERR_UNSUPPORTED, "transition tables beyond 2^32 entries");

  // lane-interleaved (32-row slice) copies of the per-configuration lists, per proton class
  const int npp_i = np * np;
  std::vector<uint32_t> cslice(nclasses + 1, 0);
  for (int c = 0; c < nclasses; ++c) cslice[c + 1] = cslice[c] + (b.h_cstart[c + 1] - b.h_cstart[c] + 31) / 32;
  const uint32_t nslices = cslice[nclasses];
  std::vector<uint32_t> sl_off(size_t(nslices) * v.ndm + 1, 0), sl_e, pps_off(nslices + 1, 0), pp_rank;
  std::vector<double> sl_c, pp_h;
  for (int c = 0; c < nclasses; ++c) {
    const uint32_t g0 = b.h_cstart[c], L = b.h_cstart[c + 1] - g0;
    if (L > 0xffff) throw Error(CG_ERR_UNSUPPORTED, "proton class longer than 65535 configurations");
    for (uint32_t sg = 0; sg < (L + 31) / 32; ++sg) {
      const uint32_t sl = cslice[c] + sg;
      for (int k = 0; k < v.ndm; ++k) {
        sl_off[size_t(sl) * v.ndm + k] = uint32_t(sl_e.size());
        uint32_t cnt = 0;
        for (uint32_t l = 0; l < 32 && sg * 32 + l < L; ++l) {
          const uint64_t g = g0 + sg * 32 + l;
          cnt = std::max(cnt, pt_off[g * v.ndm + k + 1] - pt_off[g * v.ndm + k]);
        }
        for (uint32_t j = 0; j < cnt; ++j)
          for (uint32_t l = 0; l < 32; ++l) {
            const uint32_t r = sg * 32 + l;
            uint32_t ent = uint32_t(npp_i) << 16;  // padding: weight slot npp holds 0
            double cv = 0.0;
            if (r < L) {
              const uint64_t g = g0 + r;
              const uint32_t e0 = pt_off[g * v.ndm + k];
              if (j < pt_off[g * v.ndm + k + 1] - e0) {
                const uint2 q = pt[e0 + j];
                const uint32_t bl = q.y & 0xff, dl = (q.y >> 8) & 0xff, sg1 = (q.y >> 16) & 1;
                ent = q.x | ((bl * np + dl) << 16) | (sg1 << 27);
                cv = pt_c[e0 + j];
              }
            }
            sl_e.push_back(ent);
            sl_c.push_back(cv);
          }
      }
      pps_off[sl] = uint32_t(pp_rank.size());
      uint32_t cnt = 0;
      for (uint32_t l = 0; l < 32 && sg * 32 + l < L; ++l) {
        const uint64_t g = g0 + sg * 32 + l;
        cnt = std::max(cnt, pp_off[g + 1] - pp_off[g]);
      }
      for (uint32_t j = 0; j < cnt; ++j)
        for (uint32_t l = 0; l < 32; ++l) {
          const uint32_t r = sg * 32 + l;
          uint32_t rank = 0;
          double hv = 0.0;
          if (r < L && j < pp_off[g0 + r + 1] - pp_off[g0 + r]) {
            rank = pp2[pp_off[g0 + r] + j].target;
            hv = pp2[pp_off[g0 + r] + j].h;
          }
          pp_rank.push_back(rank);
          pp_h.push_back(hv);
        }
    }
  }
  sl_off[size_t(nslices) * v.ndm] = uint32_t(sl_e.size());
  pps_off[nslices] = uint32_t(pp_rank.size());
  if (sl_e.size() >= (1ull << 32) || pp_rank.size() >= (1ull << 32))
    throw Error(CG_ERR_UNSUPPORTED, "transition tables beyond 2^32 entries");

  // interaction slices
  const size_t npp = size_t(np) * np;
  std::vector<double> W(size_t(nn) * nn * npp, 0.0), Un(size_t(nn) * nn * np, 0.0), Up(npp * nn, 0.0),
      Vd(size_t(nn) * np, 0.0);
  for (int an = 0; an < nn; ++an)
    for (int cn = 0; cn < nn; ++cn) {
      if (an == cn) continue;
      for (int bl = 0; bl < np; ++bl)
        for (int dl = 0; dl < np; ++dl) {
          if (bl == dl) continue;
          const int bg = nn + bl, dg = nn + dl;
          W[((size_t(an) * nn + cn) * np + bl) * np + dl] = an < cn ? H.V(an, bg, cn, dg) : H.V(cn, dg, an, bg);
        }
      for (int q = 0; q < np; ++q)
        Un[(size_t(an) * nn + cn) * np + q] = H.V(std::min(an, cn), nn + q, std::max(an, cn), nn + q);
    }
  for (int bl = 0; bl < np; ++bl)
    for (int dl = 0; dl < np; ++dl) {
      if (bl == dl) continue;
      for (int q = 0; q < nn; ++q)
        Up[(size_t(bl) * np + dl) * nn + q] = H.V(q, nn + std::min(bl, dl), q, nn + std::max(bl, dl));
    }
  for (int q = 0; q < nn; ++q)
    for (int bl = 0; bl < np; ++bl) Vd[size_t(q) * np + bl] = H.V(q, nn + bl, q, nn + bl);

  // generated elements per product and a largest-first block order
  std::vector<uint64_t> cls_pp(nclasses, 0), cls_dm(size_t(nclasses) * v.ndm, 0);
  for (int c = 0; c < nclasses; ++c)
    for (uint32_t g = b.h_cstart[c]; g < b.h_cstart[c + 1]; ++g) {
      cls_pp[c] += pp_off[g + 1] - pp_off[g] + pt_off[size_t(g) * v.ndm + v.dm0 + 1] - pt_off[size_t(g) * v.ndm + v.dm0];
      for (int k = 0; k < v.ndm; ++k) cls_dm[size_t(c) * v.ndm + k] += pt_off[size_t(g) * v.ndm + k + 1] - pt_off[size_t(g) * v.ndm + k];
    }
  std::vector<uint64_t> work(nblocks, 0);
  uint64_t conn = 0;
  for (int beta = 0; beta < nblocks; ++beta) {
    const uint32_t c = b.h_bclass[beta];
    uint64_t w = uint64_t(blen[beta]) * (1 + (nn_off[beta + 1] - nn_off[beta])) + cls_pp[c];
    for (uint32_t t = nt_off[beta]; t < nt_off[beta + 1]; ++t) {
      w += cls_dm[size_t(c) * v.ndm + (v.ndm - 2 - (nt[t].dmi & ~1) + (nt[t].dmi & 1))];
      if (nt[t].dmi == v.dm0) w += blen[beta];
    }
    work[beta] = w;
    conn += w;
  }
  v.connections = conn;
  std::iota(order.begin(), order.end(), 0u);
  std::stable_sort(order.begin(), order.end(), [&](uint32_t p, uint32_t q) { return work[p] > work[q]; });

  // upload
  v.bstart.upload(b.h_bstart, s);
  v.blen.upload(blen, s);
  v.bclass.upload(b.h_bclass, s);
  if (wide) {
    v.bmask64.upload(b.h_wbmask, s);
    v.bmask.alloc(1);
  } else {
    v.bmask.upload(b.h_bmask, s);
  }
  v.order.upload(order, s);
  v.cstart.upload(b.h_cstart, s);
  if (wide) {
    v.cmask64.upload(b.h_wcmask, s);
    v.cmask.alloc(1);
  } else {
    v.cmask.upload(b.h_cmasks, s);
  }
  v.nt_off.upload(nt_off, s);
  v.nt.upload(nt, s);
  v.nn_off.upload(nn_off, s);
  v.nn2.upload(nn2, s);
  v.cslice.upload(cslice, s);
  v.sl_off.upload(sl_off, s);
  v.sl_e.upload(sl_e, s);
  v.sl_c.upload(sl_c, s);
  v.pp_off.upload(pps_off, s);
  v.pp_rank.upload(pp_rank, s);
  v.pp_h.upload(pp_h, s);
  if (trunc) {
    v.gcr.upload(gcr, s);
    v.lmap.upload(lmap, s);
    v.lmap_off.upload(lmap_off, s);
    v.lmap_len.upload(lmap_len, s);
  }
  std::vector<float> sl_cf(sl_c.begin(), sl_c.end()), pp_hf(pp_h.begin(), pp_h.end());
  v.sl_cf.upload(sl_cf, s);
  v.pp_hf.upload(pp_hf, s);
  auto lo_part = [](const std::vector<double>& d, const std::vector<float>& f) {
    std::vector<float> l(d.size());
    for (size_t i = 0; i < d.size(); ++i) l[i] = float(d[i] - double(f[i]));
    return l;
  };
  v.sl_cl.upload(lo_part(sl_c, sl_cf), s);
  v.pp_hl.upload(lo_part(pp_h, pp_hf), s);
  v.W.upload(W, s);
  v.Un.upload(Un, s);
  v.Up.upload(Up, s);
  std::vector<float> Wf(W.begin(), W.end()), Unf(Un.begin(), Un.end()), Upf(Up.begin(), Up.end());
  v.Wf.upload(Wf, s);
  v.Unf.upload(Unf, s);
  v.Upf.upload(Upf, s);
  v.Wl.upload(lo_part(W, Wf), s);
  v.Unl.upload(lo_part(Un, Unf), s);
  v.Upl.upload(lo_part(Up, Upf), s);
  h.diag.alloc(std::max<uint64_t>(b.n, 1));
  if (b.n) {
    DBuf<double> dEn, dEp, dVd;
    dEn.upload(En, s);
    dEp.upload(Ep, s);
    dVd.upload(Vd, s);
    const unsigned gd = unsigned((b.n + 255) / 256);
    if (wide)
      k_virtual_diag<unsigned long long><<<gd, 256, 0, s>>>(
          b.n, nblocks, v.bstart.p, v.bclass.p, reinterpret_cast<const unsigned long long*>(v.bmask64.p), v.cstart.p,
          reinterpret_cast<const unsigned long long*>(v.cmask64.p), dEn.p, dEp.p, dVd.p, np, h.diag.p);
    else
      k_virtual_diag<uint32_t><<<gd, 256, 0, s>>>(b.n, nblocks, v.bstart.p, v.bclass.p, v.bmask.p, v.cstart.p,
                                                  v.cmask.p, dEn.p, dEp.p, dVd.p, np, h.diag.p);
    CG_CUDA(cudaGetLastError());
    count_launch();
    CG_CUDA(cudaStreamSynchronize(s));
  }
  CG_CUDA(cudaStreamSynchronize(s));
  v.err.alloc(1);
  h.virt = vp;
  h.nnz = conn;
  h.nnz_upper = 0;
  h.max_row = 0;
  h.build_seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_begin).count();
}

}  // namespace cg
