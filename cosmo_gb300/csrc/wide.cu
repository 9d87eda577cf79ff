// Valence spaces wider than the bitstring basis: a species with more than 32
// m-states (up to 64 per species, 128 in all), e.g. the spsdpf space of the
// reference's 33Al example (0s, 0p, 1s0d, 1p0f: 40 m-states per species).
//
// The reference handles any width (determinants are sorted index tuples;
// SM::MakeMBS2, include/sm/MakeMBS.cxx:414-598, and the XsysmbsOMP partitions,
// xmlshell/xmbs/XsysmbsOMP.cpp:214-300).  Here a determinant is a pair of
// 64-bit species masks.  The species configurations are enumerated on the host
// in lexicographic order by a depth-first search that drops every branch whose
// oscillator quanta can no longer stay inside the truncation (20 neutrons in
// the 40 spsdpf m-states have C(40, 20) = 1.4e11 configurations, their 0-1 hw
// window a few hundred), then bucketed into proton classes and per-neutron
// lists exactly as the bitstring basis does, so the order is the reference's.
// A determinant is located by two binary searches: its neutron mask among the
// blocks, its proton mask inside the block's list (SM::locate is a binary
// search over the whole basis, include/sm/ManyBodyStates.cxx:92-130).
//
// The Hamiltonian rows follow the element rules of the bitstring builder
// (hbuild.cu) on 128-bit occupation words: the diagonal; one particle moved
// with every other occupied orbital as spectator; two particles of one species
// moved; one neutron and one proton moved.  Each element is evaluated from the
// lower-index determinant of the pair with the forward-ordered terms and kept
// when |value| >= 1e-14 (PPMatrix2CSBBlk, include/sm/PPMatrix.cxx:571-656);
// a target outside a truncated basis is skipped.  <J-J+> and <T-T+> are the
// expectation values of the two-body operators (J+)+ J+ and (T+)+ T+, built
// as stored matrices on the same basis.
#include <algorithm>
#include <climits>
#include <cmath>
#include <map>
#include <memory>
#include <numeric>

#include "device.h"

namespace cg {

namespace {

constexpr double kDropW = 1e-14;
constexpr uint64_t kOutsideW = ~0ull - 1;
constexpr uint64_t kSpeciesCap = 1ull << 26;  // configurations per species kept on the host

// ------------------------------------------------------------------- host
// Depth-first lexicographic enumeration of the k-subsets of norb states whose
// quanta stay <= qlimit (minsum bounds what the remaining particles add).
struct SpeciesEnum {
  int norb = 0, k = 0, qlimit = INT_MAX / 4;
  const int *q = nullptr, *m2 = nullptr, *par = nullptr;
  std::vector<int> minsum;  // (norb + 1) x (k + 1): least quanta of r states among i..norb-1
  std::vector<uint64_t> mask;
  std::vector<int> msum, psum, qsum;

  void run() {
    minsum.assign(size_t(norb + 1) * (k + 1), INT_MAX / 4);
    for (int i = 0; i <= norb; ++i) {
      std::vector<int> rest(q + i, q + norb);
      std::sort(rest.begin(), rest.end());
      int s = 0;
      minsum[size_t(i) * (k + 1)] = 0;
      for (int r = 1; r <= k && r <= int(rest.size()); ++r) {
        s += rest[r - 1];
        minsum[size_t(i) * (k + 1) + r] = s;
      }
    }
    if (k <= norb) go(0, k, 0, 0, 0, 0);
  }
  void go(int start, int left, uint64_t m, int Q, int M, int P) {
    if (left == 0) {
      if (mask.size() >= kSpeciesCap) throw Error(CG_ERR_UNSUPPORTED, "species configuration space too large");
      mask.push_back(m);
      msum.push_back(M);
      psum.push_back(P);
      qsum.push_back(Q);
      return;
    }
    for (int c = start; c + left <= norb; ++c) {
      const int Q2 = Q + q[c];
      if (Q2 + minsum[size_t(c + 1) * (k + 1) + left - 1] > qlimit) continue;
      go(c + 1, left - 1, m | (1ull << c), Q2, M + m2[c], P ^ par[c]);
    }
  }
};

// ----------------------------------------------------------------- device
// 128-bit occupation word as two 64-bit words (s.p. state b at bit b & 63 of
// word b >> 6), with the few operations the element rules need.
struct Occ {
  unsigned long long w0, w1;
};
__device__ __forceinline__ Occ occ_bit(int b) {
  return b < 64 ? Occ{1ull << b, 0ull} : Occ{0ull, 1ull << (b - 64)};
}
__device__ __forceinline__ Occ operator^(Occ a, Occ b) { return Occ{a.w0 ^ b.w0, a.w1 ^ b.w1}; }
__device__ __forceinline__ Occ operator&(Occ a, Occ b) { return Occ{a.w0 & b.w0, a.w1 & b.w1}; }
__device__ __forceinline__ Occ operator~(Occ a) { return Occ{~a.w0, ~a.w1}; }
__device__ __forceinline__ bool occ_any(Occ a) { return (a.w0 | a.w1) != 0ull; }
__device__ __forceinline__ int occ_popc(Occ a) { return __popcll(a.w0) + __popcll(a.w1); }
// index of the lowest set bit (the word must not be empty)
__device__ __forceinline__ int occ_low(Occ a) {
  return a.w0 ? __ffsll((long long)a.w0) - 1 : 64 + __ffsll((long long)a.w1) - 1;
}
__device__ __forceinline__ Occ occ_drop_low(Occ a) {
  if (a.w0) a.w0 &= a.w0 - 1ull;
  else a.w1 &= a.w1 - 1ull;
  return a;
}
// bits 0 .. b-1
__device__ __forceinline__ Occ occ_below(int b) {
  if (b >= 128) return Occ{~0ull, ~0ull};
  if (b >= 64) return Occ{~0ull, b == 64 ? 0ull : ((1ull << (b - 64)) - 1ull)};
  return Occ{b == 0 ? 0ull : ((1ull << b) - 1ull), 0ull};
}
__device__ __forceinline__ int occ_popc_below(Occ a, int b) { return occ_popc(a & occ_below(b)); }

__global__ void k_wide_expand(uint64_t n, int nblocks, const uint64_t* __restrict__ bstart,
                              const uint64_t* __restrict__ bmask, const uint32_t* __restrict__ bclass,
                              const uint32_t* __restrict__ cstart, const uint64_t* __restrict__ cmask,
                              uint64_t* __restrict__ wstate) {
  const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i >= n) return;
  int lo = 0, hi = nblocks - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (bstart[mid] <= i) lo = mid; else hi = mid - 1;
  }
  wstate[2 * i] = bmask[lo];
  wstate[2 * i + 1] = cmask[cstart[bclass[lo]] + (i - bstart[lo])];
}

__global__ void k_wide_tuples(uint64_t first, uint64_t count, int N, int nn, const uint64_t* __restrict__ wstate,
                              uint16_t* __restrict__ out) {
  const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i >= count) return;
  uint64_t a = wstate[2 * (first + i)], p = wstate[2 * (first + i) + 1];
  uint16_t* o = out + i * N;
  int k = 0;
  for (; a; a &= a - 1) o[k++] = uint16_t(__ffsll((long long)a) - 1);
  for (; p; p &= p - 1) o[k++] = uint16_t(nn + __ffsll((long long)p) - 1);
}

struct WCtx {
  int ns, nn, npairs, nblocks;
  bool truncated;
  uint64_t n;
  const uint64_t* wstate;
  const uint64_t *bstart, *nkey, *pkey;
  const uint32_t *bclass, *cstart, *nblk, *prank;
  const double *e1, *v2;
  const int8_t* m2;
  const unsigned long long* mmask;  // per species x (2 kMOff + 1): 128-bit masks as (lo, hi)
};

struct WShared {
  Occ mmask[2 * (2 * kMOff + 1)];
  int16_t pidx[128 * 128];
  int8_t m2[128];
};

__device__ void load_wshared(WShared& sh, const WCtx& c) {
  for (int i = threadIdx.x; i < 2 * (2 * kMOff + 1); i += blockDim.x)
    sh.mmask[i] = Occ{c.mmask[2 * i], c.mmask[2 * i + 1]};
  for (int i = threadIdx.x; i < 128 * 128; i += blockDim.x) {
    const int a = i >> 7, b = i & 127;
    sh.pidx[i] = int16_t((a < b && b < c.ns) ? (a * c.ns - a * (a + 1) / 2 + (b - a - 1)) : -1);
  }
  for (int i = threadIdx.x; i < 128; i += blockDim.x) sh.m2[i] = i < c.ns ? c.m2[i] : 0;
  __syncthreads();
}

// neutron and proton masks of an occupation word (neutrons at bits 0 .. nn-1)
__device__ __forceinline__ void occ_split(Occ K, int nn, unsigned long long& nm, unsigned long long& pm) {
  if (nn == 0) {
    nm = 0ull;
    pm = K.w0;
  } else if (nn == 64) {
    nm = K.w0;
    pm = K.w1;
  } else {
    nm = K.w0 & ((1ull << nn) - 1ull);
    pm = (K.w0 >> nn) | (K.w1 << (64 - nn));
  }
}
__device__ __forceinline__ Occ occ_join(unsigned long long nm, unsigned long long pm, int nn) {
  if (nn == 0) return Occ{pm, 0ull};
  if (nn == 64) return Occ{nm, pm};
  return Occ{nm | (pm << nn), pm >> (64 - nn)};
}

// basis index of determinant K; kOutsideW outside a truncated basis, ~0 when
// an untruncated basis misses it (an internal error the caller flags)
__device__ uint64_t wide_index(const WCtx& c, Occ K) {
  unsigned long long nm, pm;
  occ_split(K, c.nn, nm, pm);
  const uint64_t miss = c.truncated ? kOutsideW : ~0ull;
  int lo = 0, hi = c.nblocks;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if (c.nkey[mid] < nm) lo = mid + 1; else hi = mid;
  }
  if (lo == c.nblocks || c.nkey[lo] != nm) return miss;
  const uint32_t blk = c.nblk[lo], L = c.bclass[blk];
  const uint32_t end = c.cstart[L + 1];
  uint32_t a = c.cstart[L], e = end;
  while (a < e) {
    const uint32_t mid = (a + e) >> 1;
    if (c.pkey[mid] < pm) a = mid + 1; else e = mid;
  }
  if (a == end || c.pkey[a] != pm) return miss;
  return c.bstart[blk] + c.prank[a];
}

__device__ __forceinline__ double wterm2(const WCtx& c, const WShared& sh, Occ S0, int b0, int b1, int b2, int b3) {
  const double v = __ldg(c.v2 + size_t(sh.pidx[b0 * 128 + b1]) * c.npairs + sh.pidx[b2 * 128 + b3]);
  int p = occ_popc_below(S0, b0) + occ_popc_below(S0, b1) - 1;
  const Occ I = S0 & ~(occ_bit(b0) ^ occ_bit(b1));
  p += occ_popc_below(I, b2) + occ_popc_below(I, b3);
  return (p & 1) ? -v : v;
}

__device__ __forceinline__ double wterm1(const WCtx& c, Occ S0, int x, int y) {
  const double v = __ldg(c.e1 + x * c.ns + y);
  const int p = occ_popc_below(S0, x) + occ_popc_below(S0 & ~occ_bit(x), y);
  return (p & 1) ? -v : v;
}

// emit(K, value, is_diagonal) for every element of row `row`
template <class Emit>
__device__ void visit_row_wide(const WCtx& c, const WShared& sh, uint64_t row, Emit&& emit) {
  const Occ S = occ_join(c.wstate[2 * row], c.wstate[2 * row + 1], c.nn);
  const Occ nall = occ_below(c.nn), pall = occ_below(c.ns) & ~nall;
  {
    double v = 0.0;
    for (Occ t = S; occ_any(t); t = occ_drop_low(t)) {
      const int a = occ_low(t);
      v += __ldg(c.e1 + a * c.ns + a);
    }
    for (Occ t = S; occ_any(t); t = occ_drop_low(t)) {
      const int a = occ_low(t);
      for (Occ u = occ_drop_low(t); occ_any(u); u = occ_drop_low(u)) {
        const int pab = sh.pidx[a * 128 + occ_low(u)];
        v += __ldg(c.v2 + size_t(pab) * c.npairs + pab);
      }
    }
    emit(S, v, true);
  }
  for (int sp = 0; sp < 2; ++sp) {
    const Occ all = sp ? pall : nall;
    const Occ Ss = S & all, holes = ~S & all;
    const Occ* mm = sh.mmask + sp * (2 * kMOff + 1) + kMOff;
    for (Occ t = Ss; occ_any(t); t = occ_drop_low(t)) {
      const int a = occ_low(t);
      for (Occ u = holes & mm[sh.m2[a]]; occ_any(u); u = occ_drop_low(u)) {
        const int f = occ_low(u);
        const Occ K = S ^ occ_bit(a) ^ occ_bit(f);
        const int x = a < f ? a : f, y = a < f ? f : a;
        const Occ S0 = a < f ? S : K;
        double v = wterm1(c, S0, x, y);
        for (Occ w = S & ~occ_bit(a); occ_any(w); w = occ_drop_low(w)) {
          const int sc = occ_low(w);
          v += wterm2(c, sh, S0, x < sc ? x : sc, x < sc ? sc : x, y < sc ? y : sc, y < sc ? sc : y);
        }
        emit(K, v, false);
      }
    }
    for (Occ t = Ss; occ_any(t); t = occ_drop_low(t)) {
      const int a = occ_low(t);
      for (Occ u = occ_drop_low(t); occ_any(u); u = occ_drop_low(u)) {
        const int b = occ_low(u);
        const int msum = sh.m2[a] + sh.m2[b];
        for (Occ w = holes; occ_any(w); w = occ_drop_low(w)) {
          const int cc = occ_low(w);
          const int dm = msum - sh.m2[cc];
          if (dm < -kMOff || dm > kMOff) continue;
          for (Occ z = holes & mm[dm] & ~occ_below(cc + 1); occ_any(z); z = occ_drop_low(z)) {
            const int d = occ_low(z);
            const Occ K = S ^ occ_bit(a) ^ occ_bit(b) ^ occ_bit(cc) ^ occ_bit(d);
            const bool fwd = (a < cc) || (a == cc && b < d);
            emit(K, fwd ? wterm2(c, sh, S, a, b, cc, d) : wterm2(c, sh, K, cc, d, a, b), false);
          }
        }
      }
    }
  }
  {
    const Occ Sn = S & nall, Sp = S & pall, hn = ~S & nall, hp = ~S & pall;
    const Occ* mmp = sh.mmask + (2 * kMOff + 1) + kMOff;
    for (Occ t = Sn; occ_any(t); t = occ_drop_low(t)) {
      const int a = occ_low(t);
      for (Occ w = hn; occ_any(w); w = occ_drop_low(w)) {
        const int cc = occ_low(w);
        const int dmn = sh.m2[a] - sh.m2[cc];
        for (Occ u = Sp; occ_any(u); u = occ_drop_low(u)) {
          const int b = occ_low(u);
          const int dm = dmn + sh.m2[b];
          if (dm < -kMOff || dm > kMOff) continue;
          for (Occ z = hp & mmp[dm]; occ_any(z); z = occ_drop_low(z)) {
            const int d = occ_low(z);
            const Occ K = S ^ occ_bit(a) ^ occ_bit(b) ^ occ_bit(cc) ^ occ_bit(d);
            emit(K, (a < cc) ? wterm2(c, sh, S, a, b, cc, d) : wterm2(c, sh, K, cc, d, a, b), false);
          }
        }
      }
    }
  }
}

__global__ void k_wide_count(WCtx c, uint32_t* __restrict__ counts, int* __restrict__ err) {
  __shared__ WShared sh;
  load_wshared(sh, c);
  for (uint64_t row = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; row < c.n;
       row += uint64_t(gridDim.x) * blockDim.x) {
    uint32_t k = 0;
    visit_row_wide(c, sh, row, [&](Occ K, double v, bool isdiag) {
      if (fabs(v) < kDropW) return;
      if (isdiag) { ++k; return; }
      const uint64_t col = wide_index(c, K);
      if (col == ~0ull) { atomicOr(err, 1); return; }
      if (col != kOutsideW) ++k;
    });
    counts[row] = k;
  }
}

__global__ void k_wide_fill(WCtx c, const uint64_t* __restrict__ rowptr, uint32_t* __restrict__ col,
                            double* __restrict__ val, double* __restrict__ diag) {
  __shared__ WShared sh;
  load_wshared(sh, c);
  for (uint64_t row = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; row < c.n;
       row += uint64_t(gridDim.x) * blockDim.x) {
    uint64_t p = rowptr[row];
    const uint64_t pend = rowptr[row + 1];
    double dv = 0.0;
    visit_row_wide(c, sh, row, [&](Occ K, double v, bool isdiag) {
      if (fabs(v) < kDropW) return;
      const uint64_t k = isdiag ? row : wide_index(c, K);
      if (k >= kOutsideW || p >= pend) return;
      col[p] = uint32_t(k);
      val[p] = v;
      ++p;
      if (isdiag) dv = v;
    });
    diag[row] = dv;
  }
}

// ------------------------------------------------ overlaps between two bases
// The pull forms of sf.cu on wide bases: one thread per daughter determinant,
// the parent determinant located by wide_index on the parent's tables.
constexpr int kMaxDaughterW = 16;

WCtx locate_ctx(const Basis& b) {
  WCtx c{};
  c.ns = b.ns;
  c.nn = b.nn;
  c.nblocks = int(b.h_bstart.size());
  c.truncated = b.truncated;
  c.n = b.n;
  c.wstate = b.wstate.p;
  c.bstart = b.wbstart.p;
  c.nkey = b.wnkey.p;
  c.pkey = b.wpkey.p;
  c.bclass = b.wbclass.p;
  c.cstart = b.wcstart.p;
  c.nblk = b.wnblk.p;
  c.prank = b.wprank.p;
  return c;
}

__device__ __forceinline__ void reduce_daughter(const double (&acc)[kMaxDaughterW], double* __restrict__ part,
                                                size_t slot) {
  __shared__ double red[kMaxDaughterW][256 / 32];
  const int lane = threadIdx.x & 31, wi = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < kMaxDaughterW; ++q) {
    double v = acc[q];
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(~0u, v, o);
    if (lane == 0) red[q][wi] = v;
  }
  __syncthreads();
  if (threadIdx.x < kMaxDaughterW) {
    double v = 0.0;
    for (int i = 0; i < int(blockDim.x >> 5); ++i) v += red[threadIdx.x][i];
    part[slot * kMaxDaughterW + threadIdx.x] = v;
  }
}

// <D_q| sum_t v_t a+_f a_i |P>: P = D - f + i, phase of a+_f a_i on P
__global__ void __launch_bounds__(256) k_wide_onebody(WCtx par, const uint64_t* __restrict__ dstate, uint64_t nd,
                                                      const double* __restrict__ psid, int nq,
                                                      const double* __restrict__ psip, const int2* __restrict__ tif,
                                                      const double* __restrict__ tv, int nt,
                                                      double* __restrict__ part, int* __restrict__ err) {
  double acc[kMaxDaughterW];
#pragma unroll
  for (int q = 0; q < kMaxDaughterW; ++q) acc[q] = 0.0;
  for (uint64_t row = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; row < nd;
       row += uint64_t(gridDim.x) * blockDim.x) {
    const Occ D = occ_join(dstate[2 * row], dstate[2 * row + 1], par.nn);
    double w = 0.0;
    for (int t = 0; t < nt; ++t) {
      const int2 e = tif[t];
      if (!occ_any(D & occ_bit(e.y))) continue;
      const Occ Df = D & ~occ_bit(e.y);
      if (e.x != e.y && occ_any(Df & occ_bit(e.x))) continue;
      const Occ P = e.x == e.y ? D : (Df ^ occ_bit(e.x));
      const uint64_t idx = wide_index(par, P);
      if (idx == kOutsideW) continue;
      if (idx >= par.n) { atomicOr(err, 1); continue; }
      const int ph = occ_popc_below(P, e.x) + occ_popc_below(Df, e.y);
      const double v = tv[t] * psip[idx];
      w += (ph & 1) ? -v : v;
    }
#pragma unroll
    for (int q = 0; q < kMaxDaughterW; ++q)
      if (q < nq) acc[q] += w * psid[row * nq + q];
  }
  reduce_daughter(acc, part, blockIdx.x);
}

// <D_q| a_s |P>: P = D + s, phase of the states of D below s
__global__ void __launch_bounds__(256) k_wide_sf(WCtx par, const uint64_t* __restrict__ dstate, uint64_t nd,
                                                 const double* __restrict__ psid, int nq,
                                                 const double* __restrict__ psip, const int* __restrict__ sidx,
                                                 double* __restrict__ part, int* __restrict__ err) {
  const int s = sidx[blockIdx.y];
  double acc[kMaxDaughterW];
#pragma unroll
  for (int q = 0; q < kMaxDaughterW; ++q) acc[q] = 0.0;
  for (uint64_t row = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; row < nd;
       row += uint64_t(gridDim.x) * blockDim.x) {
    const Occ D = occ_join(dstate[2 * row], dstate[2 * row + 1], par.nn);
    if (occ_any(D & occ_bit(s))) continue;
    const uint64_t idx = wide_index(par, D ^ occ_bit(s));
    if (idx == kOutsideW) continue;
    if (idx >= par.n) { atomicOr(err, 1); continue; }
    const double c = ((occ_popc_below(D, s) & 1) ? -1.0 : 1.0) * psip[idx];
#pragma unroll
    for (int q = 0; q < kMaxDaughterW; ++q)
      if (q < nq) acc[q] += c * psid[row * nq + q];
  }
  reduce_daughter(acc, part, size_t(blockIdx.y) * gridDim.x + blockIdx.x);
}

class WideRowsImpl : public WideRows {
 public:
  WideRowsImpl(const System& sys, const Operator& op, const Basis& b, cudaStream_t s) : s_(s) {
    const int ns = b.ns;
    int np = 0;
    std::vector<int32_t> pidx(size_t(ns) * ns, -1);
    for (int a = 0; a < ns; ++a)
      for (int c = a + 1; c < ns; ++c) pidx[size_t(a) * ns + c] = np++;
    std::vector<double> e1(size_t(ns) * ns, 0.0);
    for (auto& kv : op.one) {
      const int i = kv.first[0], f = kv.first[1];
      if (i < 0 || f < 0 || i >= ns || f >= ns) throw Error(CG_ERR_INTERNAL, "one-body key out of range");
      e1[size_t(i) * ns + f] = kv.second;
    }
    std::vector<double> v2(size_t(std::max(np, 1)) * std::max(np, 1), 0.0);
    for (auto& kv : op.two) {
      const Key4& k = kv.first;
      if (k[0] >= k[1] || k[2] >= k[3]) continue;  // cannot act on a determinant
      v2[size_t(pidx[size_t(k[0]) * ns + k[1]]) * np + pidx[size_t(k[2]) * ns + k[3]]] = kv.second;
    }
    std::vector<unsigned long long> mm(2 * 2 * (2 * kMOff + 1), 0ull);
    std::vector<int8_t> m2(ns);
    for (int i = 0; i < ns; ++i) {
      const int sp = i < sys.n_neutron_states ? 0 : 1;
      const int m = sys.sps[i].m2;
      if (m < -kMOff || m > kMOff) throw Error(CG_ERR_UNSUPPORTED, "|2m| too large");
      m2[i] = int8_t(m);
      const size_t e = size_t(sp) * (2 * kMOff + 1) + (m + kMOff);
      mm[2 * e + (i >> 6)] |= 1ull << (i & 63);
    }
    e1_.upload(e1, s);
    v2_.upload(v2, s);
    mm_.upload(mm, s);
    m2_.upload(m2, s);
    c_.ns = ns;
    c_.nn = b.nn;
    c_.npairs = np;
    c_.nblocks = int(b.h_bstart.size());
    c_.truncated = b.truncated;
    c_.n = b.n;
    c_.wstate = b.wstate.p;
    c_.bstart = b.wbstart.p;
    c_.nkey = b.wnkey.p;
    c_.pkey = b.wpkey.p;
    c_.bclass = b.wbclass.p;
    c_.cstart = b.wcstart.p;
    c_.nblk = b.wnblk.p;
    c_.prank = b.wprank.p;
    c_.e1 = e1_.p;
    c_.v2 = v2_.p;
    c_.m2 = m2_.p;
    c_.mmask = mm_.p;
    grid_ = unsigned(std::max<uint64_t>(1, std::min<uint64_t>((b.n + kT - 1) / kT, 152ull * 16)));
  }
  void count(uint32_t* counts, int* err) override {
    if (!c_.n) return;
    k_wide_count<<<grid_, kT, 0, s_>>>(c_, counts, err);
    CG_CUDA(cudaGetLastError());
    count_launch();
  }
  void fill(const uint64_t* rowptr, uint32_t* col, double* val, double* diag) override {
    if (!c_.n) return;
    k_wide_fill<<<grid_, kT, 0, s_>>>(c_, rowptr, col, val, diag);
    CG_CUDA(cudaGetLastError());
    count_launch();
  }

 private:
  static constexpr int kT = 128;
  cudaStream_t s_;
  WCtx c_{};
  unsigned grid_ = 1;
  DBuf<double> e1_, v2_;
  DBuf<unsigned long long> mm_;
  DBuf<int8_t> m2_;
};

}  // namespace

std::unique_ptr<WideRows> wide_rows(const System& sys, const Operator& op, const Basis& b, cudaStream_t s) {
  if (!b.wide) throw Error(CG_ERR_INTERNAL, "wide rows of a bitstring basis");
  return std::make_unique<WideRowsImpl>(sys, op, b, s);
}

void basis_build_wide(const System& sys, Basis& b) {
  CG_CUDA(cudaGetDevice(&b.device));
  if (!b.stream) CG_CUDA(cudaStreamCreateWithFlags(&b.stream, cudaStreamNonBlocking));
  cudaStream_t s = b.stream;
  b.ns = int(sys.sps.size());
  b.nn = sys.n_neutron_states;
  b.np = b.ns - b.nn;
  b.kn = sys.nv;
  b.kp = sys.zv;
  b.twom = sys.twom;
  b.parity = sys.parity;
  b.wide = true;
  if (b.nn > 64 || b.np > 64) throw Error(CG_ERR_UNSUPPORTED, "more than 64 m-states per species");
  b.sp_m2.resize(b.ns);
  b.sp_par.resize(b.ns);
  std::vector<int> q(b.ns);
  for (int i = 0; i < b.ns; ++i) {
    b.sp_m2[i] = sys.sps[i].m2;
    b.sp_par[i] = sys.sps[i].parity;
    q[i] = sp_quanta(sys.sps[i]);
  }
  const Truncation& tr = sys.trunc;
  b.truncated = tr.active();
  const int R = int(tr.rejections.size());
  // SM::CoreQuanta: the quanta of the first Nv (Zv) s.p. states in list order
  int ncore = 0, pcore = 0;
  for (int i = 0; i < std::min(b.kn, b.nn); ++i) ncore += q[i];
  for (int i = 0; i < std::min(b.kp, b.np); ++i) pcore += q[b.nn + i];
  SpeciesEnum en, ep;
  en.norb = b.nn;
  en.k = b.kn;
  en.q = q.data();
  en.m2 = b.sp_m2.data();
  en.par = b.sp_par.data();
  ep.norb = b.np;
  ep.k = b.kp;
  ep.q = q.data() + b.nn;
  ep.m2 = b.sp_m2.data() + b.nn;
  ep.par = b.sp_par.data() + b.nn;
  if (tr.hw) {
    en.qlimit = ncore + tr.hwmax;
    ep.qlimit = pcore + tr.hwmax;
  }
  en.run();
  ep.run();

  // proton classes by (2m, parity), lexicographic inside
  std::map<std::pair<int, int>, std::vector<uint32_t>> cls;
  for (size_t i = 0; i < ep.mask.size(); ++i) cls[{ep.msum[i], ep.psum[i]}].push_back(uint32_t(i));
  b.h_wpuniv = ep.mask;
  b.h_wpuniv_rank.assign(ep.mask.size(), 0);
  b.h_wpuniv_csize.assign(ep.mask.size(), 0);
  for (auto& kv : cls)
    for (size_t r = 0; r < kv.second.size(); ++r) {
      b.h_wpuniv_rank[kv.second[r]] = uint32_t(r);
      b.h_wpuniv_csize[kv.second[r]] = uint32_t(kv.second.size());
    }
  // neutron blocks in lexicographic order, each with its list of allowed
  // proton configurations (the class itself when nothing is truncated)
  std::map<std::vector<int>, uint32_t> list_id;
  std::vector<std::vector<uint32_t>> lists;
  std::vector<uint64_t> bstart;
  std::vector<uint32_t> bclass;
  b.h_wbmask.clear();
  uint64_t off = 0;
  for (size_t i = 0; i < en.mask.size(); ++i) {
    const std::pair<int, int> ckey{b.twom - en.msum[i], b.parity ^ en.psum[i]};
    auto it = cls.find(ckey);
    if (it == cls.end()) continue;
    const int qn = en.qsum[i] - ncore;
    if (tr.hw && (qn < 0 || qn > tr.hwmax)) continue;
    std::vector<int> key{ckey.first, ckey.second, tr.hw ? qn : 0};
    for (int r = 0; r < R; ++r) key.push_back(__builtin_popcountll(en.mask[i] & tr.rejections[r].nmask));
    auto lit = list_id.find(key);
    if (lit == list_id.end()) {
      std::vector<uint32_t> keep;
      for (uint32_t li : it->second) {
        const int qp = ep.qsum[li] - pcore;
        if (tr.hw && (qp < 0 || qp > tr.hwmax || qn + qp < tr.hwmin || qn + qp > tr.hwmax)) continue;
        bool ok = true;
        for (int r = 0; r < R && ok; ++r) {
          const int c = key[3 + r] + __builtin_popcountll(ep.mask[li] & tr.rejections[r].pmask);
          ok = c >= tr.rejections[r].nmin && c <= tr.rejections[r].nmax;
        }
        if (ok) keep.push_back(li);
      }
      lit = list_id.emplace(key, uint32_t(lists.size())).first;
      lists.push_back(std::move(keep));
    }
    const std::vector<uint32_t>& lst = lists[lit->second];
    if (lst.empty()) continue;
    bstart.push_back(off);
    b.h_wbmask.push_back(en.mask[i]);
    bclass.push_back(lit->second);
    off += lst.size();
  }
  if (off >= (1ull << 32)) throw Error(CG_ERR_UNSUPPORTED, "dimension >= 2^32");
  b.n = off;
  std::vector<uint32_t> cstart;
  b.h_wcmask.clear();
  for (auto& l : lists) {
    cstart.push_back(uint32_t(b.h_wcmask.size()));
    for (uint32_t li : l) b.h_wcmask.push_back(ep.mask[li]);
  }
  cstart.push_back(uint32_t(b.h_wcmask.size()));
  b.h_bstart = bstart;
  b.h_bclass = bclass;
  b.h_cstart = cstart;
  b.h_bmask.clear();
  b.h_cmasks.clear();
  // locate tables: neutron block masks sorted, list members sorted per list
  const size_t nb = bstart.size();
  std::vector<uint32_t> ord(nb);
  std::iota(ord.begin(), ord.end(), 0u);
  std::sort(ord.begin(), ord.end(), [&](uint32_t x, uint32_t y) { return b.h_wbmask[x] < b.h_wbmask[y]; });
  b.h_wnkey.resize(nb);
  b.h_wnblk.resize(nb);
  for (size_t i = 0; i < nb; ++i) {
    b.h_wnkey[i] = b.h_wbmask[ord[i]];
    b.h_wnblk[i] = ord[i];
  }
  b.h_wpkey.resize(b.h_wcmask.size());
  b.h_wprank.resize(b.h_wcmask.size());
  for (size_t L = 0; L + 1 < cstart.size(); ++L) {
    const uint32_t a = cstart[L], e = cstart[L + 1];
    std::vector<uint32_t> r(e - a);
    std::iota(r.begin(), r.end(), 0u);
    std::sort(r.begin(), r.end(), [&](uint32_t x, uint32_t y) { return b.h_wcmask[a + x] < b.h_wcmask[a + y]; });
    for (uint32_t j = 0; j < e - a; ++j) {
      b.h_wpkey[a + j] = b.h_wcmask[a + r[j]];
      b.h_wprank[a + j] = r[j];
    }
  }
  auto up64 = [&](DBuf<uint64_t>& d, const std::vector<uint64_t>& h) {
    if (h.empty()) d.alloc(1); else d.upload(h, s);
  };
  auto up32 = [&](DBuf<uint32_t>& d, const std::vector<uint32_t>& h) {
    if (h.empty()) d.alloc(1); else d.upload(h, s);
  };
  up64(b.wbstart, bstart);
  up32(b.wbclass, bclass);
  up32(b.wcstart, cstart);
  up64(b.wnkey, b.h_wnkey);
  up32(b.wnblk, b.h_wnblk);
  up64(b.wpkey, b.h_wpkey);
  up32(b.wprank, b.h_wprank);
  b.wstate.alloc(std::max<uint64_t>(2 * b.n, 2));
  if (b.n) {
    DBuf<uint64_t> dbm, dcm;
    dbm.upload(b.h_wbmask, s);
    dcm.upload(b.h_wcmask, s);
    const int T = 256;
    k_wide_expand<<<unsigned((b.n + T - 1) / T), T, 0, s>>>(b.n, int(nb), b.wbstart.p, dbm.p, b.wbclass.p,
                                                           b.wcstart.p, dcm.p, b.wstate.p);
    CG_CUDA(cudaGetLastError());
    count_launch();
  }
  CG_CUDA(cudaStreamSynchronize(s));
}

void basis_tuples_wide(const Basis& b, uint64_t first, uint64_t count, uint16_t* out) {
  const int N = b.kn + b.kp;
  const uint64_t chunk = 1ull << 24;
  DBuf<uint16_t> d(std::max<uint64_t>(std::min(count, chunk) * std::max(N, 1), 1));
  for (uint64_t c0 = 0; c0 < count; c0 += chunk) {
    const uint64_t c = std::min(chunk, count - c0);
    const int T = 256;
    k_wide_tuples<<<unsigned((c + T - 1) / T), T, 0, b.stream>>>(first + c0, c, N, b.nn, b.wstate.p, d.p);
    CG_CUDA(cudaGetLastError());
    count_launch();
    CG_CUDA(cudaMemcpyAsync(out + c0 * N, d.p, c * N * sizeof(uint16_t), cudaMemcpyDeviceToHost, b.stream));
    CG_CUDA(cudaStreamSynchronize(b.stream));
  }
}

uint64_t basis_locate_wide_host(const Basis& b, const uint16_t* t) {
  const uint64_t miss = b.n + 1;
  const int N = b.kn + b.kp;
  uint64_t nmask = 0, pmask = 0;
  int kn = 0, kp = 0, m2 = 0, par = 0;
  for (int i = 0; i < N; ++i) {
    if (i && t[i] <= t[i - 1]) return miss;
    const int x = t[i];
    if (x >= b.ns) return miss;
    if (x < b.nn) { nmask |= 1ull << x; ++kn; }
    else { pmask |= 1ull << (x - b.nn); ++kp; }
    m2 += b.sp_m2[x];
    par ^= b.sp_par[x];
  }
  if (kn != b.kn || kp != b.kp || m2 != b.twom || par != b.parity) return miss;
  auto it = std::lower_bound(b.h_wnkey.begin(), b.h_wnkey.end(), nmask);
  if (it == b.h_wnkey.end() || *it != nmask) return miss;
  const uint32_t blk = b.h_wnblk[size_t(it - b.h_wnkey.begin())], L = b.h_bclass[blk];
  auto a = b.h_wpkey.begin() + b.h_cstart[L], e = b.h_wpkey.begin() + b.h_cstart[L + 1];
  auto jt = std::lower_bound(a, e, pmask);
  if (jt == e || *jt != pmask) return miss;
  return b.h_bstart[blk] + b.h_wprank[size_t(jt - b.h_wpkey.begin())];
}

void wide_onebody_partials(const Basis& parent, const Basis& daughter, const double* psid, int nq,
                           const double* psip, const int2* tif, const double* tv, int nt, double* part,
                           unsigned grid, int* err, cudaStream_t s) {
  if (!parent.wide || !daughter.wide) throw Error(CG_ERR_ARG, "both bases must use the wide representation");
  k_wide_onebody<<<grid, 256, 0, s>>>(locate_ctx(parent), daughter.wstate.p, daughter.n, psid, nq, psip, tif, tv, nt,
                                      part, err);
  CG_CUDA(cudaGetLastError());
  count_launch();
}

void wide_sf_partials(const Basis& parent, const Basis& daughter, const double* psid, int nq, const double* psip,
                      const int* sidx, int nsidx, double* part, unsigned grid, int* err, cudaStream_t s) {
  if (!parent.wide || !daughter.wide) throw Error(CG_ERR_ARG, "both bases must use the wide representation");
  k_wide_sf<<<dim3(grid, unsigned(nsidx)), 256, 0, s>>>(locate_ctx(parent), daughter.wstate.p, daughter.n, psid, nq,
                                                        psip, sidx, part, err);
  CG_CUDA(cudaGetLastError());
  count_launch();
}

void jt_expectations_wide(const System& sys, const Basis& b, const double* vecs, int nst, double* jj, double* tt) {
  const uint64_t n = b.n;
  auto expect = [&](const Operator& op, double* out) {
    for (int k = 0; k < nst; ++k) out[k] = 0.0;
    if (!n) return;
    Hamiltonian m;
    hamiltonian_build(sys, op, b, CG_PREC_FP64, m, false);
    std::vector<double> y(n * nst);
    spmm_host(m, CG_PREC_FP64, vecs, y.data(), nst);
    for (int k = 0; k < nst; ++k) {
      double acc = 0.0;
      for (uint64_t i = 0; i < n; ++i) acc += vecs[uint64_t(k) * n + i] * y[uint64_t(k) * n + i];
      out[k] = acc;
    }
  };
  expect(square_operator(j_plus_terms(sys.sps)), jj);
  if (sys.zv > 0 && sys.nv < b.nn) expect(square_operator(t_plus_terms(sys)), tt);
  else for (int k = 0; k < nst; ++k) tt[k] = 0.0;
}

}  // namespace cg
