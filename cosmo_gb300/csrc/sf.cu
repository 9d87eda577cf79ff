// Overlaps of one-body operators between two bases on the GPU:
// spectroscopic amplitudes <D_q| a_s |P_p> for one-particle removal, the
// overlaps the reference's XSHLSF takes (xmlshell/XSHLSF.cpp:150-175) with
// PPMatrix::OverlapNH and the one-body operator a_s (include/sm/
// PPMatrix.cxx:275-302); and transition amplitudes <D_q| sum v a+_f a_i |P_p>
// of XSHLEMB's electromagnetic and beta operators (xmlshell/XSHLEMB.cpp:
// 248-270); and the occupation numbers of XSHLAO.
//
// The reference applies a_s to every parent determinant (SM::Annihilation,
// include/sm/operators.cxx:121-150: phase of the number of states below s),
// locates the result in the daughter basis and sums y[ket] * x[bra].  Here it
// runs in pull form: one thread per daughter determinant D and one grid row
// per s.p. state s whose m, charge and parity take D into the parent's sector;
// the parent determinant P = D + s is located by the colex tables of the
// parent basis (per-list ranks for a truncated basis), and the thread
// accumulates sign * psi_parent[P] * psi_daughter[D, q] for every daughter
// state q.  Per-CTA sums are added on the host in a fixed order.
#include <cmath>

#include "device.h"
#include "em.h"

namespace cg {

namespace {

constexpr int kMaxDaughter = 16;

__device__ __forceinline__ uint64_t below_sf(int b) { return b >= 64 ? ~0ull : (1ull << b) - 1ull; }

__device__ __forceinline__ uint64_t colex_sf(uint64_t mask, const uint64_t* binom) {
  uint64_t r = 0;
  int i = 1;
  while (mask) {
    const int c = __ffsll((long long)mask) - 1;
    r += binom[c * kBinom + i];
    ++i;
    mask &= mask - 1;
  }
  return r;
}

struct SfArgs {
  uint64_t nd;               // daughter dimension
  const uint64_t* dstate;    // daughter determinants (neutron bits low)
  const double* psid;        // daughter vectors, row-interleaved (row * nq + q)
  int nq;
  int nn;                    // neutron s.p. states
  uint64_t nall;             // neutron mask
  uint64_t np_;              // parent dimension
  const uint64_t* noff;      // parent basis: neutron block offsets by colex rank
  const uint32_t* pcrank;    // parent basis: proton rank by colex rank
  const uint32_t* nlist;     // truncated parent basis: list of each neutron block (null otherwise)
  const uint32_t* lrank;     // truncated parent basis: rank inside a list by proton colex rank
  uint64_t npc;
  const uint64_t* binom;
  const double* psip;        // one parent vector
  const int* sidx;           // the s.p. states of the grid rows
};

__global__ void k_sf_amplitudes(SfArgs a, double* __restrict__ part, int* __restrict__ err) {
  __shared__ double red[kMaxDaughter][256 / 32];
  const int s = a.sidx[blockIdx.y];
  double acc[kMaxDaughter];
#pragma unroll
  for (int q = 0; q < kMaxDaughter; ++q) acc[q] = 0.0;
  for (uint64_t row = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; row < a.nd;
       row += uint64_t(gridDim.x) * blockDim.x) {
    const uint64_t D = a.dstate[row];
    if ((D >> s) & 1) continue;
    const uint64_t P = D | (1ull << s);
    const uint64_t cn = colex_sf(P & a.nall, a.binom);
    const uint64_t off = a.noff[cn];
    if (off == ~0ull) continue;
    uint64_t idx;
    if (a.nlist) {  // truncated parent basis: a determinant outside it has amplitude 0
      const uint32_t r = a.lrank[uint64_t(a.nlist[cn]) * a.npc + colex_sf(P >> a.nn, a.binom)];
      if (r == ~0u) continue;
      idx = off + r;
    } else {
      idx = off + a.pcrank[colex_sf(P >> a.nn, a.binom)];
    }
    if (idx >= a.np_) { atomicOr(err, 1); continue; }
    const double c = ((__popcll(D & below_sf(s)) & 1) ? -1.0 : 1.0) * a.psip[idx];
#pragma unroll
    for (int q = 0; q < kMaxDaughter; ++q)
      if (q < a.nq) acc[q] += c * a.psid[row * a.nq + q];
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < kMaxDaughter; ++q) {
    double v = acc[q];
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(~0u, v, o);
    if (lane == 0) red[q][w] = v;
  }
  __syncthreads();
  if (threadIdx.x < kMaxDaughter) {
    double v = 0.0;
    for (int i = 0; i < int(blockDim.x >> 5); ++i) v += red[threadIdx.x][i];
    part[(size_t(blockIdx.y) * gridDim.x + blockIdx.x) * kMaxDaughter + threadIdx.x] = v;
  }
}

__global__ void k_rows_sf(uint64_t n, int nst, const double* __restrict__ src, double* __restrict__ dst) {
  const uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i >= n * nst) return;
  const uint64_t r = i / nst;
  const int k = int(i - r * nst);
  dst[i] = src[uint64_t(k) * n + r];
}

// <D_q| sum_t v_t a+_f a_i |P> for one parent vector: one thread per
// daughter determinant D and every term t whose f is occupied in D and whose
// i is free in D - f (or i = f); the parent determinant P = D - f + i is
// located by the colex tables of the parent basis and the phase is that of
// a+_f a_i acting on P (states below i in P, then below f in P - i).
struct ObArgs {
  uint64_t nd;
  const uint64_t* dstate;
  const double* psid;
  int nq;
  int nn;
  uint64_t nall;
  uint64_t np_;
  const uint64_t* noff;
  const uint32_t* pcrank;
  const uint32_t* nlist;
  const uint32_t* lrank;
  uint64_t npc;
  const uint64_t* binom;
  const double* psip;
  const int2* tif;  // per term: i, f
  const double* tv;  // per term: value
  int nt;
};

__global__ void k_onebody_amplitudes(ObArgs a, double* __restrict__ part, int* __restrict__ err) {
  __shared__ double red[kMaxDaughter][256 / 32];
  double acc[kMaxDaughter];
#pragma unroll
  for (int q = 0; q < kMaxDaughter; ++q) acc[q] = 0.0;
  for (uint64_t row = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; row < a.nd;
       row += uint64_t(gridDim.x) * blockDim.x) {
    const uint64_t D = a.dstate[row];
    double w = 0.0;
    for (int t = 0; t < a.nt; ++t) {
      const int2 e = a.tif[t];
      if (!((D >> e.y) & 1)) continue;
      const uint64_t Df = D & ~(1ull << e.y);
      if (e.x != e.y && ((Df >> e.x) & 1)) continue;
      const uint64_t P = Df | (1ull << e.x);
      const uint64_t cn = colex_sf(P & a.nall, a.binom);
      const uint64_t off = a.noff[cn];
      if (off == ~0ull) continue;
      uint64_t idx;
      if (a.nlist) {
        const uint32_t r = a.lrank[uint64_t(a.nlist[cn]) * a.npc + colex_sf(P >> a.nn, a.binom)];
        if (r == ~0u) continue;
        idx = off + r;
      } else {
        idx = off + a.pcrank[colex_sf(P >> a.nn, a.binom)];
      }
      if (idx >= a.np_) { atomicOr(err, 1); continue; }
      const int ph = __popcll(P & below_sf(e.x)) + __popcll(Df & below_sf(e.y));
      const double v = a.tv[t] * a.psip[idx];
      w += (ph & 1) ? -v : v;
    }
#pragma unroll
    for (int q = 0; q < kMaxDaughter; ++q)
      if (q < a.nq) acc[q] += w * a.psid[row * a.nq + q];
  }
  const int lane = threadIdx.x & 31, wi = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < kMaxDaughter; ++q) {
    double v = acc[q];
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(~0u, v, o);
    if (lane == 0) red[q][wi] = v;
  }
  __syncthreads();
  if (threadIdx.x < kMaxDaughter) {
    double v = 0.0;
    for (int i = 0; i < int(blockDim.x >> 5); ++i) v += red[threadIdx.x][i];
    part[size_t(blockIdx.x) * kMaxDaughter + threadIdx.x] = v;
  }
}

// Occupation numbers <psi| n_s |psi> = sum over determinants holding s of
// psi_D^2 (SM::occupation, include/sm/occupation.cxx:55-70): one thread per
// determinant adds psi_D^2 to a per-CTA shared row of s.p. states for each of
// its set bits; the CTA rows are summed on the host.
__global__ void k_occupations(uint64_t n, const uint64_t* __restrict__ state, const double* __restrict__ psi, int ns,
                              double* __restrict__ part) {
  __shared__ double occ[64];
  for (int i = threadIdx.x; i < 64; i += blockDim.x) occ[i] = 0.0;
  __syncthreads();
  for (uint64_t row = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; row < n;
       row += uint64_t(gridDim.x) * blockDim.x) {
    const double p = psi[row] * psi[row];
    for (uint64_t D = state[row]; D; D &= D - 1) atomicAdd(&occ[__ffsll((long long)D) - 1], p);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < ns; i += blockDim.x) part[size_t(blockIdx.x) * 64 + i] = occ[i];
}

// The same on a wide basis: determinants as (neutron, proton) 64-bit masks,
// proton s.p. state j at index nn + j, CTA rows of 128 s.p. states.
__global__ void k_occupations_wide(uint64_t n, const uint64_t* __restrict__ wstate, const double* __restrict__ psi,
                                   int ns, int nn, double* __restrict__ part) {
  __shared__ double occ[128];
  for (int i = threadIdx.x; i < 128; i += blockDim.x) occ[i] = 0.0;
  __syncthreads();
  for (uint64_t row = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; row < n;
       row += uint64_t(gridDim.x) * blockDim.x) {
    const double p = psi[row] * psi[row];
    for (uint64_t D = wstate[2 * row]; D; D &= D - 1) atomicAdd(&occ[__ffsll((long long)D) - 1], p);
    for (uint64_t D = wstate[2 * row + 1]; D; D &= D - 1) atomicAdd(&occ[nn + __ffsll((long long)D) - 1], p);
  }
  __syncthreads();
  for (int i = threadIdx.x; i < ns; i += blockDim.x) part[size_t(blockIdx.x) * 128 + i] = occ[i];
}

}  // namespace

void occupations(const Basis& b, const double* v, int nst, double* occ) {
  const int ns = b.ns;
  for (size_t i = 0; i < size_t(nst) * ns; ++i) occ[i] = 0.0;
  if (b.n == 0 || nst < 1) return;
  cudaStream_t st = b.stream;
  const unsigned gx = unsigned(std::min<uint64_t>((b.n + 255) / 256, 152ull * 4));
  const int stride = b.wide ? 128 : 64;
  DBuf<double> psi(b.n), part(size_t(gx) * stride);
  std::vector<double> h(part.n);
  for (int k = 0; k < nst; ++k) {
    psi.upload(v + uint64_t(k) * b.n, b.n, st);
    if (b.wide) k_occupations_wide<<<gx, 256, 0, st>>>(b.n, b.wstate.p, psi.p, ns, b.nn, part.p);
    else k_occupations<<<gx, 256, 0, st>>>(b.n, b.state.p, psi.p, ns, part.p);
    CG_CUDA(cudaGetLastError());
    count_launch();
    CG_CUDA(cudaMemcpyAsync(h.data(), part.p, h.size() * 8, cudaMemcpyDeviceToHost, st));
    CG_CUDA(cudaStreamSynchronize(st));
    for (unsigned g = 0; g < gx; ++g)
      for (int s = 0; s < ns; ++s) occ[size_t(k) * ns + s] += h[size_t(g) * stride + s];
  }
}

void onebody_amplitudes(const System& psys, const Basis& parent, const double* vp, int np, const Basis& daughter,
                        const double* vd, int nd, const std::vector<OneBodyTerm>& terms, double* amp) {
  if (np < 1 || nd < 1 || nd > kMaxDaughter) throw Error(CG_ERR_ARG, "1..16 daughter states, at least one parent state");
  if (parent.wide != daughter.wide) throw Error(CG_ERR_ARG, "parent and daughter bases of different representations");
  if (parent.ns != daughter.ns || parent.nn != daughter.nn)
    throw Error(CG_ERR_ARG, "parent and daughter bases have different valence spaces");
  if (parent.kn + parent.kp != daughter.kn + daughter.kp)
    throw Error(CG_ERR_ARG, "a one-body operator keeps the number of particles");
  const int ns = parent.ns;
  for (size_t i = 0; i < size_t(nd) * np; ++i) amp[i] = 0.0;
  // the terms that take the daughter's sector into the parent's (species
  // change, m and parity), so that P = D - f + i is always in the parent's
  // sector and its colex ranks cannot alias another sector's
  const int dn = parent.kn - daughter.kn;  // +1: a neutron becomes a proton
  std::vector<int2> tif;
  std::vector<double> tv;
  for (const OneBodyTerm& t : terms) {
    if (t.i < 0 || t.i >= ns || t.f < 0 || t.f >= ns) throw Error(CG_ERR_ARG, "one-body term outside the s.p. states");
    const bool in_ = t.i < parent.nn, fn = t.f < parent.nn;
    if (int(in_) - int(fn) != dn) continue;
    const SPState &si = psys.sps[t.i], &sf = psys.sps[t.f];
    if (sf.m2 - si.m2 != daughter.twom - parent.twom) continue;
    if ((sf.parity ^ si.parity) != (daughter.parity ^ parent.parity)) continue;
    if (t.v == 0.0) continue;
    tif.push_back(make_int2(t.i, t.f));
    tv.push_back(t.v);
  }
  if (tif.empty() || daughter.n == 0 || parent.n == 0) return;
  cudaStream_t st = parent.stream;
  DBuf<double> dcm(daughter.n * nd), psid(daughter.n * nd), pv(parent.n);
  dcm.upload(vd, daughter.n * nd, st);
  k_rows_sf<<<unsigned((daughter.n * nd + 255) / 256), 256, 0, st>>>(daughter.n, nd, dcm.p, psid.p);
  CG_CUDA(cudaGetLastError());
  count_launch();
  DBuf<int2> dtif;
  DBuf<double> dtv;
  DBuf<int> err(1);
  dtif.upload(tif, st);
  dtv.upload(tv, st);
  CG_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), st));
  ObArgs a;
  a.nd = daughter.n;
  a.dstate = daughter.state.p;
  a.psid = psid.p;
  a.nq = nd;
  a.nn = parent.nn;
  a.nall = parent.nn ? ((parent.nn == 64) ? ~0ull : ((1ull << parent.nn) - 1)) : 0;
  a.np_ = parent.n;
  a.noff = parent.noff.p;
  a.pcrank = parent.pcrank.p;
  a.nlist = parent.truncated ? parent.nlist.p : nullptr;
  a.lrank = parent.truncated ? parent.lrank.p : nullptr;
  a.npc = parent.npc;
  a.binom = parent.binom.p;
  a.tif = dtif.p;
  a.tv = dtv.p;
  a.nt = int(tif.size());
  const int T = 256;
  const unsigned gx = unsigned(std::min<uint64_t>((daughter.n + T - 1) / T, 152ull * 4));
  DBuf<double> part(size_t(gx) * kMaxDaughter);
  std::vector<double> h(part.n);
  for (int p = 0; p < np; ++p) {
    pv.upload(vp + uint64_t(p) * parent.n, parent.n, st);
    a.psip = pv.p;
    if (parent.wide) {
      wide_onebody_partials(parent, daughter, psid.p, nd, pv.p, dtif.p, dtv.p, a.nt, part.p, gx, err.p, st);
    } else {
      k_onebody_amplitudes<<<gx, T, 0, st>>>(a, part.p, err.p);
      CG_CUDA(cudaGetLastError());
      count_launch();
    }
    CG_CUDA(cudaMemcpyAsync(h.data(), part.p, h.size() * 8, cudaMemcpyDeviceToHost, st));
    CG_CUDA(cudaStreamSynchronize(st));
    for (unsigned g = 0; g < gx; ++g)
      for (int q = 0; q < nd; ++q) amp[size_t(q) * np + p] += h[size_t(g) * kMaxDaughter + q];
  }
  int herr = 0;
  CG_CUDA(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  CG_CUDA(cudaStreamSynchronize(st));
  if (herr) throw Error(CG_ERR_INTERNAL, "a one-body move left the parent basis");
}

void sf_amplitudes(const System& psys, const Basis& parent, const double* vp, int np, const Basis& daughter,
                   const double* vd, int nd, double* amp) {
  if (np < 1 || nd < 1 || nd > kMaxDaughter) throw Error(CG_ERR_ARG, "1..16 daughter states, at least one parent state");
  if (parent.wide != daughter.wide) throw Error(CG_ERR_ARG, "parent and daughter bases of different representations");
  if (parent.ns != daughter.ns || parent.nn != daughter.nn)
    throw Error(CG_ERR_ARG, "parent and daughter bases have different valence spaces");
  const int ns = parent.ns;
  const bool extra_n = parent.kn == daughter.kn + 1 && parent.kp == daughter.kp;
  const bool extra_p = parent.kp == daughter.kp + 1 && parent.kn == daughter.kn;
  if (!extra_n && !extra_p) throw Error(CG_ERR_ARG, "the parent must hold one particle more than the daughter");
  for (size_t i = 0; i < size_t(nd) * np * ns; ++i) amp[i] = 0.0;
  // s.p. states that take the daughter's sector into the parent's
  std::vector<int> sidx;
  for (int s = extra_n ? 0 : parent.nn; s < (extra_n ? parent.nn : ns); ++s)
    if (psys.sps[s].m2 == parent.twom - daughter.twom && (psys.sps[s].parity ^ daughter.parity) == parent.parity)
      sidx.push_back(s);
  if (sidx.empty() || daughter.n == 0 || parent.n == 0) return;
  cudaStream_t st = parent.stream;
  DBuf<double> dcm(daughter.n * nd), psid(daughter.n * nd), pv(parent.n);
  dcm.upload(vd, daughter.n * nd, st);
  k_rows_sf<<<unsigned((daughter.n * nd + 255) / 256), 256, 0, st>>>(daughter.n, nd, dcm.p, psid.p);
  CG_CUDA(cudaGetLastError());
  count_launch();
  DBuf<int> dsidx, err(1);
  dsidx.upload(sidx, st);
  CG_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), st));
  SfArgs a;
  a.nd = daughter.n;
  a.dstate = daughter.state.p;
  a.psid = psid.p;
  a.nq = nd;
  a.nn = parent.nn;
  a.nall = parent.nn ? ((parent.nn == 64) ? ~0ull : ((1ull << parent.nn) - 1)) : 0;
  a.np_ = parent.n;
  a.noff = parent.noff.p;
  a.pcrank = parent.pcrank.p;
  a.nlist = parent.truncated ? parent.nlist.p : nullptr;
  a.lrank = parent.truncated ? parent.lrank.p : nullptr;
  a.npc = parent.npc;
  a.binom = parent.binom.p;
  a.sidx = dsidx.p;
  const int T = 256;
  const unsigned gx = unsigned(std::min<uint64_t>((daughter.n + T - 1) / T, 152ull * 4));
  const dim3 grid(gx, unsigned(sidx.size()));
  DBuf<double> part(size_t(gx) * sidx.size() * kMaxDaughter);
  std::vector<double> h(part.n);
  for (int p = 0; p < np; ++p) {
    pv.upload(vp + uint64_t(p) * parent.n, parent.n, st);
    a.psip = pv.p;
    if (parent.wide) {
      wide_sf_partials(parent, daughter, psid.p, nd, pv.p, dsidx.p, int(sidx.size()), part.p, gx, err.p, st);
    } else {
      k_sf_amplitudes<<<grid, T, 0, st>>>(a, part.p, err.p);
      CG_CUDA(cudaGetLastError());
      count_launch();
    }
    CG_CUDA(cudaMemcpyAsync(h.data(), part.p, h.size() * 8, cudaMemcpyDeviceToHost, st));
    CG_CUDA(cudaStreamSynchronize(st));
    for (size_t y = 0; y < sidx.size(); ++y)
      for (unsigned g = 0; g < gx; ++g)
        for (int q = 0; q < nd; ++q)
          amp[(size_t(q) * np + p) * ns + sidx[y]] += h[(y * gx + g) * kMaxDaughter + q];
  }
  int herr = 0;
  CG_CUDA(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, st));
  CG_CUDA(cudaStreamSynchronize(st));
  if (herr) throw Error(CG_ERR_INTERNAL, "a + s left the parent basis");
}

}  // namespace cg
