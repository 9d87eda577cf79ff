// <J-J+> and <T-T+> of eigenvectors on the GPU (the reference's XSHLJT,
// include/xsm/XSHLJT.cxx:38-142).
//
// The reference builds the one-body raising operators J+ (SPJPlus: same orbit
// and species, m -> m + 1, value sqrt((j - m)(j + m + 1)))) and T+ (SPTPlus:
// same orbit and m, proton -> neutron, value 1; include/sm/spherical2sp.cxx:
// 629-700), applies each to the state vector bra by bra into a map of final
// determinants and takes the squared norm (PPMatrix::Sqr,
// include/sm/PPMatrix.cxx:403-411).  Here the image O psi is formed in pull
// form on the GPU: the target basis (2M + 2, or one proton turned into a
// neutron) is enumerated, and each target determinant K sums over the
// particles that O could have moved into it: S = K with y replaced by its
// lower partner x, coefficient * fermion phase of a+_y a_x on S * psi[S].  One
// thread per target row, every state vector at once; per-CTA partial sums of
// the squares are added on the host in a fixed order.
#include <cmath>

#include "device.h"

namespace cg {

namespace {

constexpr int kMaxStates = 16;

__device__ __forceinline__ uint64_t bel(int b) { return b >= 64 ? ~0ull : (1ull << b) - 1ull; }

__device__ __forceinline__ uint64_t colex_d(uint64_t mask, const uint64_t* binom) {
  uint64_t r = 0;
  int i = 1;
  while (mask) {
    int c = __ffsll((long long)mask) - 1;
    r += binom[c * kBinom + i];
    ++i;
    mask &= mask - 1;
  }
  return r;
}

struct RaiseArgs {
  uint64_t nt;               // target dimension
  const uint64_t* tstate;    // target determinants (neutron bits low)
  int nn;                    // neutron s.p. states
  uint64_t nall;             // neutron mask
  uint64_t ns_src;           // source dimension
  const uint64_t* noff;      // source basis: neutron block offsets by colex rank
  const uint32_t* pcrank;    // source basis: proton rank by colex rank
  const uint32_t* nlist;     // truncated source basis: list of each neutron block (null otherwise)
  const uint32_t* lrank;     // truncated source basis: rank inside a list by proton colex rank
  uint64_t npc;
  const uint64_t* binom;
  const int8_t* partner;     // per s.p. y: the x that O moves into y, -1 if none
  const double* coef;        // per s.p. y: the operator value for x -> y
  const double* psi;         // source vectors, row-interleaved (row * nst + k)
  int nst;
};

__global__ void k_raise_norm(RaiseArgs a, double* __restrict__ part, int* __restrict__ err) {
  __shared__ double red[kMaxStates][256 / 32];
  double acc[kMaxStates];
#pragma unroll
  for (int k = 0; k < kMaxStates; ++k) acc[k] = 0.0;
  for (uint64_t row = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; row < a.nt;
       row += uint64_t(gridDim.x) * blockDim.x) {
    const uint64_t K = a.tstate[row];
    double v[kMaxStates];
#pragma unroll
    for (int k = 0; k < kMaxStates; ++k) v[k] = 0.0;
    for (uint64_t t = K; t; t &= t - 1) {
      const int y = __ffsll((long long)t) - 1;
      const int x = a.partner[y];
      if (x < 0 || ((K >> x) & 1)) continue;
      const uint64_t S = K ^ (1ull << y) ^ (1ull << x);
      const uint64_t cn = colex_d(S & a.nall, a.binom);
      const uint64_t off = a.noff[cn];
      uint64_t idx;
      if (a.nlist) {  // truncated source basis: a source outside it has amplitude 0
        if (off == ~0ull) continue;
        const uint32_t r = a.lrank[uint64_t(a.nlist[cn]) * a.npc + colex_d(S >> a.nn, a.binom)];
        if (r == ~0u) continue;
        idx = off + r;
      } else {
        idx = off == ~0ull ? ~0ull : off + a.pcrank[colex_d(S >> a.nn, a.binom)];
      }
      if (idx >= a.ns_src) { atomicOr(err, 1); continue; }
      const int p = __popcll(S & bel(x)) + __popcll((S & ~(1ull << x)) & bel(y));
      const double c = (p & 1) ? -a.coef[y] : a.coef[y];
#pragma unroll
      for (int k = 0; k < kMaxStates; ++k)
        if (k < a.nst) v[k] += c * a.psi[idx * a.nst + k];
    }
#pragma unroll
    for (int k = 0; k < kMaxStates; ++k) acc[k] += v[k] * v[k];
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < kMaxStates; ++k) {
    double s = acc[k];
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(~0u, s, o);
    if (lane == 0) red[k][w] = s;
  }
  __syncthreads();
  if (threadIdx.x < kMaxStates) {
    double s = 0.0;
    for (int i = 0; i < int(blockDim.x >> 5); ++i) s += red[threadIdx.x][i];
    part[size_t(blockIdx.x) * kMaxStates + threadIdx.x] = s;
  }
}

__global__ void k_rows_of(uint64_t n, int nst, const double* __restrict__ src, double* __restrict__ dst) {
  uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i >= n * nst) return;
  uint64_t r = i / nst;
  int k = int(i - r * nst);
  dst[i] = src[uint64_t(k) * n + r];
}

// ||O psi_k||^2 for every state; O described by partner/coef; target basis tb.
void raise_norms(const Basis& src, const Basis& tb, const std::vector<int8_t>& partner, const std::vector<double>& coef,
                 const DBuf<double>& psi, int nst, double* out, cudaStream_t s) {
  for (int k = 0; k < nst; ++k) out[k] = 0.0;
  if (tb.n == 0) return;
  DBuf<int8_t> dpart;
  DBuf<double> dcoef;
  dpart.upload(partner, s);
  dcoef.upload(coef, s);
  RaiseArgs a;
  a.nt = tb.n;
  a.tstate = tb.state.p;
  a.nn = src.nn;
  a.nall = src.nn ? ((src.nn == 64) ? ~0ull : ((1ull << src.nn) - 1)) : 0;
  a.ns_src = src.n;
  a.noff = src.noff.p;
  a.pcrank = src.pcrank.p;
  a.nlist = src.truncated ? src.nlist.p : nullptr;
  a.lrank = src.truncated ? src.lrank.p : nullptr;
  a.npc = src.npc;
  a.binom = src.binom.p;
  a.partner = dpart.p;
  a.coef = dcoef.p;
  a.psi = psi.p;
  a.nst = nst;
  const int T = 256;
  const unsigned grid = unsigned(std::min<uint64_t>((tb.n + T - 1) / T, 152ull * 8));
  DBuf<double> part(size_t(grid) * kMaxStates);
  DBuf<int> err(1);
  CG_CUDA(cudaMemsetAsync(err.p, 0, sizeof(int), s));
  k_raise_norm<<<grid, T, 0, s>>>(a, part.p, err.p);
  CG_CUDA(cudaGetLastError());
  count_launch();
  std::vector<double> h(size_t(grid) * kMaxStates);
  int herr = 0;
  CG_CUDA(cudaMemcpyAsync(h.data(), part.p, h.size() * 8, cudaMemcpyDeviceToHost, s));
  CG_CUDA(cudaMemcpyAsync(&herr, err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
  CG_CUDA(cudaStreamSynchronize(s));
  if (herr) throw Error(CG_ERR_INTERNAL, "raising operator left the source basis");
  for (unsigned g = 0; g < grid; ++g)
    for (int k = 0; k < nst; ++k) out[k] += h[size_t(g) * kMaxStates + k];
}

}  // namespace

void jt_expectations(const System& sys, const Basis& b, const double* vecs, int nst, double* jj, double* tt) {
  if (nst < 1 || nst > kMaxStates) throw Error(CG_ERR_ARG, "1..16 states per call");
  if (b.wide) {
    jt_expectations_wide(sys, b, vecs, nst, jj, tt);
    return;
  }
  cudaStream_t s = b.stream;
  const uint64_t n = b.n;
  const int ns = b.ns, nn = b.nn;
  DBuf<double> cm(n * nst), psi(n * nst);
  cm.upload(vecs, n * nst, s);
  if (n) {
    k_rows_of<<<unsigned((n * nst + 255) / 256), 256, 0, s>>>(n, nst, cm.p, psi.p);
    CG_CUDA(cudaGetLastError());
    count_launch();
  }
  // J+: a+_{m+1} a_m within one orbit and species, sqrt((j - m)(j + m + 2)) / 2 in doubled units
  {
    std::vector<int8_t> partner(64, -1);
    std::vector<double> coef(64, 0.0);
    for (int y = 0; y < ns; ++y)
      for (int x = 0; x < ns; ++x) {
        const SPState &X = sys.sps[x], &Y = sys.sps[y];
        if (X.level == Y.level && X.tz2 == Y.tz2 && X.m2 + 2 == Y.m2) {
          partner[y] = int8_t(x);
          coef[y] = std::sqrt(double(X.j2 - X.m2) * double(X.j2 + X.m2 + 2)) / 2.0;
        }
      }
    System st = sys;
    st.twom = sys.twom + 2;
    Basis tb;
    basis_build(st, tb);
    raise_norms(b, tb, partner, coef, psi, nst, jj, s);
  }
  // T+: proton -> neutron in the same orbit and m, value 1
  {
    for (int k = 0; k < nst; ++k) tt[k] = 0.0;
    if (sys.zv > 0 && sys.nv < nn) {
      std::vector<int8_t> partner(64, -1);
      std::vector<double> coef(64, 0.0);
      for (int y = 0; y < nn; ++y)
        for (int x = nn; x < ns; ++x) {
          const SPState &X = sys.sps[x], &Y = sys.sps[y];
          if (X.level == Y.level && X.m2 == Y.m2 && X.n == Y.n && X.l == Y.l && X.j2 == Y.j2 &&
              X.parity == Y.parity && X.t2 == Y.t2 && X.tz2 + 2 == Y.tz2) {
            partner[y] = int8_t(x);
            coef[y] = std::sqrt(double(X.t2 - X.tz2) * double(X.t2 + X.tz2 + 2)) / 2.0;
          }
        }
      System st = sys;
      st.nv = sys.nv + 1;
      st.zv = sys.zv - 1;
      Basis tb;
      basis_build(st, tb);
      raise_norms(b, tb, partner, coef, psi, nst, tt, s);
    }
  }
}

int jj_spin(double x, int two_m) {
  // 2J from <J-J+> = J(J+1) - M(M+1): 2J = sqrt(4x + 2M(2M+2) + 1) - 1, accepted when J + M is an
  // integer within 0.1 (SM::JJSpin, include/sm/QN.cxx:40-60)
  const double s2 = std::sqrt(4.0 * x + double(two_m) * double(two_m + 2) + 1.0) - 1.0;
  const double t = 0.5 * (s2 + double(two_m));
  if (std::fabs(t - std::round(t)) < 0.1) return int(std::lround(s2));
  return -1;
}

}  // namespace cg
