// H + lambda * J-J+ builder on the GPU (count -> scan -> fill -> per-row sort).
//
// The reference builds each upper-triangle row by applying every operator term
// to the bra (SM::ActFermiOperator, include/sm/cioperators.cxx:36-62), summing
// into a map keyed by the final determinant, locating it in the basis upward
// from the bra (SM::locate, include/sm/ManyBodyStates.cxx:92) and dropping
// |value| < 1e-14 (PPMatrix2CSBBlk, include/sm/PPMatrix.cxx:571-656, :621).
//
// Here one thread owns one row and enumerates the determinants it connects to
// by at most two particle-hole moves, per species, with bitstring arithmetic:
//   diagonal; one particle moved a -> f (same species, same m) with every other
//   occupied orbital as spectator; two same-species particles moved; one
//   neutron and one proton moved.
// Every element is evaluated from the lower-index determinant of the pair with
// the forward-ordered terms (the upper-triangle convention of the reference),
// so both triangles are written from the same FP64 number and the upper
// triangle equals the reference's row.  The fermionic phase of a term
// (b0 < b1 annihilated, b2 < b3 created) applied to occupation S is
//   parity(#S below b0 + #S below b1 - 1 + #I below b2 + #I below b3),
// I = S without b0, b1, which is what SM::Annihilation / SM::Creation
// (include/sm/operators.cxx:121-187) accumulate.  Terms of one element are
// summed in the reference's operator order: one-body term first, then the
// two-body terms with the spectator ascending.
#include <algorithm>
#include <chrono>

#include "device.h"
#include "tiled.h"

namespace cg {

Hamiltonian::~Hamiltonian() {
  if (stream) cudaStreamDestroy(stream);
}

void upload_operator(const System& sys, const Operator& op, DevOperator& d, cudaStream_t s) {
  const int ns = int(sys.sps.size());
  d.ns = ns;
  std::vector<int32_t> pidx(ns * ns, -1);
  int np = 0;
  for (int a = 0; a < ns; ++a)
    for (int b = a + 1; b < ns; ++b) pidx[a * ns + b] = np++;
  d.npairs = np;
  std::vector<double> e1(ns * ns, 0.0);
  for (auto& kv : op.one) {
    int i = kv.first[0], f = kv.first[1];
    if (i < 0 || f < 0 || i >= ns || f >= ns) throw Error(CG_ERR_INTERNAL, "one-body key out of range");
    e1[i * ns + f] = kv.second;
  }
  std::vector<double> v2(size_t(std::max(np, 1)) * std::max(np, 1), 0.0);
  for (auto& kv : op.two) {
    const Key4& k = kv.first;
    // keys with a repeated index can never act on a determinant (the
    // reference's Annihilation/locate reject them), so they carry no element
    if (k[0] >= k[1] || k[2] >= k[3]) continue;
    v2[size_t(pidx[k[0] * ns + k[1]]) * np + pidx[k[2] * ns + k[3]]] = kv.second;
  }
  std::vector<uint64_t> mm(2 * (2 * kMOff + 1), 0);
  for (int i = 0; i < ns; ++i) {
    int sp = i < sys.n_neutron_states ? 0 : 1;
    int m = sys.sps[i].m2;
    if (m < -kMOff || m > kMOff) throw Error(CG_ERR_UNSUPPORTED, "|2m| too large");
    mm[sp * (2 * kMOff + 1) + m + kMOff] |= 1ull << i;
  }
  d.e1.upload(e1, s);
  d.v2.upload(v2, s);
  d.pidx.upload(pidx, s);
  d.mmask.upload(mm, s);
}

namespace {

struct Ctx {
  int ns, nn, npairs;
  uint64_t nall;     // mask of neutron s.p. states
  uint64_t pall;     // mask of proton s.p. states (global bits)
  uint64_t n;
  const uint64_t* state;
  const uint64_t* noff;
  const uint32_t* pcrank;
  const uint32_t* nlist;  // truncated basis: list of each neutron block (null when not truncated)
  const uint32_t* lrank;  // truncated basis: rank inside a list by proton colex rank, ~0u if absent
  uint64_t npc;
  const double* e1;
  const double* v2;
  const uint64_t* mmask;
  const int8_t* m2;  // per s.p. (device)
};

constexpr double kDrop = 1e-14;

struct Shared {
  uint64_t binom[33 * 33];  // C(a, b), a, b <= 32
  int16_t pidx[64 * 64];
  int8_t m2[64];
  uint64_t mmask[2 * (2 * kMOff + 1)];
};

__device__ __forceinline__ uint64_t below(int b) { return b >= 64 ? ~0ull : (1ull << b) - 1ull; }

__device__ __forceinline__ uint64_t colex(uint64_t mask, const uint64_t* binom) {
  uint64_t r = 0;
  int i = 1;
  while (mask) {
    int c = __ffsll((long long)mask) - 1;
    r += binom[c * 33 + i];
    ++i;
    mask &= mask - 1;
  }
  return r;
}

// Index of determinant K.  In an untruncated basis an M- and parity-conserving
// operator never leaves it, so ~0 marks an internal error the caller flags; a
// truncated basis drops the determinants outside it (kOutside: the matrix is
// the operator projected on the basis, as the reference's PPMatrix2CSBBlk
// skips a ket that SM::locate does not find, include/sm/PPMatrix.cxx:571-656).
constexpr uint64_t kOutside = ~0ull - 1;
__device__ __forceinline__ uint64_t ket_index(const Ctx& c, const Shared& sh, uint64_t K) {
  uint64_t kn = K & c.nall, kp = K >> c.nn;
  const uint64_t cn = colex(kn, sh.binom);
  uint64_t off = c.noff[cn];
  if (c.nlist) {
    if (off == ~0ull) return kOutside;
    const uint32_t r = c.lrank[uint64_t(c.nlist[cn]) * c.npc + colex(kp, sh.binom)];
    return r == ~0u ? kOutside : off + r;
  }
  if (off == ~0ull) return ~0ull;
  uint64_t idx = off + c.pcrank[colex(kp, sh.binom)];
  return idx < c.n ? idx : ~0ull;
}

// forward two-body term (b0 < b1 annihilated, b2 < b3 created) on S0
__device__ __forceinline__ double term2(const Ctx& c, const Shared& sh, uint64_t S0, int b0, int b1, int b2,
                                        int b3) {
  double v = __ldg(c.v2 + size_t(sh.pidx[b0 * 64 + b1]) * c.npairs + sh.pidx[b2 * 64 + b3]);
  int p = __popcll(S0 & below(b0)) + __popcll(S0 & below(b1)) - 1;
  uint64_t I = S0 & ~((1ull << b0) | (1ull << b1));
  p += __popcll(I & below(b2)) + __popcll(I & below(b3));
  return (p & 1) ? -v : v;
}

// forward one-body term x -> y on S0
__device__ __forceinline__ double term1(const Ctx& c, uint64_t S0, int x, int y) {
  double v = __ldg(c.e1 + x * c.ns + y);
  int p = __popcll(S0 & below(x)) + __popcll((S0 & ~(1ull << x)) & below(y));
  return (p & 1) ? -v : v;
}

// Visit every stored element of row `row`; emit(col, value) for |value| >= 1e-14.
template <class Emit>
__device__ void visit_row(const Ctx& c, const Shared& sh, uint64_t row, Emit&& emit) {
  const uint64_t S = c.state[row];
  // diagonal: one-body terms (i, i) ascending, then two-body (a, b, a, b) ascending
  {
    double v = 0.0;
    for (uint64_t t = S; t; t &= t - 1) {
      int a = __ffsll((long long)t) - 1;
      v += __ldg(c.e1 + a * c.ns + a);
    }
    for (uint64_t t = S; t; t &= t - 1) {
      int a = __ffsll((long long)t) - 1;
      for (uint64_t u = t & (t - 1); u; u &= u - 1) {
        int b = __ffsll((long long)u) - 1;
        int pab = sh.pidx[a * 64 + b];
        v += __ldg(c.v2 + size_t(pab) * c.npairs + pab);
      }
    }
    emit(row, v, true);
  }
  for (int sp = 0; sp < 2; ++sp) {
    const uint64_t all = sp ? c.pall : c.nall;
    const uint64_t Ss = S & all, holes = ~S & all;
    const uint64_t* mm = sh.mmask + sp * (2 * kMOff + 1) + kMOff;
    // one particle a -> f, same species and m, all other occupied orbitals as spectators
    for (uint64_t t = Ss; t; t &= t - 1) {
      int a = __ffsll((long long)t) - 1;
      for (uint64_t u = holes & mm[sh.m2[a]]; u; u &= u - 1) {
        int f = __ffsll((long long)u) - 1;
        uint64_t K = S ^ (1ull << a) ^ (1ull << f);
        int x = a < f ? a : f, y = a < f ? f : a;
        uint64_t S0 = a < f ? S : K;
        double v = term1(c, S0, x, y);
        for (uint64_t w = S & ~(1ull << a); w; w &= w - 1) {
          int sc = __ffsll((long long)w) - 1;
          int b0 = x < sc ? x : sc, b1 = x < sc ? sc : x;
          int b2 = y < sc ? y : sc, b3 = y < sc ? sc : y;
          v += term2(c, sh, S0, b0, b1, b2, b3);
        }
        emit(ket_index(c, sh, K), v, false);
      }
    }
    // two particles of this species a < b -> c < d
    for (uint64_t t = Ss; t; t &= t - 1) {
      int a = __ffsll((long long)t) - 1;
      for (uint64_t u = t & (t - 1); u; u &= u - 1) {
        int b = __ffsll((long long)u) - 1;
        int msum = sh.m2[a] + sh.m2[b];
        for (uint64_t w = holes; w; w &= w - 1) {
          int cc = __ffsll((long long)w) - 1;
          int dm = msum - sh.m2[cc];
          if (dm < -kMOff || dm > kMOff) continue;
          for (uint64_t z = holes & mm[dm] & ~below(cc + 1); z; z &= z - 1) {
            int d = __ffsll((long long)z) - 1;
            uint64_t K = S ^ (1ull << a) ^ (1ull << b) ^ (1ull << cc) ^ (1ull << d);
            bool fwd = (a < cc) || (a == cc && b < d);
            double v = fwd ? term2(c, sh, S, a, b, cc, d) : term2(c, sh, K, cc, d, a, b);
            emit(ket_index(c, sh, K), v, false);
          }
        }
      }
    }
  }
  // one neutron a -> cc and one proton b -> d
  {
    const uint64_t Sn = S & c.nall, Sp = S & c.pall;
    const uint64_t hn = ~S & c.nall, hp = ~S & c.pall;
    const uint64_t* mmp = sh.mmask + (2 * kMOff + 1) + kMOff;
    for (uint64_t t = Sn; t; t &= t - 1) {
      int a = __ffsll((long long)t) - 1;
      for (uint64_t w = hn; w; w &= w - 1) {
        int cc = __ffsll((long long)w) - 1;
        int dmn = sh.m2[a] - sh.m2[cc];
        for (uint64_t u = Sp; u; u &= u - 1) {
          int b = __ffsll((long long)u) - 1;
          int dm = dmn + sh.m2[b];
          if (dm < -kMOff || dm > kMOff) continue;
          for (uint64_t z = hp & mmp[dm]; z; z &= z - 1) {
            int d = __ffsll((long long)z) - 1;
            uint64_t K = S ^ (1ull << a) ^ (1ull << b) ^ (1ull << cc) ^ (1ull << d);
            double v = (a < cc) ? term2(c, sh, S, a, b, cc, d) : term2(c, sh, K, cc, d, a, b);
            emit(ket_index(c, sh, K), v, false);
          }
        }
      }
    }
  }
}

__device__ void load_shared(Shared& sh, const Ctx& c, const uint64_t* binom64) {
  for (int i = threadIdx.x; i < 33 * 33; i += blockDim.x) sh.binom[i] = binom64[(i / 33) * kBinom + (i % 33)];
  for (int i = threadIdx.x; i < 64 * 64; i += blockDim.x) {
    int a = i / 64, b = i % 64;
    sh.pidx[i] = int16_t((a < b && b < c.ns) ? (a * c.ns - a * (a + 1) / 2 + (b - a - 1)) : -1);
  }
  for (int i = threadIdx.x; i < 64; i += blockDim.x) sh.m2[i] = i < c.ns ? c.m2[i] : 0;
  for (int i = threadIdx.x; i < 2 * (2 * kMOff + 1); i += blockDim.x) sh.mmask[i] = c.mmask[i];
  __syncthreads();
}

__global__ void k_count(Ctx c, const uint64_t* binom64, uint32_t* __restrict__ counts, int* __restrict__ err) {
  __shared__ Shared sh;
  load_shared(sh, c, binom64);
  for (uint64_t row = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; row < c.n;
       row += uint64_t(gridDim.x) * blockDim.x) {
    uint32_t k = 0;
    visit_row(c, sh, row, [&](uint64_t col, double v, bool) {
      if (col == ~0ull) { atomicOr(err, 1); return; }
      if (col == kOutside) return;
      k += (fabs(v) >= kDrop);
    });
    counts[row] = k;
  }
}

__global__ void k_fill(Ctx c, const uint64_t* binom64, const uint64_t* __restrict__ rowptr,
                       uint32_t* __restrict__ col, double* __restrict__ val, double* __restrict__ diag) {
  __shared__ Shared sh;
  load_shared(sh, c, binom64);
  for (uint64_t row = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; row < c.n;
       row += uint64_t(gridDim.x) * blockDim.x) {
    uint64_t p = rowptr[row];
    double dv = 0.0;
    visit_row(c, sh, row, [&](uint64_t k, double v, bool isdiag) {
      if (k >= kOutside) return;
      if (fabs(v) >= kDrop) {
        col[p] = uint32_t(k);
        val[p] = v;
        ++p;
        if (isdiag) dv = v;
      }
    });
    diag[row] = dv;
  }
}

// Block-wise exclusive scan of u32 counts into u64 offsets (pass 1: local scan
// + block totals; pass 2 adds the scanned block totals).
constexpr int kScanT = 256, kScanItems = 8, kScanTile = kScanT * kScanItems;

__global__ void k_scan_local(const uint32_t* __restrict__ in, uint64_t n, uint64_t* __restrict__ out,
                             uint64_t* __restrict__ tile_sum) {
  __shared__ uint64_t s[kScanT];
  uint64_t base = uint64_t(blockIdx.x) * kScanTile + uint64_t(threadIdx.x) * kScanItems;
  uint64_t v[kScanItems], run = 0;
  for (int i = 0; i < kScanItems; ++i) {
    v[i] = (base + i < n) ? in[base + i] : 0;
    run += v[i];
  }
  s[threadIdx.x] = run;
  __syncthreads();
  for (int off = 1; off < kScanT; off <<= 1) {
    uint64_t t = threadIdx.x >= off ? s[threadIdx.x - off] : 0;
    __syncthreads();
    s[threadIdx.x] += t;
    __syncthreads();
  }
  uint64_t excl = s[threadIdx.x] - run;
  for (int i = 0; i < kScanItems; ++i) {
    if (base + i < n) out[base + i] = excl;
    excl += v[i];
  }
  if (threadIdx.x == kScanT - 1) tile_sum[blockIdx.x] = s[kScanT - 1];
}

__global__ void k_scan_add(uint64_t* __restrict__ out, uint64_t n, const uint64_t* __restrict__ tile_off) {
  uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x;
  if (i < n) out[i] += tile_off[i / kScanTile];
}

// One CTA per row: bitonic sort of (col, position) keys in shared memory, then
// write columns and values (FP64, or FP32 hi + lo) in ascending column order.
__global__ void k_sort_rows(uint64_t n, const uint64_t* __restrict__ rowptr, uint32_t* __restrict__ col,
                            const double* __restrict__ val, double* __restrict__ out64, float* __restrict__ hi,
                            float* __restrict__ lo, unsigned long long* __restrict__ upper_count, int min_len) {
  extern __shared__ uint64_t skey[];
  __shared__ unsigned long long up_blk;
  if (threadIdx.x == 0) up_blk = 0;
  __syncthreads();
  for (uint64_t row = blockIdx.x; row < n; row += gridDim.x) {
    uint64_t b = rowptr[row], e = rowptr[row + 1];
    int len = int(e - b);
    if (len < min_len) continue;  // sorted by k_sort_rows_w (uniform across the CTA)
    int L = 1;
    while (L < len) L <<= 1;
    for (int i = threadIdx.x; i < L; i += blockDim.x)
      skey[i] = i < len ? ((uint64_t(col[b + i]) << 32) | uint32_t(i)) : ~0ull;
    __syncthreads();
    for (int k = 2; k <= L; k <<= 1)
      for (int j = k >> 1; j > 0; j >>= 1) {
        for (int i = threadIdx.x; i < L; i += blockDim.x) {
          int ixj = i ^ j;
          if (ixj > i) {
            uint64_t x = skey[i], y = skey[ixj];
            bool up = (i & k) == 0;
            if ((x > y) == up) { skey[i] = y; skey[ixj] = x; }
          }
        }
        __syncthreads();
      }
    unsigned up = 0;
    // gather values first (all reads of the row before any write)
    double* sval = reinterpret_cast<double*>(skey + L);
    for (int i = threadIdx.x; i < len; i += blockDim.x) sval[i] = val[b + uint32_t(skey[i])];
    __syncthreads();
    for (int i = threadIdx.x; i < len; i += blockDim.x) {
      uint32_t cc = uint32_t(skey[i] >> 32);
      col[b + i] = cc;
      double v = sval[i];
      if (out64) out64[b + i] = v;
      if (hi) {
        float h = float(v);
        hi[b + i] = h;
        lo[b + i] = float(v - double(h));
      }
      up += (cc >= row);
    }
    if (up) atomicAdd(&up_blk, (unsigned long long)up);
    __syncthreads();
  }
  __syncthreads();
  if (threadIdx.x == 0 && up_blk) atomicAdd(upper_count, up_blk);
}

// Per-row sort for rows of at most 1024 entries in matrices of fewer than
// 2^22 rows: one warp per row, the row's keys (column << 10 | position) held
// 32 per lane in registers (lane l: positions 32 l .. 32 l + 31) and sorted
// by a bitonic network whose stages of distance >= 32 exchange registers
// between lanes by shuffles and whose shorter stages swap within a lane; then
// columns and values are written in order.  Columns are unique within a row,
// so the order is the column order.  Rows that do not fit are left to
// k_sort_rows.
__global__ void __launch_bounds__(256, 2) k_sort_rows_w(uint64_t n, const uint64_t* __restrict__ rowptr,
                                                     uint32_t* __restrict__ col, const double* __restrict__ val,
                                                     double* __restrict__ out64, float* __restrict__ hi,
                                                     float* __restrict__ lo, unsigned long long* __restrict__ upper_count) {
  const int lane = threadIdx.x & 31;
  const uint64_t w0 = (blockIdx.x * uint64_t(blockDim.x) + threadIdx.x) >> 5;
  const uint64_t nw = (uint64_t(gridDim.x) * blockDim.x) >> 5;
  unsigned long long up = 0;
  for (uint64_t row = w0; row < n; row += nw) {
    const uint64_t b = rowptr[row];
    const int len = int(rowptr[row + 1] - b);
    if (len > 1024) continue;
    uint32_t v[32];
#pragma unroll
    for (int i = 0; i < 32; ++i) {
      const int pos = lane * 32 + i;
      v[i] = pos < len ? (col[b + pos] << 10) | uint32_t(pos) : 0xffffffffu;
    }
#pragma unroll
    for (int k = 2; k <= 1024; k <<= 1) {
#pragma unroll
      for (int j = k >> 1; j > 0; j >>= 1) {
        if (j >= 32) {
          const int lm = j >> 5;
          const bool lower = (lane & lm) == 0;
#pragma unroll
          for (int i = 0; i < 32; ++i) {
            const bool asc = ((lane * 32 + i) & k) == 0;
            const uint32_t o = __shfl_xor_sync(0xffffffffu, v[i], lm);
            v[i] = (asc == lower) ? min(v[i], o) : max(v[i], o);
          }
        } else {
#pragma unroll
          for (int i = 0; i < 32; ++i) {
            if (i & j) continue;
            const bool asc = ((lane * 32 + i) & k) == 0;
            const uint32_t a = v[i], c = v[i | j];
            if ((a > c) == asc) {
              v[i] = c;
              v[i | j] = a;
            }
          }
        }
      }
    }
#pragma unroll
    for (int i = 0; i < 32; ++i) {
      const int pos = lane * 32 + i;
      if (pos < len) {
        const uint32_t c = v[i] >> 10;
        const double x = val[b + (v[i] & 1023u)];
        col[b + pos] = c;
        if (out64) out64[b + pos] = x;
        if (hi) {
          const float h = float(x);
          hi[b + pos] = h;
          lo[b + pos] = float(x - double(h));
        }
        up += c >= row;
      }
    }
  }
  for (int o = 16; o; o >>= 1) up += __shfl_xor_sync(0xffffffffu, up, o);
  if (lane == 0 && up) atomicAdd(upper_count, up);
}

__global__ void k_max_u32(const uint32_t* __restrict__ a, uint64_t n, unsigned* __restrict__ out) {
  unsigned m = 0;
  for (uint64_t i = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; i < n; i += uint64_t(gridDim.x) * blockDim.x)
    m = max(m, a[i]);
  for (int o = 16; o; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

}  // namespace

void hamiltonian_build(const System& sys, const Operator& op, const Basis& b, int precision, Hamiltonian& h,
                       bool tiled_copy) {
  if (precision != CG_PREC_FP64 && precision != CG_PREC_FP32)
    throw Error(CG_ERR_ARG, "Hamiltonian precision must be CG_PREC_FP64 or CG_PREC_FP32");
  CG_CUDA(cudaGetDevice(&h.device));
  if (h.device != b.device) throw Error(CG_ERR_ARG, "basis lives on another device");
  if (!h.stream) CG_CUDA(cudaStreamCreateWithFlags(&h.stream, cudaStreamNonBlocking));
  cudaStream_t s = h.stream;
  h.precision = precision;
  h.n = b.n;
  if (b.n >= (1ull << 32)) throw Error(CG_ERR_UNSUPPORTED, "dimension >= 2^32 needs the on-the-fly product");
  cudaEvent_t e0, e1;
  CG_CUDA(cudaEventCreate(&e0));
  CG_CUDA(cudaEventCreate(&e1));
  CG_CUDA(cudaEventRecord(e0, s));

  DevOperator dop;
  std::unique_ptr<WideRows> wide;
  std::vector<int8_t> m2(b.ns);
  for (int i = 0; i < b.ns; ++i) m2[i] = int8_t(b.sp_m2[i]);
  DBuf<int8_t> dm2;
  dm2.upload(m2, s);
  Ctx c{};
  if (b.wide) {
    wide = wide_rows(sys, op, b, s);  // valence spaces of more than 32 m-states per species (wide.cu)
  } else {
    upload_operator(sys, op, dop, s);
    c.ns = b.ns;
    c.nn = b.nn;
    c.npairs = dop.npairs;
    c.nall = b.nn ? ((b.nn == 64) ? ~0ull : ((1ull << b.nn) - 1)) : 0;
    c.pall = (b.ns == 64 ? ~0ull : ((1ull << b.ns) - 1)) & ~c.nall;
    c.n = b.n;
    c.state = b.state.p;
    c.noff = b.noff.p;
    c.pcrank = b.pcrank.p;
    c.nlist = b.truncated ? b.nlist.p : nullptr;
    c.lrank = b.truncated ? b.lrank.p : nullptr;
    c.npc = b.npc;
    c.e1 = dop.e1.p;
    c.v2 = dop.v2.p;
    c.mmask = dop.mmask.p;
    c.m2 = dm2.p;
  }

  const uint64_t n = b.n;
  DBuf<uint32_t> counts(std::max<uint64_t>(n, 1));
  int T = 128;
  unsigned grid = unsigned(std::min<uint64_t>((n + T - 1) / T, 152ull * 64));
  if (grid == 0) grid = 1;
  DBuf<int> derr(1);
  CG_CUDA(cudaMemsetAsync(derr.p, 0, sizeof(int), s));
  if (wide) {
    wide->count(counts.p, derr.p);
  } else {
    k_count<<<grid, T, 0, s>>>(c, b.binom.p, counts.p, derr.p);
    CG_CUDA(cudaGetLastError());
    count_launch();
  }
  int herr = 0;
  CG_CUDA(cudaMemcpyAsync(&herr, derr.p, sizeof(int), cudaMemcpyDeviceToHost, s));

  // rowptr = exclusive scan of counts, rowptr[n] = nnz
  h.rowptr.alloc(n + 1);
  uint64_t ntiles = (n + kScanTile - 1) / kScanTile;
  DBuf<uint64_t> tsum(std::max<uint64_t>(ntiles, 1));
  if (n) {
    k_scan_local<<<unsigned(ntiles), kScanT, 0, s>>>(counts.p, n, h.rowptr.p, tsum.p);
    CG_CUDA(cudaGetLastError());
    count_launch();
  }
  std::vector<uint64_t> ht(ntiles);
  if (ntiles) CG_CUDA(cudaMemcpyAsync(ht.data(), tsum.p, ntiles * 8, cudaMemcpyDeviceToHost, s));
  DBuf<unsigned> dmax(1);
  CG_CUDA(cudaMemsetAsync(dmax.p, 0, 4, s));
  if (n) k_max_u32<<<304, 256, 0, s>>>(counts.p, n, dmax.p);
  unsigned maxrow = 0;
  CG_CUDA(cudaMemcpyAsync(&maxrow, dmax.p, 4, cudaMemcpyDeviceToHost, s));
  CG_CUDA(cudaStreamSynchronize(s));
  if (herr) throw Error(CG_ERR_INTERNAL, "operator connects a determinant outside the basis");
  uint64_t run = 0;
  for (auto& x : ht) { uint64_t t = x; x = run; run += t; }
  h.nnz = run;
  h.max_row = int(maxrow);
  if (ntiles) {
    tsum.upload(ht, s);
    k_scan_add<<<unsigned((n + 255) / 256), 256, 0, s>>>(h.rowptr.p, n, tsum.p);
    CG_CUDA(cudaGetLastError());
    count_launch();
  }
  CG_CUDA(cudaMemcpyAsync(h.rowptr.p + n, &h.nnz, 8, cudaMemcpyHostToDevice, s));
  counts.release();

  h.col.alloc(std::max<uint64_t>(h.nnz, 1));
  DBuf<double> tmpval(std::max<uint64_t>(h.nnz, 1));
  h.diag.alloc(std::max<uint64_t>(n, 1));
  if (n && wide) {
    wide->fill(h.rowptr.p, h.col.p, tmpval.p, h.diag.p);
  } else if (n) {
    k_fill<<<grid, T, 0, s>>>(c, b.binom.p, h.rowptr.p, h.col.p, tmpval.p, h.diag.p);
    CG_CUDA(cudaGetLastError());
    count_launch();
  }
  if (precision == CG_PREC_FP64) {
    h.val64.alloc(std::max<uint64_t>(h.nnz, 1));
  } else {
    h.hi.alloc(std::max<uint64_t>(h.nnz, 1));
    h.lo.alloc(std::max<uint64_t>(h.nnz, 1));
  }
  int L = 1;
  while (L < h.max_row) L <<= 1;
  size_t smem = size_t(L) * 16;
  if (smem > 200 * 1024) throw Error(CG_ERR_UNSUPPORTED, "row longer than the per-row sort supports");
  if (smem > 48 * 1024)
    CG_CUDA(cudaFuncSetAttribute(k_sort_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
  DBuf<unsigned long long> dup(1);
  CG_CUDA(cudaMemsetAsync(dup.p, 0, 8, s));
  if (n) {
    // rows of up to 1024 entries: warp-per-row register sort; longer rows
    // (or 2^22 rows and more, whose columns need more than 22 key bits):
    // CTA-per-row shared-memory sort
    const bool warp_sort = n < (1ull << 22);
    if (warp_sort) {
      const unsigned wg = unsigned(std::min<uint64_t>((n * 32 + 255) / 256, 152ull * 64));
      k_sort_rows_w<<<wg, 256, 0, s>>>(n, h.rowptr.p, h.col.p, tmpval.p, h.val64.p, h.hi.p, h.lo.p, dup.p);
      CG_CUDA(cudaGetLastError());
      count_launch();
    }
    if (!warp_sort || h.max_row > 1024) {
      int st = std::min(256, std::max(32, L / 2));
      unsigned sg = unsigned(std::min<uint64_t>(n, 152ull * 16));
      k_sort_rows<<<sg, st, smem, s>>>(n, h.rowptr.p, h.col.p, tmpval.p, h.val64.p, h.hi.p, h.lo.p, dup.p,
                                       warp_sort ? 1025 : 0);
      CG_CUDA(cudaGetLastError());
      count_launch();
    }
  }
  unsigned long long up = 0;
  CG_CUDA(cudaMemcpyAsync(&up, dup.p, 8, cudaMemcpyDeviceToHost, s));
  CG_CUDA(cudaEventRecord(e1, s));
  CG_CUDA(cudaStreamSynchronize(s));
  h.nnz_upper = up;
  float ms = 0;
  CG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
  h.build_seconds = ms * 1e-3;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  h.blocks = b.h_bstart;
  h.blocks.push_back(b.n);
  if (precision == CG_PREC_FP32 && tiled_copy && h.nnz >= kTiledMinEntries) {
    // block-tiled copy for the 8-vector product, blocks = neutron blocks
    const auto t0 = std::chrono::steady_clock::now();
    tiled_build(h, h.blocks);
    h.build_seconds += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
}

void hamiltonian_upper_rows(const Hamiltonian& h, uint64_t row0, uint64_t nrows, uint64_t* rowptr, uint32_t* cols,
                            double* vals) {
  if (row0 + nrows > h.n) throw Error(CG_ERR_ARG, "row range outside the matrix");
  std::vector<uint64_t> rp(nrows + 1);
  CG_CUDA(cudaMemcpy(rp.data(), h.rowptr.p + row0, (nrows + 1) * 8, cudaMemcpyDeviceToHost));
  uint64_t b = rp[0], e = rp[nrows];
  std::vector<uint32_t> c(e - b);
  std::vector<double> v;
  std::vector<float> fh, fl;
  if (e > b) CG_CUDA(cudaMemcpy(c.data(), h.col.p + b, (e - b) * 4, cudaMemcpyDeviceToHost));
  if (cols && vals && e > b) {
    if (h.precision == CG_PREC_FP64) {
      v.resize(e - b);
      CG_CUDA(cudaMemcpy(v.data(), h.val64.p + b, (e - b) * 8, cudaMemcpyDeviceToHost));
    } else {
      fh.resize(e - b);
      fl.resize(e - b);
      CG_CUDA(cudaMemcpy(fh.data(), h.hi.p + b, (e - b) * 4, cudaMemcpyDeviceToHost));
      CG_CUDA(cudaMemcpy(fl.data(), h.lo.p + b, (e - b) * 4, cudaMemcpyDeviceToHost));
    }
  }
  uint64_t k = 0;
  rowptr[0] = 0;
  for (uint64_t r = 0; r < nrows; ++r) {
    for (uint64_t j = rp[r] - b; j < rp[r + 1] - b; ++j) {
      if (c[j] < row0 + r) continue;
      if (cols && vals) {
        cols[k] = c[j];
        vals[k] = h.precision == CG_PREC_FP64 ? v[j] : double(fh[j]) + double(fl[j]);
      }
      ++k;
    }
    rowptr[r + 1] = k;
  }
}

}  // namespace cg
