// Device-side objects shared by the kernels: the resident basis, the stored
// Hamiltonian and the interaction tables, plus CUDA error plumbing.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "cosmo_gb300.h"
#include "model.h"

namespace cg {

#define CG_CUDA(call)                                                                            \
  do {                                                                                           \
    cudaError_t e_ = (call);                                                                     \
    if (e_ != cudaSuccess)                                                                       \
      throw ::cg::Error(e_ == cudaErrorMemoryAllocation ? CG_ERR_NOMEM : CG_ERR_CUDA,            \
                        std::string(#call) + ": " + cudaGetErrorString(e_) + " (" __FILE__ ":" + \
                            std::to_string(__LINE__) + ")");                                     \
  } while (0)

// Kernel launches issued by this library (for benchmark accounting).
uint64_t& launch_counter();
inline void count_launch(uint64_t k = 1) { launch_counter() += k; }

// Owning device buffer.
template <class T>
struct DBuf {
  T* p = nullptr;
  size_t n = 0;
  DBuf() = default;
  explicit DBuf(size_t count) { alloc(count); }
  DBuf(const DBuf&) = delete;
  DBuf& operator=(const DBuf&) = delete;
  DBuf(DBuf&& o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
  DBuf& operator=(DBuf&& o) noexcept {
    if (this != &o) { release(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
    return *this;
  }
  ~DBuf() { release(); }
  void alloc(size_t count) {
    release();
    if (count) CG_CUDA(cudaMalloc(&p, count * sizeof(T)));
    n = count;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  void upload(const T* h, size_t count, cudaStream_t s = 0) {
    if (count) CG_CUDA(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
  }
  void upload(const std::vector<T>& h, cudaStream_t s = 0) {
    if (n < h.size()) alloc(h.size());
    upload(h.data(), h.size(), s);
  }
  size_t bytes() const { return n * sizeof(T); }
};

// Binomial table in constant memory, C(a, b) for a, b < 65.
constexpr int kBinom = 65;

// ------------------------------------------------------------------ basis
// Per-species bitstring description: a species has `norb` m-scheme states
// (bits 0..norb-1 of its mask) and `k` particles.  A configuration's colex rank
// (sum over set bits c_i, ascending, of C(c_i, i+1)) indexes the small lookup
// tables; the basis order itself is the reference's lexicographic order.
struct SpeciesTables {
  int norb = 0, k = 0;
  uint64_t nconf = 0;              // C(norb, k)
  std::vector<uint32_t> lex_mask;  // configurations in lexicographic order
  std::vector<int> lex_m2, lex_par;
};

struct Basis {
  int device = 0;
  int ns = 0, nn = 0, np = 0;  // s.p. states: total, neutron, proton
  int kn = 0, kp = 0;          // particles per species
  int twom = 0, parity = 0;
  uint64_t n = 0;
  SpeciesTables neut, prot;
  std::vector<int> sp_m2, sp_par;  // per global s.p. index
  // device tables
  DBuf<uint64_t> state;            // per basis state: combined mask (neutron bits low, proton bits << nn)
  DBuf<uint64_t> noff;             // by neutron colex rank: first index of that neutron block, ~0 if none
  DBuf<uint32_t> pcrank;           // by proton colex rank: rank inside its (2m, parity) class
  DBuf<uint64_t> binom;            // kBinom x kBinom
  // neutron blocks (basis order) and proton classes, host copies
  std::vector<uint64_t> h_bstart;  // first index of each neutron block
  std::vector<uint32_t> h_bmask;   // neutron mask of each block
  std::vector<uint32_t> h_bclass;  // proton class of each block
  std::vector<uint32_t> h_cstart;  // first position of each proton class in h_cmasks
  std::vector<uint32_t> h_cmasks;  // proton masks, class by class, rank order
  // truncated bases: a neutron block holds the proton configurations of its
  // class that the truncation allows with it, a list fixed by the neutron
  // configuration's quanta and rejection counts; h_bclass then numbers these
  // lists (h_cstart / h_cmasks hold them) and the in-block rank is
  // lrank[list * npc + colex(p)] (~0u: not in the list)
  bool truncated = false;
  uint64_t npc = 0;                // proton configurations (colex ranks)
  DBuf<uint32_t> nlist;            // by neutron colex rank: list of its block, ~0u if none
  DBuf<uint32_t> lrank;            // lists x npc
  std::vector<uint32_t> h_nlist, h_lrank;
  // valence spaces with a species of more than 32 m-states (wide.cu): a
  // determinant is a pair of 64-bit species masks; blocks and lists as above
  // (h_bstart, h_bclass, h_cstart) with 64-bit masks, located by binary search
  bool wide = false;
  DBuf<uint64_t> wstate;                     // 2 per basis state: neutron mask, proton mask
  std::vector<uint64_t> h_wbmask, h_wcmask;  // block neutron masks; list members in h_cstart order
  std::vector<uint64_t> h_wnkey, h_wpkey;    // block neutron masks sorted; list members sorted per list
  std::vector<uint32_t> h_wnblk, h_wprank;   // block of each sorted neutron mask; rank of each sorted member
  DBuf<uint64_t> wbstart, wnkey, wpkey;
  DBuf<uint32_t> wbclass, wcstart, wnblk, wprank;
  // every enumerated proton configuration (lexicographic) with its rank in, and
  // the size of, its (2m, parity) class (the on-the-fly product's class ranks)
  std::vector<uint64_t> h_wpuniv;
  std::vector<uint32_t> h_wpuniv_rank, h_wpuniv_csize;
  // host copies used for locate and .mbs output
  std::vector<uint64_t> h_noff;
  std::vector<uint32_t> h_pcrank;
  std::vector<uint64_t> h_binom;
  cudaStream_t stream = nullptr;
  ~Basis();
};

// the bitstring basis, or the wide one (wide.cu) when a species has more than 32 m-states
void basis_build(const System& sys, Basis& b);
// the wide representation for any system (up to 64 m-states per species)
void basis_build_wide(const System& sys, Basis& b);
void basis_tuples_wide(const Basis& b, uint64_t first, uint64_t count, uint16_t* out);
uint64_t basis_locate_wide_host(const Basis& b, const uint16_t* tuple);
void jt_expectations_wide(const System& sys, const Basis& b, const double* vecs, int nst, double* jj, double* tt);
// per-CTA partial sums of the pull-form overlaps (sf.cu) on wide bases: the
// one-body transition amplitudes (part[cta * 16 + q]) and the removal
// amplitudes (part[(s * grid + cta) * 16 + q]), 256 threads per CTA
void wide_onebody_partials(const Basis& parent, const Basis& daughter, const double* psid, int nq,
                           const double* psip, const int2* tif, const double* tv, int nt, double* part,
                           unsigned grid, int* err, cudaStream_t s);
void wide_sf_partials(const Basis& parent, const Basis& daughter, const double* psid, int nq, const double* psip,
                      const int* sidx, int nsidx, double* part, unsigned grid, int* err, cudaStream_t s);
uint64_t colex_host(uint64_t mask, const std::vector<uint64_t>& binom);

// <J-J+> = ||J+ psi||^2 and <T-T+> = ||T+ psi||^2 of nst host vectors (state k at vecs + k*n).
void jt_expectations(const System& sys, const Basis& b, const double* vecs, int nst, double* jj, double* tt);
// amp[(q * np + p) * ns + s] = <D_q| a_s |P_p> (sf.cu)
void sf_amplitudes(const System& psys, const Basis& parent, const double* vp, int np, const Basis& daughter,
                   const double* vd, int nd, double* amp);
// amp[q * np + p] = <D_q| sum_t v_t a+_f a_i |P_p> (sf.cu); nd <= 16
struct OneBodyTerm;
void onebody_amplitudes(const System& psys, const Basis& parent, const double* vp, int np, const Basis& daughter,
                        const double* vd, int nd, const std::vector<OneBodyTerm>& terms, double* amp);
// occ[k * ns + s] = <psi_k| n_s |psi_k> for nst host vectors (sf.cu)
void occupations(const Basis& b, const double* v, int nst, double* occ);
// twice the spin from <J-J+> and twice the projection; -1 if not (half-)integer within 0.1
int jj_spin(double x, int two_m);
void basis_tuples(const Basis& b, uint64_t first, uint64_t count, uint16_t* out);
uint64_t basis_locate_host(const Basis& b, const uint16_t* tuple);

// ----------------------------------------------------------- interaction
struct DevOperator {
  int ns = 0, npairs = 0;
  DBuf<double> e1;      // ns x ns, forward one-body terms (i <= f)
  DBuf<double> v2;      // npairs x npairs, forward two-body terms
  DBuf<int32_t> pidx;   // ns x ns pair index for a < b
  DBuf<uint64_t> mmask; // per species (2) x per 2m value (kMOff*2+1): mask of s.p. states
};
constexpr int kMOff = 64;  // 2m in [-64, 64]

void upload_operator(const System& sys, const Operator& op, DevOperator& d, cudaStream_t s);

// ----------------------------------------------------------- Hamiltonian
// Launch shape of the FP32 product (chosen by spmm_autotune).
struct SpmmTuning {
  int warps = 16;       // warps per CTA
  int ctas_per_sm = 2;  // resident CTAs per SM the grid is sized for
  bool tuned = false;
};
struct SpmmCandidate {
  int warps, ctas_per_sm;
  float ms;
};

struct VirtualOp;
struct TiledOp;
struct Hamiltonian {
  int device = 0;
  int precision = CG_PREC_FP64;
  uint64_t n = 0, nnz = 0, nnz_upper = 0;
  int max_row = 0;
  double build_seconds = 0;
  DBuf<uint64_t> rowptr;  // n + 1
  DBuf<uint32_t> col;     // nnz
  DBuf<double> val64;     // nnz (CG_PREC_FP64)
  DBuf<float> hi, lo;     // nnz (CG_PREC_FP32)
  DBuf<double> diag;      // n
  SpmmTuning tuning;
  std::shared_ptr<VirtualOp> virt;  // set for the on-the-fly product (nothing stored)
  std::shared_ptr<TiledOp> tiled;   // block-tiled copy of the FP32 values (8-vector product)
  std::vector<uint64_t> blocks;     // neutron-block starts (+ n) when built from a basis
  bool use_tiled = true;            // route 8-vector FP32 products through `tiled` when present
  cudaStream_t stream = nullptr;
  ~Hamiltonian();
  uint64_t device_bytes() const;  // HBM held by the matrix (or the on-the-fly tables)
};

// Rows of H on a wide basis (wide.cu): per-row element counts, then the
// elements (unsorted columns) and the diagonal, as the bitstring builder's
// count and fill passes.
struct WideRows {
  virtual ~WideRows() = default;
  virtual void count(uint32_t* counts, int* err) = 0;
  virtual void fill(const uint64_t* rowptr, uint32_t* col, double* val, double* diag) = 0;
};
std::unique_ptr<WideRows> wide_rows(const System& sys, const Operator& op, const Basis& b, cudaStream_t s);

// tiled_copy: also build the block-tiled copy of an FP32 matrix (tiled.h)
void hamiltonian_build(const System& sys, const Operator& op, const Basis& b, int precision, Hamiltonian& h,
                       bool tiled_copy = true);
void hamiltonian_upper_rows(const Hamiltonian& h, uint64_t row0, uint64_t nrows, uint64_t* rowptr, uint32_t* cols,
                            double* vals);
// stored H from a .HH file (both triangles rebuilt from the stored upper rows)
void hamiltonian_read_hh(const std::string& path, int precision, Hamiltonian& h);

// ------------------------------------------------------------------ SpMM
// Row-interleaved operands: element (i, k) at x[i*ldx + k].
void spmm_launch(const Hamiltonian& h, int precision, const void* x, int ldx, void* y, int ldy, int m,
                 cudaStream_t s);
// FP32 product of m <= 16 vectors from a staging block whose rows are 32-byte
// aligned and padded with zero vectors to 8 or 16 (ldx >= 8 or 16); only the
// first m outputs of each row are stored.
void spmm_f32_padded(const Hamiltonian& h, const float* x, int ldx, float* y, int ldy, int m, cudaStream_t s);
std::vector<SpmmCandidate> spmm_autotune(Hamiltonian& h, int m, int reps);
// Double-float product with its staging area in a static device array (no
// allocation); h.n must not exceed spmm_refine_static_max_rows().
void spmm_refine_static(const Hamiltonian& h, const double* x, int ldx, double* y, int ldy, int m,
                        cudaStream_t s);
uint64_t spmm_refine_static_max_rows();
// Random 32-byte gathers per second from a table of `rows` 32-byte rows.
double gather_probe(int device, uint64_t rows, int share);
// Refinement product Y = H X (FP64 in and out, any m) computed in double-float
// FP32 arithmetic from the stored (hi, lo) values; stage holds n x 16 floats.
void spmm_refine_df(const Hamiltonian& h, const double* x, int ldx, double* y, int ldy, int m, float* stage,
                    cudaStream_t s);
// Host column-major doubles in and out (vector k at k*n), any m >= 1.
void spmm_host(const Hamiltonian& h, int precision, const double* x, double* y, int m);

}  // namespace cg
