/*
 * cosmo_gb300 — C ABI of the GB300 (sm_103a) configuration-interaction hot path.
 *
 * Plain C: opaque handles, plain pointers and sizes, every call returns a
 * status (0 = CG_OK, negative = error; the message is in cg_last_error()).
 * Nothing throws across this boundary.  Handles are bound to the CUDA device
 * that was current when they were created; calls on one handle are not
 * thread-safe.  All large objects (basis, Hamiltonian, Davidson vectors) stay
 * resident in HBM; host buffers are only touched by the calls that take them.
 *
 * Each entry point names the reference interface it replaces (paths are
 * relative to the reference project, alvolya/cosmo).
 */
#ifndef COSMO_GB300_H
#define COSMO_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
typedef int32_t cg_status;
#define CG_OK 0
#define CG_ERR_ARG (-1)
#define CG_ERR_IO (-2)
#define CG_ERR_PARSE (-3)
#define CG_ERR_CUDA (-4)
#define CG_ERR_NOMEM (-5)
#define CG_ERR_UNSUPPORTED (-6)
#define CG_ERR_NOT_CONVERGED (-7)
#define CG_ERR_TIMEOUT (-8)
#define CG_ERR_NO_DEVICE (-9)
#define CG_ERR_INTERNAL (-10)

/* precision of a stored Hamiltonian / of an SpMM call */
#define CG_PREC_FP64 0   /* FP64 values, FP64 vectors                        */
#define CG_PREC_FP32 1   /* FP32 values and vectors, FP32 accumulation          */
#define CG_PREC_REFINE 2 /* FP32 hi + FP32 lo values (~FP64), FP64 vectors    */

/* Last error message of the calling thread ("" if none). */
const char* cg_last_error(void);
/* ABI version (major * 100 + minor). */
int32_t cg_version(void);
/* Number of CUDA devices visible, or a negative status. */
int32_t cg_device_count(void);
/* Kernel launches this library has issued in this process (monotonic). */
uint64_t cg_launch_count(void);

/* --------------------------------------------------------------- problem */
/* Host-side CI problem: valence space, s.p. states, system quantum numbers and
 * the forward-ordered m-scheme operator terms ESP (one-body) and VSPX
 * (two-body, including lambda * J-J+).
 * Replaces SM::Make(sps, XMLNode) (include/xsm/xSingleParticleStates.cxx:26)
 * and xReadSPInt(ESP, VSPX, ...) (include/xsm/xReadSPInt.cxx:24). */
typedef struct cg_problem cg_problem;

typedef struct {
  int32_t n_sps;          /* m-scheme s.p. states                          */
  int32_t n_neutron_sps;  /* sps [0, n_neutron_sps) are neutrons           */
  int32_t nv, zv;         /* valence neutrons, protons                     */
  int32_t twom;           /* 2 * Jz                                        */
  int32_t parity;         /* 0 '+', 1 '-'                                  */
  int32_t has_jj;         /* matrix JJ attribute present                   */
  double jj;              /* lambda                                        */
  int64_t n_one_body;     /* ESP terms                                     */
  int64_t n_two_body;     /* VSPX terms                                    */
} cg_problem_info;

/* system_name may be NULL when the XML holds one <system>. */
cg_status cg_problem_load_xml(const char* xml_path, const char* system_name, cg_problem** out);

/* A problem from explicit operator terms, as SM::PPMatrix is assembled from
 * any set of MBOperator components (include/sm/PPMatrix.cxx:42-60, pushed in
 * include/xsm/DEXHVcsb.cxx:47-49).  sps: n_sps rows of 8 int32 in the layout of
 * cg_problem_sps (neutron states first, at most 64 per species); keys are
 * forward ordered as in cg_problem_one_body / cg_problem_two_body. */
typedef struct {
  int32_t n_sps, n_neutron_sps;
  const int32_t* sps;
  int32_t nv, zv, twom, parity;
  int64_t n_one_body;
  const int32_t* one_keys;
  const double* one_vals;
  int64_t n_two_body;
  const int32_t* two_keys;
  const double* two_vals;
} cg_problem_desc;
cg_status cg_problem_create(const cg_problem_desc* desc, cg_problem** out);
void cg_problem_destroy(cg_problem* p);
cg_status cg_problem_get_info(const cg_problem* p, cg_problem_info* info);
/* n_sps rows of 8 int32: level n l 2j 2m 2t 2tz parity (SPS, include/sm/SingleParticleStates.cxx:36). */
cg_status cg_problem_sps(const cg_problem* p, int32_t* table);
/* Operator terms in key order: keys[2*k], vals[k] (ESP) / keys[4*k], vals[k] (VSPX). */
cg_status cg_problem_one_body(const cg_problem* p, int32_t* keys, double* vals);
cg_status cg_problem_two_body(const cg_problem* p, int32_t* keys, double* vals);

/* ----------------------------------------------------------------- basis */
/* M-scheme Slater-determinant basis, enumerated on the GPU from per-species
 * bitstrings; index order is the reference's lexicographic order of sorted
 * s.p. tuples.  Replaces SM::MakeMBS2 (include/sm/MakeMBS.cxx:186) and the
 * Xsysmbs/XsysmbsOMP tools (xmlshell/xmbs/XsysmbsOMP.cpp:323).  A system with
 * a basis truncation (hwmax attribute, <hwrejection> or <rejection> children,
 * XsysmbsOMP.cpp:214-300) gets the truncated basis in the same order as the
 * reference's: neutron configurations in lexicographic order, each followed
 * by the proton configurations the truncation allows with it. */
typedef struct cg_basis cg_basis;

cg_status cg_basis_build(const cg_problem* p, cg_basis** out);
/* A valence space with more than 32 m-states in a species (up to 64 per
 * species, e.g. the spsdpf space: 40) gets the wide representation: species
 * configurations enumerated on the host in the reference's order, pruned by
 * the truncation's oscillator quanta (an untruncated species of more than
 * 2^26 configurations is refused), determinants as pairs of 64-bit species
 * masks located by binary search (SM::locate, include/sm/ManyBodyStates.cxx:
 * 92-130).  Same order, .mbs bytes, stored Hamiltonian, Davidson, <J-J+> /
 * <T-T+>, occupations, XSHLSF / XSHLEMB amplitudes, batched solves and the
 * on-the-fly product as the bitstring basis.  cg_basis_build_wide builds that
 * representation for any system (the two agree on every system both take). */
cg_status cg_basis_build_wide(const cg_problem* p, cg_basis** out);
cg_status cg_basis_is_wide(const cg_basis* b, int32_t* wide);
void cg_basis_destroy(cg_basis* b);
/* dimension n and particle number N */
cg_status cg_basis_dims(const cg_basis* b, uint64_t* n, int32_t* nparticles);
/* count states from `first` as sorted uint16 tuples (count * N values), host buffer.
 * Same content as Many_Body_States::z (include/sm/ManyBodyStates.cxx:43-49). */
cg_status cg_basis_states(const cg_basis* b, uint64_t first, uint64_t count, uint16_t* tuples);
/* state -> index, the reference's SM::locate (include/sm/ManyBodyStates.cxx:92);
 * out[k] = n + 1 when tuple k is not in the basis (same sentinel). */
cg_status cg_basis_locate(const cg_basis* b, const uint16_t* tuples, uint64_t count, uint64_t* out);
/* write the .mbs file: int32 N, uint64 n, n*N uint16
 * (Many_Body_States::Write, include/sm/ManyBodyStates.cxx:199-206) */
cg_status cg_basis_write_mbs(const cg_basis* b, const char* path);

/* ----------------------------------------------------------- Hamiltonian */
/* H + lambda * J-J+ built on the GPU (count -> scan -> fill -> per-row sort):
 * every pair of determinants differing by at most two particle-hole moves,
 * fermionic phases by popcount, |H_ij| < 1e-14 dropped like PPMatrix2CSBBlk
 * (include/sm/PPMatrix.cxx:571-656, drop at :621).  Both triangles are stored
 * (row-sliced CSR with 32-bit columns); each element is computed once from the
 * lower-index determinant with the forward operator, so H is exactly symmetric
 * and its upper triangle is the reference's CSB content.
 * precision: CG_PREC_FP64 stores FP64 values; CG_PREC_FP32 stores FP32 hi and
 * FP32 lo = fl(h - hi) so the same matrix serves CG_PREC_FP32 and
 * CG_PREC_REFINE products. */
typedef struct cg_hamiltonian cg_hamiltonian;

typedef struct {
  uint64_t n;
  uint64_t nnz_full;     /* stored entries, both triangles              */
  uint64_t nnz_upper;    /* entries with col >= row (reference CSB nnz) */
  int32_t precision;     /* CG_PREC_FP64 or CG_PREC_FP32                 */
  int32_t max_row;       /* longest row                                 */
  uint64_t device_bytes; /* HBM held by the matrix                      */
  double build_seconds;  /* device time of the build                    */
} cg_hamiltonian_info;

cg_status cg_hamiltonian_build(const cg_problem* p, const cg_basis* b, int32_t precision, cg_hamiltonian** out);
/* On-the-fly H + lambda * J-J+ (nothing stored), SM::PPMatrix
 * (include/sm/PPMatrix.cxx:42-152) as used by DEXHVJT (davidson/DEXHVJT.cpp:36-78):
 * the product regenerates every element per call from the basis bitstrings and
 * the interaction, through per-species transition tables (neutron blocks x
 * proton classes of the M-scheme basis; in a truncated basis the allowed proton
 * configurations of each neutron block, targets outside the basis dropped as
 * the reference's locate drops them).  The handle works with every product
 * and Davidson call: CG_PREC_FP32 products compute in FP32, CG_PREC_FP64 and
 * CG_PREC_REFINE products in FP64; precision only sets the default of
 * cg_spmm calls.  info.nnz_full = elements generated per product and vector,
 * info.nnz_upper = 0; cg_hamiltonian_upper_rows / write_hh are unsupported. */
cg_status cg_hamiltonian_build_virtual(const cg_problem* p, const cg_basis* b, int32_t precision,
                                       cg_hamiltonian** out);
cg_status cg_hamiltonian_is_virtual(const cg_hamiltonian* h, int32_t* is_virtual);
void cg_hamiltonian_destroy(cg_hamiltonian* h);
cg_status cg_hamiltonian_get_info(const cg_hamiltonian* h, cg_hamiltonian_info* info);
/* FP64 diagonal, host buffer of n (SparseMatrixCSB::ReadDiagonal, include/tav/csbmatrix.cxx:393). */
cg_status cg_hamiltonian_diagonal(const cg_hamiltonian* h, double* diag);
/* Upper triangle (col >= row) of rows [row0, row0 + nrows), columns ascending.
 * rowptr has nrows + 1 entries (relative to the first exported row); when cols
 * is NULL only rowptr is filled.  Values are the stored values widened to FP64
 * (hi + lo for CG_PREC_FP32 matrices). */
cg_status cg_hamiltonian_upper_rows(const cg_hamiltonian* h, uint64_t row0, uint64_t nrows, uint64_t* rowptr,
                                    uint32_t* cols, double* vals);
/* .HH row-sparse file: uint64 n, then per row uint32 nz, uint64 ind[nz], double
 * elem[nz] (upper triangle incl. diagonal), PPMatrix::Write (include/sm/PPMatrix.cxx:413-465). */
cg_status cg_hamiltonian_write_hh(const cg_hamiltonian* h, const char* path);
/* A stored Hamiltonian from a .HH file (the davidson_vfile input: SparseMatrix::Read,
 * include/tav/sparse.cxx:402-445; each off-diagonal pair stored once, applied to
 * both triangles as SparseMatrix::TimesMatrix does, :274-291). */
cg_status cg_hamiltonian_read_hh(const char* path, int32_t precision, cg_hamiltonian** out);
/* Stream used by this handle's kernels (cudaStream_t), for event timing. */
void* cg_hamiltonian_stream(const cg_hamiltonian* h);

/* ------------------------------------------------------------------ SpMM */
/* y = H x for m vectors on host buffers, both n x m column-major (vector k at
 * offset k*n) as SparseMatrixCSB::TimesMatrix(ftyp* y, ftyp* x, m)
 * (include/tav/csbmatrix.cxx:680) and MatB::MatrixBase::TimesMatrix
 * (include/kdav/matrixbase.h:17).  precision selects the product:
 * CG_PREC_FP64 (FP64 matrix), CG_PREC_FP32 or CG_PREC_REFINE (FP32 matrix). */
cg_status cg_spmm(const cg_hamiltonian* h, const double* x, double* y, int32_t m, int32_t precision);
/* Device-resident product on the handle's stream: x and y are row-interleaved
 * n x ld arrays (element (i, k) at i*ld + k) of float (CG_PREC_FP32) or double
 * (CG_PREC_FP64, CG_PREC_REFINE); columns [0, m) are used.  Asynchronous. */
cg_status cg_spmm_device(const cg_hamiltonian* h, const void* x, int32_t ldx, void* y, int32_t ldy, int32_t m,
                         int32_t precision);

/* Allocation-free FP64 product, no counterpart in the reference: y = H x for
 * m = 1..16 vectors, x and y device FP64 buffers, row-interleaved (x[i*ldx + k]),
 * computed by the double-float kernel of CG_PREC_REFINE from an FP32 (hi + lo)
 * matrix, enqueued on the handle's stream (the call returns before it finishes).
 * The kernel's staging area is a fixed 8 MiB device array inside the library
 * instead of a device allocation, so this call allocates no memory; it serves
 * callers that cannot allocate: a host eigensolver whose stored matrix and
 * vector basis already hold the device's memory, or one that must not stall
 * other streams (cudaMalloc/cudaFree can synchronize the device).
 * Limits: n <= 131,072 rows (8 MiB / 64 bytes a row; larger matrices are
 * rejected with CG_ERR_ARG: use cg_spmm_device or cg_spmm).  The first call on
 * each device looks up the array's device address (set-up); make that first
 * call before any stream capture begins.  Every call on a device shares the
 * one array (nothing in it needs to start at zero): calls whose work can
 * overlap on the device (other streams, other threads, other handles) race on
 * it and give wrong results, so order them, e.g. by synchronizing the previous
 * call's stream first. */
cg_status cg_spmm_refine_static(const cg_hamiltonian* h, const double* x, int32_t ldx, double* y, int32_t ldy,
                                int32_t m);
/* Row limit of cg_spmm_refine_static (131,072). */
cg_status cg_spmm_refine_static_max_rows(uint64_t* rows);
/* Launch-shape autotuner of the FP32 product: times every candidate (warps per
 * CTA x CTAs per SM, each CTA on one contiguous row range) with `nvec` vectors
 * on this matrix, keeps the fastest in the handle, and reports all candidates
 * (arrays of capacity *n_candidates on entry, count on return). */
cg_status cg_spmm_autotune(cg_hamiltonian* h, int32_t nvec, int32_t reps, int32_t* n_candidates, int32_t* warps,
                           int32_t* ctas_per_sm, float* ms);
/* Calibration: random 32-byte gathers per second on the current device from a
 * table of `rows` 32-byte rows (share = lanes reading consecutive rows).  The
 * stored-H SpMM's dominant traffic is one such gather per stored entry. */
cg_status cg_gather_ceiling(uint64_t rows, int32_t share, double* gathers_per_second);
/* Set (e.g. from a cached tuning) or read the launch shape of the FP32 product. */
cg_status cg_spmm_set_tuning(cg_hamiltonian* h, int32_t warps, int32_t ctas_per_sm);
cg_status cg_spmm_get_tuning(const cg_hamiltonian* h, int32_t* warps, int32_t* ctas_per_sm, int32_t* tuned);
/* Storage the FP32 product of up to 8 vectors reads.  An FP32 matrix built
 * from a basis also holds a block-tiled copy: tiles = (neutron block, neutron
 * block) pairs, 16-bit in-tile columns, x of the column block staged in shared
 * memory per tile.  The reference's counterpart is its fixed CSB blocking
 * (PPMatrix2CSBBlk, include/sm/PPMatrix.cxx:571-656); the choice of format has
 * no counterpart there.  The copy is built with the matrix from 2^26 stored
 * entries up, and on request (cg_spmm_set_format(h, CG_FORMAT_TILED)) below.
 * cg_spmm_autotune picks the faster format when the copy exists (its tiled
 * candidate is reported with ctas_per_sm = 0). */
#define CG_FORMAT_ROWS 0
#define CG_FORMAT_TILED 1
typedef struct {
  int32_t format;          /* CG_FORMAT_ROWS or CG_FORMAT_TILED (in use for <= 8 FP32 vectors) */
  int32_t tiled_available; /* the block-tiled copy exists */
  int32_t warps, stages;   /* tiled product: consumer warps per CTA, ring slots */
  int32_t slices_per_warp; /* tiled product: 32-row slices per consumer warp */
  int32_t reserved;
  uint64_t entries;        /* tiled entries stored, including the slice padding */
  uint64_t units;          /* staged units (tile, entry-group range) */
  uint64_t meta_bytes;     /* per-unit descriptors and run offsets read by one product */
  uint64_t device_bytes;   /* HBM held by the tiled copy */
  uint64_t ident_tiles;    /* scaled-identity tiles (one value each, x read in place) */
  uint64_t ident_entries;  /* stored entries those tiles stand for */
} cg_spmm_format_info;
cg_status cg_spmm_set_format(cg_hamiltonian* h, int32_t format);
cg_status cg_spmm_get_format(const cg_hamiltonian* h, cg_spmm_format_info* info);
/* Launch shape of the tiled product (e.g. from a cached tuning): 32-row slices
 * per consumer warp (1..4, at most 31 consumer warps) and ring slots (2..7,
 * within 227 KB of shared memory). */
cg_status cg_spmm_set_tiled_shape(cg_hamiltonian* h, int32_t slices_per_warp, int32_t stages);

/* -------------------------------------------------------------- Davidson */
/* Block Davidson for the lowest eigenpairs (Davidson-Liu with diagonal
 * preconditioning, classical Gram-Schmidt with re-orthogonalisation, restart by
 * collapse), the algorithm of dvdrvr2 (include/kdav/fsdavidson.cxx:615-775)
 * driven by DavidsonDiagonalization (include/kdav/davidson.cxx:168-225).
 * All vectors, the projection and the small eigensolve stay on the GPU.
 * precision CG_PREC_FP64: FP64 matrix and vectors throughout.
 * precision CG_PREC_FP32: FP32 matrix and vectors, FP64 projections, then FP64
 *   refinement sweeps (CG_PREC_REFINE products) until resid <= tol_resid. */
typedef struct {
  int32_t nstates;   /* eigenpairs wanted (nume)                          */
  int32_t block;     /* vectors added per iteration (mblock)              */
  int32_t lim;       /* maximum basis size before collapse (limmax; <= 128) */
  int32_t maxiter;   /* iteration cap (0: max(40*nstates, 200) as the reference) */
  double crite;      /* eigenvalue-change threshold (reference 1e-15)     */
  double critc;      /* Ritz-coefficient threshold (reference 1e-12)      */
  double critr;      /* residual-norm threshold (reference 1e-8)          */
  double ortho;      /* re-orthogonalisation threshold (reference 1e-9)   */
  double tol_resid;  /* stop when every wanted residual norm <= tol_resid (0: use critr only) */
  double switch_resid; /* FP32 phase hands over to FP64 refinement below this residual */
  int32_t precision; /* CG_PREC_FP64 or CG_PREC_FP32 (must match the matrix) */
  int32_t verbose;   /* 0 silent, 1 per-iteration line on stderr          */
  int32_t ortho_block; /* FP64 only: 0 = one vector at a time as the reference,
                          1 = block Gram-Schmidt (the FP32 phase always uses blocks) */
  int32_t algorithm; /* -1 (default): 0 for FP64, 1 for FP32;
                        0: the reference control flow (convergence bookkeeping of
                        Test_Convergence, collapse to nstates vectors);
                        1: residual-driven block Davidson: every wanted residual is
                        re-checked each iteration, restarts keep `keep` Ritz vectors */
  int32_t keep;      /* algorithm 1: Ritz vectors kept at a restart (0: 2 * nstates; at most 64) */
  int32_t precond;   /* algorithm 1: 1 = diagonal preconditioner (lambda - H_ii), 0 = none */
  int32_t refine_lim;   /* mixed solve: basis limit of the FP64 refinement phase (0: lim) */
  int32_t refine_keep;  /* mixed solve: Ritz vectors kept at its restarts (0: keep; at most 64) */
  int32_t ortho_pip;    /* algorithm 1 (default 1): orthogonalise each new block by two
                           passes of block Gram-Schmidt with Pythagorean inner products,
                           the Cholesky-QR of the block folded into the same update
                           (per pass one X^T Y and one X G over basis + block); falls back
                           to the classical two passes + Cholesky-QR twice when the block
                           is nearly inside the basis.  0: always the classical form. */
  int32_t refine_block; /* mixed solve: vectors added per refinement iteration (0: block) */
  int32_t refine_fp32_corrections; /* mixed solve, algorithm 1 (default 1): in the refinement
                           phase only the starting vectors are multiplied in double-float;
                           the correction blocks use the FP32 product (they enter the Ritz
                           vectors with coefficients of the order of the residual), and the
                           converged Ritz vectors are multiplied again in double-float, their
                           residuals checked, iterating on with double-float products if one
                           is above tol_resid (also when the largest residual has not dropped
                           by 10 % for 4 iterations: tol_resid below the FP32 products' noise).
                           0: every refinement product in double-float. */
} cg_davidson_params;

typedef struct {
  int32_t iterations;        /* outer iterations (all phases)                */
  int32_t refine_iterations; /* of which FP64 refinement                     */
  int64_t matvecs;           /* vectors multiplied by H                      */
  int32_t restarts;          /* collapses                                    */
  int32_t converged;         /* wanted pairs with resid <= tolerance         */
  int32_t ierr;              /* reference-style error code (1024 ortho, 2048 maxiter) */
  double seconds;            /* wall time of the solve                       */
  double spmm_seconds;       /* device time in SpMM                          */
} cg_davidson_stats;

void cg_davidson_defaults(cg_davidson_params* prm, int32_t nstates);
/* eig, de (|last change|), resid: nstates doubles; vecs: NULL or nstates*n
 * doubles (vector k at k*n); init: NULL or n_init*n doubles used as starting
 * vectors (Davidson::InitVectors, include/kdav/cdavidson.cpp:386). */
cg_status cg_davidson(const cg_hamiltonian* h, const cg_davidson_params* prm, const double* init, int32_t n_init,
                      double* eig, double* de, double* resid, double* vecs, cg_davidson_stats* stats);

/* ------------------------------------------------------------- batches */
/* Many independent problems solved together (no counterpart in the reference,
 * which runs one system per DEXHVJTcsb call, davidson/DEXHVJTcsb.cpp:36-77):
 * every basis and stored FP32 (hi + lo) H is built on the GPU and concatenated
 * block-diagonally; problems of dimension <= 64 are diagonalised exactly by a
 * batched Jacobi kernel, the others run one lockstep block Davidson (FP32
 * vectors and products with FP64 projections to switch_resid, then FP64 with
 * the hi + lo product to tol_resid) whose iterations are CUDA graphs covering
 * all problems; a problem whose nstates residuals are below the tolerance is
 * frozen (skipped by every later kernel) until the slowest one finishes. */
typedef struct cg_batch cg_batch;
typedef struct {
  int32_t nstates;      /* eigenpairs per problem, 1..8 (default 5) */
  int32_t block;        /* vectors added per iteration, nstates..8 (default 8) */
  int32_t lim;          /* basis limit <= 40 (default 40) */
  int32_t keep;         /* Ritz vectors kept at a restart, >= block (default 16) */
  int32_t maxiter;      /* per precision phase (default 300) */
  double tol_resid;     /* default 1e-5 */
  double switch_resid;  /* default 1e-4 */
  int32_t use_graph;    /* 1: replay captured CUDA graphs (default) */
} cg_batch_params;
typedef struct {
  int32_t iterations_fp32, iterations_fp64;
  uint64_t graph_launches;   /* iterations replayed as one graph launch each */
  int32_t graph_kernels;     /* kernels in the largest iteration graph */
  uint64_t launches;         /* kernel launches of the solve, graph replays included */
  double seconds, build_seconds;
  int32_t spmm_warps;        /* launch shape the autotuner chose for the block-diagonal product at */
  int32_t spmm_ctas_per_sm;  /* cg_batch_create (warps per CTA, resident CTAs per SM) */
  double spmm_tune_seconds;  /* time the autotuner took (inside build_seconds) */
} cg_batch_stats;
cg_status cg_batch_create(const cg_problem* const* problems, int32_t count, cg_batch** out);
void cg_batch_destroy(cg_batch* b);
cg_status cg_batch_defaults(cg_batch_params* prm);
/* dimension of each problem (count values) */
cg_status cg_batch_dims(const cg_batch* b, uint64_t* dims);
/* eig, resid: count * nstates (NaN where a problem has fewer states); nconv:
 * per problem, states with resid <= tol_resid; stats may be NULL. */
cg_status cg_batch_solve(cg_batch* b, const cg_batch_params* prm, double* eig, double* resid, int32_t* nconv,
                         cg_batch_stats* stats);

/* ----------------------------------------------------- spin and isospin */
/* <J-J+> = ||J+ psi||^2 and <T-T+> = ||T+ psi||^2 of nstates (1..16) vectors of
 * the basis (host, state k at vecs + k*n, the .EE layout), the computation of
 * XSHLJT (include/xsm/XSHLJT.cxx:94-126): PPMatrix::Sqr (include/sm/PPMatrix.cxx:
 * 403-411) of the one-body J+ (SPJPlus) and T+ (SPTPlus, proton -> neutron),
 * include/sm/spherical2sp.cxx:629-700.  Computed on the GPU in FP64. */
cg_status cg_jt_expectations(const cg_basis* b, const double* vecs, int32_t nstates, double* jj, double* tt);
/* 2J from <J-J+> and 2M (SM::JJSpin, include/sm/QN.cxx:40-60): -1 when J + M is
 * not an integer within 0.1. */
int32_t cg_jj_spin(double jj, int32_t two_m);

/* ------------------------------------------------ spectroscopic factors */
/* One-particle removal amplitudes <D_q| a_s |P_p> for every s.p. state s, the
 * overlaps of XSHLSF (xmlshell/XSHLSF.cpp:150-175: PPMatrix::OverlapNH,
 * include/sm/PPMatrix.cxx:275-302, of the one-body operator a_s).  parent: a
 * basis with one neutron or one proton more than daughter, same valence space;
 * vp: np parent vectors, vd: nd daughter vectors (1..16), host, vector k at
 * v + k*n (the .EE layout).  amp: nd * np * n_sps values, amp[(q*np + p)*n_sps
 * + s]; 0 for the states s that cannot connect the two (M, charge, parity)
 * sectors.  Computed on the GPU in FP64. */
cg_status cg_sf_amplitudes(const cg_basis* parent, const double* vp, int32_t np, const cg_basis* daughter,
                           const double* vd, int32_t nd, double* amp);
/* The XSHLSF tool (xmlshell/XSHLSF.cpp:40-222): every <state> of the parent
 * system (parent_xml; parent_system may be NULL when the file holds one system)
 * against every <state> of the daughter system (daughter_xml, NULL: the same
 * file), the vectors read from the .EE files their <wavefunction file id>
 * names; spectroscopic factors written to out_path (NULL: none) per orbital l,
 * or per s.p. state (2j, A, SF) when full is nonzero; a report on stdout. */
cg_status cg_xshlsf(const char* parent_xml, const char* parent_system, const char* daughter_xml,
                    const char* daughter_system, const char* out_path, int32_t full);

/* --------------------------------------- electromagnetic / beta transitions */
/* Flags of cg_xshlemb / cg_transition_terms. */
#define CG_EMB_WEISSKOPF 1      /* -w: B also in Weisskopf units (E, M) */
#define CG_EMB_UNITS 2          /* -u: B in e^2 fm^2L / mu_N^2 fm^(2L-2), oscillator length on moments */
#define CG_EMB_LOGFT 4          /* -ft: log ft (6145 s, g_A = 1.27) */
#define CG_EMB_PHASE_INFINITY 8 /* -p: oscillator radial functions positive at infinity */
/* The m-scheme terms v a+_f a_i of the transition operator of the
 * <operator> node (op_name, or the first one when NULL) of an XML file, for the
 * projection kappa (m_f = m_i + 2 kappa in doubled units), on the s.p. states
 * of system_name: ElectricSPMultipole / MagneticSPMultipole / BetaJAMultipole
 * with oscillator radial integrals, SPTPlus + Hermitian2FullOperator for F
 * (include/sm/EMspherical2sp.cxx, include/xsm/xmlemb.cxx:121-206).  Writes up
 * to cap terms into (i, f, v) and their number into *count (CG_ERR_ARG when
 * cap is too small; NULL arrays with cap 0 only count).  Host only. */
cg_status cg_transition_terms(const char* xml_path, const char* system_name, const char* op_name, int32_t kappa,
                              int32_t flags, int32_t* i, int32_t* f, double* v, int32_t cap, int32_t* count);
/* Transition amplitudes <D_q| sum_t v_t a+_f a_i |P_p> of a one-body operator
 * between two bases with the same number of particles (the overlaps XSHLEMB
 * takes with PPMatrix::OverlapNH, include/sm/PPMatrix.cxx:275-302): vp, vd
 * host vectors (.EE layout), nd 1..16; amp[q*np + p].  On the GPU in FP64. */
cg_status cg_onebody_amplitudes(const cg_basis* parent, const double* vp, int32_t np, const cg_basis* daughter,
                                const double* vd, int32_t nd, const int32_t* i, const int32_t* f, const double* v,
                                int32_t nterms, double* amp);
/* The XSHLEMB tool (xmlshell/XSHLEMB.cpp:116-372): B(op) of the <operator>
 * node of parent_xml (op_name, or the first one when NULL) from every <state>
 * of the parent system to every <state> of the daughter system (daughter_xml,
 * NULL: the parent file), written as <transition> and <moment> children of the
 * parent's states into out_xml (NULL: parent_xml itself); flags CG_EMB_*;
 * a report on stdout.  Radial overlaps from files are refused (CG_ERR_UNSUPPORTED). */
cg_status cg_xshlemb(const char* parent_xml, const char* parent_system, const char* daughter_xml,
                     const char* daughter_system, const char* out_xml, int32_t flags, const char* op_name);
/* XSHLJT (xmlshell/XSHLJT.cpp, include/xsm/XSHLJT.cxx:38-142): the first nstates
 * (all when <= 0) eigenpairs of ee_path get 2J and 2T from <J-J+> / <T-T+>
 * computed on the GPU, E minus lambda*(J-M)(J+M+2)/4 when the system's matrix
 * carries JJ = lambda, and a <state J P T E dE name Ex><wavefunction Jz Tz file
 * id/></state> node each in the system of xml_path (SM::AddState +
 * SM::OrganizeStates, include/xsm/xState.cxx:113-236), written to xml_out (or
 * in place when NULL).  2Tz is Nv - Zv.  n_added (may be NULL) receives the
 * number of states recorded after the system's J / T filters. */
cg_status cg_xshljt(const char* xml_path, const char* system_name, const char* ee_path, int32_t nstates,
                    const char* xml_out, int32_t* n_added);

/* Occupation numbers <psi_k| n_s |psi_k> of every s.p. state (SM::occupation,
 * include/sm/occupation.cxx:55-70) for nst host vectors (.EE layout) of a
 * basis: occ[k * n_sps + s].  On the GPU in FP64. */
cg_status cg_occupations(const cg_basis* b, const double* vecs, int32_t nst, double* occ);
/* The XSHLAO tool (xmlshell/XSHLAO.cpp:22-101): per <state> of the system, the
 * occupation of every orbital of the valence space, neutrons and protons
 * apart, as <occupation name N Z/> children, written to out_xml (NULL: the
 * input file); a report on stdout. */
cg_status cg_xshlao(const char* xml_path, const char* system_name, const char* out_xml);

/* The Xlevels tool (xmlshell/Xlevels.cpp:60-134): the <state> nodes of every
 * space (<nucleus>, else <system>) of nfiles XML files organized together
 * (energy order, names J P (k), Ex from the lowest) and listed on stdout one
 * per line, "name T=T Ex E" plus the experimental Ex of a <data> child and
 * the mean shift and RMS; the organized states written to out_xml when not
 * NULL.  Host only. */
cg_status cg_xlevels(const char* const* files, int32_t nfiles, const char* out_xml);

/* Exact diagonalization of a small stored matrix: every eigenpair of the
 * full symmetric matrix in FP64, ascending (eig: n values; vecs: n vectors of
 * n, state k at vecs + k*n, or NULL).  The path the reference's DXHV takes
 * instead of Davidson when the dimension is at most its limit
 * (include/xsm/DEXHVcsb.cxx:80-110, Eigen's SelfAdjointEigenSolver; here the
 * Householder + implicit QL solver of the Davidson's projected problems on
 * the host).  Stored matrices only (CG_ERR_UNSUPPORTED on the fly), n <= 8192
 * (CG_ERR_ARG above); eigenvector signs are the solver's own. */
cg_status cg_dense_eigensolve(const cg_hamiltonian* h, double* eig, double* vecs);

/* ------------------------------------------------------------ file I/O */
/* .EE eigenpair file: uint32 count, then per state double E, dE, resid,
 * uint64 n, double v[n] (Davidson::Save, include/kdav/cdavidson.cpp:327-368). */
cg_status cg_write_ee(const char* path, int32_t nstates, uint64_t n, const double* eig, const double* de,
                      const double* resid, const double* vecs);

#ifdef __cplusplus
}
#endif
#endif /* COSMO_GB300_H */
