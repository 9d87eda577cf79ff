/*
 * CPU ORACLE — test infrastructure only.  Never shipped, never on the product
 * path: only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline arm
 * load this library, and only as the parity reference or the timed CPU baseline.
 *
 * A plain-C (+OpenMP) restatement of the reference CoSMo algorithms on the CI
 * hot path, each function citing the reference code it follows:
 *   oracle_basis          SM::MakeMBS2 (include/sm/MakeMBS.cxx:186-410)
 *   oracle_build_upper    PPMatrix2CSBBlk rows (include/sm/PPMatrix.cxx:571-656)
 *                         via SM::ActFermiOperator (include/sm/cioperators.cxx:36-62),
 *                         SM::Annihilation / SM::Creation (include/sm/operators.cxx:121-187)
 *                         and SM::locate (include/sm/ManyBodyStates.cxx:92-130)
 *   oracle_csb_*          SparseMatrixCSB and its pull-form TimesMatrix
 *                         (include/tav/csbmatrix.cxx:128-336, 623-663)
 *   oracle_davidson       DavidsonDiagonalization + dvdrvr2
 *                         (include/kdav/davidson.cxx:168-225, include/kdav/fsdavidson.cxx)
 * Parity of this oracle is pinned against outputs of the reference itself
 * (oracle/_ref, tests/golden/).
 */
#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define OR_MAXN 64

/* ------------------------------------------------------------------ basis */
/* MakeMBS2, fermion branch: lexicographic odometer over sorted N-tuples with
 * the exact Mmax/Tmax pruning; states with sum(Jz) == jz, sum(Tz) == tz and
 * parity == par are written.  Returns n, writes at most cap states. */
uint64_t oracle_basis(int ns, const int* m2, const int* tz2, const int* pa, int N, int jz, int tz, int par,
                      uint16_t* out, uint64_t cap) {
  if (N > ns || N > OR_MAXN) return 0;
  int mmax[OR_MAXN + 1], tmax[OR_MAXN + 1], lst[OR_MAXN * 2], cur[OR_MAXN], msum[OR_MAXN], tsum[OR_MAXN];
  int tmp[256];
  for (int i = 0; i < ns; ++i) tmp[i] = m2[i];
  for (int i = 1; i < ns; ++i)
    for (int j = i; j > 0 && tmp[j - 1] > tmp[j]; --j) { int t = tmp[j]; tmp[j] = tmp[j - 1]; tmp[j - 1] = t; }
  mmax[0] = 0;
  for (int k = 1; k <= N; ++k) mmax[k] = mmax[k - 1] + tmp[ns - k];
  for (int i = 0; i < ns; ++i) tmp[i] = tz2[i];
  for (int i = 1; i < ns; ++i)
    for (int j = i; j > 0 && tmp[j - 1] > tmp[j]; --j) { int t = tmp[j]; tmp[j] = tmp[j - 1]; tmp[j - 1] = t; }
  tmax[0] = 0;
  for (int k = 1; k <= N; ++k) tmax[k] = tmax[k - 1] + tmp[ns - k];
  (void)lst;
  int JZ = 0, TZ = 0, LL = 1;
  for (int i = 0; i < N; ++i) { cur[i] = i; JZ += m2[i]; TZ += tz2[i]; LL ^= pa[i]; }
  uint64_t n = 0;
  for (;;) {
    if (JZ == jz && TZ == tz && (LL ^ par)) {
      if (n < cap) for (int i = 0; i < N; ++i) out[n * N + i] = (uint16_t)cur[i];
      ++n;
    }
    msum[0] = 0;
    tsum[0] = 0;
    for (int i = 0; i < N - 1; ++i) { msum[i + 1] = msum[i] + m2[cur[i]]; tsum[i + 1] = tsum[i] + tz2[cur[i]]; }
    int moved = 0;
    for (int i = N - 1; i >= 0; --i) {
      if (abs(jz - msum[i]) > mmax[N - i]) continue;
      if (abs(tz - tsum[i]) > tmax[N - i]) continue;
      if ((ns - 1 - cur[i]) < (N - i)) continue;
      for (int j = N - 1; j >= i; --j) {
        JZ -= m2[cur[j]]; TZ -= tz2[cur[j]]; LL ^= pa[cur[j]];
        cur[j] = cur[i] + j + 1 - i;
        JZ += m2[cur[j]]; TZ += tz2[cur[j]]; LL ^= pa[cur[j]];
      }
      moved = 1;
      break;
    }
    if (!moved) break;
    if (N == 0) break;
  }
  return n;
}

/* ------------------------------------------------------ fermion operators */
/* SM::Annihilation: remove the ordered operator indices from the ordered
 * state, phase ^= (number of kept elements before each removed one) & 1. */
static int annihilate(int* phase, int* nk, uint16_t* ket, int nopr, const uint16_t* opr, int nbra, const uint16_t* bra) {
  if (nopr > nbra) return 0;
  int nnf = 0, nni = 0;
  for (int nno = 0; nno < nopr; ++nno) {
    while (nni < nbra && bra[nni] < opr[nno]) ket[nnf++] = bra[nni++];
    if (nni >= nbra || bra[nni] != opr[nno]) return 0;
    ++nni;
    *phase ^= (nnf & 1);
  }
  while (nni < nbra) ket[nnf++] = bra[nni++];
  *nk = nbra - nopr;
  return 1;
}
/* SM::Creation: merge the ordered operator indices into the ordered state,
 * phase ^= (number of state elements before each inserted one) & 1; a repeated
 * index fails. */
static int create(int* phase, int* nk, uint16_t* ket, int nopr, const uint16_t* opr, int nbra, const uint16_t* bra) {
  int nnf = 0, nni = 0, nno = 0, Nk = nbra + nopr;
  while (nnf < Nk) {
    if (nni == nbra) { ket[nnf++] = opr[nno++]; *phase ^= (nni & 1); continue; }
    if (nno == nopr) { ket[nnf++] = bra[nni++]; continue; }
    if (bra[nni] < opr[nno]) { ket[nnf++] = bra[nni++]; continue; }
    if (bra[nni] > opr[nno]) { ket[nnf++] = opr[nno++]; *phase ^= (nni & 1); continue; }
    return 0;
  }
  *nk = Nk;
  return 1;
}

static int cmp_tuple(int N, const uint16_t* a, const uint16_t* b) {
  for (int i = 0; i < N; ++i) { if (a[i] < b[i]) return -1; if (a[i] > b[i]) return 1; }
  return 0;
}
/* SM::locate with lower limit jl (search upward); n + 1 when absent. */
static uint64_t locate(uint64_t n, int N, const uint16_t* z, const uint16_t* a, uint64_t jl) {
  uint64_t ju = n, jm;
  int happy = cmp_tuple(N, a, z + jl * N);
  jm = jl;
  if (happy * cmp_tuple(N, a, z + (ju - 1) * N) > 0) return n + 1;
  while (happy != 0) {
    jm = (ju + jl) >> 1;
    if (jm == jl) return n + 1;
    happy = cmp_tuple(N, a, z + jm * N);
    if (happy == 1) jl = jm; else ju = jm;
  }
  return jm;
}

/* -------------------------------------------------------------- H rows */
typedef struct { uint16_t st[OR_MAXN]; double v; } fin_t;

/* Operator terms in the reference's STensor key order.  one: keys[2*k]
 * (annihilated, created); two: keys[4*k] (b0 < b1 annihilated, b2 < b3
 * created).  For speed the two-body terms are grouped by their annihilated
 * pair (key order is preserved inside and across groups): a term whose pair is
 * not occupied fails SM::Annihilation anyway, so skipping it changes nothing. */
typedef struct {
  int ns;
  int64_t n1, n2;
  const int32_t* k1; const double* v1;
  const int32_t* k2; const double* v2;
  int64_t* pstart;  /* ns*ns + 1 prefix over annihilated pairs a*ns+b */
} ops_t;

static void ops_index(ops_t* o) {
  int ns = o->ns;
  o->pstart = (int64_t*)calloc((size_t)ns * ns + 1, sizeof(int64_t));
  for (int64_t k = 0; k < o->n2; ++k) o->pstart[o->k2[4 * k] * ns + o->k2[4 * k + 1] + 1]++;
  for (int i = 0; i < ns * ns; ++i) o->pstart[i + 1] += o->pstart[i];
}

/* One upper row: all final states of ESP then VSPX acting on the bra (map
 * accumulation in term order), located upward from the bra, |v| < 1e-14
 * dropped.  Returns the entry count; cols/vals receive them in column order. */
static int64_t hrow(const ops_t* o, uint64_t n, int N, const uint16_t* z, uint64_t bra, fin_t* buf, int64_t bufcap,
                    uint32_t* cols, double* vals) {
  const uint16_t* s = z + bra * N;
  int64_t nf = 0;
  uint16_t mid[OR_MAXN], fin[OR_MAXN];
  /* one-body */
  for (int64_t k = 0; k < o->n1; ++k) {
    uint16_t a = (uint16_t)o->k1[2 * k], c = (uint16_t)o->k1[2 * k + 1];
    int ph = 0, q, q2;
    if (!annihilate(&ph, &q, mid, 1, &a, N, s)) continue;
    if (!create(&ph, &q2, fin, 1, &c, q, mid)) continue;
    if (nf >= bufcap) return -1;
    memcpy(buf[nf].st, fin, sizeof(uint16_t) * N);
    buf[nf++].v = ph ? -o->v1[k] : o->v1[k];
  }
  /* two-body, grouped by occupied annihilated pair (ascending key order) */
  for (int i = 0; i < N; ++i)
    for (int j = i + 1; j < N; ++j) {
      int p = s[i] * o->ns + s[j];
      for (int64_t k = o->pstart[p]; k < o->pstart[p + 1]; ++k) {
        uint16_t an[2] = {(uint16_t)o->k2[4 * k], (uint16_t)o->k2[4 * k + 1]};
        uint16_t cr[2] = {(uint16_t)o->k2[4 * k + 2], (uint16_t)o->k2[4 * k + 3]};
        int ph = 0, q, q2;
        if (!annihilate(&ph, &q, mid, 2, an, N, s)) continue;
        if (!create(&ph, &q2, fin, 2, cr, q, mid)) continue;
        if (nf >= bufcap) return -1;
        memcpy(buf[nf].st, fin, sizeof(uint16_t) * N);
        buf[nf++].v = ph ? -o->v2[k] : o->v2[k];
      }
    }
  /* merge equal final states: a stable merge sort keeps each group in term order */
  {
    /* stable merge sort on buf */
    fin_t* tmpb = (fin_t*)malloc(sizeof(fin_t) * (size_t)(nf ? nf : 1));
    for (int64_t w = 1; w < nf; w <<= 1) {
      for (int64_t lo = 0; lo < nf; lo += 2 * w) {
        int64_t m = lo + w < nf ? lo + w : nf, hi = lo + 2 * w < nf ? lo + 2 * w : nf;
        int64_t a = lo, b = m, t = lo;
        while (a < m && b < hi) tmpb[t++] = (cmp_tuple(N, buf[b].st, buf[a].st) < 0) ? buf[b++] : buf[a++];
        while (a < m) tmpb[t++] = buf[a++];
        while (b < hi) tmpb[t++] = buf[b++];
      }
      memcpy(buf, tmpb, sizeof(fin_t) * (size_t)nf);
    }
    free(tmpb);
  }
  int64_t ne = 0;
  uint64_t locket = bra;
  for (int64_t k = 0; k < nf;) {
    double v = 0.0;
    int64_t e = k;
    while (e < nf && cmp_tuple(N, buf[e].st, buf[k].st) == 0) v += buf[e++].v;
    uint64_t ket = locate(n, N, z, buf[k].st, locket);
    k = e;
    if (ket == n + 1) continue;
    if (fabs(v) < 1e-14) continue;
    locket = ket;
    if (cols) { cols[ne] = (uint32_t)ket; vals[ne] = v; }
    ++ne;
  }
  return ne;
}

/* Upper triangle of H (rows of PPMatrix2CSBBlk) as CSR.  Two passes: counts,
 * then fill.  rowptr has n + 1 entries; cols/vals may be NULL on the first
 * call to obtain rowptr.  Returns nnz or -1 on overflow of a row buffer. */
int64_t oracle_build_upper(int ns, int64_t n1, const int32_t* k1, const double* v1, int64_t n2, const int32_t* k2,
                           const double* v2, uint64_t n, int N, const uint16_t* z, uint64_t* rowptr, uint32_t* cols,
                           double* vals, int nthreads) {
  ops_t o = {ns, n1, n2, k1, v1, k2, v2, NULL};
  ops_index(&o);
  const int64_t cap = 1 << 20;
  int bad = 0;
  if (nthreads > 0) omp_set_num_threads(nthreads);
  if (!cols) {
#pragma omp parallel
    {
      fin_t* buf = (fin_t*)malloc(sizeof(fin_t) * cap);
#pragma omp for schedule(dynamic, 64)
      for (int64_t r = 0; r < (int64_t)n; ++r) {
        int64_t c = hrow(&o, n, N, z, (uint64_t)r, buf, cap, NULL, NULL);
        if (c < 0) bad = 1;
        rowptr[r + 1] = (uint64_t)(c < 0 ? 0 : c);
      }
      free(buf);
    }
    rowptr[0] = 0;
    for (uint64_t r = 0; r < n; ++r) rowptr[r + 1] += rowptr[r];
  } else {
#pragma omp parallel
    {
      fin_t* buf = (fin_t*)malloc(sizeof(fin_t) * cap);
#pragma omp for schedule(dynamic, 64)
      for (int64_t r = 0; r < (int64_t)n; ++r) {
        int64_t c = hrow(&o, n, N, z, (uint64_t)r, buf, cap, cols + rowptr[r], vals + rowptr[r]);
        if (c < 0) bad = 1;
      }
      free(buf);
    }
  }
  free(o.pstart);
  return bad ? -1 : (int64_t)rowptr[n];
}

/* ------------------------------------------------------------------- CSB */
/* Upper-triangle CSB with square br x br blocks, br = floor(sqrt(n)) + 1
 * (include/xsm/DEXHVcsb.cxx:64), u16 local (row, col) and FP64 values. */
typedef struct {
  uint64_t n;
  int br, nb;
  uint64_t* bstart;  /* nb*nb + 1, block (i, j) at i*nb + j, entries in row order */
  uint16_t* lr;
  uint16_t* lc;
  double* val;
} oracle_csb;

oracle_csb* oracle_csb_from_upper(uint64_t n, const uint64_t* rowptr, const uint32_t* cols, const double* vals) {
  oracle_csb* m = (oracle_csb*)calloc(1, sizeof(oracle_csb));
  m->n = n;
  m->br = (int)(sqrt((double)n)) + 1;
  m->nb = (int)((n + m->br - 1) / m->br);
  size_t nbb = (size_t)m->nb * m->nb;
  m->bstart = (uint64_t*)calloc(nbb + 1, sizeof(uint64_t));
  uint64_t nnz = rowptr[n];
  for (uint64_t r = 0; r < n; ++r)
    for (uint64_t k = rowptr[r]; k < rowptr[r + 1]; ++k) m->bstart[(r / m->br) * m->nb + cols[k] / m->br + 1]++;
  for (size_t b = 0; b < nbb; ++b) m->bstart[b + 1] += m->bstart[b];
  uint64_t* fill = (uint64_t*)malloc(sizeof(uint64_t) * (nbb ? nbb : 1));
  memcpy(fill, m->bstart, sizeof(uint64_t) * nbb);
  m->lr = (uint16_t*)malloc(2 * (nnz ? nnz : 1));
  m->lc = (uint16_t*)malloc(2 * (nnz ? nnz : 1));
  m->val = (double*)malloc(8 * (nnz ? nnz : 1));
  for (uint64_t r = 0; r < n; ++r)
    for (uint64_t k = rowptr[r]; k < rowptr[r + 1]; ++k) {
      size_t b = (r / m->br) * m->nb + cols[k] / m->br;
      uint64_t p = fill[b]++;
      m->lr[p] = (uint16_t)(r % m->br);
      m->lc[p] = (uint16_t)(cols[k] % m->br);
      m->val[p] = vals[k];
    }
  free(fill);
  return m;
}

void oracle_csb_free(oracle_csb* m) {
  if (!m) return;
  free(m->bstart); free(m->lr); free(m->lc); free(m->val); free(m);
}

/* Pull-form symmetric product, SparseMatrixCSB::TimesMatrix
 * (include/tav/csbmatrix.cxx:623-663): block row j gathers B_ij^T x_i for
 * i < j and B_ji x_i for i >= j; a diagonal block applies both halves.
 * x, y: n x m column-major (vector k at k*n). */
void oracle_csb_times_matrix(const oracle_csb* M, const double* x, double* y, int m, int nthreads) {
  const uint64_t n = M->n;
  const int br = M->br, nb = M->nb;
  if (nthreads > 0) omp_set_num_threads(nthreads);
  memset(y, 0, sizeof(double) * n * (size_t)m);
#pragma omp parallel for schedule(dynamic, 1)
  for (int j = 0; j < nb; ++j) {
    for (int i = 0; i < nb; ++i) {
      if (i < j) {
        size_t b = (size_t)i * nb + j;
        for (int im = 0; im < m; ++im) {
          double* yy = y + (size_t)im * n + (size_t)j * br;
          const double* xx = x + (size_t)im * n + (size_t)i * br;
          for (uint64_t k = M->bstart[b]; k < M->bstart[b + 1]; ++k) yy[M->lc[k]] += M->val[k] * xx[M->lr[k]];
        }
      } else {
        size_t b = (size_t)j * nb + i;
        for (int im = 0; im < m; ++im) {
          double* yy = y + (size_t)im * n + (size_t)j * br;
          const double* xx = x + (size_t)im * n + (size_t)i * br;
          if (i == j) {
            for (uint64_t k = M->bstart[b]; k < M->bstart[b + 1]; ++k) {
              yy[M->lr[k]] += M->val[k] * xx[M->lc[k]];
              if (M->lr[k] != M->lc[k]) yy[M->lc[k]] += M->val[k] * xx[M->lr[k]];
            }
          } else {
            for (uint64_t k = M->bstart[b]; k < M->bstart[b + 1]; ++k) yy[M->lr[k]] += M->val[k] * xx[M->lc[k]];
          }
        }
      }
    }
  }
}

/* diagonal of the upper CSR (ReadDiagonal) */
void oracle_diagonal(uint64_t n, const uint64_t* rowptr, const uint32_t* cols, const double* vals, double* d) {
  for (uint64_t r = 0; r < n; ++r) {
    d[r] = 0.0;
    for (uint64_t k = rowptr[r]; k < rowptr[r + 1]; ++k)
      if (cols[k] == r) d[r] = vals[k];
  }
}
