/*
 * CPU ORACLE — test infrastructure only (see cosmo_oracle.c).
 *
 * Block Davidson restated from the reference: DavidsonDiagonalization
 * (include/kdav/davidson.cxx:168-225) and dvdrvr2 with its helpers
 * (include/kdav/fsdavidson.cxx:21-775): setup_2d unit start vectors,
 * DiagonalizeS, Test_Convergence, Add_Vectors_To_Basis (residual, diagonal
 * preconditioner guarded at 1e-13), Orthogonalize_Basis (classical
 * Gram-Schmidt repeated while the overlap exceeds `ortho`), collapse at lim.
 * Vectors are FP64, one array per basis vector as in the reference; the matrix
 * product is the pull-form CSB product of cosmo_oracle.c.  A wall-time budget
 * lets the CPU baseline time a bounded number of iterations.
 */
#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef struct oracle_csb oracle_csb;
void oracle_csb_times_matrix(const oracle_csb* M, const double* x, double* y, int m, int nthreads);

static double wall(void) { return omp_get_wtime(); }

/* cyclic Jacobi eigensolver, ascending eigenvalues, eigenvectors as columns of z */
static void jacobi(int n, double* a, double* w, double* z) {
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) z[i * n + j] = (i == j);
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0.0, tot = 0.0;
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) {
        tot += a[i * n + j] * a[i * n + j];
        if (i != j) off += a[i * n + j] * a[i * n + j];
      }
    if (off <= 1e-30 * tot || off == 0.0) break;
    for (int p = 0; p < n; ++p)
      for (int q = p + 1; q < n; ++q) {
        double apq = a[p * n + q];
        if (fabs(apq) < 1e-300) continue;
        double th = (a[q * n + q] - a[p * n + p]) / (2.0 * apq);
        double t = (th >= 0 ? 1.0 : -1.0) / (fabs(th) + sqrt(th * th + 1.0));
        double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
        for (int k = 0; k < n; ++k) {
          double akp = a[k * n + p], akq = a[k * n + q];
          a[k * n + p] = c * akp - s * akq;
          a[k * n + q] = s * akp + c * akq;
        }
        for (int k = 0; k < n; ++k) {
          double apk = a[p * n + k], aqk = a[q * n + k];
          a[p * n + k] = c * apk - s * aqk;
          a[q * n + k] = s * apk + c * aqk;
        }
        for (int k = 0; k < n; ++k) {
          double zkp = z[k * n + p], zkq = z[k * n + q];
          z[k * n + p] = c * zkp - s * zkq;
          z[k * n + q] = s * zkp + c * zkq;
        }
      }
  }
  /* sort ascending (selection, stable on ties) */
  int* idx = (int*)malloc(sizeof(int) * n);
  for (int i = 0; i < n; ++i) idx[i] = i;
  for (int i = 0; i < n; ++i) {
    int m = i;
    for (int j = i + 1; j < n; ++j)
      if (a[idx[j] * n + idx[j]] < a[idx[m] * n + idx[m]]) m = j;
    int t = idx[i]; idx[i] = idx[m]; idx[m] = t;
  }
  double* zz = (double*)malloc(sizeof(double) * n * n);
  for (int k = 0; k < n; ++k) {
    w[k] = a[idx[k] * n + idx[k]];
    for (int i = 0; i < n; ++i) zz[i * n + k] = z[i * n + idx[k]];
  }
  memcpy(z, zz, sizeof(double) * n * n);
  free(zz);
  free(idx);
}

/* Deterministic dot product: fixed chunks summed in chunk order (an OpenMP
 * reduction combines thread partials in completion order, which would make the
 * iteration trace vary from run to run). */
#define DOT_CHUNK 65536
static double dot(uint64_t n, const double* a, const double* b) {
  int64_t nch = (int64_t)((n + DOT_CHUNK - 1) / DOT_CHUNK);
  double part_stack[64];
  double* part = nch <= 64 ? part_stack : (double*)malloc(sizeof(double) * nch);
#pragma omp parallel for schedule(static)
  for (int64_t ch = 0; ch < nch; ++ch) {
    uint64_t lo = (uint64_t)ch * DOT_CHUNK, hi = lo + DOT_CHUNK < n ? lo + DOT_CHUNK : n;
    double s = 0.0;
    for (uint64_t i = lo; i < hi; ++i) s += a[i] * b[i];
    part[ch] = s;
  }
  double s = 0.0;
  for (int64_t ch = 0; ch < nch; ++ch) s += part[ch];
  if (part != part_stack) free(part);
  return s;
}

typedef struct {
  uint64_t n;
  int lim, nume;
  double** b;
  double** ab;
} vecs_t;

/* columns kp of x (list of vectors) combined: out[j] = sum_k z[k*ld + j] x[k] for j < m (in place safe) */
static void combine(uint64_t n, double** x, int kp, const double* z, int ldz, int m) {
#pragma omp parallel
  {
    double* t = (double*)malloc(sizeof(double) * m);
#pragma omp for schedule(static)
    for (int64_t i = 0; i < (int64_t)n; ++i) {
      for (int j = 0; j < m; ++j) {
        double s = 0.0;
        for (int k = 0; k < kp; ++k) s += z[k * ldz + j] * x[k][i];
        t[j] = s;
      }
      for (int j = 0; j < m; ++j) x[j][i] = t[j];
    }
    free(t);
  }
}

/* AB[c0:c0+m] = H B[c0:c0+m]; S rows for the new vectors */
static void add_ab_s(const oracle_csb* M, vecs_t* V, int c0, int m, double* S, int nthreads, int64_t* nmv) {
  uint64_t n = V->n;
  double* x = (double*)malloc(sizeof(double) * n * m);
  double* y = (double*)malloc(sizeof(double) * n * m);
  for (int k = 0; k < m; ++k) memcpy(x + (size_t)k * n, V->b[c0 + k], sizeof(double) * n);
  oracle_csb_times_matrix(M, x, y, m, nthreads);
  for (int k = 0; k < m; ++k) memcpy(V->ab[c0 + k], y + (size_t)k * n, sizeof(double) * n);
  free(x);
  free(y);
  *nmv += m;
  for (int c = 0; c < m; ++c) {
    int i = c0 + c;
    for (int j = 0; j <= i; ++j) {
      double v = dot(n, V->b[j], V->ab[i]);
      S[i * V->lim + j] = v;
      S[j * V->lim + i] = v;
    }
  }
}

/* Orthogonalize_Basis; returns 0 on restart */
static int ortho_seq(vecs_t* V, int basis_dim, int* nncv, double ortho) {
  uint64_t n = V->n;
  int iv = 1, icur = basis_dim;
  double* sc = (double*)malloc(sizeof(double) * (V->lim + 1));
  while (iv <= *nncv) {
    double dprev = 1.0e7;
    int again;
    do {
      again = 0;
      int k = basis_dim + iv - 1;
      double dcur = 0.0;
      for (int j = 0; j < k; ++j) {
        sc[j] = dot(n, V->b[j], V->b[icur]);
        if (fabs(sc[j]) > dcur) dcur = fabs(sc[j]);
      }
      double* v = V->b[icur];
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < (int64_t)n; ++i) {
        double t = v[i];
        for (int j = 0; j < k; ++j) t -= sc[j] * V->b[j][i];
        v[i] = t;
      }
      if (dcur >= ortho) {
        if (dcur > dprev) { *nncv = iv - 1; free(sc); return 0; }
        dprev = dcur;
        again = 1;
      }
    } while (again);
    double nr = sqrt(dot(n, V->b[icur], V->b[icur]));
    if (nr < 1e-14) {
      if (basis_dim + *nncv - 1 != icur) memcpy(V->b[icur], V->b[basis_dim + *nncv - 1], sizeof(double) * n);
      --*nncv;
    } else {
      double f = 1.0 / nr;
      double* v = V->b[icur];
#pragma omp parallel for schedule(static)
      for (int64_t i = 0; i < (int64_t)n; ++i) v[i] *= f;
      ++icur;
      ++iv;
    }
  }
  free(sc);
  return 1;
}

/* Returns ierr (reference codes); fills eig/de/resid (nume) and vectors
 * (nume x n, may be NULL).  time_budget > 0 stops after that many seconds
 * (ierr 4096 marks a budget stop); *iters and *per_iter report the work done.
 * iter_end (maxiter entries, may be NULL) receives the wall time of the end of
 * every iteration, from the start of the first one; *collapses (may be NULL)
 * the number of basis collapses (restarts at the basis limit). */
int oracle_davidson(const oracle_csb* M, const double* diag, uint64_t n, int nume, int mblock, int lim, int maxiter,
                    double crite, double critc, double critr, double ortho, double* eig, double* de, double* resid,
                    double* vout, int* iters, int64_t* matvecs, int nthreads, double time_budget, double* per_iter,
                    double* first_iter_start, double* iter_end, int* collapses) {
  if (nthreads > 0) omp_set_num_threads(nthreads);
  vecs_t V = {n, lim, nume, (double**)malloc(sizeof(double*) * lim), (double**)malloc(sizeof(double*) * lim)};
  for (int k = 0; k < lim; ++k) {
    V.b[k] = (double*)calloc(n, sizeof(double));
    V.ab[k] = (double*)calloc(n, sizeof(double));
  }
  double* S = (double*)calloc((size_t)lim * lim, sizeof(double));
  double* eigs = (double*)calloc(lim, sizeof(double));
  double* old = (double*)calloc(lim, sizeof(double));
  double* zv = (double*)calloc((size_t)lim * lim, sizeof(double));
  double* a = (double*)calloc((size_t)lim * lim, sizeof(double));
  double* w = (double*)calloc(lim, sizeof(double));
  int* icv = (int*)calloc(nume, sizeof(int));
  int* incv = (int*)calloc(lim, sizeof(int));
  double* rowlast = (double*)calloc(lim, sizeof(double));
  int64_t nmv = 0;
  /* setup_2d: unit vectors at the nume lowest diagonals, first index on ties */
  {
    char* used = (char*)calloc(n, 1);
    for (int k = 0; k < nume; ++k) {
      uint64_t imin = n;
      for (uint64_t j = 0; j < n; ++j)
        if (!used[j] && (imin == n || diag[j] < diag[imin])) imin = j;
      used[imin] = 1;
      V.b[k][imin] = 1.0;
    }
    free(used);
  }
  int kpass = nume, nncv = kpass, nloops = 0, ierr = 0, done = 0, first = 1, hit_cap = 1;
  if (collapses) *collapses = 0;
  add_ab_s(M, &V, 0, kpass, S, nthreads, &nmv);
  double t_start = wall();
  if (first_iter_start) *first_iter_start = t_start;
  int kz = kpass; /* dimension of zv */
  do {
    for (int i = 0; i < nume; ++i) old[i] = eigs[i];
    for (int i = 0; i < kpass; ++i)
      for (int j = 0; j < kpass; ++j) a[i * kpass + j] = S[i * lim + j];
    jacobi(kpass, a, w, zv);
    kz = kpass;
    for (int i = 0; i < nume; ++i) eigs[i] = w[i];
    /* Test_Convergence */
    int nnce = 0;
    for (int i = 0; i < nume; ++i)
      if (fabs(old[i] - eigs[i]) >= crite) ++nnce;
    if (nnce == 0) done = 1;
    else {
      int cnt = 0;
      for (int i = 0; i < nume; ++i) {
        if (icv[i]) continue;
        double tmax = fabs(zv[(kpass - 1) * kz + i]);
        for (int l = 1; l <= nncv - 1; ++l) {
          double t = fabs(zv[(kpass - l - 1) * kz + i]);
          if (t > tmax) tmax = t;
        }
        if (tmax < critc) icv[i] = 1;
        else { incv[cnt] = i; rowlast[cnt] = tmax; ++cnt; }
      }
      nncv = cnt;
      done = (cnt == 0);
      for (int i = 0; i < cnt; ++i) {
        int mx = i;
        for (int j = i + 1; j < cnt; ++j)
          if (rowlast[j] > rowlast[mx]) mx = j;
        double tr = rowlast[i]; rowlast[i] = rowlast[mx]; rowlast[mx] = tr;
        int ti = incv[i]; incv[i] = incv[mx]; incv[mx] = ti;
      }
    }
    if (done || (uint64_t)kpass >= n) { hit_cap = 0; break; }
    if (kpass == lim) {
      if (collapses) ++*collapses;
      combine(n, V.b, lim, zv, kz, nume);
      combine(n, V.ab, lim, zv, kz, nume);
      memset(S, 0, sizeof(double) * lim * lim);
      for (int i = 0; i < nume; ++i) S[i * lim + i] = eigs[i];
      memset(zv, 0, sizeof(double) * lim * lim);
      for (int i = 0; i < nume; ++i) zv[i * nume + i] = 1.0;
      kz = nume;
      kpass = nume;
    }
    /* Add_Vectors_To_Basis */
    int limadd = lim < mblock + kpass ? lim : mblock + kpass;
    int nadded = 0, icvc = 0, early = 0, icur = kpass;
    for (int i = 0; i < nncv; ++i) {
      int st = incv[i];
      double* r = V.b[icur];
      double lam = eigs[st];
#pragma omp parallel for schedule(static)
      for (int64_t q = 0; q < (int64_t)n; ++q) {
        double sb = 0.0, sa = 0.0;
        for (int k = 0; k < kpass; ++k) {
          double c = zv[k * kz + st];
          sb += V.b[k][q] * c;
          sa += V.ab[k][q] * c;
        }
        r[q] = sa - lam * sb;
      }
      double ss = sqrt(dot(n, r, r));
      if (ss < critr) {
        ++icvc;
        icv[st] = 1;
        if (icvc < nncv) continue;
        early = 1;
        break;
      }
      incv[nadded++] = st;
      if (nadded + kpass == limadd) break;
      ++icur;
    }
    int restart = 0;
    if (early) done = 1;
    else {
      nncv = nadded;
      for (int i = 0; i < nncv; ++i) {
        double* r = V.b[kpass + i];
        double lam = eigs[incv[i]];
#pragma omp parallel for schedule(static)
        for (int64_t q = 0; q < (int64_t)n; ++q) {
          double dg = lam - diag[q];
          r[q] = (fabs(dg) > 1e-13) ? r[q] / dg : r[q] / 1e-13;
        }
      }
      restart = !ortho_seq(&V, kpass, &nncv, ortho);
    }
    if (!restart) first = 1;
    else if (first) {
      first = 0;
      combine(n, V.b, kpass, zv, kz, nume);
      combine(n, V.ab, kpass, zv, kz, nume);
      memset(S, 0, sizeof(double) * lim * lim);
      for (int i = 0; i < nume; ++i) { S[i * lim + i] = eigs[i]; eigs[i] = 1e30; }
      memset(zv, 0, sizeof(double) * lim * lim);
      for (int i = 0; i < nume; ++i) zv[i * nume + i] = 1.0;
      kz = nume;
      kpass = nume;
      continue;
    } else { ierr += 1024; hit_cap = 0; break; }
    if (done || nncv == 0) { hit_cap = 0; break; }
    add_ab_s(M, &V, kpass, nncv, S, nthreads, &nmv);
    kpass += nncv;
    if (iter_end) iter_end[nloops] = wall() - t_start;
    ++nloops;
    if (time_budget > 0 && wall() - t_start > time_budget) { ierr += 4096; break; }
  } while (nloops < maxiter);
  double t_end = wall();
  if (hit_cap && !(ierr & 4096)) ierr += 2048;
  if (hit_cap) kpass -= nncv;
  for (int i = 0; i < nume; ++i) { de[i] = fabs(old[i] - eigs[i]); eig[i] = eigs[i]; }
  if (kpass != nume) {
    combine(n, V.b, kpass, zv, kz, nume);
    combine(n, V.ab, kpass, zv, kz, nume);
  }
  double* rtmp = (double*)malloc(sizeof(double) * n);
  for (int i = 0; i < nume; ++i) {
    const double* b = V.b[i];
    const double* ab = V.ab[i];
    double lam = eigs[i];
#pragma omp parallel for schedule(static)
    for (int64_t q = 0; q < (int64_t)n; ++q) rtmp[q] = ab[q] - lam * b[q];
    resid[i] = sqrt(dot(n, rtmp, rtmp));
    if (vout) memcpy(vout + (size_t)i * n, V.b[i], sizeof(double) * n);
  }
  free(rtmp);
  if (iters) *iters = nloops;
  if (matvecs) *matvecs = nmv;
  if (per_iter) *per_iter = nloops ? (t_end - t_start) / nloops : 0.0;
  for (int k = 0; k < lim; ++k) { free(V.b[k]); free(V.ab[k]); }
  free(V.b); free(V.ab); free(S); free(eigs); free(old); free(zv); free(a); free(w); free(icv); free(incv);
  free(rowlast);
  return ierr;
}
