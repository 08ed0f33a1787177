/*
 * ks_oracle.c -- CPU restatement of SLEPc 3.22's Krylov-Schur path, used as the ORACLE.
 *
 * TEST INFRASTRUCTURE ONLY: the reference results for the CUDA path's tests and the timed CPU baseline.  Nothing under
 * slepc_gb300/ links, loads or calls this file.  Written from the reference's algorithms in our own code:
 *
 *   Krylov-Schur restart loop ........ src/eps/impls/krylov/krylovschur/krylovschur.c:227-337
 *   setup defaults (ncv, mpd, max_it)  src/eps/interface/epssetup.c:648-671, krylovschur.c:93-117
 *   convergence test / marker ........ src/eps/impls/krylov/epskrylov.c:207-295, epsdefault.c:224-302
 *   Lanczos / Arnoldi factorisation .. src/sys/classes/bv/interface/bvkrylov.c:56-226
 *   CGS1 + IFNEEDED refinement ....... src/sys/classes/bv/interface/bvorthog.c:32-217,380-427
 *   norm estimate / safe sqrt ........ include/slepc/private/bvimpl.h:121-141,346-415
 *   restart V*Q (BVMultInPlace) ...... src/sys/classes/bv/interface/bvblas.c:74-106, bvops.c:220-245
 *   DSHEP (arrow->tridiag, QR, sort)   src/sys/classes/ds/impls/hep/dshep.c:137-426,643-670
 *   DSNHEP (Hessenberg, Schur, sort) . src/sys/classes/ds/impls/dsutil.c:21-171, nhep/dsnhep.c:101-166,303-425
 *   truncation size (2x2 blocks) ..... src/sys/classes/ds/interface/dsops.c:329-344
 *   insertion sort / column perm ..... src/sys/classes/ds/interface/dspriv.c:172-270
 *   sorting criteria ................. src/sys/slepcsc.c:40-245
 *   solve driver / final sort ........ src/eps/interface/epssolve.c:119-208
 *   NHEP eigenvectors (V*X) .......... src/eps/interface/epsdefault.c:105-169
 *
 * The LAPACK routines the reference calls (lartg, steqr, gehrd/orghr, hseqr, lanv2, trexc/laexc, trevc) are not
 * under the reference tree; they are restated here from their published algorithms:
 *   - Givens rotation with r = sign(f)*hypot(f,g)  (LAPACK 3.10 la_lartg convention)
 *   - symmetric tridiagonal implicit QL with Wilkinson shift (Bowdler, Martin, Reinsch, Wilkinson 1968)
 *   - Householder reduction to Hessenberg form; Francis implicit double-shift QR (Francis 1961)
 *   - 2x2 standardisation of real Schur blocks (Bai & Demmel; LAPACK dlanv2 conventions)
 *   - direct swapping of adjacent Schur blocks (Bai & Demmel 1993), QR of [-X; I] for the Sylvester solution
 *   - back substitution for quasi-triangular eigenvectors (LAPACK dtrevc conventions: x(k) = 1, pair sign)
 * Rounding therefore differs from the reference's LAPACK at the 1e-15 level; the Krylov iteration is the same.
 *
 * Random vectors (breakdown restarts, no initial space): splitmix64 uniform[-1,1]; the reference uses PetscRandom.
 */
#include "ks_oracle.h"

#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define DEPS DBL_EPSILON
#define IDX(i, j, ld) ((size_t)(i) + (size_t)(j) * (size_t)(ld))

static double now_s(void) {
  struct timespec t;
  clock_gettime(CLOCK_MONOTONIC, &t);
  return (double)t.tv_sec + 1e-9 * (double)t.tv_nsec;
}

static unsigned long long splitmix64(unsigned long long *s) {
  unsigned long long z = (*s += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
static double urand_pm1(unsigned long long *s) {
  return (double)(splitmix64(s) >> 11) * (2.0 / 9007199254740992.0) - 1.0;
}

/* ------------------------------------------------------------------------------------------------------------
 * Sorting criteria (slepcsc.c:152-245).  Returns -1 if a goes first, 1 if b goes first, 0 if tied.
 * ------------------------------------------------------------------------------------------------------------ */
static int sc_compare(int which, double target, double ar, double ai, double br, double bi) {
  double a, b;
  switch (which) {
    /* SlepcCompareTargetMagnitude / SlepcCompareTargetReal (slepcsc.c:240-267), real scalars */
    case KSOR_TARGET_MAGNITUDE: a = hypot(ar - target, ai); b = hypot(br - target, bi); return a > b ? 1 : (a < b ? -1 : 0);
    case KSOR_TARGET_REAL: a = fabs(ar - target); b = fabs(br - target); return a > b ? 1 : (a < b ? -1 : 0);
    case KSOR_LARGEST_MAGNITUDE: a = hypot(ar, ai); b = hypot(br, bi); return a < b ? 1 : (a > b ? -1 : 0);
    case KSOR_SMALLEST_MAGNITUDE: a = hypot(ar, ai); b = hypot(br, bi); return a > b ? 1 : (a < b ? -1 : 0);
    case KSOR_LARGEST_REAL: a = ar; b = br; return a < b ? 1 : (a > b ? -1 : 0);
    case KSOR_SMALLEST_REAL: a = ar; b = br; return a > b ? 1 : (a < b ? -1 : 0);
    case KSOR_LARGEST_IMAGINARY: a = fabs(ai); b = fabs(bi); return a < b ? 1 : (a > b ? -1 : 0);
    case KSOR_SMALLEST_IMAGINARY: a = fabs(ai); b = fabs(bi); return a > b ? 1 : (a < b ? -1 : 0);
    default: return 0;
  }
}

/* ------------------------------------------------------------------------------------------------------------
 * Small dense kernels
 * ------------------------------------------------------------------------------------------------------------ */
static void givens(double f, double g, double *c, double *s, double *r) {
  if (g == 0.0) { *c = 1.0; *s = 0.0; *r = f; }
  else if (f == 0.0) { *c = 0.0; *s = copysign(1.0, g); *r = fabs(g); }
  else {
    double d = hypot(f, g);
    *c = fabs(f) / d;
    *r = copysign(d, f);
    *s = g / *r;
  }
}
/* x' = c x + s y ; y' = c y - s x  (BLAS rot) over n entries with strides */
static void rot(int n, double *x, int incx, double *y, int incy, double c, double s) {
  for (int i = 0; i < n; i++) {
    double xi = x[(size_t)i * incx], yi = y[(size_t)i * incy];
    x[(size_t)i * incx] = c * xi + s * yi;
    y[(size_t)i * incy] = c * yi - s * xi;
  }
}
static double nrm2(int n, const double *x) {
  double scale = 0.0, ssq = 1.0;
  for (int i = 0; i < n; i++) {
    if (x[i] != 0.0) {
      double a = fabs(x[i]);
      if (scale < a) { ssq = 1.0 + ssq * (scale / a) * (scale / a); scale = a; }
      else ssq += (a / scale) * (a / scale);
    }
  }
  return scale * sqrt(ssq);
}

/* ------------------------------------------------------------------------------------------------------------
 * DSHEP pieces
 * ------------------------------------------------------------------------------------------------------------ */

/* Arrowhead -> tridiagonal by Givens rotations chased to the top-left corner (dshep.c:221-262). The arrow is in
 * the last row/column: d[0..n-1] diagonal, e[0..n-2] couplings of rows 0..n-2 with row n-1. */
static void arrow_to_tridiag(int n, double *d, double *e, double *Q, int ld) {
  if (n <= 2) return;
  for (int j = 0; j < n - 2; j++) {
    double c, s, r;
    /* rotation in the (j, j+1) plane removes e[j] against e[j+1] */
    givens(e[j + 1], e[j], &c, &s, &r);
    e[j + 1] = r;
    s = -s;
    double dj = d[j], dj1 = d[j + 1];
    e[j] = c * s * (dj1 - dj);
    d[j + 1] = s * s * dj + c * c * dj1;
    d[j] = c * c * dj + s * s * dj1;
    rot(j + 2, Q + IDX(0, j, ld), 1, Q + IDX(0, j + 1, ld), 1, c, s);
    /* chase the fill-in up to the corner */
    for (int i = j - 1; i >= 0; i--) {
      double off = -s * e[i];
      e[i] = c * e[i];
      givens(e[i + 1], off, &c, &s, &r);
      e[i + 1] = r;
      s = -s;
      double t = (d[i] - d[i + 1]) * s - 2.0 * c * e[i];
      double p = s * t;
      d[i + 1] += p;
      d[i] -= p;
      e[i] = -e[i] - c * t;
      rot(j + 2, Q + IDX(0, i, ld), 1, Q + IDX(0, i + 1, ld), 1, c, s);
    }
  }
}

/* Symmetric tridiagonal eigenproblem by implicit QL with Wilkinson shifts, accumulating the rotations into
 * the columns of Q (nq rows).  d[0..n-1], e[0..n-2] couples i,i+1 (e[n-1] used as workspace).  Eigenvalues are
 * returned in ascending order with Q's columns permuted alike (the steqr contract).  Returns 0 or failure. */
static int tridiag_ql(int n, double *d, double *e, double *Q, int ld, int nq) {
  if (n <= 0) return 0;
  double saved_last = e[n - 1];
  e[n - 1] = 0.0;
  int maxit = 30 * n;
  int total = 0;
  for (int l = 0; l < n; l++) {
    for (;;) {
      int m;
      for (m = l; m < n - 1; m++) {
        double dd = fabs(d[m]) + fabs(d[m + 1]);
        if (fabs(e[m]) <= DEPS * dd) break;
      }
      if (m == l) break;
      if (++total > maxit) { e[n - 1] = saved_last; return 1; }
      double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
      double r = hypot(g, 1.0);
      g = d[m] - d[l] + e[l] / (g + copysign(r, g));
      double s = 1.0, c = 1.0, p = 0.0;
      int i;
      for (i = m - 1; i >= l; i--) {
        double f = s * e[i], b = c * e[i];
        r = hypot(f, g);
        e[i + 1] = r;
        if (r == 0.0) { d[i + 1] -= p; e[m] = 0.0; break; }
        s = f / r;
        c = g / r;
        g = d[i + 1] - p;
        r = (d[i] - g) * s + 2.0 * c * b;
        p = s * r;
        d[i + 1] = g + p;
        g = c * r - b;
        double *qi = Q + IDX(0, i, ld), *qi1 = Q + IDX(0, i + 1, ld);
        for (int k = 0; k < nq; k++) {
          double t = qi1[k];
          qi1[k] = s * qi[k] + c * t;
          qi[k] = c * qi[k] - s * t;
        }
      }
      if (r == 0.0 && i >= l) continue;
      d[l] -= p;
      e[l] = g;
      e[m] = 0.0;
    }
  }
  /* ascending order, selection sort with column swaps */
  for (int i = 0; i < n - 1; i++) {
    int k = i;
    double p = d[i];
    for (int j = i + 1; j < n; j++) if (d[j] < p) { k = j; p = d[j]; }
    if (k != i) {
      d[k] = d[i];
      d[i] = p;
      double *a = Q + IDX(0, i, ld), *b = Q + IDX(0, k, ld);
      for (int r2 = 0; r2 < nq; r2++) { double t = a[r2]; a[r2] = b[r2]; b[r2] = t; }
    }
  }
  e[n - 1] = saved_last;
  return 0;
}

/* Insertion sort of real eigenvalues on [l, t) (dspriv.c:226-245) */
static void sort_real_perm(int which, double target, int l, int t, const double *eig, int *perm) {
  for (int i = l + 1; i < t; i++) {
    double re = eig[perm[i]];
    int j = i - 1;
    int res = sc_compare(which, target, re, 0.0, eig[perm[j]], 0.0);
    while (res < 0 && j >= l) {
      int tmp = perm[j]; perm[j] = perm[j + 1]; perm[j + 1] = tmp;
      j--;
      if (j >= l) res = sc_compare(which, target, re, 0.0, eig[perm[j]], 0.0);
    }
  }
}

/* Apply a permutation to columns [istart,iend) of Q (rows 0..nrows-1), dspriv.c:250-270 */
static void permute_columns(int istart, int iend, int nrows, double *Q, int ld, int *perm) {
  for (int i = istart; i < iend; i++) {
    int p = perm[i];
    if (p != i) {
      int j = i + 1;
      while (perm[j] != i) j++;
      perm[j] = p;
      perm[i] = i;
      double *a = Q + IDX(0, p, ld), *b = Q + IDX(0, i, ld);
      for (int k = 0; k < nrows; k++) { double t = a[k]; a[k] = b[k]; b[k] = t; }
    }
  }
}

typedef struct {
  int ld, n, l, k, t;
  int state; /* 0 raw, 1 intermediate, 2 condensed, 3 truncated */
  double *d, *e; /* HEP compact storage (ld each) */
  double *A;     /* NHEP dense (ld x ld) */
  double *Q;     /* ld x ld */
  double *X;     /* ld x ld eigenvectors */
  int *perm;
  double *work;
} ds_t;

enum { ST_RAW = 0, ST_INTERMEDIATE = 1, ST_CONDENSED = 2, ST_TRUNCATED = 3 };

static void ds_identity(ds_t *ds) {
  memset(ds->Q, 0, sizeof(double) * (size_t)ds->ld * ds->ld);
  for (int i = 0; i < ds->n; i++) ds->Q[IDX(i, i, ds->ld)] = 1.0;
}

/* DSSolve_HEP_QR (dshep.c:383-426) with DSIntermediate_HEP (dshep.c:267-321), compact storage */
static int ds_hep_solve(ds_t *ds, double *wr, double *wi) {
  int n = ds->n, l = ds->l, ld = ds->ld;
  int n1 = ds->k - l + 1;
  if (n1 < 0) n1 = 0;
  ds_identity(ds);
  double *Qoff = ds->Q + IDX(l, l, ld);
  if (ds->state < ST_INTERMEDIATE) arrow_to_tridiag(n1, ds->d + l, ds->e + l, Qoff, ld);
  for (int i = 0; i < l; i++) wr[i] = ds->d[i];
  int info = tridiag_ql(n - l, ds->d + l, ds->e + l, Qoff, ld, n - l);
  if (info) return 1;
  for (int i = l; i < n; i++) wr[i] = ds->d[i];
  for (int i = 0; i < n - 1; i++) ds->e[i] = 0.0;
  if (wi) for (int i = l; i < n; i++) wi[i] = 0.0;
  ds->state = ST_CONDENSED;
  return 0;
}

/* DSSort_HEP (dshep.c:323-347) */
static void ds_hep_sort(ds_t *ds, int which, double target, double *wr) {
  int n = ds->n, l = ds->l;
  for (int i = 0; i < n; i++) ds->perm[i] = i;
  sort_real_perm(which, target, l, ds->t, ds->d, ds->perm);
  for (int i = l; i < n; i++) wr[i] = ds->d[ds->perm[i]];
  permute_columns(l, n, n, ds->Q, ds->ld, ds->perm);
  for (int i = l; i < n; i++) ds->d[i] = wr[i];
}

/* DSUpdateExtraRow_HEP, compact (dshep.c:349-381) */
static void ds_hep_extrarow(ds_t *ds) {
  int n = ds->n, ld = ds->ld;
  double beta = ds->e[n - 1];
  for (int i = 0; i < n; i++) ds->e[i] = beta * ds->Q[IDX(n - 1, i, ld)];
  ds->k = n;
}

/* ------------------------------------------------------------------------------------------------------------
 * DSNHEP pieces
 * ------------------------------------------------------------------------------------------------------------ */

/* Householder vector for x[0..m-1]: returns tau and overwrites x with v (v[0] = 1) and beta in *beta. */
static double house(int m, double *x, double *beta) {
  double alpha = x[0];
  double xn = m > 1 ? nrm2(m - 1, x + 1) : 0.0;
  if (xn == 0.0) { *beta = alpha; x[0] = 1.0; return 0.0; }
  double b = -copysign(hypot(alpha, xn), alpha);
  double tau = (b - alpha) / b;
  double sc = 1.0 / (alpha - b);
  for (int i = 1; i < m; i++) x[i] *= sc;
  x[0] = 1.0;
  *beta = b;
  return tau;
}

/* Reduce A (n x n, ld) to upper Hessenberg form from column ilo (0-based) on; accumulate into Q (n x n).
 * Rows/columns before ilo are assumed upper triangular already (gehrd with ILO = ilo+1). */
static void hessenberg(int n, int ilo, double *A, int ld, double *Q, double *v) {
  for (int c = ilo; c < n - 2; c++) {
    int m = n - c - 1;
    for (int i = 0; i < m; i++) v[i] = A[IDX(c + 1 + i, c, ld)];
    double beta;
    double tau = house(m, v, &beta);
    if (tau == 0.0) continue;
    /* left: rows c+1..n-1, columns c..n-1 */
    for (int j = c; j < n; j++) {
      double s = 0.0;
      for (int i = 0; i < m; i++) s += v[i] * A[IDX(c + 1 + i, j, ld)];
      s *= tau;
      for (int i = 0; i < m; i++) A[IDX(c + 1 + i, j, ld)] -= s * v[i];
    }
    /* right: rows 0..n-1, columns c+1..n-1 */
    for (int i = 0; i < n; i++) {
      double s = 0.0;
      for (int j = 0; j < m; j++) s += A[IDX(i, c + 1 + j, ld)] * v[j];
      s *= tau;
      for (int j = 0; j < m; j++) A[IDX(i, c + 1 + j, ld)] -= s * v[j];
    }
    for (int i = 0; i < n; i++) {
      double s = 0.0;
      for (int j = 0; j < m; j++) s += Q[IDX(i, c + 1 + j, ld)] * v[j];
      s *= tau;
      for (int j = 0; j < m; j++) Q[IDX(i, c + 1 + j, ld)] -= s * v[j];
    }
    A[IDX(c + 1, c, ld)] = beta;
    for (int i = 1; i < m; i++) A[IDX(c + 1 + i, c, ld)] = 0.0;
  }
}

/* Standardise a 2x2 block [a b; c d]: on return either c == 0 (real pair) or a == d and b*c < 0 (complex pair).
 * The block is transformed as G^T [a b; c d] G with G = [cs -sn; sn cs]. */
static void std2x2(double *a, double *b, double *c, double *d, double *cs, double *sn) {
  const double eps = DEPS;
  if (*c == 0.0) { *cs = 1.0; *sn = 0.0; return; }
  if (*b == 0.0) {
    *cs = 0.0; *sn = 1.0;
    double t = *d; *d = *a; *a = t; *b = -*c; *c = 0.0;
    return;
  }
  if ((*a - *d) == 0.0 && copysign(1.0, *b) != copysign(1.0, *c)) { *cs = 1.0; *sn = 0.0; return; }
  double temp = *a - *d;
  double p = 0.5 * temp;
  double bcmax = fmax(fabs(*b), fabs(*c));
  double bcmis = fmin(fabs(*b), fabs(*c)) * copysign(1.0, *b) * copysign(1.0, *c);
  double scale = fmax(fabs(p), bcmax);
  double z = (p / scale) * p + (bcmax / scale) * bcmis;
  if (z >= 4.0 * eps) {
    /* real eigenvalues: compute a and d */
    z = p + copysign(sqrt(scale) * sqrt(z), p);
    *a = *d + z;
    *d = *d - (bcmax / z) * bcmis;
    double tau = hypot(*c, z);
    *cs = z / tau;
    *sn = *c / tau;
    *b = *b - *c;
    *c = 0.0;
  } else {
    /* complex or nearly equal real eigenvalues: make the diagonal equal */
    double sigma = *b + *c;
    double tau = hypot(sigma, temp);
    *cs = sqrt(0.5 * (1.0 + fabs(sigma) / tau));
    *sn = -(p / (tau * *cs)) * copysign(1.0, sigma);
    double aa = *a * *cs + *b * *sn, bb = -*a * *sn + *b * *cs;
    double cc = *c * *cs + *d * *sn, dd = -*c * *sn + *d * *cs;
    *a = aa * *cs + cc * *sn;
    *b = bb * *cs + dd * *sn;
    *c = -aa * *sn + cc * *cs;
    *d = -bb * *sn + dd * *cs;
    temp = 0.5 * (*a + *d);
    *a = temp;
    *d = temp;
    if (*c != 0.0) {
      if (*b != 0.0) {
        if (copysign(1.0, *b) == copysign(1.0, *c)) {
          /* real eigenvalues after all: reduce to upper triangular */
          double sab = sqrt(fabs(*b)), sac = sqrt(fabs(*c));
          p = copysign(sab * sac, *c);
          tau = 1.0 / sqrt(fabs(*b + *c));
          *a = temp + p;
          *d = temp - p;
          *b = *b - *c;
          *c = 0.0;
          double cs1 = sab * tau, sn1 = sac * tau;
          temp = *cs * cs1 - *sn * sn1;
          *sn = *cs * sn1 + *sn * cs1;
          *cs = temp;
        }
      } else {
        *b = -*c;
        *c = 0.0;
        temp = *cs;
        *cs = -*sn;
        *sn = temp;
      }
    }
  }
}

/* Standardise the 2x2 block at (i, i+1) of T and propagate the rotation to the rest of T and to Q (n rows). */
static void std_block(int n, double *T, int ld, double *Q, int nq, int i) {
  double a = T[IDX(i, i, ld)], b = T[IDX(i, i + 1, ld)], c = T[IDX(i + 1, i, ld)], d = T[IDX(i + 1, i + 1, ld)];
  double cs, sn;
  std2x2(&a, &b, &c, &d, &cs, &sn);
  T[IDX(i, i, ld)] = a; T[IDX(i, i + 1, ld)] = b; T[IDX(i + 1, i, ld)] = c; T[IDX(i + 1, i + 1, ld)] = d;
  if (i + 2 < n) rot(n - i - 2, T + IDX(i, i + 2, ld), ld, T + IDX(i + 1, i + 2, ld), ld, cs, sn);
  if (i > 0) rot(i, T + IDX(0, i, ld), 1, T + IDX(0, i + 1, ld), 1, cs, sn);
  if (Q) rot(nq, Q + IDX(0, i, ld), 1, Q + IDX(0, i + 1, ld), 1, cs, sn);
}

/* Apply a Householder reflector I - tau v v^T (v of length m acting on indices r0..r0+m-1) from both sides of
 * H (full rows 0..n-1 for the right side, columns c0..n-1 for the left side) and to Q. */
static void refl_left(double *H, int ld, int r0, int m, int c0, int c1, const double *v, double tau) {
  for (int j = c0; j <= c1; j++) {
    double s = 0.0;
    for (int i = 0; i < m; i++) s += v[i] * H[IDX(r0 + i, j, ld)];
    s *= tau;
    for (int i = 0; i < m; i++) H[IDX(r0 + i, j, ld)] -= s * v[i];
  }
}
static void refl_right(double *H, int ld, int c0, int m, int r0, int r1, const double *v, double tau) {
  for (int i = r0; i <= r1; i++) {
    double s = 0.0;
    for (int j = 0; j < m; j++) s += H[IDX(i, c0 + j, ld)] * v[j];
    s *= tau;
    for (int j = 0; j < m; j++) H[IDX(i, c0 + j, ld)] -= s * v[j];
  }
}

/* Real Schur form of the upper Hessenberg H (n x n) whose rows/columns before ilo are already triangular, by
 * Francis double-shift QR; full T (wantt) and Schur vectors accumulated into Q.  Returns 0 or failure. */
static int francis_schur(int n, int ilo, double *H, int ld, double *Q, double *wr, double *wi) {
  const double eps = DEPS;
  const double smlnum = DBL_MIN * ((double)n / eps);
  int ihi = n - 1;
  int its = 0, totits = 0, maxtot = 40 * (n > 10 ? n : 10);
  double v[3];
  for (int i = ilo + 2; i < n; i++) for (int j = ilo; j < i - 1; j++) H[IDX(i, j, ld)] = 0.0;
  while (ihi >= ilo) {
    int l;
    /* look for a single small subdiagonal element */
    for (l = ihi; l > ilo; l--) {
      double hll = fabs(H[IDX(l, l - 1, ld)]);
      if (hll <= smlnum) break;
      double tst = fabs(H[IDX(l - 1, l - 1, ld)]) + fabs(H[IDX(l, l, ld)]);
      if (tst == 0.0) {
        if (l - 2 >= ilo) tst += fabs(H[IDX(l - 1, l - 2, ld)]);
        if (l + 1 <= ihi) tst += fabs(H[IDX(l + 1, l, ld)]);
      }
      if (hll <= eps * tst) {
        /* Ahues & Tisseur conservative test */
        double ab = fmax(hll, fabs(H[IDX(l - 1, l, ld)]));
        double ba = fmin(hll, fabs(H[IDX(l - 1, l, ld)]));
        double aa = fmax(fabs(H[IDX(l, l, ld)]), fabs(H[IDX(l - 1, l - 1, ld)] - H[IDX(l, l, ld)]));
        double bb = fmin(fabs(H[IDX(l, l, ld)]), fabs(H[IDX(l - 1, l - 1, ld)] - H[IDX(l, l, ld)]));
        double s = aa + ab;
        if (ba * (ab / s) <= fmax(smlnum, eps * (bb * (aa / s)))) break;
      }
    }
    if (l > ilo) H[IDX(l, l - 1, ld)] = 0.0;
    if (l >= ihi) {
      /* 1x1 block converged */
      wr[ihi] = H[IDX(ihi, ihi, ld)];
      wi[ihi] = 0.0;
      ihi -= 1;
      its = 0;
      continue;
    }
    if (l == ihi - 1) {
      /* 2x2 block converged: standardise */
      std_block(n, H, ld, Q, n, l);
      double a = H[IDX(l, l, ld)], b = H[IDX(l, l + 1, ld)], c = H[IDX(l + 1, l, ld)], d = H[IDX(l + 1, l + 1, ld)];
      wr[l] = a;
      wr[l + 1] = d;
      if (c == 0.0) { wi[l] = 0.0; wi[l + 1] = 0.0; }
      else { wi[l] = sqrt(fabs(b)) * sqrt(fabs(c)); wi[l + 1] = -wi[l]; }
      ihi -= 2;
      its = 0;
      continue;
    }
    if (++totits > maxtot) return 1;
    its++;
    /* shifts */
    double h11, h12, h21, h22;
    if (its == 10) {
      double s = fabs(H[IDX(l + 1, l, ld)]) + fabs(H[IDX(l + 2, l + 1, ld)]);
      h11 = 0.75 * s + H[IDX(l, l, ld)];
      h12 = -0.4375 * s;
      h21 = s;
      h22 = h11;
    } else if (its == 20) {
      double s = fabs(H[IDX(ihi, ihi - 1, ld)]) + fabs(H[IDX(ihi - 1, ihi - 2, ld)]);
      h11 = 0.75 * s + H[IDX(ihi, ihi, ld)];
      h12 = -0.4375 * s;
      h21 = s;
      h22 = h11;
    } else {
      h11 = H[IDX(ihi - 1, ihi - 1, ld)];
      h21 = H[IDX(ihi, ihi - 1, ld)];
      h12 = H[IDX(ihi - 1, ihi, ld)];
      h22 = H[IDX(ihi, ihi, ld)];
    }
    double s = fabs(h11) + fabs(h12) + fabs(h21) + fabs(h22);
    double rt1r, rt1i, rt2r, rt2i;
    if (s == 0.0) { rt1r = rt1i = rt2r = rt2i = 0.0; }
    else {
      h11 /= s; h21 /= s; h12 /= s; h22 /= s;
      double tr = (h11 + h22) / 2.0;
      double det = (h11 - tr) * (h22 - tr) - h12 * h21;
      double rtdisc = sqrt(fabs(det));
      if (det >= 0.0) {
        rt1r = tr * s; rt2r = rt1r; rt1i = rtdisc * s; rt2i = -rt1i;
      } else {
        rt1r = tr + rtdisc; rt2r = tr - rtdisc;
        if (fabs(rt1r - h22) <= fabs(rt2r - h22)) { rt1r *= s; rt2r = rt1r; }
        else { rt2r *= s; rt1r = rt2r; }
        rt1i = rt2i = 0.0;
      }
    }
    /* first column of (H - s1)(H - s2) on the active window, scaled */
    int m = l;
    {
      double h21s = H[IDX(m + 1, m, ld)];
      double sc = fabs(H[IDX(m, m, ld)] - rt2r) + fabs(rt2i) + fabs(h21s);
      h21s /= sc;
      v[0] = h21s * H[IDX(m, m + 1, ld)] + (H[IDX(m, m, ld)] - rt1r) * ((H[IDX(m, m, ld)] - rt2r) / sc) - rt1i * (rt2i / sc);
      v[1] = h21s * (H[IDX(m, m, ld)] + H[IDX(m + 1, m + 1, ld)] - rt1r - rt2r);
      v[2] = h21s * H[IDX(m + 2, m + 1, ld)];
      sc = fabs(v[0]) + fabs(v[1]) + fabs(v[2]);
      v[0] /= sc; v[1] /= sc; v[2] /= sc;
    }
    /* bulge chase */
    for (int k = m; k <= ihi - 1; k++) {
      int nr = (3 < ihi - k + 1) ? 3 : ihi - k + 1;
      if (k > m) {
        for (int i = 0; i < nr; i++) v[i] = H[IDX(k + i, k - 1, ld)];
      }
      double beta;
      double tau = house(nr, v, &beta);
      if (k > m) {
        H[IDX(k, k - 1, ld)] = beta;
        H[IDX(k + 1, k - 1, ld)] = 0.0;
        if (k < ihi - 1) H[IDX(k + 2, k - 1, ld)] = 0.0;
      }
      if (tau != 0.0) {
        refl_left(H, ld, k, nr, k, n - 1, v, tau);
        int r1 = (k + 3 < ihi) ? k + 3 : ihi;
        refl_right(H, ld, k, nr, 0, r1, v, tau);
        refl_right(Q, ld, k, nr, 0, n - 1, v, tau);
      }
    }
  }
  return 0;
}

/* Solve the small Sylvester equation T11 X - X T22 = B (n1, n2 in {1,2}) via its Kronecker system with
 * complete pivoting; tiny pivots are perturbed to smin (as dlasy2 does). X is n1 x n2, column-major ldx=2. */
static void sylv_small(int n1, int n2, const double *T11, int l1, const double *T22, int l2, const double *B,
                       int lb, double *X, double smin) {
  int m = n1 * n2;
  double K[4][4], rhs[4];
  int colp[4];
  for (int i = 0; i < m; i++) for (int j = 0; j < m; j++) K[i][j] = 0.0;
  /* unknown index u = r + c*n1 (X(r,c)) */
  for (int c = 0; c < n2; c++)
    for (int r = 0; r < n1; r++) {
      int u = r + c * n1;
      rhs[u] = B[r + c * lb];
      for (int k = 0; k < n1; k++) K[u][k + c * n1] += T11[r + k * l1];
      for (int k = 0; k < n2; k++) K[u][r + k * n1] -= T22[k + c * l2];
    }
  for (int i = 0; i < m; i++) colp[i] = i;
  for (int p = 0; p < m; p++) {
    int bi = p, bj = p;
    double best = -1.0;
    for (int i = p; i < m; i++) for (int j = p; j < m; j++) if (fabs(K[i][j]) > best) { best = fabs(K[i][j]); bi = i; bj = j; }
    if (bi != p) { for (int j = 0; j < m; j++) { double t = K[p][j]; K[p][j] = K[bi][j]; K[bi][j] = t; } double t = rhs[p]; rhs[p] = rhs[bi]; rhs[bi] = t; }
    if (bj != p) { for (int i = 0; i < m; i++) { double t = K[i][p]; K[i][p] = K[i][bj]; K[i][bj] = t; } int t = colp[p]; colp[p] = colp[bj]; colp[bj] = t; }
    if (fabs(K[p][p]) < smin) K[p][p] = smin;
    for (int i = p + 1; i < m; i++) {
      double f = K[i][p] / K[p][p];
      for (int j = p; j < m; j++) K[i][j] -= f * K[p][j];
      rhs[i] -= f * rhs[p];
    }
  }
  double y[4];
  for (int i = m - 1; i >= 0; i--) {
    double s = rhs[i];
    for (int j = i + 1; j < m; j++) s -= K[i][j] * y[j];
    y[i] = s / K[i][i];
  }
  for (int i = 0; i < m; i++) {
    int u = colp[i];
    X[(u % n1) + (u / n1) * 2] = y[i];
  }
}

/* Swap the adjacent diagonal blocks of sizes n1 (at j1) and n2 (at j1+n1) of the real Schur form T (n x n),
 * updating Q (nq rows).  Returns 0 on success, 1 if the swap was rejected as too ill-conditioned. */
static int swap_blocks(int n, double *T, int ld, double *Q, int nq, int j1, int n1, int n2) {
  const double eps = DEPS;
  if (n1 == 1 && n2 == 1) {
    int j2 = j1 + 1;
    double t11 = T[IDX(j1, j1, ld)], t22 = T[IDX(j2, j2, ld)];
    double cs, sn, r;
    givens(T[IDX(j1, j2, ld)], t22 - t11, &cs, &sn, &r);
    if (j2 + 1 < n) rot(n - j2 - 1, T + IDX(j1, j2 + 1, ld), ld, T + IDX(j2, j2 + 1, ld), ld, cs, sn);
    if (j1 > 0) rot(j1, T + IDX(0, j1, ld), 1, T + IDX(0, j2, ld), 1, cs, sn);
    T[IDX(j1, j1, ld)] = t22;
    T[IDX(j2, j2, ld)] = t11;
    rot(nq, Q + IDX(0, j1, ld), 1, Q + IDX(0, j2, ld), 1, cs, sn);
    return 0;
  }
  int m = n1 + n2;
  double D[16], dnorm = 0.0;
  for (int j = 0; j < m; j++) for (int i = 0; i < m; i++) { D[i + j * 4] = T[IDX(j1 + i, j1 + j, ld)]; dnorm = fmax(dnorm, fabs(D[i + j * 4])); }
  double smin = fmax(eps * dnorm, DBL_MIN / eps);
  double thresh = fmax(20.0 * eps * dnorm, DBL_MIN / eps);
  /* T11 X - X T22 = T12 */
  double X[4];
  sylv_small(n1, n2, D, 4, D + n1 + n1 * 4, 4, D + n1 * 4, 4, X, smin);
  /* orthogonal G whose first n2 columns span [-X; I] (the invariant subspace of T22) */
  double M[4][2];
  for (int c = 0; c < n2; c++) {
    for (int r = 0; r < n1; r++) M[r][c] = -X[r + c * 2];
    for (int r = 0; r < n2; r++) M[n1 + r][c] = (r == c) ? 1.0 : 0.0;
  }
  double G[16];
  for (int i = 0; i < 16; i++) G[i] = 0.0;
  for (int i = 0; i < m; i++) G[i + i * 4] = 1.0;
  for (int c = 0; c < n2; c++) {
    double v[4], beta;
    int len = m - c;
    for (int i = 0; i < len; i++) v[i] = M[c + i][c];
    double tau = house(len, v, &beta);
    if (tau == 0.0) continue;
    /* apply to remaining columns of M */
    for (int cc = c; cc < n2; cc++) {
      double s = 0.0;
      for (int i = 0; i < len; i++) s += v[i] * M[c + i][cc];
      s *= tau;
      for (int i = 0; i < len; i++) M[c + i][cc] -= s * v[i];
    }
    /* G = G * (I - tau v v^T) on columns c.. */
    for (int i = 0; i < m; i++) {
      double s = 0.0;
      for (int j = 0; j < len; j++) s += G[i + (c + j) * 4] * v[j];
      s *= tau;
      for (int j = 0; j < len; j++) G[i + (c + j) * 4] -= s * v[j];
    }
  }
  /* D2 = G^T D G; check the block that must vanish */
  double W[16], D2[16];
  for (int i = 0; i < m; i++) for (int j = 0; j < m; j++) { double s = 0.0; for (int k = 0; k < m; k++) s += D[i + k * 4] * G[k + j * 4]; W[i + j * 4] = s; }
  for (int i = 0; i < m; i++) for (int j = 0; j < m; j++) { double s = 0.0; for (int k = 0; k < m; k++) s += G[k + i * 4] * W[k + j * 4]; D2[i + j * 4] = s; }
  double resid = 0.0;
  for (int i = n2; i < m; i++) for (int j = 0; j < n2; j++) resid = fmax(resid, fabs(D2[i + j * 4]));
  if (resid > thresh) return 1;
  /* apply G to T (rows j1..j1+m-1 from the left over columns j1..n-1; columns from the right over rows 0..j1+m-1) */
  double tmp[4];
  for (int j = j1; j < n; j++) {
    for (int i = 0; i < m; i++) { double s = 0.0; for (int k = 0; k < m; k++) s += G[k + i * 4] * T[IDX(j1 + k, j, ld)]; tmp[i] = s; }
    for (int i = 0; i < m; i++) T[IDX(j1 + i, j, ld)] = tmp[i];
  }
  for (int i = 0; i < j1 + m; i++) {
    for (int j = 0; j < m; j++) { double s = 0.0; for (int k = 0; k < m; k++) s += T[IDX(i, j1 + k, ld)] * G[k + j * 4]; tmp[j] = s; }
    for (int j = 0; j < m; j++) T[IDX(i, j1 + j, ld)] = tmp[j];
  }
  for (int i = 0; i < nq; i++) {
    for (int j = 0; j < m; j++) { double s = 0.0; for (int k = 0; k < m; k++) s += Q[IDX(i, j1 + k, ld)] * G[k + j * 4]; tmp[j] = s; }
    for (int j = 0; j < m; j++) Q[IDX(i, j1 + j, ld)] = tmp[j];
  }
  for (int i = n2; i < m; i++) for (int j = 0; j < n2; j++) T[IDX(j1 + i, j1 + j, ld)] = 0.0;
  /* re-standardise the moved blocks */
  if (n2 == 2) std_block(n, T, ld, Q, nq, j1);
  else T[IDX(j1 + 1, j1, ld)] = 0.0;
  if (n1 == 2) std_block(n, T, ld, Q, nq, j1 + n2);
  return 0;
}

/* Move the diagonal block starting at ifst to position ilst (0-based, ifst > ilst here) by adjacent swaps,
 * as dtrexc does for the "move up" direction.  Returns 0 or 1 (rejected swap). */
static int schur_move(int n, double *T, int ld, double *Q, int nq, int ifst, int ilst) {
  /* normalise to the first row of each block */
  if (ifst > 0 && T[IDX(ifst, ifst - 1, ld)] != 0.0) ifst--;
  int nbf = (ifst < n - 1 && T[IDX(ifst + 1, ifst, ld)] != 0.0) ? 2 : 1;
  if (ilst > 0 && T[IDX(ilst, ilst - 1, ld)] != 0.0) ilst--;
  int here = ifst;
  while (here > ilst) {
    int nbnext = (here >= 2 && T[IDX(here - 1, here - 2, ld)] != 0.0) ? 2 : 1;
    if (swap_blocks(n, T, ld, Q, nq, here - nbnext, nbnext, nbf)) return 1;
    /* a 2x2 block may have split into two 1x1 blocks during the swap */
    if (nbf == 2 && T[IDX(here - nbnext + 1, here - nbnext, ld)] == 0.0) nbf = 1;
    here -= nbnext;
  }
  return 0;
}

/* Eigenvalues from the (standardised) quasi-triangular T for rows [from, n) */
static void schur_eigs(int n, const double *T, int ld, int from, double *wr, double *wi) {
  for (int j = from; j < n; j++) {
    wr[j] = T[IDX(j, j, ld)];
    if (j < n - 1 && T[IDX(j + 1, j, ld)] != 0.0) {
      wi[j] = sqrt(fabs(T[IDX(j + 1, j, ld)])) * sqrt(fabs(T[IDX(j, j + 1, ld)]));
      wr[j + 1] = wr[j];
      wi[j + 1] = -wi[j];
      j++;
    } else wi[j] = 0.0;
  }
}

/* DSSolve_NHEP_Private (dsutil.c:21-87) */
static int ds_nhep_solve(ds_t *ds, double *wr, double *wi) {
  int n = ds->n, ld = ds->ld, l = ds->l;
  double *A = ds->A, *Q = ds->Q;
  memset(Q, 0, sizeof(double) * (size_t)ld * ld);
  for (int i = 0; i < n; i++) Q[IDX(i, i, ld)] = 1.0;
  if (n == 1) { wr[0] = A[0]; wi[0] = 0.0; ds->state = ST_CONDENSED; return 0; }
  if (ds->state < ST_INTERMEDIATE) hessenberg(n, l, A, ld, Q, ds->work);
  int info = francis_schur(n, l, A, ld, Q, wr, wi);
  if (info) return 1;
  for (int j = 0; j < l; j++) {
    if (j == n - 1 || A[IDX(j + 1, j, ld)] == 0.0) { wr[j] = A[IDX(j, j, ld)]; wi[j] = 0.0; }
    else {
      wr[j] = A[IDX(j, j, ld)];
      wr[j + 1] = wr[j];
      wi[j] = sqrt(fabs(A[IDX(j + 1, j, ld)])) * sqrt(fabs(A[IDX(j, j + 1, ld)]));
      wi[j + 1] = -wi[j];
      j++;
    }
  }
  /* hseqr leaves eigenvalues in diagonal order; rebuild them from the standardised T */
  schur_eigs(n, A, ld, l, wr, wi);
  ds->state = ST_CONDENSED;
  return 0;
}

/* DSSort_NHEP_Total (dsutil.c:93-171): selection sort with block moves */
static int ds_nhep_sort(ds_t *ds, int which, double target, double *wr, double *wi) {
  int n = ds->n, ld = ds->ld;
  for (int i = ds->l; i < n - 1; i++) {
    double re = wr[i], im = wi[i];
    int pos = 0;
    int j = i + 1;
    if (im != 0.0) j = i + 2;
    for (; j < n; j++) {
      if (sc_compare(which, target, re, im, wr[j], wi[j]) > 0) { re = wr[j]; im = wi[j]; pos = j; }
      if (wi[j] != 0.0) j++;
    }
    if (pos) {
      if (schur_move(n, ds->A, ld, ds->Q, n, pos, i)) return 1;
      schur_eigs(n, ds->A, ld, i, wr, wi);
    }
    if (wi[i] != 0.0) i++;
  }
  return 0;
}

/* DSUpdateExtraRow_NHEP (dsnhep.c:318-340) */
static void ds_nhep_extrarow(ds_t *ds) {
  int n = ds->n, ld = ds->ld;
  double *x = ds->work, *A = ds->A, *Q = ds->Q;
  for (int i = 0; i < n; i++) x[i] = A[IDX(n, i, ld)];
  for (int i = 0; i < n; i++) {
    double s = 0.0;
    for (int j = 0; j < n; j++) s += Q[IDX(j, i, ld)] * x[j];
    A[IDX(n, i, ld)] = s;
  }
  ds->k = n;
}

/* Right eigenvector of the quasi-triangular T (n x n) for the block starting at k (dtrevc conventions): writes
 * xr (and xi for a complex pair, eigenvalue with positive imaginary part) of length n (zero below the block). */
static void quasi_tri_eigvec(int n, const double *T, int ld, int k, double *xr, double *xi, int *is_complex) {
  const double eps = DEPS;
  double tnorm = 0.0;
  for (int j = 0; j < n; j++) for (int i = 0; i <= j + 1 && i < n; i++) tnorm = fmax(tnorm, fabs(T[IDX(i, j, ld)]));
  double smin = fmax(eps * tnorm, DBL_MIN / eps);
  for (int i = 0; i < n; i++) { xr[i] = 0.0; if (xi) xi[i] = 0.0; }
  int cplx = (k < n - 1 && T[IDX(k + 1, k, ld)] != 0.0);
  *is_complex = cplx;
  if (!cplx) {
    double lam = T[IDX(k, k, ld)];
    xr[k] = 1.0;
    for (int i = k - 1; i >= 0; i--) {
      if (i > 0 && T[IDX(i, i - 1, ld)] != 0.0) {
        /* 2x2 block (i-1, i) */
        double r0 = 0.0, r1 = 0.0;
        for (int j = i + 1; j <= k; j++) { r0 -= T[IDX(i - 1, j, ld)] * xr[j]; r1 -= T[IDX(i, j, ld)] * xr[j]; }
        double a = T[IDX(i - 1, i - 1, ld)] - lam, b = T[IDX(i - 1, i, ld)];
        double c = T[IDX(i, i - 1, ld)], d = T[IDX(i, i, ld)] - lam;
        double det = a * d - b * c;
        if (fabs(det) < smin) det = copysign(smin, det);
        xr[i - 1] = (r0 * d - b * r1) / det;
        xr[i] = (a * r1 - c * r0) / det;
        i--;
      } else {
        double s = 0.0;
        for (int j = i + 1; j <= k; j++) s -= T[IDX(i, j, ld)] * xr[j];
        double den = T[IDX(i, i, ld)] - lam;
        if (fabs(den) < smin) den = smin;
        xr[i] = s / den;
      }
      double mx = 0.0;
      for (int j = i; j <= k; j++) mx = fmax(mx, fabs(xr[j]));
      if (mx > 1e150) for (int j = 0; j <= k; j++) xr[j] /= mx;
    }
  } else {
    /* complex pair at (k, k+1): lambda = wr + i*wi with wi > 0 */
    int ki = k + 1;
    double wr = T[IDX(k, k, ld)];
    double wim = sqrt(fabs(T[IDX(k, ki, ld)])) * sqrt(fabs(T[IDX(ki, k, ld)]));
    if (fabs(T[IDX(k, ki, ld)]) >= fabs(T[IDX(ki, k, ld)])) {
      xr[k] = 1.0;
      xi[ki] = wim / T[IDX(k, ki, ld)];
    } else {
      xr[k] = -wim / T[IDX(ki, k, ld)];
      xi[ki] = 1.0;
    }
    xr[ki] = 0.0;
    xi[k] = 0.0;
    for (int i = k - 1; i >= 0; i--) {
      if (i > 0 && T[IDX(i, i - 1, ld)] != 0.0) {
        double r0r = 0.0, r0i = 0.0, r1r = 0.0, r1i = 0.0;
        for (int j = i + 1; j <= ki; j++) {
          r0r -= T[IDX(i - 1, j, ld)] * xr[j]; r0i -= T[IDX(i - 1, j, ld)] * xi[j];
          r1r -= T[IDX(i, j, ld)] * xr[j]; r1i -= T[IDX(i, j, ld)] * xi[j];
        }
        /* [a b; c d] complex shift by lambda: a' = a - wr - i wim */
        double ar = T[IDX(i - 1, i - 1, ld)] - wr, ai = -wim, b = T[IDX(i - 1, i, ld)];
        double c = T[IDX(i, i - 1, ld)], dr = T[IDX(i, i, ld)] - wr, di = -wim;
        /* det = a d - b c (complex) */
        double detr = ar * dr - ai * di - b * c, deti = ar * di + ai * dr;
        double dd = detr * detr + deti * deti;
        if (dd < smin * smin) { detr = smin; deti = 0.0; dd = smin * smin; }
        /* x0 = (r0 d - b r1)/det ; x1 = (a r1 - c r0)/det */
        double nr = r0r * dr - r0i * di - b * r1r, ni = r0r * di + r0i * dr - b * r1i;
        xr[i - 1] = (nr * detr + ni * deti) / dd;
        xi[i - 1] = (ni * detr - nr * deti) / dd;
        nr = ar * r1r - ai * r1i - c * r0r;
        ni = ar * r1i + ai * r1r - c * r0i;
        xr[i] = (nr * detr + ni * deti) / dd;
        xi[i] = (ni * detr - nr * deti) / dd;
        i--;
      } else {
        double sr = 0.0, si = 0.0;
        for (int j = i + 1; j <= ki; j++) { sr -= T[IDX(i, j, ld)] * xr[j]; si -= T[IDX(i, j, ld)] * xi[j]; }
        double denr = T[IDX(i, i, ld)] - wr, deni = -wim;
        double dd = denr * denr + deni * deni;
        if (dd < smin * smin) { denr = smin; deni = 0.0; dd = smin * smin; }
        xr[i] = (sr * denr + si * deni) / dd;
        xi[i] = (si * denr - sr * deni) / dd;
      }
      double mx = 0.0;
      for (int j = i; j <= ki; j++) mx = fmax(mx, fabs(xr[j]) + fabs(xi[j]));
      if (mx > 1e150) for (int j = 0; j <= ki; j++) { xr[j] /= mx; xi[j] /= mx; }
    }
  }
}

/* DSVectors_NHEP_Eigen_Some (dsnhep.c:101-166): eigenvector k, back-transformed with Q when condensed,
 * normalised; rnorm = |x(n-1)|.  *k advances past a complex pair. */
static void ds_nhep_vector(ds_t *ds, int *k, double *rnorm) {
  int n = ds->n, ld = ds->ld;
  double *Y = ds->X + IDX(0, *k, ld);
  double *yr = ds->work, *yi = ds->work + ld;
  int cplx;
  quasi_tri_eigvec(n, ds->A, ld, *k, yr, yi, &cplx);
  if (ds->state >= ST_CONDENSED) {
    for (int i = 0; i < n; i++) {
      double s = 0.0, t = 0.0;
      for (int j = 0; j < n; j++) { s += ds->Q[IDX(i, j, ld)] * yr[j]; if (cplx) t += ds->Q[IDX(i, j, ld)] * yi[j]; }
      Y[i] = s;
      if (cplx) Y[i + ld] = t;
    }
    double nrm = nrm2(n, Y);
    if (cplx) nrm = hypot(nrm, nrm2(n, Y + ld));
    for (int i = 0; i < n; i++) { Y[i] /= nrm; if (cplx) Y[i + ld] /= nrm; }
  } else {
    for (int i = 0; i < n; i++) { Y[i] = yr[i]; if (cplx) Y[i + ld] = yi[i]; }
  }
  if (rnorm) *rnorm = cplx ? hypot(Y[n - 1], Y[n - 1 + ld]) : fabs(Y[n - 1]);
  if (cplx) (*k)++;
}

/* DSVectors_NHEP_Eigen_All: all eigenvectors of T (back-transformed with Q when condensed), normalised */
static void ds_nhep_vectors_all(ds_t *ds) {
  int n = ds->n, ld = ds->ld;
  for (int k = 0; k < n; k++) {
    double *Y = ds->X + IDX(0, k, ld);
    double *yr = ds->work, *yi = ds->work + ld;
    int cplx;
    quasi_tri_eigvec(n, ds->A, ld, k, yr, yi, &cplx);
    if (ds->state >= ST_CONDENSED) {
      for (int i = 0; i < n; i++) {
        double s = 0.0, t = 0.0;
        for (int j = 0; j < n; j++) { s += ds->Q[IDX(i, j, ld)] * yr[j]; if (cplx) t += ds->Q[IDX(i, j, ld)] * yi[j]; }
        Y[i] = s;
        if (cplx) Y[i + ld] = t;
      }
    } else {
      for (int i = 0; i < n; i++) { Y[i] = yr[i]; if (cplx) Y[i + ld] = yi[i]; }
    }
    double nrm = nrm2(n, Y);
    if (cplx) nrm = hypot(nrm, nrm2(n, Y + ld));
    for (int i = 0; i < n; i++) { Y[i] /= nrm; if (cplx) Y[i + ld] /= nrm; }
    if (cplx) k++;
  }
}

typedef struct {
  int n; const int *rp, *ci; const double *va;
} csr_t;

/* ------------------------------------------------------------------------------------------------------------
 * BV: basis of m columns of length n (column-major, ld = n) with the reference's coefficient buffer layout:
 * column j of `h` (length m+1) holds the orthogonalisation coefficients of vector j, h[j] its norm.
 * ------------------------------------------------------------------------------------------------------------ */
typedef struct {
  int n, m;
  double *V;
  double *h;   /* (m+1) x (m+1) */
  double *c;   /* scratch coefficients (m+1) */
  double eta;
  int refine;  /* 0 never, 1 ifneeded, 2 always */
  int nthreads;
  unsigned long long rng;
  long long npasses;
  const double *bw;  /* diagonal of the inner-product matrix B (BVSetMatrix), NULL: Euclidean */
  const csr_t *bm;   /* or a general inner-product matrix B (CSR) */
  double *bt;        /* scratch for B w (n) */
  int nc;            /* constraint columns (the deflation space, BVInsertConstraints), orthonormal, before V */
  double *W;         /* n x nc */
  double *cw;        /* their coefficients (nc) */
} bv_t;

#define VCOL(bv, j) ((bv)->V + (size_t)(j) * (size_t)(bv)->n)

/* c[0..j-1] = V[:,0:j]^T w, c[j] = w^T w  (BVDotColumnInc, bvorthog.c:32-47); with an inner-product matrix B the
 * dots are against B w (BV_IPMatMult, bvimpl.h:147-157), B diagonal here */
static void bv_dot_inc_b(bv_t *bv, int j, const double *w, double *c);
void ksor_spmv(int n, const int *rowptr, const int *colidx, const double *vals, const double *x, double *y,
               int nthreads);
static void bv_dot_inc_general(bv_t *bv, int j, const double *w, double *c);
static void bv_dot_inc(bv_t *bv, int j, const double *w, double *c) {
  if (bv->bw) { bv_dot_inc_b(bv, j, w, c); return; }
  if (bv->bm) { bv_dot_inc_general(bv, j, w, c); return; }
  int n = bv->n;
  for (int i = 0; i <= j; i++) c[i] = 0.0;
#pragma omp parallel num_threads(bv->nthreads)
  {
    double loc[1024];
    double *lp = (j + 1 <= 1024) ? loc : (double *)calloc((size_t)j + 1, sizeof(double));
    for (int i = 0; i <= j; i++) lp[i] = 0.0;
#pragma omp for schedule(static)
    for (int r0 = 0; r0 < n; r0 += 256) {
      int r1 = r0 + 256 < n ? r0 + 256 : n;
      for (int i = 0; i < j; i++) {
        const double *vi = VCOL(bv, i);
        double s = 0.0;
        for (int r = r0; r < r1; r++) s += vi[r] * w[r];
        lp[i] += s;
      }
      double s = 0.0;
      for (int r = r0; r < r1; r++) s += w[r] * w[r];
      lp[j] += s;
    }
#pragma omp critical
    for (int i = 0; i <= j; i++) c[i] += lp[i];
    if (lp != loc) free(lp);
  }
}

static void bv_dot_inc_b(bv_t *bv, int j, const double *w, double *c) {
  int n = bv->n;
  const double *b = bv->bw;
  for (int i = 0; i <= j; i++) c[i] = 0.0;
#pragma omp parallel num_threads(bv->nthreads)
  {
    double loc[1024];
    double *lp = (j + 1 <= 1024) ? loc : (double *)calloc((size_t)j + 1, sizeof(double));
    for (int i = 0; i <= j; i++) lp[i] = 0.0;
#pragma omp for schedule(static)
    for (int r0 = 0; r0 < n; r0 += 256) {
      int r1 = r0 + 256 < n ? r0 + 256 : n;
      for (int i = 0; i < j; i++) {
        const double *vi = VCOL(bv, i);
        double s = 0.0;
        for (int r = r0; r < r1; r++) s += vi[r] * (b[r] * w[r]);
        lp[i] += s;
      }
      double s = 0.0;
      for (int r = r0; r < r1; r++) s += w[r] * (b[r] * w[r]);
      lp[j] += s;
    }
#pragma omp critical
    for (int i = 0; i <= j; i++) c[i] += lp[i];
    if (lp != loc) free(lp);
  }
}

/* the same with a general B: t = B w (BV_IPMatMult, a MatMult), then V^T t and w^T t */
static void bv_dot_inc_general(bv_t *bv, int j, const double *w, double *c) {
  int n = bv->n;
  const double *t = bv->bt;
  ksor_spmv(n, bv->bm->rp, bv->bm->ci, bv->bm->va, w, bv->bt, bv->nthreads);
  for (int i = 0; i <= j; i++) c[i] = 0.0;
#pragma omp parallel num_threads(bv->nthreads)
  {
    double loc[1024];
    double *lp = (j + 1 <= 1024) ? loc : (double *)calloc((size_t)j + 1, sizeof(double));
    for (int i = 0; i <= j; i++) lp[i] = 0.0;
#pragma omp for schedule(static)
    for (int r0 = 0; r0 < n; r0 += 256) {
      int r1 = r0 + 256 < n ? r0 + 256 : n;
      for (int i = 0; i < j; i++) {
        const double *vi = VCOL(bv, i);
        double s = 0.0;
        for (int r = r0; r < r1; r++) s += vi[r] * t[r];
        lp[i] += s;
      }
      double s = 0.0;
      for (int r = r0; r < r1; r++) s += w[r] * t[r];
      lp[j] += s;
    }
#pragma omp critical
    for (int i = 0; i <= j; i++) c[i] += lp[i];
    if (lp != loc) free(lp);
  }
}

/* w -= V[:,0:j] c  (BVMultColumn / gemv "N") */
static void bv_mult_sub(bv_t *bv, int j, double *w, const double *c) {
  int n = bv->n;
#pragma omp parallel for schedule(static) num_threads(bv->nthreads)
  for (int r0 = 0; r0 < n; r0 += 256) {
    int r1 = r0 + 256 < n ? r0 + 256 : n;
    for (int i = 0; i < j; i++) {
      const double *vi = VCOL(bv, i);
      double ci = c[i];
      for (int r = r0; r < r1; r++) w[r] -= vi[r] * ci;
    }
  }
}

static double vec_norm(int n, const double *w, int nthreads) {
  double s = 0.0;
#pragma omp parallel for reduction(+ : s) num_threads(nthreads)
  for (int r = 0; r < n; r++) s += w[r] * w[r];
  return sqrt(s);
}

/* the norm of the BV's inner product (BVNormColumn with a matrix: sqrt(w^T B w)) */
static double bv_vec_norm(const bv_t *bv, const double *w) {
  if (bv->bm) {
    ksor_spmv(bv->n, bv->bm->rp, bv->bm->ci, bv->bm->va, w, bv->bt, bv->nthreads);
    double s = 0.0;
    for (int r = 0; r < bv->n; r++) s += w[r] * bv->bt[r];
    return sqrt(s > 0.0 ? s : 0.0);
  }
  if (!bv->bw) return vec_norm(bv->n, w, bv->nthreads);
  double s = 0.0;
#pragma omp parallel for reduction(+ : s) num_threads(bv->nthreads)
  for (int r = 0; r < bv->n; r++) s += w[r] * (bv->bw[r] * w[r]);
  return sqrt(s);
}

/* One CGS pass (BVOrthogonalizeCGS1, bvorthog.c:91-132).  Returns 0, or an error code for a negative inner
 * product (BV_SafeSqrt).  onorm/norm optional. */
/* constraint part of one CGS pass (BVOrthogonalizeCGS1 runs over columns -nc..j-1, bvorthog.c): cw = W^T w against
 * the same w as the basis dots, subtracted with them, and counted in the square sum */
static void bv_constraint_dots(bv_t *bv, const double *w) {
  for (int i = 0; i < bv->nc; i++) {
    const double *wi = bv->W + (size_t)i * bv->n;
    double s = 0.0;
    for (int r = 0; r < bv->n; r++) s += wi[r] * w[r];
    bv->cw[i] = s;
  }
}
static void bv_constraint_sub(bv_t *bv, double *w) {
  for (int i = 0; i < bv->nc; i++) {
    const double *wi = bv->W + (size_t)i * bv->n;
    for (int r = 0; r < bv->n; r++) w[r] -= wi[r] * bv->cw[i];
  }
}

static int bv_cgs1(bv_t *bv, int j, double *h, double *onorm, double *norm) {
  double *w = VCOL(bv, j), *c = bv->c;
  double beta = 0.0;
  bv->npasses++;
  bv_dot_inc(bv, j, w, c);
  bv_constraint_dots(bv, w);
  if (onorm || norm) {
    double alpha = c[j];
    if (alpha < -10.0 * DEPS) return 62; /* PETSC_ERR_USER_INPUT: invalid inner product */
    beta = alpha < 0.0 ? 0.0 : sqrt(alpha);
  }
  bv_mult_sub(bv, j, w, c);
  bv_constraint_sub(bv, w);
  if (onorm) *onorm = beta;
  if (norm) {
    double sum = 0.0;
    for (int i = 0; i < bv->nc; i++) sum += bv->cw[i] * bv->cw[i];
    for (int i = 0; i < j; i++) sum += c[i] * c[i];
    double nn = beta * beta - sum;
    if (nn <= 0.0) *norm = bv_vec_norm(bv, w);
    else *norm = sqrt(nn);
  }
  for (int i = 0; i < j; i++) h[i] += c[i];
  return 0;
}

/* BVOrthogonalizeGS (bvorthog.c:145-217) on column j; h = coefficient column j */
static int bv_orthogonalize_gs(bv_t *bv, int j, double *nrm_out, int *lindep) {
  double *h = bv->h + (size_t)j * (bv->m + 1);
  double onrm = 0.0, nrm = 0.0;
  int err;
  for (int i = 0; i < j; i++) h[i] = 0.0;
  if (bv->refine == 1) {
    if ((err = bv_cgs1(bv, j, h, &onrm, &nrm))) return err;
    int l = 1;
    while (l < 3 && nrm != 0.0 && fabs(nrm) < bv->eta * fabs(onrm)) {
      l++;
      if ((err = bv_cgs1(bv, j, h, &onrm, &nrm))) return err;
    }
    *lindep = !(nrm != 0.0 && fabs(nrm) >= bv->eta * fabs(onrm));
  } else if (bv->refine == 0) {
    if ((err = bv_cgs1(bv, j, h, NULL, NULL))) return err;
    nrm = bv_vec_norm(bv, VCOL(bv, j));
    *lindep = (nrm == 0.0);
  } else {
    if ((err = bv_cgs1(bv, j, h, NULL, NULL))) return err;
    if ((err = bv_cgs1(bv, j, h, &onrm, &nrm))) return err;
    *lindep = !(nrm != 0.0 && fabs(nrm) >= bv->eta * fabs(onrm));
  }
  *nrm_out = nrm;
  h[j] = *lindep ? 0.0 : nrm;
  return 0;
}

static void bv_scale(bv_t *bv, int j, double a) {
  double *w = VCOL(bv, j);
#pragma omp parallel for num_threads(bv->nthreads)
  for (int r = 0; r < bv->n; r++) w[r] *= a;
}

/* BVOrthonormalizeColumn (bvorthog.c:380-427) with replace = FALSE */
static int bv_orthonormalize(bv_t *bv, int j, double *nrm, int *lindep) {
  int err = bv_orthogonalize_gs(bv, j, nrm, lindep);
  if (err) return err;
  if (*nrm != 1.0 && *nrm != 0.0) bv_scale(bv, j, 1.0 / *nrm);
  return 0;
}

static void bv_random_column(bv_t *bv, int j) {
  double *w = VCOL(bv, j);
  for (int r = 0; r < bv->n; r++) w[r] = urand_pm1(&bv->rng);
}

/* V[:, s:e] = V[:, a:b] * Q[a:b, s:e]  (BVMultInPlace with active columns [a,b), bvblas.c:74-106) */
static void bv_mult_in_place(bv_t *bv, const double *Q, int ldq, int a, int b, int s, int e) {
  int n = bv->n, kk = b - a, nn = e - s;
  if (nn <= 0 || kk <= 0) return;
#pragma omp parallel num_threads(bv->nthreads)
  {
    const int BS = 64;
    double *work = (double *)malloc(sizeof(double) * (size_t)BS * nn);
#pragma omp for schedule(static)
    for (int r0 = 0; r0 < n; r0 += BS) {
      int rb = r0 + BS < n ? BS : n - r0;
      for (int c = 0; c < nn; c++) {
        double *wc = work + (size_t)c * BS;
        for (int r = 0; r < rb; r++) wc[r] = 0.0;
        for (int k = 0; k < kk; k++) {
          double q = Q[IDX(a + k, s + c, ldq)];
          const double *vk = VCOL(bv, a + k) + r0;
          for (int r = 0; r < rb; r++) wc[r] += vk[r] * q;
        }
      }
      for (int c = 0; c < nn; c++) memcpy(VCOL(bv, s + c) + r0, work + (size_t)c * BS, sizeof(double) * rb);
    }
    free(work);
  }
}

void ksor_spmv(int n, const int *rowptr, const int *colidx, const double *vals, const double *x, double *y,
               int nthreads) {
#pragma omp parallel for schedule(static, 1024) num_threads(nthreads > 0 ? nthreads : 1)
  for (int r = 0; r < n; r++) {
    double s = 0.0;
    for (int p = rowptr[r]; p < rowptr[r + 1]; p++) s += vals[p] * x[colidx[p]];
    y[r] = s;
  }
}

/* ------------------------------------------------------------------------------------------------------------
 * The Krylov-Schur solver
 * ------------------------------------------------------------------------------------------------------------ */

/* DSTranslateHarmonic_NHEP, translation (dsnhep.c:466-507): g = (A - tau I)^T \ (beta e_n), A(:, n-1) += beta g,
 * returns gamma = sqrt(1 + g'g).  The reference factors A - tau I (getrf) and solves with its transpose (getrs "C");
 * here the transpose is factored with partial pivoting, which solves the same system. */
static int harmonic_translate(ds_t *ds, double tau, double beta, double *g, double *gamma) {
  int n = ds->n, ld = ds->ld;
  double *B = (double *)malloc(sizeof(double) * (size_t)n * n);
  if (!B) return 55;
  for (int j = 0; j < n; j++)
    for (int i = 0; i < n; i++) B[i + (size_t)j * n] = ds->A[IDX(j, i, ld)] - (i == j ? tau : 0.0);
  for (int i = 0; i < n; i++) g[i] = 0.0;
  g[n - 1] = beta;
  int err = 0;
  for (int c = 0; c < n; c++) {
    int p = c;
    for (int i = c + 1; i < n; i++) if (fabs(B[i + (size_t)c * n]) > fabs(B[p + (size_t)c * n])) p = i;
    if (B[p + (size_t)c * n] == 0.0) { err = 76; break; }
    if (p != c) {
      for (int j = 0; j < n; j++) { double t = B[c + (size_t)j * n]; B[c + (size_t)j * n] = B[p + (size_t)j * n]; B[p + (size_t)j * n] = t; }
      double t = g[c]; g[c] = g[p]; g[p] = t;
    }
    for (int i = c + 1; i < n; i++) {
      double f = B[i + (size_t)c * n] / B[c + (size_t)c * n];
      for (int j = c + 1; j < n; j++) B[i + (size_t)j * n] -= f * B[c + (size_t)j * n];
      g[i] -= f * g[c];
    }
  }
  if (!err)
    for (int i = n - 1; i >= 0; i--) {
      double s = g[i];
      for (int j = i + 1; j < n; j++) s -= B[i + (size_t)j * n] * g[j];
      g[i] = s / B[i + (size_t)i * n];
    }
  free(B);
  if (err) return err;
  for (int i = 0; i < n; i++) ds->A[IDX(i, n - 1, ld)] += g[i] * beta;
  *gamma = hypot(1.0, nrm2(n, g));
  return 0;
}

/* DSTranslateHarmonic_NHEP, recovery (dsnhep.c:508-535) with DSSetDimensions(n, k, l): ghat = -Q(:,0:k+l)' g;
 * A(i, j) += ghat_i Q(n-1, j) beta for i < k+l, k <= j < k+l; g <- g + Q(:,0:k+l) ghat; gamma = sqrt(1 + g'g);
 * the extra row entries k..k+l-1 are multiplied by gamma. */
static void harmonic_recover(ds_t *ds, int k, int l, double beta, double *g, double *gamma) {
  int n = ds->n, ld = ds->ld, ncol = k + l;
  double *gh = ds->work;
  for (int j = 0; j < ncol; j++) {
    double s = 0.0;
    for (int i = 0; i < n; i++) s += ds->Q[IDX(i, j, ld)] * g[i];
    gh[j] = -s;
  }
  for (int i = 0; i < ncol; i++)
    for (int j = k; j < ncol; j++) ds->A[IDX(i, j, ld)] += gh[i] * ds->Q[IDX(n - 1, j, ld)] * beta;
  for (int i = 0; i < n; i++) {
    double s = 0.0;
    for (int j = 0; j < ncol; j++) s += ds->Q[IDX(i, j, ld)] * gh[j];
    g[i] += s;
  }
  *gamma = hypot(1.0, nrm2(n, g));
  for (int j = k; j < ncol; j++) ds->A[IDX(n, j, ld)] *= *gamma;
}

/* BVMatLanczos / BVMatArnoldi (bvkrylov.c:56-226): steps j = k..m-1 */
/* STApply of STSHIFT with shift 0 (st/impls/shift/shift.c): w = A v, then w = B^-1 w for a generalised problem (a
 * direct solve with the diagonal B: one division per entry) */
/* the operator of STSHIFT with shift 0: A, or B^-1 A with a direct solve with B -- a division per entry for a
 * diagonal B, or a dense LU factorisation with partial pivoting for a general one (the reference's default
 * KSPPREONLY + PCLU) */
typedef struct {
  const double *bdiv;     /* diagonal B, or NULL */
  const double *lu;       /* general B: n x n row-major LU factors (unit lower L below the diagonal), or NULL */
  const int *piv;         /* its row interchanges */
} stop_t;

/* LU factorisation with partial pivoting (Doolittle, row interchanges as in LAPACK's getrf); 0, or the first
 * zero pivot + 1 */
static int lu_factor(int n, double *a, int *piv) {
  for (int k = 0; k < n; k++) {
    int p = k;
    for (int i = k + 1; i < n; i++)
      if (fabs(a[(size_t)i * n + k]) > fabs(a[(size_t)p * n + k])) p = i;
    piv[k] = p;
    if (a[(size_t)p * n + k] == 0.0) return k + 1;
    if (p != k)
      for (int j = 0; j < n; j++) {
        double t = a[(size_t)k * n + j];
        a[(size_t)k * n + j] = a[(size_t)p * n + j];
        a[(size_t)p * n + j] = t;
      }
    const double d = a[(size_t)k * n + k];
    for (int i = k + 1; i < n; i++) {
      double l = a[(size_t)i * n + k] / d;
      a[(size_t)i * n + k] = l;
      if (l != 0.0)
        for (int j = k + 1; j < n; j++) a[(size_t)i * n + j] -= l * a[(size_t)k * n + j];
    }
  }
  return 0;
}

static void lu_solve(int n, const double *a, const int *piv, double *x) {
  for (int k = 0; k < n; k++)
    if (piv[k] != k) {
      double t = x[k];
      x[k] = x[piv[k]];
      x[piv[k]] = t;
    }
  for (int i = 1; i < n; i++) {
    double s = x[i];
    for (int j = 0; j < i; j++) s -= a[(size_t)i * n + j] * x[j];
    x[i] = s;
  }
  for (int i = n - 1; i >= 0; i--) {
    double s = x[i];
    for (int j = i + 1; j < n; j++) s -= a[(size_t)i * n + j] * x[j];
    x[i] = s / a[(size_t)i * n + i];
  }
}

static void st_apply(const csr_t *A, const stop_t *op, const double *v, double *w, int nthreads) {
  ksor_spmv(A->n, A->rp, A->ci, A->va, v, w, nthreads);
  if (op->bdiv)
    for (int r = 0; r < A->n; r++) w[r] /= op->bdiv[r];
  else if (op->lu)
    lu_solve(A->n, op->lu, op->piv, w);
}

static int krylov_factor(bv_t *bv, const csr_t *A, const stop_t *op, int hermitian, ds_t *ds, int k, int *m,
                         double *beta, int *breakdown, long long *nsteps) {
  int lindep = 0, err;
  double nrm = 0.0;
  int j;
  for (j = k; j < *m; j++) {
    st_apply(A, op, VCOL(bv, j), VCOL(bv, j + 1), bv->nthreads);
    (*nsteps)++;
    if ((err = bv_orthonormalize(bv, j + 1, &nrm, &lindep))) return err;
    if (lindep) { *m = j + 1; break; }
  }
  *beta = nrm;
  *breakdown = lindep;
  int ld = ds->ld, hs = bv->m + 1;
  if (hermitian) {
    for (j = k; j < *m; j++) {
      ds->d[j] = bv->h[(size_t)(j + 1) * hs + j];
      ds->e[j] = bv->h[(size_t)(j + 1) * hs + j + 1];
    }
  } else {
    for (j = k; j < *m - 1; j++)
      for (int i = 0; i < j + 2; i++) ds->A[IDX(i, j, ld)] = bv->h[(size_t)(j + 1) * hs + i];
    for (int i = 0; i < *m; i++) ds->A[IDX(i, *m - 1, ld)] = bv->h[(size_t)(*m) * hs + i];
    if (ld > *m) ds->A[IDX(*m, *m - 1, ld)] = bv->h[(size_t)(*m) * hs + *m];
  }
  return 0;
}

int ksor_solve(int n, const int *rowptr, const int *colidx, const double *vals,
               int hermitian, int which, int nev, int ncv, int mpd, double tol, int max_it,
               double keep, int lock, int nthreads, const double *v0, unsigned long long seed,
               double time_budget_s,
               int *info, int ncv_cap, double *eigr_out, double *eigi_out, double *errest_out, double *X,
               int harmonic, double target) {
  return ksor_solve_gen(n, rowptr, colidx, vals, NULL, hermitian, which, nev, ncv, mpd, tol, max_it, keep, lock,
                        nthreads, v0, seed, time_budget_s, info, ncv_cap, eigr_out, eigi_out, errest_out, X, harmonic,
                        target, KSOR_CONV_REL, 0.0, 0.0, 1);
}

/* the deflation space of the next solve (EPSSetDeflationSpace, epssetup.c:523-560): nds vectors of length n,
 * column-major; the caller keeps them alive until the solve returns */
static int g_defl_n = 0;
static const double *g_defl = NULL;
void ksor_set_deflation(int nds, const double *W) {
  g_defl_n = W ? nds : 0;
  g_defl = W;
}

/* BVInsertConstraints (bvbasic.c): each vector orthonormalised against the ones kept before it (classical
 * Gram-Schmidt, refined if needed, as BVOrthonormalizeColumn); a linearly dependent one is dropped */
static void insert_constraints(bv_t *bv, int nds, const double *U) {
  const int n = bv->n;
  bv->nc = 0;
  for (int k = 0; k < nds; k++) {
    double *w = bv->W + (size_t)bv->nc * n;
    memcpy(w, U + (size_t)k * n, sizeof(double) * n);
    double onrm = 0.0, nrm = 0.0;
    for (int pass = 0; pass < 3; pass++) {
      double a = 0.0, sum = 0.0;
      for (int r = 0; r < n; r++) a += w[r] * w[r];
      bv_constraint_dots(bv, w);
      bv_constraint_sub(bv, w);
      for (int i = 0; i < bv->nc; i++) sum += bv->cw[i] * bv->cw[i];
      onrm = sqrt(a);
      nrm = (a - sum > 0.0) ? sqrt(a - sum) : nrm2(n, w);
      if (!(nrm != 0.0 && nrm < bv->eta * onrm)) break;
    }
    if (nrm == 0.0 || nrm < bv->eta * onrm) continue;  /* linearly dependent */
    for (int r = 0; r < n; r++) w[r] /= nrm;
    bv->nc++;
  }
}

static ksor_monitor_fn g_monitor = NULL;
static void *g_monitor_ctx = NULL;
void ksor_set_monitor(ksor_monitor_fn fn, void *ctx) {
  g_monitor = fn;
  g_monitor_ctx = ctx;
}

static int solve_impl(int n, const int *rowptr, const int *colidx, const double *vals, const double *bdiag,
                      const csr_t *bcsr, int hermitian, int which, int nev, int ncv, int mpd, double tol, int max_it,
                      double keep, int lock, int nthreads, const double *v0, unsigned long long seed,
                      double time_budget_s, int *info, int ncv_cap, double *eigr_out, double *eigi_out,
                      double *errest_out, double *X, int harmonic, double target, int conv, double nrma,
                      double nrmb, int purify);

int ksor_solve_gen(int n, const int *rowptr, const int *colidx, const double *vals, const double *bdiag,
                   int hermitian, int which, int nev, int ncv, int mpd, double tol, int max_it,
                   double keep, int lock, int nthreads, const double *v0, unsigned long long seed,
                   double time_budget_s,
                   int *info, int ncv_cap, double *eigr_out, double *eigi_out, double *errest_out, double *X,
                   int harmonic, double target, int conv, double nrma, double nrmb, int purify) {
  return solve_impl(n, rowptr, colidx, vals, bdiag, NULL, hermitian, which, nev, ncv, mpd, tol, max_it, keep, lock,
                    nthreads, v0, seed, time_budget_s, info, ncv_cap, eigr_out, eigi_out, errest_out, X, harmonic,
                    target, conv, nrma, nrmb, purify);
}

int ksor_solve_genb(int n, const int *rowptr, const int *colidx, const double *vals, const int *browptr,
                    const int *bcolidx, const double *bvals, int hermitian, int which, int nev, int ncv, int mpd,
                    double tol, int max_it, double keep, int lock, int nthreads, const double *v0,
                    unsigned long long seed, double time_budget_s, int *info, int ncv_cap, double *eigr_out,
                    double *eigi_out, double *errest_out, double *X, int harmonic, double target, int conv,
                    double nrma, double nrmb, int purify) {
  const csr_t B = {n, browptr, bcolidx, bvals};
  return solve_impl(n, rowptr, colidx, vals, NULL, &B, hermitian, which, nev, ncv, mpd, tol, max_it, keep, lock,
                    nthreads, v0, seed, time_budget_s, info, ncv_cap, eigr_out, eigi_out, errest_out, X, harmonic,
                    target, conv, nrma, nrmb, purify);
}

static int solve_impl(int n, const int *rowptr, const int *colidx, const double *vals, const double *bdiag,
                      const csr_t *bcsr, int hermitian, int which, int nev, int ncv, int mpd, double tol, int max_it,
                      double keep, int lock, int nthreads, const double *v0, unsigned long long seed,
                      double time_budget_s, int *info, int ncv_cap, double *eigr_out, double *eigi_out,
                      double *errest_out, double *X, int harmonic, double target, int conv, double nrma,
                      double nrmb, int purify) {
  double t_start = now_s();
  /* generalised problems (epssetup.c:321-329): B^-1 A, with the B-inner product when Hermitian (GHEP); start
   * vectors forced into the range of the operator and eigenvectors purified for GHEP (epssolve.c:855-862,
   * epsdefault.c:28-50) */
  const int ghep = (bdiag || bcsr) && hermitian;
  const csr_t Acsr = {n, rowptr, colidx, vals};
  stop_t op = {bdiag, NULL, NULL};
  double *lu = NULL;
  int *piv = NULL;
  /* EPSSolve_KrylovSchur_Default (krylovschur.c:238-239): harmonic extraction runs the non-symmetric variant */
  if (harmonic) hermitian = 0;
  if (n <= 0 || nev <= 0) return 63;
  /* EPSSetUp clamps the dimensions to the problem size (epssetup.c:337-338); ncv = n is a full basis whose last
   * factorisation step breaks down with every eigenvalue converged */
  if (nev > n) nev = n;
  if (ncv > n) ncv = n;
  if (nthreads <= 0) nthreads = 1;
  /* EPSSetDimensions_Default (epssetup.c:648-671) */
  if (ncv <= 0) {
    if (mpd > 0) ncv = (n < nev + mpd) ? n : nev + mpd;
    else if (nev < 500) { int t = 2 * nev > nev + 15 ? 2 * nev : nev + 15; ncv = n < t ? n : t; }
    else { mpd = 500; ncv = n < nev + mpd ? n : nev + mpd; }
  } else if (!(ncv >= nev + 1 || (ncv == nev && ncv == n))) return 62;
  if (mpd <= 0) mpd = ncv;
  if (ncv > nev + mpd) return 62;
  if (max_it <= 0) max_it = (2 * n / ncv) > 100 ? 2 * n / ncv : 100;
  if (tol <= 0.0) tol = 1e-8;
  if (keep <= 0.0) keep = 0.5;
  if (ncv_cap < ncv) return 60;

  int ld = ncv + 1;
  bv_t bv = {0};
  bv.n = n; bv.m = ncv + 1; bv.eta = 0.7071; bv.refine = 1; bv.nthreads = nthreads;
  bv.rng = seed ? seed : 0x5eed;
  bv.bw = ghep ? bdiag : NULL;
  bv.bm = ghep ? bcsr : NULL;
  bv.V = (double *)calloc((size_t)n * bv.m, sizeof(double));
  if (g_defl_n > 0) {
    if (bdiag || bcsr) { free(bv.V); return 56; } /* deflation spaces of generalised problems: not restated */
    bv.W = (double *)calloc((size_t)n * g_defl_n, sizeof(double));
    bv.cw = (double *)calloc((size_t)g_defl_n, sizeof(double));
    insert_constraints(&bv, g_defl_n, g_defl);
  }
  bv.h = (double *)calloc((size_t)(bv.m + 1) * (bv.m + 1), sizeof(double));
  bv.c = (double *)calloc((size_t)bv.m + 1, sizeof(double));
  ds_t ds = {0};
  ds.ld = ld;
  ds.d = (double *)calloc(ld, sizeof(double));
  ds.e = (double *)calloc(ld, sizeof(double));
  ds.A = (double *)calloc((size_t)ld * ld, sizeof(double));
  ds.Q = (double *)calloc((size_t)ld * ld, sizeof(double));
  ds.X = (double *)calloc((size_t)ld * ld, sizeof(double));
  ds.perm = (int *)calloc(ld, sizeof(int));
  ds.work = (double *)calloc((size_t)4 * ld, sizeof(double));
  double *eigr = (double *)calloc(ld, sizeof(double)), *eigi = (double *)calloc(ld, sizeof(double));
  double *errest = (double *)calloc(ld, sizeof(double));
  int *perm = (int *)calloc(ld, sizeof(int));
  double *hg = (double *)calloc(ld, sizeof(double));
  int err = 0, reason = KSOR_ITERATING, its = 0, nconv = 0;
  long long nsteps = 0;
  if (!bv.V || !bv.h || !bv.c || !ds.A || !ds.Q || !ds.X) { err = 55; goto done; }
  if (bcsr) {
    /* the dense LU of B (n^2 doubles: the oracle's general-B path is for test sizes) */
    if (n > 8192) { err = 56; goto done; }
    lu = (double *)calloc((size_t)n * n, sizeof(double));
    piv = (int *)calloc((size_t)n, sizeof(int));
    bv.bt = (double *)calloc((size_t)n, sizeof(double));
    if (!lu || !piv || !bv.bt) { err = 55; goto done; }
    for (int r = 0; r < n; r++)
      for (int p = bcsr->rp[r]; p < bcsr->rp[r + 1]; p++) lu[(size_t)r * n + bcsr->ci[p]] += bcsr->va[p];
    if (lu_factor(n, lu, piv)) { err = 71; goto done; } /* PETSC_ERR_MAT_LU_ZRPVT: B is singular */
    op.lu = lu;
    op.piv = piv;
  }

  /* start vector: EPSSetInitialSpace copy, or a random one; then orthonormalise (EPSGetStartVector) */
  if (v0) memcpy(bv.V, v0, sizeof(double) * n);
  else bv_random_column(&bv, 0);
  if (ghep) {
    double *t = (double *)malloc(sizeof(double) * n);
    memcpy(t, bv.V, sizeof(double) * n);
    st_apply(&Acsr, &op, t, bv.V, nthreads);
    free(t);
  }
  if (bv.nc) {
    /* EPSGetStartVector (epssolve.c): orthonormalised against the deflation space */
    double nrm = 0.0;
    int lindep = 0;
    if ((err = bv_orthonormalize(&bv, 0, &nrm, &lindep))) goto done;
    if (lindep || nrm == 0.0) { err = 77; goto done; } /* the initial vector belongs to the deflation space */
  } else {
    double nrm = bv_vec_norm(&bv, bv.V);
    if (nrm == 0.0) { err = 77; goto done; } /* initial vector is zero */
    bv_scale(&bv, 0, 1.0 / nrm);
  }

  int l = 0;
  while (reason == KSOR_ITERATING) {
    its++;
    int nv = nconv + mpd < ncv ? nconv + mpd : ncv;
    /* DSSetDimensions(nv, nconv, nconv+l) */
    ds.n = nv; ds.t = nv; ds.l = nconv; ds.k = nconv + l;
    double beta = 0.0;
    int breakdown = 0;
    err = krylov_factor(&bv, &Acsr, &op, hermitian, &ds, nconv + l, &nv, &beta, &breakdown, &nsteps);
    if (err) goto done;
    ds.n = nv; ds.t = nv; ds.l = nconv; ds.k = nconv + l;
    ds.state = l ? ST_RAW : ST_INTERMEDIATE;
    /* translation of the Krylov decomposition for harmonic extraction (krylovschur.c:270-271) */
    double gamma = 1.0;
    if (harmonic) {
      if ((err = harmonic_translate(&ds, target, beta, hg, &gamma))) goto done;
      ds.state = ST_RAW;
    }
    /* solve, sort, extra row */
    if (hermitian) {
      if (ds_hep_solve(&ds, eigr, eigi)) { err = 76; goto done; }
      ds_hep_sort(&ds, which, target, eigr);
      ds_hep_extrarow(&ds);
    } else {
      if (ds_nhep_solve(&ds, eigr, eigi)) { err = 76; goto done; }
      if (ds_nhep_sort(&ds, which, target, eigr, eigi)) { err = 76; goto done; }
      ds_nhep_extrarow(&ds);
    }
    /* EPSKrylovConvergence (epskrylov.c:207-295) */
    int k, marker = -1;
    for (k = nconv; k < nv; k++) {
      double re = eigr[k], im = eigi[k];
      int newk = k;
      double resnorm;
      if (hermitian) resnorm = fabs(ds.Q[IDX(nv - 1, k, ld)]);
      else ds_nhep_vector(&ds, &newk, &resnorm);
      resnorm *= beta * gamma;  /* corrf = gamma (epskrylov.c:265) */
      double w = hypot(re, im);
      /* EPSConvergedRelative / Absolute / Norm (epsdefault.c:224-256) */
      if (conv == KSOR_CONV_ABS) errest[k] = resnorm;
      else if (conv == KSOR_CONV_NORM) errest[k] = resnorm / (nrma + w * nrmb);
      else errest[k] = (w != 0.0) ? resnorm / w : DBL_MAX;
      if (marker == -1 && errest[k] >= tol) marker = k;
      if (newk == k + 1) { errest[k + 1] = errest[k]; k++; }
      if (marker != -1) break;
    }
    if (marker != -1) k = marker;
    /* EPSMonitor (krylovschur.c, after EPSKrylovConvergence): its, nconv, all nv values and estimates */
    if (g_monitor) g_monitor(its, k, eigr, eigi, errest, nv, g_monitor_ctx);
    /* EPSStoppingBasic */
    if (k >= nev) reason = KSOR_CONVERGED_TOL;
    else if (its >= max_it) reason = KSOR_DIVERGED_ITS;
    if (time_budget_s > 0.0 && now_s() - t_start > time_budget_s && reason == KSOR_ITERATING) reason = 99;
    int nconv_new = k;
    /* update l */
    if (reason != KSOR_ITERATING || breakdown || k == nv) l = 0;
    else {
      l = (int)((nv - k) * keep);
      if (l < 1) l = 1;
      if (!hermitian && ds.A[IDX(k + l, k + l - 1, ld)] != 0.0) {
        if (k + l < nv - 1) l++;
        else l--;
      }
    }
    if (!lock && l > 0) { l += k; k = 0; }
    if (reason == KSOR_ITERATING) {
      if (breakdown || k == nv) {
        if (k < nev) {
          /* EPSGetStartVector(k): random vector orthogonalised against V[:,0:k] */
          bv_random_column(&bv, k);
          if (ghep) {
            double *t = (double *)malloc(sizeof(double) * n);
            memcpy(t, VCOL(&bv, k), sizeof(double) * n);
            st_apply(&Acsr, &op, t, VCOL(&bv, k), nthreads);
            free(t);
          }
          double nrm;
          int ld2;
          if ((err = bv_orthogonalize_gs(&bv, k, &nrm, &ld2))) goto done;
          if (ld2 || nrm == 0.0) reason = KSOR_DIVERGED_BREAKDOWN;
          else bv_scale(&bv, k, 1.0 / nrm);
        }
      } else {
        if (harmonic) {
          /* undo the translation (krylovschur.c:306-316): gamma u^ = u - V(:,0:nv) g~ */
          harmonic_recover(&ds, k, l, beta, hg, &gamma);
          double *u = VCOL(&bv, nv);
          for (int i = 0; i < n; i++) {
            double s = 0.0;
            for (int j = 0; j < nv; j++) s += VCOL(&bv, j)[i] * hg[j];
            u[i] = (u[i] - s) / gamma;
          }
        }
        /* DSTruncate(k+l) */
        int nn = k + l;
        if (!hermitian) {
          for (int i = nconv; i < nn; i++) ds.A[IDX(nn, i, ld)] = ds.A[IDX(ds.n, i, ld)];
          for (int i = nconv; i < ds.n; i++) ds.A[IDX(ds.n, i, ld)] = 0.0;
        }
        ds.k = nn; ds.t = ds.n; ds.n = nn;
        ds.state = ST_TRUNCATED;
      }
    }
    /* V(:,nconv:k+l) = V(:,nconv:nv) * Q(nconv:nv, nconv:k+l) */
    bv_mult_in_place(&bv, ds.Q, ld, nconv, nv, nconv, k + l);
    if (reason == KSOR_ITERATING && !breakdown) memcpy(VCOL(&bv, k + l), VCOL(&bv, nv), sizeof(double) * n);
    nconv = k;
    (void)nconv_new;
  }
  /* DSTruncate(nconv, trim) */
  ds.n = nconv; ds.l = 0; ds.k = 0; ds.t = nconv;
  ds.state = ST_RAW;
  /* EPSComputeVectors: NHEP -> V = V * X with X eigenvectors of the leading Schur block */
  if (!hermitian && nconv > 0) {
    for (int i = 0; i < nconv; i++) for (int j = 0; j < nconv; j++) ds.X[IDX(i, j, ld)] = 0.0;
    ds_nhep_vectors_all(&ds);
    bv_mult_in_place(&bv, ds.X, ld, 0, nconv, 0, nconv);
  }
  /* EPS_Purify + BVNormalize for GHEP: x = B^-1 A x / ||B^-1 A x||_B */
  if (ghep && purify && nconv > 0) {
    double *t = (double *)malloc(sizeof(double) * n);
    for (int j = 0; j < nconv; j++) {
      memcpy(t, VCOL(&bv, j), sizeof(double) * n);
      st_apply(&Acsr, &op, t, VCOL(&bv, j), nthreads);
      double nrm = bv_vec_norm(&bv, VCOL(&bv, j));
      if (nrm > 0.0) bv_scale(&bv, j, 1.0 / nrm);
    }
    free(t);
  }
  /* reorder conjugate pairs (positive imaginary first) and final sort (epssolve.c:160-178) */
  for (int i = 0; i < nconv - 1; i++) {
    if (eigi[i] != 0.0) {
      if (eigi[i] < 0.0) { eigi[i] = -eigi[i]; eigi[i + 1] = -eigi[i + 1]; bv_scale(&bv, i + 1, -1.0); }
      i++;
    }
  }
  for (int i = 0; i < ncv; i++) perm[i] = i;
  /* SlepcSortEigenvalues (slepcsc.c:89-140) */
  for (int i = nconv - 1; i >= 0; i--) {
    double re = eigr[perm[i]], im = eigi[perm[i]];
    int j = i + 1;
    if (im != 0.0) { i--; im = eigi[perm[i]]; }
    while (j < nconv) {
      if (sc_compare(which, target, re, im, eigr[perm[j]], eigi[perm[j]]) <= 0) break;
      int tmp;
      if (im == 0.0) {
        if (eigi[perm[j]] == 0.0) { tmp = perm[j - 1]; perm[j - 1] = perm[j]; perm[j] = tmp; j++; }
        else { tmp = perm[j - 1]; perm[j - 1] = perm[j]; perm[j] = perm[j + 1]; perm[j + 1] = tmp; j += 2; }
      } else {
        if (eigi[perm[j]] == 0.0) { tmp = perm[j - 2]; perm[j - 2] = perm[j]; perm[j] = perm[j - 1]; perm[j - 1] = tmp; j++; }
        else { tmp = perm[j - 2]; perm[j - 2] = perm[j]; perm[j] = tmp; tmp = perm[j - 1]; perm[j - 1] = perm[j + 1]; perm[j + 1] = tmp; j += 2; }
      }
    }
  }
  /* outputs in sorted order.  X[:,i] = V[:,perm[i]]: for a complex pair (eigi[i] > 0, eigi[i+1] < 0) the two
   * columns are the real and imaginary parts, which is what BV_GetEigenvector (bvimpl.h:421-444) reads. */
  for (int i = 0; i < nconv; i++) {
    int p = perm[i];
    eigr_out[i] = eigr[p];
    eigi_out[i] = eigi[p];
    errest_out[i] = errest[p];
    if (X) memcpy(X + (size_t)i * n, VCOL(&bv, p), sizeof(double) * n);
  }
done:
  if (info) {
    memset(info, 0, sizeof(int) * KSOR_INFO_LEN);
    info[KSOR_INFO_NCONV] = nconv;
    info[KSOR_INFO_ITS] = its;
    info[KSOR_INFO_REASON] = reason;
    info[KSOR_INFO_NSTEPS] = (int)nsteps;
    info[KSOR_INFO_NPASSES] = (int)bv.npasses;
    info[KSOR_INFO_NCV] = ncv;
    info[KSOR_INFO_MPD] = mpd;
    info[KSOR_INFO_MAXIT] = max_it;
  }
  free(bv.V); free(bv.h); free(bv.c); free(bv.bt); free(bv.W); free(bv.cw); free(lu); free(piv);
  free(ds.d); free(ds.e); free(ds.A); free(ds.Q); free(ds.X); free(ds.perm); free(ds.work);
  free(eigr); free(eigi); free(errest); free(perm); free(hg);
  return err;
}

/* ------------------------------------------------------------------------------------------------------------
 * DS test entry points
 * ------------------------------------------------------------------------------------------------------------ */
int ksor_ds_hep(int n, int l, int k, int ld, const double *d, const double *e, int state_raw, int which,
                int extrarow, double *wr, double *Q, double *e_out) {
  ds_t ds = {0};
  ds.ld = ld; ds.n = n; ds.l = l; ds.k = k; ds.t = n;
  ds.d = (double *)calloc(ld, sizeof(double));
  ds.e = (double *)calloc(ld, sizeof(double));
  ds.Q = Q;
  ds.perm = (int *)calloc(ld, sizeof(int));
  memcpy(ds.d, d, sizeof(double) * n);
  memcpy(ds.e, e, sizeof(double) * n);
  ds.state = state_raw ? ST_RAW : ST_INTERMEDIATE;
  int err = ds_hep_solve(&ds, wr, NULL);
  if (!err) {
    ds_hep_sort(&ds, which, 0.0, wr);
    if (extrarow) ds_hep_extrarow(&ds);
    if (e_out) memcpy(e_out, ds.e, sizeof(double) * n);
  }
  free(ds.d); free(ds.e); free(ds.perm);
  return err;
}

int ksor_ds_nhep(int n, int ld, double *A, int state_intermediate, int which, int extrarow,
                 double *wr, double *wi, double *Q, int vec_index, double *rnorm, double *X) {
  ds_t ds = {0};
  ds.ld = ld; ds.n = n; ds.l = 0; ds.k = 0; ds.t = n;
  ds.A = A; ds.Q = Q;
  ds.X = (double *)calloc((size_t)ld * ld, sizeof(double));
  ds.work = (double *)calloc((size_t)4 * ld, sizeof(double));
  ds.state = state_intermediate ? ST_INTERMEDIATE : ST_RAW;
  int err = ds_nhep_solve(&ds, wr, wi);
  if (!err) err = ds_nhep_sort(&ds, which, 0.0, wr, wi);
  if (!err) {
    if (extrarow) ds_nhep_extrarow(&ds);
    if (vec_index >= 0 && rnorm) { int j = vec_index; ds_nhep_vector(&ds, &j, rnorm); }
    if (X) {
      ds_nhep_vectors_all(&ds);
      memcpy(X, ds.X, sizeof(double) * (size_t)ld * ld);
    }
  }
  free(ds.X); free(ds.work);
  return err;
}

int ksor_schur(int n, int ld, double *A, double *Q, double *wr, double *wi) {
  double *work = (double *)calloc((size_t)ld, sizeof(double));
  memset(Q, 0, sizeof(double) * (size_t)ld * ld);
  for (int i = 0; i < n; i++) Q[IDX(i, i, ld)] = 1.0;
  hessenberg(n, 0, A, ld, Q, work);
  int err = francis_schur(n, 0, A, ld, Q, wr, wi);
  if (!err) schur_eigs(n, A, ld, 0, wr, wi);
  free(work);
  return err;
}
