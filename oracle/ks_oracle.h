/*
 * ks_oracle.h -- CPU restatement of SLEPc 3.22's Krylov-Schur path (the oracle).
 *
 * TEST INFRASTRUCTURE ONLY.  This library is what the CUDA path is compared against in the tests, and the
 * timed CPU baseline.  Only tests/, __graft_entry__.smoke() and bench.py's cpu_baseline / reference arm may
 * load it.  The product (slepc_gb300/) never links, loads or calls it.
 *
 * All arithmetic is IEEE FP64 (plus OpenMP over rows for SpMV, Gram-Schmidt and the restart product).
 */
#ifndef KS_ORACLE_H
#define KS_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* which: same numbering as SLEPc's EPSWhich (include/slepceps.h:109) */
enum { KSOR_LARGEST_MAGNITUDE = 1, KSOR_SMALLEST_MAGNITUDE, KSOR_LARGEST_REAL, KSOR_SMALLEST_REAL,
       KSOR_LARGEST_IMAGINARY, KSOR_SMALLEST_IMAGINARY, KSOR_TARGET_MAGNITUDE, KSOR_TARGET_REAL };

/* converged reasons (include/slepceps.h:174-180) */
enum { KSOR_CONVERGED_TOL = 1, KSOR_DIVERGED_ITS = -1, KSOR_DIVERGED_BREAKDOWN = -2, KSOR_ITERATING = 0 };

/* info[] slots filled by ksor_solve */
enum { KSOR_INFO_NCONV = 0, KSOR_INFO_ITS, KSOR_INFO_REASON, KSOR_INFO_NSTEPS, KSOR_INFO_NPASSES,
       KSOR_INFO_NCV, KSOR_INFO_MPD, KSOR_INFO_MAXIT, KSOR_INFO_LEN = 16 };

/* Full Krylov-Schur solve (EPSSolve with EPSKRYLOVSCHUR, ST shift 0, Ritz or harmonic extraction).
 *   CSR matrix (n, rowptr[n+1], colidx[nnz], vals[nnz]); hermitian selects Lanczos+DSHEP vs Arnoldi+DSNHEP.
 *   ncv/mpd/max_it <= 0 select the reference defaults.  keep <= 0 selects 0.5.  lock: 1 locking, 0 not.
 *   v0: start vector (n), copied into V[:,0] as EPSSetInitialSpace does; NULL draws a random one.
 *   Outputs: info[KSOR_INFO_LEN]; eigr/eigi/errest (capacity ncv_cap) in final sorted order;
 *   X (n x ncv_cap column-major, may be NULL) receives the eigenvectors in the same order (complex pairs as
 *   consecutive real/imag columns, as in the reference's V layout).
 *   time_budget_s > 0 stops after that many seconds (reason stays ITERATING): used for bounded CPU samples.
 *   harmonic: harmonic Rayleigh-Ritz extraction for the given target (EPSSetExtraction(EPS_HARMONIC),
 *   EPSSetTarget); target also serves the target sorting criteria.
 * Returns 0 on success, nonzero error code otherwise. */
int ksor_solve(int n, const int *rowptr, const int *colidx, const double *vals,
               int hermitian, int which, int nev, int ncv, int mpd, double tol, int max_it,
               double keep, int lock, int nthreads, const double *v0, unsigned long long seed,
               double time_budget_s,
               int *info, int ncv_cap, double *eigr, double *eigi, double *errest, double *X,
               int harmonic, double target);

/* convergence tests (EPSConv, include/slepceps.h) */
enum { KSOR_CONV_ABS = 0, KSOR_CONV_REL = 1, KSOR_CONV_NORM = 2 };

/* ksor_solve for A x = k B x with a diagonal B (bdiag[n]; NULL: standard problem), as the reference runs it with
 * STSHIFT (shift 0) and a direct solve with B: the operator B^-1 A, the B-inner product and purified eigenvectors
 * when hermitian (EPS_GHEP), the Euclidean inner product otherwise (EPS_GNHEP).  conv selects the convergence test
 * (nrma, nrmb: the norms of EPS_CONV_NORM); purify applies to EPS_GHEP.  Eigenvectors X are B-normalised. */
int ksor_solve_gen(int n, const int *rowptr, const int *colidx, const double *vals, const double *bdiag,
                   int hermitian, int which, int nev, int ncv, int mpd, double tol, int max_it,
                   double keep, int lock, int nthreads, const double *v0, unsigned long long seed,
                   double time_budget_s,
                   int *info, int ncv_cap, double *eigr, double *eigi, double *errest, double *X,
                   int harmonic, double target, int conv, double nrma, double nrmb, int purify);

/* ksor_solve_gen for a general B in CSR (B rowptr/colidx/vals): the direct solve with B is a dense LU factorisation
 * with partial pivoting (n <= 8192; a singular B returns 71), and for hermitian (EPS_GHEP) the B-inner products
 * multiply by B in CSR. */
int ksor_solve_genb(int n, const int *rowptr, const int *colidx, const double *vals, const int *browptr,
                    const int *bcolidx, const double *bvals, int hermitian, int which, int nev, int ncv, int mpd,
                    double tol, int max_it, double keep, int lock, int nthreads, const double *v0,
                    unsigned long long seed, double time_budget_s, int *info, int ncv_cap, double *eigr,
                    double *eigi, double *errest, double *X, int harmonic, double target, int conv, double nrma,
                    double nrmb, int purify);

/* A monitor called by the solves after every restart, as EPSMonitor is (epsmon.c:40-48): restart count, number
 * converged, the nest current values and error estimates.  NULL turns it off.  Not thread-safe (one global). */
typedef void (*ksor_monitor_fn)(int its, int nconv, const double *eigr, const double *eigi, const double *errest,
                                int nest, void *ctx);
void ksor_set_monitor(ksor_monitor_fn fn, void *ctx);
/* the deflation space of the next solves (EPSSetDeflationSpace): nds column-major vectors of length n, orthonormalised
 * on entry to each solve; NULL clears it.  Standard problems only (a generalised one returns 56). */
void ksor_set_deflation(int nds, const double *W);

/* y = A x (CSR), the operation MatMult performs for AIJ. */
void ksor_spmv(int n, const int *rowptr, const int *colidx, const double *vals, const double *x, double *y,
               int nthreads);

/* DSHEP compact test (src/sys/classes/ds/tests/test3.c): d[n], e[n] (arrow/tridiagonal couplings), dims (n,l,k)
 * leading dimension ld; state_raw=1 reduces the arrow first.  Solves, sorts by `which`, optionally updates the
 * extra row.  Outputs wr[n] (sorted), Q (ld x ld), e_out[n] (extra row if requested). */
int ksor_ds_hep(int n, int l, int k, int ld, const double *d, const double *e, int state_raw, int which,
                int extrarow, double *wr, double *Q, double *e_out);

/* DSNHEP test (src/sys/classes/ds/tests/test1.c): A is ld x ld col-major (extra row at row n if extrarow).
 * state_intermediate=1 means A is already Hessenberg.  Solves (Schur), sorts by `which`, optionally updates the
 * extra row, then returns rnorm of eigenvector vec_index and all eigenvectors X (ld x ld).
 * A and Q are overwritten with the sorted Schur form / Schur vectors. */
int ksor_ds_nhep(int n, int ld, double *A, int state_intermediate, int which, int extrarow,
                 double *wr, double *wi, double *Q, int vec_index, double *rnorm, double *X);

/* Dense real Schur form with sorting only (used by unit tests of the restated LAPACK pieces). */
int ksor_schur(int n, int ld, double *A, double *Q, double *wr, double *wi);

#ifdef __cplusplus
}
#endif
#endif
