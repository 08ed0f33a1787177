/*
 * slepc_gb300.h -- GB300-specific entry points that have no counterpart in the reference.
 *
 * They select the arithmetic of the bandwidth-bound kernels, expose device-resident results and report
 * per-solve statistics (Krylov steps, restarts, kernel time), for programs that want more than the SLEPc API.
 */
#ifndef SLEPC_GB300_H
#define SLEPC_GB300_H

#include "slepceps.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Arithmetic of the Gram-Schmidt, restart and residual kernels.
 *   EPS_GB300_ARITH_PAIR (default): FP64 storage; products and sums on FP32 pairs with error-free
 *       transformations (relative error per product below 2^-46), the only form that reaches the HBM roofline on
 *       GB300, whose FP64 pipe runs at about 1.2 TFLOP/s.
 *   EPS_GB300_ARITH_F64: plain IEEE FP64 fused multiply-add everywhere (slower on GB300). */
/*   EPS_GB300_ARITH_F32: the precision form.  Operator values and the Krylov basis are stored in FP32 (half the
 *       bytes of the memory-bound SpMV and Gram-Schmidt); every dot product, norm and accumulation is still formed
 *       exactly in FP32 pairs, the orthogonalisation coefficients, DS and residuals stay FP64.  The FP32 basis
 *       limits this phase to about 1e-7, so it runs to max(tol, 1e-6); each converged pair is then rechecked in
 *       FP64 (||A x - lambda x|| / |lambda|), and if one fails tol an FP64-class refinement sweep (a pair-storage
 *       solve started from the sum of the phase-1 Ritz vectors) finishes to tol.  EPSGB300GetStats reports the
 *       steps of each phase. */
typedef enum { EPS_GB300_ARITH_PAIR = 0, EPS_GB300_ARITH_F64 = 1, EPS_GB300_ARITH_F32 = 2 } EPSGB300Arith;
PetscErrorCode EPSGB300SetArithmetic(EPS eps, EPSGB300Arith arith);
PetscErrorCode EPSGB300GetArithmetic(EPS eps, EPSGB300Arith *arith);

/* Solver of the symmetric projected problem inside EPSSolve.
 *   EPS_GB300_DS_AUTO (default): EPS_GB300_DS_REFINED while its accuracy checks pass; from the first restart whose
 *       pairs fail the check (that restart redone by the QR solver), EPS_GB300_DS_QR for the rest of the solve.
 *       Problems whose wanted end is well separated keep the fast solver; dense clusters (the 3-D Laplacians) cost
 *       one extra attempt per solve and follow the QR solver's iteration exactly.
 *   EPS_GB300_DS_QR: the reference's algorithm (arrowhead reduction, implicit QL) in FP64 in one thread
 *       block.
 *   EPS_GB300_DS_REFINED: FP32 arrowhead reduction and implicit QL, then FP64 eigenvector refinement (Ogita-Aishima
 *       iterations with clustered eigenvalues diagonalised by Jacobi, and a Newton-Schulz step), whose matrix
 *       products run on the whole GPU, then an accuracy check of every pair; a restart whose pairs fail the check is
 *       solved again by the QR solver (EPSGB300Stats.ds_fallbacks counts them).  Faster when the wanted end of the
 *       spectrum is well separated; on dense clusters (the 3-D Laplacians) every restart falls back.
 * The non-Hermitian solver and the DS object always use the FP64 algorithms. */
typedef enum { EPS_GB300_DS_REFINED = 0, EPS_GB300_DS_QR = 1, EPS_GB300_DS_AUTO = 2 } EPSGB300DSMethod;
/* default: EPS_GB300_DS_AUTO; option -eps_gb300_ds auto|refined|qr */

/* Gram-Schmidt of IEEE-double storage (EPS_GB300_ARITH_F64) inside EPSSolve.  No counterpart in the reference, whose
 * orthogonalisation (BVOrthogonalizeCGS1, src/sys/classes/bv/interface/bvorthog.c:91-132) calls FP64 BLAS gemv.
 *   EPS_GB300_GS_FMA: IEEE FP64 FMA in every product (bound by GB300's FP64 pipe near 2.4 TB/s).
 *   EPS_GB300_GS_TENSOR: every product of the two Gram-Schmidt halves exact on the FP16 tensor cores (an
 *       error-free split of each value's 55/56-bit fixed point, against its column/tile exponent, into byte or
 *       7-bit slices), the slice sums recombined as exact integers, rounded once per chunk of at most 512 rows and
 *       accumulated in double-double: more accurate than FP64 FMA.  On the 128^3 Laplacian it is still slower
 *       than the FMA kernels (the slicing on the CUDA cores bounds it).
 *   EPS_GB300_GS_INTEGER: every product exact on the integer pipes (each value's 54-bit fixed point against its
 *       column/tile exponent as two 27-bit halves, four 32 x 32 -> 64-bit multiply-adds per product, exact 64- and
 *       128-bit integer sums), rounded once per row (update half) or per thread's share of a column (dot half) and
 *       merged in double-double: as accurate as the tensor form, without the FP64 pipe's bound (on the 128^3
 *       Laplacian the two halves run at 2.8 and 3.0 TB/s against 2.3 for the FMA kernels).
 *   EPS_GB300_GS_AUTO (default): EPS_GB300_GS_INTEGER for solves whose factorisation segments run as direct
 *       launches, EPS_GB300_GS_FMA for those replayed from CUDA graphs (EPSGB300SetGraphCapture: by default the
 *       problems of at most 262144 rows, where launch gaps matter more than the Gram-Schmidt rate).
 * The exact forms are used for the symmetric (Lanczos) variant with the tcgen05 restart and no deflation space, and
 * run as direct launches; the other cases use the FMA kernels.  Option -eps_gb300_gs auto|integer|fma|tensor. */
typedef enum { EPS_GB300_GS_TENSOR = 0, EPS_GB300_GS_FMA = 1, EPS_GB300_GS_INTEGER = 2, EPS_GB300_GS_AUTO = 3 }
    EPSGB300GSMethod;
PetscErrorCode EPSGB300SetGSMethod(EPS eps, EPSGB300GSMethod method);
PetscErrorCode EPSGB300GetGSMethod(EPS eps, EPSGB300GSMethod *method);
PetscErrorCode EPSGB300SetProjectedSolver(EPS eps, EPSGB300DSMethod method);
PetscErrorCode EPSGB300GetProjectedSolver(EPS eps, EPSGB300DSMethod *method);

/* Kernel of the thick restart V(:, s:s+N) = V(:, a:a+K) Q for the pair-storage basis.
 *   EPS_GB300_RESTART_TENSOR (default): the bf16 tensor cores, to FP64-class accuracy by an error-free split of V
 *       (eight 7-bit slices) and Q (seven) (Ozaki scheme): the 35 slice products of the eight levels kept
 *       accumulate exactly in FP32 and are recombined in FP32 pairs (relative error about 2^-47, as the pair
 *       arithmetic).  It runs on tcgen05.mma with TMEM accumulators (EPS_GB300_RESTART_TCGEN05).
 *   EPS_GB300_RESTART_MMA_SYNC, EPS_GB300_RESTART_TCGEN05: that product on mma.sync (registers) or on tcgen05.mma
 *       (TMEM accumulators) explicitly.  Both give bit-identical results.
 *   EPS_GB300_RESTART_PAIR: FP32-pair arithmetic on the CUDA cores.
 * The reference's BVMultInPlace (bvblas.c:74-106) is a DGEMM.  Option -eps_gb300_restart
 * tensor|pair|mma_sync|tcgen05. */
typedef enum { EPS_GB300_RESTART_TENSOR = 0, EPS_GB300_RESTART_PAIR = 1, EPS_GB300_RESTART_MMA_SYNC = 2,
               EPS_GB300_RESTART_TCGEN05 = 3 } EPSGB300RestartMethod;
PetscErrorCode EPSGB300SetRestartMethod(EPS eps, EPSGB300RestartMethod method);

/* Wall-time budget of EPSSolve in seconds (0, the default: none).  Checked after each restart; when it has run out
 * the solve stops with EPS_DIVERGED_ITS and the pairs converged so far.  A stopping test of the kind
 * EPSSetStoppingTestFunction installs in the reference (epsdefault.c:290-302), for time-bounded callers. */
PetscErrorCode EPSGB300SetTimeLimit(EPS eps, PetscReal seconds);

/* Factorisation segments as CUDA graphs.  The launch sequence of one Krylov factorisation segment (from column k
 * to nv: SpMV and the two Gram-Schmidt halves per step, then the final reorthogonalisation) depends only on k, nv
 * and the EPS's buffers, so a segment seen a second time is captured once and replayed afterwards: the kernels and
 * their results are the same, without the per-launch host work between them.  mode -1 (default): on for problems
 * of at most 262144 rows, where launch gaps are a visible share of each step; 0: off; 1: on.  Graphs are dropped
 * by EPSSetUp and EPSDestroy.  Off while per-kernel profiling is on.  Option -eps_gb300_graphs -1|0|1. */
PetscErrorCode EPSGB300SetGraphCapture(EPS eps, PetscInt mode);

/* CUDA device ordinal used by this EPS (default: the current device at EPSCreate). */
PetscErrorCode EPSGB300SetDevice(EPS eps, int device);

/* Statistics of the last EPSSolve. */
typedef struct {
  long long krylov_steps;    /* operator applications inside factorisations */
  long long restarts;        /* outer iterations */
  double solve_seconds;      /* wall time of EPSSolve (device synchronised) */
  double bytes_moved;        /* algorithmic HBM bytes of the factorisations and restarts */
  double setup_seconds;      /* EPSSetUp: allocation and matrix upload */
  long long kernel_launches; /* CUDA kernels launched by the last EPSSolve */
  double solve_device_ms;    /* EPSSolve measured with CUDA events on the EPS stream */
  long long precision_steps;    /* EPS_GB300_ARITH_F32: Krylov steps of the FP32-storage phase (included above) */
  long long precision_restarts; /* EPS_GB300_ARITH_F32: restarts of the FP32-storage phase */
  long long ds_fallbacks;       /* restarts whose mixed-precision projected solve failed its accuracy check and was
                                   redone by the FP64 QR solver */
  long long graph_segments;     /* factorisation segments replayed from captured CUDA graphs */
  long long gs_exact;           /* 1 when the Gram-Schmidt pair ran with exact products (EPS_GB300_GS_TENSOR or
                                   EPS_GB300_GS_INTEGER took effect), else 0 */
} EPSGB300Stats;
PetscErrorCode EPSGB300GetStats(EPS eps, EPSGB300Stats *stats);

/* Per-kernel-class timing of the next EPSSolve calls: CUDA events recorded around every launch on the EPS stream.
 * Classes: 0 SpMV, 1 Gram-Schmidt dot half, 2 Gram-Schmidt update half, 3 thick restart, 4 projected problem.
 * EPSGB300GetProfile returns the summed device time (ms), the algorithmic HBM bytes and the launch count. */
typedef enum { EPS_GB300_K_SPMV = 0, EPS_GB300_K_GS_DOT, EPS_GB300_K_GS_UPDATE, EPS_GB300_K_RESTART, EPS_GB300_K_DS,
               EPS_GB300_K_COUNT } EPSGB300KernelClass;
PetscErrorCode EPSGB300SetProfiling(EPS eps, PetscBool on);
PetscErrorCode EPSGB300GetProfile(EPS eps, EPSGB300KernelClass cls, double *ms, double *bytes, long long *launches);

/* The converged eigenvectors on the device, as IEEE doubles, without a host copy: column i (leading dimension *ld)
 * is the vector EPSGetEigenvector(eps, i, ...) returns in Vr (for EPS_GHEP the eigenvector x itself); a complex
 * pair listed as i, i+1 has its real part in column i and its imaginary part in column i+1, as the reference's
 * basis after EPSComputeVectors_Schur (src/eps/interface/epsdefault.c:105-169).  The values are converted from the
 * basis' storage format (FP32 pairs in the default arithmetic, FP32 in the precision form) into an EPS-owned FP64
 * array on the first call after each EPSSolve; the pointer stays valid until the next EPSSolve, EPSSetUp, EPSReset
 * or EPSDestroy.  Counterpart of EPSGetEigenvector (src/eps/interface/epssolve.c:516) for all i at once. */
PetscErrorCode EPSGB300GetDeviceEigenvectors(EPS eps, const double **X, PetscInt *ld);
/* The same array as EPSGB300GetDeviceEigenvectors (kept for existing callers). */
PetscErrorCode EPSGB300GetDeviceBasis(EPS eps, const double **V, PetscInt *ld);

/* Solve `count` eigenproblems together: every EPS is configured as for EPSSolve (operators, problem type,
 * dimensions, tolerances, which, initial space) and left in the state EPSSolve would leave it, so EPSGetConverged,
 * EPSGetEigenpair, EPSGetIterationNumber and EPSGetConvergedReason read the results.  No counterpart in the
 * reference (whose unit of work is one EPSSolve, krylovschur.c:227-337); each problem runs the same algorithm.
 * The batch advances one Krylov step of every unconverged problem per kernel launch and runs a restart cycle of all
 * of them as one CUDA graph; a problem's arithmetic depends only on the problem, so its results are the same in
 * any batch, including a batch of one.  Requirements: pair arithmetic (the default), ncv <= 143, one device,
 * standard problems with Ritz extraction and no deflation space.
 * The symmetric projected problems use the FP64 QR solver (EPS_GB300_DS_QR). */
PetscErrorCode EPSGB300SolveBatch(PetscInt count, EPS *eps);

/* Serving: a request loop on its own host thread that solves eigenproblems as they arrive (continuous batching).
 * EPSGB300ServerSubmit takes a configured EPS (operators, problem type, dimensions, tolerances, which, initial
 * space; EPSSetUp is done by the server) and returns at once; the request is admitted when its footprint
 * n (ncv+1) 8 + nnz 12 bytes fits the HBM budget next to the solves already admitted (a request larger than the
 * budget is admitted alone), joins the solves on the GPU at their next restart cycle, and is retired when its
 * restart loop ends.  EPSGB300ServerWait blocks until the EPS holds its results (timeout < 0: no limit), after which
 * the usual EPSGet* calls read them and EPSGB300GetStats' solve_seconds is the latency from submission to result.
 * The client must not touch a submitted EPS until Wait reports it done.  Results do not depend on what else is
 * served at the same time.  max_requests bounds the solves admitted at once, max_ncv the ncv of any request
 * (<= 143).  Destroy waits for every submitted request.  No counterpart in the reference. */
typedef struct _p_EPSGB300Server *EPSGB300Server;
typedef struct {
  long long submitted, completed, failed, queued, live, max_live, cycles;
  double bytes_in_use, peak_bytes;
} EPSGB300ServerStats;
PetscErrorCode EPSGB300ServerCreate(double hbm_budget_bytes, PetscInt max_requests, PetscInt max_ncv,
                                    EPSGB300Server *server);
PetscErrorCode EPSGB300ServerSubmit(EPSGB300Server server, EPS eps);
PetscErrorCode EPSGB300ServerWait(EPSGB300Server server, EPS eps, double timeout_seconds, PetscBool *done);
PetscErrorCode EPSGB300ServerGetStats(EPSGB300Server server, EPSGB300ServerStats *stats);
/* Stop serving: queued and in-flight requests end at once with PETSC_ERR_ARG_WRONGSTATE (their Wait returns it). */
PetscErrorCode EPSGB300ServerCancel(EPSGB300Server server);
PetscErrorCode EPSGB300ServerDestroy(EPSGB300Server *server);

/* Tuning of the batched engine: Gram-Schmidt tiles (512 rows) per virtual block for each size bucket b, which
 * holds n in [2^(b+9), 2^(b+10)) (b = 0..13).  The table fixes each problem's summation partition, so results are
 * reproducible for a given table.  EPSGB300BatchTune measures buckets first..last on one restart cycle of a batch
 * that fills the GPU, trying 1, 2, 4, 8, 16 and 32 tiles, and keeps the fastest. */
PetscErrorCode EPSGB300BatchTune(PetscInt first_bucket, PetscInt last_bucket);
PetscErrorCode EPSGB300BatchGetTuning(PetscInt *tiles, PetscInt count);
PetscErrorCode EPSGB300BatchSetTuning(const PetscInt *tiles, PetscInt count);

/* Orthogonality ||V^T V - I||_max of the first nconv columns, computed on the device in FP64. */
PetscErrorCode EPSGB300OrthogonalityError(EPS eps, PetscReal *err);

/* y[0..k) = V(:, 0:k)^T x, with V (n x k, column-major, leading dimension ldv, 16-byte aligned, ldv even), x (n) and
 * y (k) all in device memory, computed by the same kernel and arithmetic as BVDotVec -- and allocating nothing.
 * No counterpart in the reference.  It is for callers that cannot allocate device memory while they run: programs
 * that reserve the GPU's memory up front for their own pool allocator, and time-critical loops that cannot take the
 * implicit device synchronisation of cudaMalloc/cudaFree.  Its scratch (partial sums, counter, staging; 344,448
 * bytes) is a fixed static device array that every GPU loading this library holds until the process exits.  The
 * first call on a device is a warm-up: it looks up that array's address and, with CUDA's lazy module loading, may
 * make the driver load this library's kernels and allocate driver memory for them; make it before reserving your
 * memory pool, before entering the time-critical loop, and before any stream capture.  Later calls allocate
 * nothing.  Limits: k <= 256 (larger k returns PETSC_ERR_ARG_OUTOFRANGE); any n (the kernel's grid is capped at
 * 160 blocks, which loop over the rows).  The call is asynchronous on `stream` (a
 * cudaStream_t, NULL for the legacy default stream).  All calls share the one scratch array: calls that overlap on
 * the GPU (different streams, or different host threads without ordering) race and must be serialised by the
 * caller. */
PetscErrorCode BVGB300DotVecNoAlloc(const double *V, PetscInt ldv, PetscInt n, PetscInt k, const double *x, double *y,
                                    void *stream);

#ifdef __cplusplus
}
#endif
#endif
