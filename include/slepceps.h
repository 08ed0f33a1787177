/*
 * slepceps.h -- EPS (eigenvalue problem solver) subset: the Krylov-Schur path on one GB300.
 *
 * Same prototypes, enum values and argument meanings as SLEPc 3.22's include/slepceps.h (:186-274) for the calls a
 * program needs to run EPSKRYLOVSCHUR on a standard Hermitian (EPS_HEP) or non-Hermitian (EPS_NHEP) problem with
 * Ritz extraction: create, set operators/type/dimensions/tolerances/which/initial space, solve, read eigenpairs,
 * errors and convergence data, destroy.  Errors are PETSc error codes (0 = success); failure to converge is not an
 * error but a negative EPSConvergedReason.  One CUDA stream per EPS; distinct EPS objects may be driven from
 * distinct host threads.
 */
#ifndef SLEPC_GB300_SLEPCEPS_H
#define SLEPC_GB300_SLEPCEPS_H

#include "petsc_subset.h"
#include "slepcbv.h"
#include "slepcds.h"
#include "slepcst.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct _p_EPS *EPS;
typedef const char *EPSType;
#define EPSKRYLOVSCHUR "krylovschur"
/* the other solver types' names (slepceps.h:31-56), so that programs which compare or select types compile;
 * EPSSetType accepts EPSKRYLOVSCHUR only */
#define EPSPOWER "power"
#define EPSSUBSPACE "subspace"
#define EPSARNOLDI "arnoldi"
#define EPSLANCZOS "lanczos"
#define EPSGD "gd"
#define EPSJD "jd"
#define EPSRQCG "rqcg"
#define EPSLOBPCG "lobpcg"
#define EPSCISS "ciss"
#define EPSLYAPII "lyapii"
#define EPSLAPACK "lapack"
#define EPSARPACK "arpack"
typedef enum { EPS_POWER_SHIFT_CONSTANT, EPS_POWER_SHIFT_RAYLEIGH, EPS_POWER_SHIFT_WILKINSON } EPSPowerShiftType;
extern const char *EPSPowerShiftTypes[];
typedef enum { EPS_LANCZOS_REORTHOG_LOCAL, EPS_LANCZOS_REORTHOG_FULL, EPS_LANCZOS_REORTHOG_SELECTIVE,
               EPS_LANCZOS_REORTHOG_PERIODIC, EPS_LANCZOS_REORTHOG_PARTIAL,
               EPS_LANCZOS_REORTHOG_DELAYED } EPSLanczosReorthogType;
extern const char *EPSLanczosReorthogTypes[];

typedef enum { EPS_HEP = 1, EPS_GHEP, EPS_NHEP, EPS_GNHEP, EPS_PGNHEP, EPS_GHIEP, EPS_BSE } EPSProblemType;
typedef enum { EPS_RITZ, EPS_HARMONIC, EPS_HARMONIC_RELATIVE, EPS_HARMONIC_RIGHT, EPS_HARMONIC_LARGEST,
               EPS_REFINED, EPS_REFINED_HARMONIC } EPSExtraction;
typedef enum { EPS_LARGEST_MAGNITUDE = 1, EPS_SMALLEST_MAGNITUDE, EPS_LARGEST_REAL, EPS_SMALLEST_REAL,
               EPS_LARGEST_IMAGINARY, EPS_SMALLEST_IMAGINARY, EPS_TARGET_MAGNITUDE, EPS_TARGET_REAL,
               EPS_TARGET_IMAGINARY, EPS_ALL, EPS_WHICH_USER } EPSWhich;
typedef enum { EPS_CONVERGED_TOL = 1, EPS_CONVERGED_USER = 2, EPS_DIVERGED_ITS = -1, EPS_DIVERGED_BREAKDOWN = -2,
               EPS_DIVERGED_SYMMETRY_LOST = -3, EPS_CONVERGED_ITERATING = 0 } EPSConvergedReason;
typedef enum { EPS_ERROR_ABSOLUTE, EPS_ERROR_RELATIVE, EPS_ERROR_BACKWARD } EPSErrorType;
typedef enum { EPS_CONV_ABS, EPS_CONV_REL, EPS_CONV_NORM, EPS_CONV_USER } EPSConv;

/* SlepcInitialize / SlepcFinalize (src/sys/slepcinit.c): no-op shims */
PetscErrorCode SlepcInitialize(int *argc, char ***argv, const char file[], const char help[]);
PetscErrorCode SlepcFinalize(void);

/* life cycle: src/eps/interface/epsbasic.c:48-158 */
PetscErrorCode EPSCreate(MPI_Comm comm, EPS *eps);
PetscErrorCode EPSDestroy(EPS *eps);
PetscErrorCode EPSReset(EPS eps);
PetscErrorCode EPSSetType(EPS eps, EPSType type);
PetscErrorCode EPSGetType(EPS eps, EPSType *type);
/* problem definition: epssetup.c:470-520 (EPSSetOperators), epsopts.c.  B != NULL gives a generalised problem
 * A x = lambda B x (EPS_GHEP or EPS_GNHEP; EPS_GNHEP is the default with B).  B must be diagonal here -- positive
 * for EPS_GHEP, nonzero for EPS_GNHEP -- and the solve runs Krylov-Schur on an operator with the same Krylov spaces
 * as the reference's B^-1 A with the B-inner product (STSHIFT, shift 0); other B return PETSC_ERR_SUP. */
PetscErrorCode EPSSetOperators(EPS eps, Mat A, Mat B);
PetscErrorCode EPSGetOperators(EPS eps, Mat *A, Mat *B);
PetscErrorCode EPSSetProblemType(EPS eps, EPSProblemType type);
PetscErrorCode EPSGetProblemType(EPS eps, EPSProblemType *type);
/* extraction (epsopts.c:1090-1130): EPS_RITZ, or EPS_HARMONIC for eigenvalues near the target (krylovschur.c:238-240,
 * 270-319: the Krylov decomposition is translated for the target before each projected solve and recovered before
 * the restart); the target serves EPS_TARGET_MAGNITUDE / EPS_TARGET_REAL (epsopts.c:560-600) */
PetscErrorCode EPSSetExtraction(EPS eps, EPSExtraction extr);
PetscErrorCode EPSGetExtraction(EPS eps, EPSExtraction *extr);
PetscErrorCode EPSSetTarget(EPS eps, PetscScalar target);
PetscErrorCode EPSGetTarget(EPS eps, PetscScalar *target);
PetscErrorCode EPSSetDimensions(EPS eps, PetscInt nev, PetscInt ncv, PetscInt mpd);     /* epsopts.c:392-417 */
PetscErrorCode EPSGetDimensions(EPS eps, PetscInt *nev, PetscInt *ncv, PetscInt *mpd);
PetscErrorCode EPSSetTolerances(EPS eps, PetscReal tol, PetscInt maxits);               /* epsopts.c:300-323 */
PetscErrorCode EPSGetTolerances(EPS eps, PetscReal *tol, PetscInt *maxits);
/* convergence test (epsopts.c:640-700, epsdefault.c:180-230): EPS_CONV_REL (default) errest/|k|, EPS_CONV_ABS
 * errest, EPS_CONV_NORM errest/(||A|| + |k| ||B||) with infinity norms; EPS_CONV_USER is not provided */
PetscErrorCode EPSSetConvergenceTest(EPS eps, EPSConv conv);
PetscErrorCode EPSGetConvergenceTest(EPS eps, EPSConv *conv);
/* purification of the eigenvectors of EPS_GHEP (epsdefault.c:28-50): x <- B^-1 A x, B-normalised (default on) */
PetscErrorCode EPSSetPurify(EPS eps, PetscBool purify);
PetscErrorCode EPSGetPurify(EPS eps, PetscBool *purify);
PetscErrorCode EPSSetWhichEigenpairs(EPS eps, EPSWhich which);
PetscErrorCode EPSGetWhichEigenpairs(EPS eps, EPSWhich *which);
PetscErrorCode EPSSetInitialSpace(EPS eps, PetscInt n, Vec is[]);                          /* epssetup.c:592 */
PetscErrorCode EPSSetFromOptions(EPS eps);
/* options prefix (epsopts.c:1320-1400): the EPS's options are then -<prefix>eps_...; -st_type other than shift and
 * nonzero -st_shift are PETSC_ERR_SUP (the spectral transformation is the shift of 0) */
PetscErrorCode EPSSetOptionsPrefix(EPS eps, const char prefix[]);
PetscErrorCode EPSAppendOptionsPrefix(EPS eps, const char prefix[]);
PetscErrorCode EPSGetOptionsPrefix(EPS eps, const char *prefix[]);
/* Krylov-Schur knobs: krylovschur.c:339-489 */
PetscErrorCode EPSKrylovSchurSetRestart(EPS eps, PetscReal keep);
PetscErrorCode EPSKrylovSchurGetRestart(EPS eps, PetscReal *keep);
PetscErrorCode EPSKrylovSchurSetLocking(EPS eps, PetscBool lock);
PetscErrorCode EPSKrylovSchurGetLocking(EPS eps, PetscBool *lock);
/* setup and solve: epssetup.c:286-418, epssolve.c:119-208 */
PetscErrorCode EPSSetUp(EPS eps);
PetscErrorCode EPSSolve(EPS eps);
/* results: epssolve.c:240-420, 742-815 */
PetscErrorCode EPSGetConverged(EPS eps, PetscInt *nconv);
PetscErrorCode EPSGetConvergedReason(EPS eps, EPSConvergedReason *reason);
PetscErrorCode EPSGetIterationNumber(EPS eps, PetscInt *its);
PetscErrorCode EPSGetEigenpair(EPS eps, PetscInt i, PetscScalar *eigr, PetscScalar *eigi, Vec Vr, Vec Vi);
PetscErrorCode EPSGetEigenvalue(EPS eps, PetscInt i, PetscScalar *eigr, PetscScalar *eigi);
PetscErrorCode EPSGetEigenvector(EPS eps, PetscInt i, Vec Vr, Vec Vi);
PetscErrorCode EPSGetErrorEstimate(EPS eps, PetscInt i, PetscReal *errest);
PetscErrorCode EPSComputeError(EPS eps, PetscInt i, EPSErrorType type, PetscReal *error);
/* text reports of the solution (epsview.c:243-262, 297-447, 603-617); a NULL viewer means stdout */
PetscErrorCode EPSConvergedReasonView(EPS eps, PetscViewer viewer);
PetscErrorCode EPSErrorView(EPS eps, EPSErrorType etype, PetscViewer viewer);
PetscErrorCode EPSValuesView(EPS eps, PetscViewer viewer);
PetscErrorCode EPSView(EPS eps, PetscViewer viewer); /* epsview.c:40-190; option -eps_view (after EPSSolve) */
/* monitors (epsmon.c): called after every restart with the restart count, the number converged, the nest current
 * Ritz values (operator scaling undone) and their error estimates.  Up to 5 per EPS.  The built-ins print one line
 * per restart to the viewer of their PetscViewerAndFormat: the first unconverged value (EPSMonitorFirst, option
 * -eps_monitor), all values (EPSMonitorAll, -eps_monitor_all), or each value as it converges (EPSMonitorConverged,
 * -eps_monitor_conv, whose context comes from EPSMonitorConvergedCreate). */
typedef PetscErrorCode EPSMonitorFn(EPS eps, PetscInt its, PetscInt nconv, PetscScalar eigr[], PetscScalar eigi[],
                                    PetscReal errest[], PetscInt nest, void *ctx);
PetscErrorCode EPSMonitorSet(EPS eps, EPSMonitorFn *monitor, void *mctx, PetscCtxDestroyFn *monitordestroy);
PetscErrorCode EPSMonitorCancel(EPS eps);
PetscErrorCode EPSMonitorFirst(EPS eps, PetscInt its, PetscInt nconv, PetscScalar eigr[], PetscScalar eigi[],
                               PetscReal errest[], PetscInt nest, PetscViewerAndFormat *vf);
PetscErrorCode EPSMonitorAll(EPS eps, PetscInt its, PetscInt nconv, PetscScalar eigr[], PetscScalar eigi[],
                             PetscReal errest[], PetscInt nest, PetscViewerAndFormat *vf);
PetscErrorCode EPSMonitorConverged(EPS eps, PetscInt its, PetscInt nconv, PetscScalar eigr[], PetscScalar eigi[],
                                   PetscReal errest[], PetscInt nest, PetscViewerAndFormat *vf);
PetscErrorCode EPSMonitorConvergedCreate(PetscViewer viewer, PetscViewerFormat format, void *ctx,
                                         PetscViewerAndFormat **vf);
PetscErrorCode EPSMonitorConvergedDestroy(PetscViewerAndFormat **vf);
PetscErrorCode EPSGetBV(EPS eps, BV *V);
PetscErrorCode EPSGetST(EPS eps, ST *st); /* the shift-0 transformation (slepcst.h) */
/* options of other solver types, as SLEPc dispatches them on a Krylov-Schur EPS: the setters do nothing
 * (PetscTryMethod), the getters return PETSC_ERR_SUP (PetscUseMethod) */
PetscErrorCode EPSPowerSetShiftType(EPS eps, EPSPowerShiftType shift);
PetscErrorCode EPSPowerGetShiftType(EPS eps, EPSPowerShiftType *shift);
PetscErrorCode EPSLanczosSetReorthog(EPS eps, EPSLanczosReorthogType reorthog);
PetscErrorCode EPSLanczosGetReorthog(EPS eps, EPSLanczosReorthogType *reorthog);
PetscErrorCode EPSGDSetDoubleExpansion(EPS eps, PetscBool doubleexp);
PetscErrorCode EPSGDGetDoubleExpansion(EPS eps, PetscBool *doubleexp);
/* balancing (epsopts.c:1010-1090) and the stopping test (epsopts.c:780-860).  The balancing settings are stored and
 * checked as the reference does; a Hermitian problem is never balanced (epssetup.c:378-385), and EPSSetUp returns
 * PETSC_ERR_SUP for one-sided or two-sided balancing of a non-Hermitian problem.  The stopping test is
 * EPS_STOP_BASIC; other values return PETSC_ERR_SUP.  Track-all is stored (the error estimates of all current
 * values are computed in any case). */
typedef enum { EPS_BALANCE_NONE, EPS_BALANCE_ONESIDE, EPS_BALANCE_TWOSIDE, EPS_BALANCE_USER } EPSBalance;
extern const char *EPSBalanceTypes[];
typedef enum { EPS_STOP_BASIC, EPS_STOP_USER, EPS_STOP_THRESHOLD } EPSStop;
PetscErrorCode EPSSetBalance(EPS eps, EPSBalance bal, PetscInt its, PetscReal cutoff);
PetscErrorCode EPSGetBalance(EPS eps, EPSBalance *bal, PetscInt *its, PetscReal *cutoff);
PetscErrorCode EPSSetStoppingTest(EPS eps, EPSStop stop);
PetscErrorCode EPSGetStoppingTest(EPS eps, EPSStop *stop);
PetscErrorCode EPSSetTrackAll(EPS eps, PetscBool trackall);
PetscErrorCode EPSGetTrackAll(EPS eps, PetscBool *trackall);
/* a deflation space (epsdefl.c) is not provided: an empty one is accepted */
PetscErrorCode EPSSetDeflationSpace(EPS eps, PetscInt n, Vec v[]);
/* problem properties after EPSSetProblemType (epsbasic.c:1000-1080) */
PetscErrorCode EPSIsHermitian(EPS eps, PetscBool *is);
PetscErrorCode EPSIsGeneralized(EPS eps, PetscBool *is);
PetscErrorCode EPSIsPositive(EPS eps, PetscBool *is);
PetscErrorCode EPSGetDS(EPS eps, DS *ds);

#ifdef __cplusplus
}
#endif
#endif
