/*
 * slepcst.h -- ST (spectral transformation) subset.
 *
 * Same names and enum strings as SLEPc 3.22's include/slepcst.h (:42-103).  The Krylov-Schur path here runs the
 * shift transformation with shift 0 (STSHIFT; the operator is A, or the generalised operator of EPSSetOperators):
 * EPSGetST returns that object so that programs which query or confirm it work unchanged.  The transformations that
 * need linear solves (sinvert, cayley, precond, filter, shell) and nonzero shifts return PETSC_ERR_SUP.
 */
#ifndef SLEPC_GB300_SLEPCST_H
#define SLEPC_GB300_SLEPCST_H

#include "petsc_subset.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct _p_ST *ST;
typedef const char *STType;
#define STSHELL "shell"
#define STSHIFT "shift"
#define STSINVERT "sinvert"
#define STCAYLEY "cayley"
#define STPRECOND "precond"
#define STFILTER "filter"

PetscErrorCode STSetType(ST st, STType type);
PetscErrorCode STGetType(ST st, STType *type);
PetscErrorCode STSetShift(ST st, PetscScalar shift);
PetscErrorCode STGetShift(ST st, PetscScalar *shift);
PetscErrorCode STGetNumMatrices(ST st, PetscInt *n);
PetscErrorCode STView(ST st, PetscViewer viewer);
/* the linear solver of the transformation: the shift of 0 has none to run, so its iteration count is 0 */
typedef struct _p_KSP *KSP;
PetscErrorCode STGetKSP(ST st, KSP *ksp);
PetscErrorCode KSPGetTotalIterations(KSP ksp, PetscInt *its);
PetscErrorCode KSPSetTolerances(KSP ksp, PetscReal rtol, PetscReal abstol, PetscReal dtol, PetscInt maxits);

#ifdef __cplusplus
}
#endif
#endif
