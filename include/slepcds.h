/*
 * slepcds.h -- DS (projected dense problem) subset used by the Krylov-Schur path, solved on the GPU in FP64.
 *
 * Same prototypes and argument meanings as SLEPc 3.22's include/slepcds.h for the DSHEP (compact arrow-tridiagonal)
 * and DSNHEP types.  Matrices live in host memory between calls (DSGetArray / DSGetArrayReal); DSSolve copies them to
 * the device, runs the device solver (the same code the eigensolver uses inside its loop) and copies them back.
 */
#ifndef SLEPC_GB300_SLEPCDS_H
#define SLEPC_GB300_SLEPCDS_H

#include "petsc_subset.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct _p_DS *DS;
typedef const char *DSType;
#define DSHEP "hep"
#define DSNHEP "nhep"

typedef enum { DS_STATE_RAW, DS_STATE_INTERMEDIATE, DS_STATE_CONDENSED, DS_STATE_TRUNCATED } DSStateType; /* :69 */
typedef enum { DS_MAT_A, DS_MAT_B, DS_MAT_C, DS_MAT_T, DS_MAT_D, DS_MAT_Q, DS_MAT_Z, DS_MAT_X, DS_MAT_Y,
               DS_MAT_U, DS_MAT_V, DS_MAT_W } DSMatType;                                                  /* :107 */

/* Sorting criterion (include/slepcsc.h): only the comparison function is used (RG and map are not supported). */
typedef PetscErrorCode (*SlepcSCCompareFn)(PetscScalar, PetscScalar, PetscScalar, PetscScalar, PetscInt *, void *);
struct _n_SlepcSC {
  SlepcSCCompareFn comparison;
  void *comparisonctx;
  void *map;
  void *mapobj;
  void *rg;
};
typedef struct _n_SlepcSC *SlepcSC;
PetscErrorCode SlepcCompareLargestMagnitude(PetscScalar, PetscScalar, PetscScalar, PetscScalar, PetscInt *, void *);
PetscErrorCode SlepcCompareSmallestMagnitude(PetscScalar, PetscScalar, PetscScalar, PetscScalar, PetscInt *, void *);
PetscErrorCode SlepcCompareLargestReal(PetscScalar, PetscScalar, PetscScalar, PetscScalar, PetscInt *, void *);
PetscErrorCode SlepcCompareSmallestReal(PetscScalar, PetscScalar, PetscScalar, PetscScalar, PetscInt *, void *);
PetscErrorCode SlepcCompareLargestImaginary(PetscScalar, PetscScalar, PetscScalar, PetscScalar, PetscInt *, void *);
PetscErrorCode SlepcCompareSmallestImaginary(PetscScalar, PetscScalar, PetscScalar, PetscScalar, PetscInt *, void *);

/* life cycle and dimensions: src/sys/classes/ds/interface/dsbasic.c, dsops.c:130-165 */
PetscErrorCode DSCreate(MPI_Comm comm, DS *ds);
PetscErrorCode DSSetType(DS ds, DSType type);
PetscErrorCode DSGetType(DS ds, DSType *type);  /* dsbasic.c:275; NULL until a type is set */
PetscErrorCode DSView(DS ds, PetscViewer viewer); /* type line (dsbasic.c DSView, ASCII) */
PetscErrorCode DSAllocate(DS ds, PetscInt ld);
PetscErrorCode DSGetLeadingDimension(DS ds, PetscInt *ld);
PetscErrorCode DSSetDimensions(DS ds, PetscInt n, PetscInt l, PetscInt k);
PetscErrorCode DSGetDimensions(DS ds, PetscInt *n, PetscInt *l, PetscInt *k, PetscInt *t);
PetscErrorCode DSSetState(DS ds, DSStateType state);
PetscErrorCode DSGetState(DS ds, DSStateType *state);
PetscErrorCode DSSetCompact(DS ds, PetscBool comp);
PetscErrorCode DSSetExtraRow(DS ds, PetscBool ext);
PetscErrorCode DSGetSlepcSC(DS ds, SlepcSC *sc);
PetscErrorCode DSGetArray(DS ds, DSMatType m, PetscScalar *a[]);
PetscErrorCode DSRestoreArray(DS ds, DSMatType m, PetscScalar *a[]);
PetscErrorCode DSGetArrayReal(DS ds, DSMatType m, PetscReal *a[]);
PetscErrorCode DSRestoreArrayReal(DS ds, DSMatType m, PetscReal *a[]);
PetscErrorCode DSDestroy(DS *ds);
/* DSSolve (dsops.c:723-742 -> dshep.c:383-426 / dsutil.c:21-87): eigenvalues in eigr (eigi for DSNHEP) */
PetscErrorCode DSSolve(DS ds, PetscScalar eigr[], PetscScalar eigi[]);
/* DSSort (dsops.c:777-800 -> dshep.c:323-347 / dsutil.c:93-171); rr, ri, k must be NULL */
PetscErrorCode DSSort(DS ds, PetscScalar eigr[], PetscScalar eigi[], PetscScalar rr[], PetscScalar ri[], PetscInt *k);
/* DSUpdateExtraRow (dsops.c:964 -> dshep.c:349-381 / dsnhep.c:318-340) */
PetscErrorCode DSUpdateExtraRow(DS ds);
/* DSTruncate (dsops.c:232 -> dshep.c:643-670 / dsnhep.c:394-425) */
PetscErrorCode DSTruncate(DS ds, PetscInt n, PetscBool trim);
/* DSVectors (dsops.c:931 -> dshep.c:137-172 / dsnhep.c:101-232): DS_MAT_X only */
PetscErrorCode DSVectors(DS ds, DSMatType mat, PetscInt *j, PetscReal *rnorm);

#ifdef __cplusplus
}
#endif
#endif
