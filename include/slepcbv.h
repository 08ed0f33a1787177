/*
 * slepcbv.h -- BV (basis vectors) subset used by the Krylov-Schur path, backed by device-resident storage.
 *
 * Same prototypes and argument meanings as SLEPc 3.22's include/slepcbv.h.  A BV here is an n x m column-major
 * FP64 array in GPU memory (the reference's default BVMAT type, bvmat.c); host Vec arguments are copied in and
 * out.  Each entry point names the reference interface it replaces.
 */
#ifndef SLEPC_GB300_SLEPCBV_H
#define SLEPC_GB300_SLEPCBV_H

#include "petsc_subset.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct _p_BV *BV;

typedef enum { BV_ORTHOG_CGS, BV_ORTHOG_MGS } BVOrthogType;                                     /* slepcbv.h:59 */
typedef enum { BV_ORTHOG_REFINE_IFNEEDED, BV_ORTHOG_REFINE_NEVER, BV_ORTHOG_REFINE_ALWAYS } BVOrthogRefineType; /* :71 */
typedef enum { BV_ORTHOG_BLOCK_GS, BV_ORTHOG_BLOCK_CHOL, BV_ORTHOG_BLOCK_TSQR, BV_ORTHOG_BLOCK_TSQRCHOL,
               BV_ORTHOG_BLOCK_SVQB } BVOrthogBlockType;                                          /* :84 */

/* object life cycle: src/sys/classes/bv/interface/bvbasic.c (BVCreate, BVSetSizes, BVDestroy) */
PetscErrorCode BVCreate(MPI_Comm comm, BV *bv);
PetscErrorCode BVSetSizes(BV bv, PetscInt n, PetscInt N, PetscInt m);
PetscErrorCode BVGetSizes(BV bv, PetscInt *n, PetscInt *N, PetscInt *m);
PetscErrorCode BVDestroy(BV *bv);
/* active columns [l, k): bvbasic.c:421 */
PetscErrorCode BVSetActiveColumns(BV bv, PetscInt l, PetscInt k);
PetscErrorCode BVGetActiveColumns(BV bv, PetscInt *l, PetscInt *k);
/* orthogonalisation settings: bvbasic.c:864-902 (CGS only; MGS is refused with PETSC_ERR_SUP) */
PetscErrorCode BVSetOrthogonalization(BV bv, BVOrthogType type, BVOrthogRefineType refine, PetscReal eta,
                                      BVOrthogBlockType block);
/* column copies to/from host vectors: bvbasic.c:1871 (BVCopyColumn), bvops.c (BVInsertVec, BVCopyVec) */
PetscErrorCode BVInsertVec(BV V, PetscInt j, Vec w);
PetscErrorCode BVCopyVec(BV V, PetscInt j, Vec v);
PetscErrorCode BVCopyColumn(BV V, PetscInt j, PetscInt i);
PetscErrorCode BVScaleColumn(BV bv, PetscInt j, PetscScalar alpha);
PetscErrorCode BVSetRandomColumn(BV bv, PetscInt j);

/* y = V(:,l:k)^T x over the active columns (bvglobal.c:151-187; BVDotVec_BLAS_CUDA, bvcuda.cu:204-264).
 * m = k - l results are written to the host array m. */
PetscErrorCode BVDotVec(BV X, Vec y, PetscScalar m[]);
/* y = beta*y + alpha*V(:,l:k) q (bvops.c:110-163; BVMultVec_BLAS_CUDA, bvcuda.cu:45-60) */
PetscErrorCode BVMultVec(BV X, PetscScalar alpha, PetscScalar beta, Vec y, PetscScalar q[]);
/* V(:,s:e) = V(:,l:k) Q(l:k, s:e) (bvops.c:220-245; BVMultInPlace_BLAS_CUDA, bvcuda.cu:65-112).  Q is a dense Mat
 * with at least k rows; the product runs on the device in place with no temporary basis copy. */
PetscErrorCode BVMultInPlace(BV V, Mat Q, PetscInt s, PetscInt e);
/* norms of the active block or of one column (bvglobal.c:498-829; BVNorm_BLAS_CUDA, bvcuda.cu:290-303);
 * NORM_2 of a block is refused as in the reference; NORM_FROBENIUS, NORM_1 and NORM_INFINITY are supported. */
PetscErrorCode BVNorm(BV bv, NormType type, PetscReal *val);
PetscErrorCode BVNormColumn(BV bv, PetscInt j, NormType type, PetscReal *val);
/* orthonormalise column j against columns 0..j-1 (bvorthog.c:380-427) */
PetscErrorCode BVOrthonormalizeColumn(BV bv, PetscInt j, PetscBool replace, PetscReal *norm, PetscBool *lindep);
/* Krylov factorisations over columns k..m-1 (bvkrylov.c:56-113 and :165-226).  H (dense Mat, at least m x m,
 * ldh > m for the extra row) receives the Hessenberg matrix; T (m x 2 dense) the diagonal and off-diagonal. */
PetscErrorCode BVMatArnoldi(BV V, Mat A, Mat H, PetscInt k, PetscInt *m, PetscReal *beta, PetscBool *breakdown);
PetscErrorCode BVMatLanczos(BV V, Mat A, Mat T, PetscInt k, PetscInt *m, PetscReal *beta, PetscBool *breakdown);

#ifdef __cplusplus
}
#endif
#endif
