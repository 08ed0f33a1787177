/*
 * petsc_subset.h -- the part of PETSc's C API that SLEPc's Krylov-Schur path is typed on.
 *
 * PETSc is not part of this library.  These are the names, argument meanings and error conventions of the PETSc
 * calls that the reference's EPS/BV/DS interfaces take and return (Mat, Vec, PetscErrorCode, PetscScalar = double,
 * PetscReal = double, PetscInt = 32-bit, PetscBool), so that C code written against SLEPc's API compiles against
 * this library unchanged.  Everything is backed by libslepc_gb300.so.
 *
 * Matrices: CSR ("AIJ") created from caller-owned host arrays with MatCreateSeqAIJWithArrays (the arrays must
 * outlive the Mat, as in PETSc), and small dense matrices (MatCreateSeqDense) for BVMultInPlace.  Vectors:
 * host arrays (VecCreateSeq / VecCreateSeqWithArray).  The eigensolver copies what it needs to device memory.
 */
#ifndef SLEPC_GB300_PETSC_SUBSET_H
#define SLEPC_GB300_PETSC_SUBSET_H

#include <float.h>
#include <math.h>
#include <stddef.h>
#include <stdio.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int PetscErrorCode;
typedef int PetscInt;
typedef int PetscMPIInt;
typedef int PetscBLASInt;
typedef double PetscScalar;
typedef double PetscReal;
typedef enum { PETSC_FALSE = 0, PETSC_TRUE = 1 } PetscBool;
typedef int MPI_Comm; /* one process per GPU: communicators carry no information here */

#define MPI_COMM_WORLD ((MPI_Comm)0)
#define MPI_COMM_SELF ((MPI_Comm)1)
#define PETSC_COMM_WORLD MPI_COMM_WORLD
#define PETSC_COMM_SELF MPI_COMM_SELF

/* "let the library decide" and "keep the current value" markers (PETSc 3.22 conventions) */
#define PETSC_DECIDE (-1)
#define PETSC_DETERMINE PETSC_DECIDE
#define PETSC_DEFAULT (-2)
#define PETSC_CURRENT (-2)
#define PETSC_UNLIMITED (-3)
#define PETSC_NULL_INTEGER ((PetscInt *)0)

/* error codes (numbering of petscerror.h) */
#define PETSC_SUCCESS 0
#define PETSC_ERR_MEM 55
#define PETSC_ERR_SUP 56
#define PETSC_ERR_ORDER 58
#define PETSC_ERR_ARG_SIZ 60
#define PETSC_ERR_ARG_WRONG 62
#define PETSC_ERR_ARG_OUTOFRANGE 63
#define PETSC_ERR_FILE_OPEN 65
#define PETSC_ERR_FILE_READ 66
#define PETSC_ERR_FILE_WRITE 67
#define PETSC_ERR_ARG_WRONGSTATE 73
#define PETSC_ERR_ARG_INCOMP 75
#define PETSC_ERR_LIB 76
#define PETSC_ERR_PLIB 77
#define PETSC_ERR_FILE_UNEXPECTED 79
#define PETSC_ERR_CONV_FAILED 82
#define PETSC_ERR_USER 83
#define PETSC_ERR_ARG_NULL 85
#define PETSC_ERR_USER_INPUT 91
#define PETSC_ERR_GPU_RESOURCE 96
#define PETSC_ERR_GPU 97

typedef enum { NORM_1 = 0, NORM_2 = 1, NORM_FROBENIUS = 2, NORM_INFINITY = 3, NORM_1_AND_2 = 4 } NormType;

typedef struct _p_Mat *Mat;
typedef struct _p_Vec *Vec;
typedef struct _p_PetscViewer *PetscViewer;
typedef enum { FILE_MODE_UNDEFINED = -1, FILE_MODE_READ = 0, FILE_MODE_WRITE, FILE_MODE_APPEND } PetscFileMode;
#define MAT_FILE_CLASSID 1211216
#define VEC_FILE_CLASSID 1211214

/* --- the basics programs written against PETSc use (petscsys.h, petscmath.h, petscerror.h) --- */
#define PetscInt_FMT "d"
#define PETSC_MACHINE_EPSILON DBL_EPSILON
#define PETSC_SMALL 1.e-10
#define PETSC_MAX_REAL DBL_MAX
#define PETSC_MIN_REAL (-DBL_MAX)
#define PETSC_PI 3.14159265358979323846
#define PetscMax(a, b) (((a) < (b)) ? (b) : (a))
#define PetscMin(a, b) (((a) < (b)) ? (a) : (b))
#define PetscAbs(a) (((a) >= 0) ? (a) : (-(a)))
#define PetscAbsInt(a) (((a) < 0) ? (-(a)) : (a))
#define PetscAbsReal(a) fabs(a)
#define PetscAbsScalar(a) fabs(a)
#define PetscRealPart(a) (a)
#define PetscImaginaryPart(a) ((PetscReal)0.0)
#define PetscConj(a) (a)
#define PetscSqrtReal(a) sqrt(a)
#define PetscSqrtScalar(a) sqrt(a)
#define PetscLogReal(a) log(a)
#define PetscLogScalar(a) log(a)
#define PetscExpReal(a) exp(a)
#define PetscCosReal(a) cos(a)
#define PetscSinReal(a) sin(a)
#define PetscPowReal(a, b) pow(a, b)
#define PetscSqr(a) ((a) * (a))
/* error handling: a failing call prints where it failed and returns its code from the caller */
void PetscGB300ReportError(PetscErrorCode ierr, const char *call, const char *file, int line);
#define PetscCall(...)                                                                \
  do {                                                                                \
    PetscErrorCode ierr_petsc_call_ = (__VA_ARGS__);                                  \
    if (ierr_petsc_call_) {                                                           \
      PetscGB300ReportError(ierr_petsc_call_, #__VA_ARGS__, __FILE__, __LINE__);      \
      return ierr_petsc_call_;                                                        \
    }                                                                                 \
  } while (0)
#define PetscCheck(cond, comm, ierr, ...)                                             \
  do {                                                                                \
    if (!(cond)) {                                                                    \
      fprintf(stderr, __VA_ARGS__);                                                   \
      fprintf(stderr, "\n");                                                          \
      return ierr;                                                                    \
    }                                                                                 \
  } while (0)
#define SETERRQ(comm, ierr, ...)                                                      \
  do {                                                                                \
    fprintf(stderr, __VA_ARGS__);                                                     \
    fprintf(stderr, "\n");                                                            \
    return ierr;                                                                      \
  } while (0)
#define PetscFunctionBegin
#define PetscFunctionBeginUser
#define PetscFunctionReturn(x) return (x)
#define PETSC_MAX_PATH_LEN 4096
PetscErrorCode PetscStrcmp(const char a[], const char b[], PetscBool *flg);
/* MPI on one process: rank 0 of 1 */
#define MPI_SUCCESS 0
int MPI_Comm_rank(MPI_Comm comm, int *rank);
int MPI_Comm_size(MPI_Comm comm, int *size);
#define PetscCallMPI(...) PetscCall(__VA_ARGS__)
/* random numbers (PetscRandom): uniform in [0, 1) from a counter-based splitmix64 stream; PETSc's default generator
 * is another one, so the values differ from PETSc's for the same seed */
typedef struct _p_PetscRandom *PetscRandom;
PetscErrorCode PetscRandomCreate(MPI_Comm comm, PetscRandom *r);
PetscErrorCode PetscRandomSetFromOptions(PetscRandom r);
PetscErrorCode PetscRandomSetSeed(PetscRandom r, unsigned long seed);
PetscErrorCode PetscRandomSeed(PetscRandom r);
PetscErrorCode PetscRandomGetValue(PetscRandom r, PetscScalar *value);
PetscErrorCode PetscRandomDestroy(PetscRandom *r);
PetscErrorCode PetscRandomSetInterval(PetscRandom r, PetscScalar low, PetscScalar high);
PetscErrorCode PetscRandomGetValueReal(PetscRandom r, PetscReal *value);
PetscErrorCode PetscStrendswith(const char a[], const char b[], PetscBool *flg);
/* one process owns everything: a PETSC_DECIDE size becomes the other one */
PetscErrorCode PetscSplitOwnership(MPI_Comm comm, PetscInt *n, PetscInt *N);
#define PETSC_ERR_WRONG_MPI_SIZE 94
/* type of an object (EPS: "krylovschur", ST: "shift", Mat: "seqaij" or "seqdense") against one name, or against a
 * list of names ended by "" */
PetscErrorCode PetscObjectTypeCompare(void *obj, const char type[], PetscBool *same);
PetscErrorCode PetscObjectTypeCompareAny(void *obj, PetscBool *match, const char type[], ...);
/* output on the first (only) process */
PetscErrorCode PetscPrintf(MPI_Comm comm, const char format[], ...);
/* the options database is the argument list given to SlepcInitialize/PetscInitialize (PetscOptions: NULL) */
typedef void *PetscOptions;
PetscErrorCode PetscOptionsHasName(PetscOptions options, const char pre[], const char name[], PetscBool *set);
PetscErrorCode PetscOptionsGetInt(PetscOptions options, const char pre[], const char name[], PetscInt *ivalue,
                                  PetscBool *set);
PetscErrorCode PetscOptionsGetReal(PetscOptions options, const char pre[], const char name[], PetscReal *dvalue,
                                   PetscBool *set);
PetscErrorCode PetscOptionsGetScalar(PetscOptions options, const char pre[], const char name[], PetscScalar *dvalue,
                                     PetscBool *set);
PetscErrorCode PetscOptionsGetBool(PetscOptions options, const char pre[], const char name[], PetscBool *ivalue,
                                   PetscBool *set);
PetscErrorCode PetscOptionsGetString(PetscOptions options, const char pre[], const char name[], char string[],
                                     size_t len, PetscBool *set);

/* SlepcInitialize/PetscInitialize: a no-op shim (selects the current CUDA device lazily). */
PetscErrorCode PetscInitialize(int *argc, char ***argv, const char file[], const char help[]);
PetscErrorCode PetscFinalize(void);

/* Error text of the last failing call on this thread (library extension; PETSc prints a traceback instead). */
const char *PetscGB300LastError(void);

/* --- Mat (petscmat.h) --- */
/* CSR matrix over caller-owned arrays i[m+1], j[nnz], a[nnz]; column indices of a row in ascending order. */
PetscErrorCode MatCreateSeqAIJWithArrays(MPI_Comm comm, PetscInt m, PetscInt n, PetscInt i[], PetscInt j[],
                                         PetscScalar a[], Mat *A);
/* Dense column-major matrix; data may be NULL (the library allocates and zeroes it). */
PetscErrorCode MatCreateSeqDense(MPI_Comm comm, PetscInt m, PetscInt n, PetscScalar data[], Mat *A);
PetscErrorCode MatDenseGetArray(Mat A, PetscScalar **array);
PetscErrorCode MatDenseRestoreArray(Mat A, PetscScalar **array);
PetscErrorCode MatDenseGetLDA(Mat A, PetscInt *lda);
PetscErrorCode MatGetSize(Mat A, PetscInt *m, PetscInt *n);
PetscErrorCode MatGetValue(Mat A, PetscInt row, PetscInt col, PetscScalar *v);
PetscErrorCode MatMult(Mat A, Vec x, Vec y);
PetscErrorCode MatNorm(Mat A, NormType type, PetscReal *nrm);
PetscErrorCode MatCreateVecs(Mat A, Vec *right, Vec *left);
PetscErrorCode MatDestroy(Mat *A);
/* Assembly (petscmat.h), sequential AIJ: MatCreate + MatSetSizes (+ MatSetFromOptions / MatSetUp / preallocation,
 * accepted), MatSetValue(s) with INSERT_VALUES or ADD_VALUES (negative indices skipped, as in PETSc), then
 * MatAssemblyBegin/End builds the CSR arrays (columns ascending, duplicates combined in call order).  Values may be
 * set again after assembly (new nonzeros included) and take effect at the next MatAssemblyEnd.  A matrix made by
 * MatCreateSeqAIJWithArrays becomes library-owned when modified (the caller's arrays are left as they were). */
typedef enum { NOT_SET_VALUES, INSERT_VALUES, ADD_VALUES, MAX_VALUES, MIN_VALUES } InsertMode;
typedef enum { MAT_FINAL_ASSEMBLY = 0, MAT_FLUSH_ASSEMBLY = 1 } MatAssemblyType;
typedef enum { MAT_SYMMETRIC, MAT_HERMITIAN, MAT_STRUCTURALLY_SYMMETRIC, MAT_SPD, MAT_NEW_NONZERO_LOCATIONS,
               MAT_NEW_NONZERO_ALLOCATION_ERR, MAT_IGNORE_ZERO_ENTRIES, MAT_KEEP_NONZERO_PATTERN,
               MAT_SYMMETRY_ETERNAL } MatOption;
#define MATAIJ "aij"
#define MATSEQAIJ "seqaij"
PetscErrorCode MatSetSizes(Mat A, PetscInt m, PetscInt n, PetscInt M, PetscInt N);
PetscErrorCode MatSetUp(Mat A);
PetscErrorCode MatSeqAIJSetPreallocation(Mat A, PetscInt nz, const PetscInt nnz[]);
PetscErrorCode MatGetOwnershipRange(Mat A, PetscInt *rstart, PetscInt *rend);
PetscErrorCode MatGetLocalSize(Mat A, PetscInt *m, PetscInt *n);
PetscErrorCode MatSetValue(Mat A, PetscInt i, PetscInt j, PetscScalar v, InsertMode mode);
PetscErrorCode MatSetValues(Mat A, PetscInt m, const PetscInt idxm[], PetscInt n, const PetscInt idxn[],
                            const PetscScalar v[], InsertMode mode);
PetscErrorCode MatAssemblyBegin(Mat A, MatAssemblyType type);
PetscErrorCode MatAssemblyEnd(Mat A, MatAssemblyType type);
PetscErrorCode MatAssembled(Mat A, PetscBool *assembled);
PetscErrorCode MatSetOption(Mat A, MatOption op, PetscBool flg);
PetscErrorCode MatZeroEntries(Mat A);
PetscErrorCode MatScale(Mat A, PetscScalar a);
PetscErrorCode MatShift(Mat A, PetscScalar a);
typedef enum { MAT_DO_NOT_COPY_VALUES, MAT_COPY_VALUES, MAT_SHARE_NONZERO_PATTERN } MatDuplicateOption;
typedef enum { DIFFERENT_NONZERO_PATTERN, SUBSET_NONZERO_PATTERN, SAME_NONZERO_PATTERN, UNKNOWN_NONZERO_PATTERN } MatStructure;
PetscErrorCode MatDuplicate(Mat A, MatDuplicateOption op, Mat *B);
PetscErrorCode MatDiagonalSet(Mat A, Vec D, InsertMode mode);
/* CSR arrays of an AIJ matrix, read-only (shift must be 0; the arrays stay valid until the Mat is destroyed). */
PetscErrorCode MatGetRowIJ(Mat A, PetscInt shift, PetscBool symmetric, PetscBool inodecompressed, PetscInt *n,
                           const PetscInt *ia[], const PetscInt *ja[], PetscBool *done);
PetscErrorCode MatRestoreRowIJ(Mat A, PetscInt shift, PetscBool symmetric, PetscBool inodecompressed, PetscInt *n,
                               const PetscInt *ia[], const PetscInt *ja[], PetscBool *done);
PetscErrorCode MatSeqAIJGetArrayRead(Mat A, const PetscScalar *array[]);
PetscErrorCode MatSeqAIJRestoreArrayRead(Mat A, const PetscScalar *array[]);

/* --- binary files (petscviewer.h, MatLoad/MatView/VecLoad/VecView): PETSc's big-endian binary format, so the
 * reference's data files (share/slepc/datafiles/matrices/NAME.petsc) load unchanged.  MatCreate gives an empty AIJ
 * matrix that MatLoad fills and then owns. --- */
PetscErrorCode PetscViewerBinaryOpen(MPI_Comm comm, const char name[], PetscFileMode mode, PetscViewer *viewer);
PetscErrorCode PetscViewerDestroy(PetscViewer *viewer);
PetscErrorCode MatCreate(MPI_Comm comm, Mat *A);
PetscErrorCode MatSetType(Mat A, const char *type);
PetscErrorCode MatSetFromOptions(Mat A);
PetscErrorCode MatLoad(Mat A, PetscViewer viewer);
PetscErrorCode MatView(Mat A, PetscViewer viewer);
PetscErrorCode VecLoad(Vec x, PetscViewer viewer);
PetscErrorCode VecView(Vec x, PetscViewer viewer);

/* --- ASCII viewers (petscviewer.h): text reports on stdout or a file, with a format stack.  The format names are
 * PETSc's; only DEFAULT, ASCII_INFO, ASCII_INFO_DETAIL and FAILED change what the EPS reports print.  Binary-file
 * calls (MatLoad, MatView, VecLoad, VecView) on an ASCII viewer return PETSC_ERR_SUP. --- */
typedef enum { PETSC_VIEWER_DEFAULT, PETSC_VIEWER_ASCII_MATLAB, PETSC_VIEWER_ASCII_MATHEMATICA, PETSC_VIEWER_ASCII_IMPL,
               PETSC_VIEWER_ASCII_INFO, PETSC_VIEWER_ASCII_INFO_DETAIL, PETSC_VIEWER_ASCII_COMMON,
               PETSC_VIEWER_ASCII_SYMMODU, PETSC_VIEWER_ASCII_INDEX, PETSC_VIEWER_ASCII_DENSE,
               PETSC_VIEWER_ASCII_MATRIXMARKET, PETSC_VIEWER_FAILED } PetscViewerFormat;
PetscViewer PETSC_VIEWER_STDOUT_(MPI_Comm comm);
#define PETSC_VIEWER_STDOUT_WORLD PETSC_VIEWER_STDOUT_(PETSC_COMM_WORLD)
#define PETSC_VIEWER_STDOUT_SELF PETSC_VIEWER_STDOUT_(PETSC_COMM_SELF)
PetscErrorCode PetscViewerASCIIGetStdout(MPI_Comm comm, PetscViewer *viewer);
PetscErrorCode PetscViewerASCIIOpen(MPI_Comm comm, const char name[], PetscViewer *viewer);
PetscErrorCode PetscViewerPushFormat(PetscViewer viewer, PetscViewerFormat format);
PetscErrorCode PetscViewerPopFormat(PetscViewer viewer);
PetscErrorCode PetscViewerGetFormat(PetscViewer viewer, PetscViewerFormat *format);
PetscErrorCode PetscViewerASCIIPrintf(PetscViewer viewer, const char format[], ...);

/* a viewer with the format a monitor prints in (petscviewer.h), and the context-destroy callback type */
typedef struct {
  PetscViewer viewer;
  PetscViewerFormat format;
  void *data; /* monitor-private state (EPSMonitorConverged: the previous nconv) */
} PetscViewerAndFormat;
PetscErrorCode PetscViewerAndFormatCreate(PetscViewer viewer, PetscViewerFormat format, PetscViewerAndFormat **vf);
PetscErrorCode PetscViewerAndFormatDestroy(PetscViewerAndFormat **vf);
typedef PetscErrorCode PetscCtxDestroyFn(void **ctx);

/* object names (PetscObjectSetName): kept for EPS objects, whose MATLAB-format reports print them */
typedef void *PetscObject;
PetscErrorCode PetscObjectSetName(PetscObject obj, const char name[]);
PetscErrorCode PetscObjectGetName(PetscObject obj, const char *name[]);

/* --- Vec (petscvec.h) --- */
PetscErrorCode VecCreate(MPI_Comm comm, Vec *v);
PetscErrorCode VecSetSizes(Vec v, PetscInt n, PetscInt N);
PetscErrorCode VecSetFromOptions(Vec v);
PetscErrorCode VecSetValue(Vec v, PetscInt i, PetscScalar y, InsertMode mode);
PetscErrorCode VecSetValues(Vec v, PetscInt ni, const PetscInt ix[], const PetscScalar y[], InsertMode mode);
PetscErrorCode VecAssemblyBegin(Vec v);
PetscErrorCode VecAssemblyEnd(Vec v);
PetscErrorCode VecZeroEntries(Vec v);
PetscErrorCode VecDuplicateVecs(Vec v, PetscInt m, Vec *V[]);
PetscErrorCode VecDestroyVecs(PetscInt m, Vec *V[]);
PetscErrorCode VecPlaceArray(Vec v, const PetscScalar array[]);
PetscErrorCode VecResetArray(Vec v);
PetscErrorCode VecConjugate(Vec v);
PetscErrorCode VecGetOwnershipRange(Vec v, PetscInt *low, PetscInt *high);
PetscErrorCode VecSetRandom(Vec v, PetscRandom r);
/* SLEPc's VecCheckOrthonormality (src/sys/vec/vecutil.c): lev = max |Y_j^T B X_i - delta_ij| over the nx x ny Gram
 * matrix (Y = X when y is NULL, B = I when NULL); the viewer is not used */
PetscErrorCode VecCheckOrthonormality(Vec x[], PetscInt nx, Vec y[], PetscInt ny, Mat B, PetscViewer viewer,
                                      PetscReal *lev);
PetscErrorCode VecCreateSeq(MPI_Comm comm, PetscInt n, Vec *v);
PetscErrorCode VecCreateSeqWithArray(MPI_Comm comm, PetscInt bs, PetscInt n, const PetscScalar array[], Vec *v);
PetscErrorCode VecDuplicate(Vec v, Vec *newv);
PetscErrorCode VecGetSize(Vec v, PetscInt *n);
PetscErrorCode VecGetArray(Vec v, PetscScalar **a);
PetscErrorCode VecRestoreArray(Vec v, PetscScalar **a);
PetscErrorCode VecGetArrayRead(Vec v, const PetscScalar **a);
PetscErrorCode VecRestoreArrayRead(Vec v, const PetscScalar **a);
PetscErrorCode VecSet(Vec v, PetscScalar alpha);
PetscErrorCode VecCopy(Vec x, Vec y);
PetscErrorCode VecScale(Vec v, PetscScalar alpha);
PetscErrorCode VecAXPY(Vec y, PetscScalar alpha, Vec x);
PetscErrorCode VecDot(Vec x, Vec y, PetscScalar *val);
PetscErrorCode VecNorm(Vec v, NormType type, PetscReal *nrm);
PetscErrorCode VecDestroy(Vec *v);

#ifdef __cplusplus
}
#endif
#endif
